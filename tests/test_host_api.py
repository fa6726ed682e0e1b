"""CPU checks of the host mirror: FEM::reset (fem.rs:155-169) and add_displacement
(methods_for_bc_data_handle.rs:176-203), single and bulk.  No device work happens before the first add,
so these run without a GPU: the handle swap, the new sizes and the kept node limit, and the imposed DOFs,
values and messages against a sequential loop over a stand-in node table."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError


def test_reset_sizes_vectors_and_keeps_tolerances_and_limit():
    g = FEM(1e-9, 1e-11, 5)
    h0 = g.handle.value
    g.reset(8)
    assert g.handle.value and g.handle.value != h0
    assert (g.rel_tol, g.abs_tol, g.nodes_number) == (1e-9, 1e-11, 8)
    assert g._node_limit == 5
    assert g.node_count() == 0 and g.element_counts() == (0, 0, 0)
    assert np.array_equal(g.displacements_vector(), np.zeros(48))
    g.reset(2)
    assert g.nodes_number == 2 and g._node_limit == 5
    assert g.displacements_vector().shape == (12,)
    g.close()
    assert g.handle is None


class _Nodes:
    """stands in for the node table of a handle (the add_nodes upload needs a GPU): node numbers in index order"""

    def __init__(self, g):
        self.numbers = []
        g.node_count = lambda: len(self.numbers)
        g.index_node_numbers = lambda: np.array(self.numbers, np.uint32)


def _sequential(numbers, imposed, values, calls):
    """add_displacement (methods_for_bc_data_handle.rs:176-203) one item at a time: node lookup by number,
    the node's DOF 6 * index + p, refusal of a DOF imposed before"""
    index = {n: i for i, n in enumerate(numbers)}
    done = 0
    for n, p, v in calls:
        if n not in index:
            return done, f"Node with number {n} does not exist!"
        k = 6 * index[n] + p
        if imposed[k]:
            return done, f"Displacement {FEM.DOF_PARAMETERS[p]} already applied to node {n}!"
        imposed[k] = 1
        values[k] = v
        done += 1
    return done, None


def test_add_displacement_single_and_bulk_messages():
    g = FEM(1e-12, 1e-12, 10)
    nodes = _Nodes(g)
    nodes.numbers += [5, 3, 9]
    g.add_displacement(3, "Y", 0.5)
    assert g.displacements_vector()[7] == 0.5 and g._imposed()[7] == 1
    with pytest.raises(FEMError, match=r"^Displacement Y already applied to node 3!$"):
        g.add_displacement(3, 1, 0.0)
    with pytest.raises(FEMError, match=r"^Node with number 7 does not exist!$"):
        g.add_displacements([9, 7], ["ThZ", "X"], [1.0, 2.0])
    assert g._imposed()[6 * 2 + 5] == 1  # the item before the failure stays imposed
    with pytest.raises(FEMError, match=r"^Displacement Z already applied to node 5!$"):
        g.add_displacements([5, 5], "Z", 0.0)  # a repeat inside one call
    assert g.add_displacements([], [], []) == 0
    with pytest.raises(FEMError):
        g.add_displacements([5], [6], [0.0])


@pytest.mark.parametrize("seed", range(4))
def test_add_displacements_match_a_sequential_loop(seed):
    rng = np.random.default_rng(seed)
    cap = 30000
    g = FEM(1e-12, 1e-12, cap)
    nodes = _Nodes(g)
    pool = rng.permutation(np.arange(1, 10 * cap, dtype=np.int64))
    imposed, values = np.zeros(6 * cap, np.uint8), np.zeros(6 * cap)
    used = 0
    for step in range(40):
        grow = int(rng.choice([0, 1, 37, 2000, 9000]))  # small tails and growth past a re-sort
        grow = min(grow, cap - used)
        nodes.numbers += [int(x) for x in pool[used:used + grow]]
        used += grow
        m = int(rng.integers(1, 400))
        known = np.asarray(nodes.numbers or [1], np.int64)
        numbers = np.where(rng.random(m) < 0.995, rng.choice(known, m), rng.choice(pool[used:used + 50] if used < cap
                                                                                     else [0], m))
        dofs = rng.integers(0, 6, m)
        vals = rng.standard_normal(m)
        want_n, want_msg = _sequential(nodes.numbers, imposed, values, zip(numbers.tolist(), dofs.tolist(), vals))
        if want_msg is None:
            assert g.add_displacements(numbers, dofs, vals) == m
        else:
            with pytest.raises(FEMError) as e:
                g.add_displacements(numbers, dofs, vals)
            assert str(e.value) == want_msg
        np.testing.assert_array_equal(g._imposed(), imposed)
        np.testing.assert_array_equal(g.displacements_vector(), values)


def test_extract_global_analysis_result_rows():
    """(node number, DOF, displacement, load) for every DOF of every node in node index order
    (methods_for_global_analysis.rs:361-387), with Python ints, names and floats as the crate's tuples"""
    g = FEM(1e-12, 1e-12, 5)
    nodes = _Nodes(g)
    nodes.numbers += [7, 2, 40]
    rng = np.random.default_rng(0)
    forces = rng.standard_normal(30)
    g.forces_vector = lambda: forces.copy()
    g.add_displacements([2, 40], ["ThY", "X"], [0.25, -1.5])
    got = g.extract_global_analysis_result()
    disp = g.displacements_vector()
    want = [(n, FEM.DOF_PARAMETERS[d], float(disp[6 * i + d]), float(forces[6 * i + d]))
            for i, n in enumerate(nodes.numbers) for d in range(6)]
    assert got == want
    assert all(type(r[0]) is int and type(r[1]) is str and type(r[2]) is float and type(r[3]) is float for r in got)
    assert got[6 + 4] == (2, "ThY", 0.25, float(forces[10]))


def test_extract_elements_analysis_result_rows():
    """(element number, [(component, value), ...]) for the trusses, the beams, then the plates, in call order
    (methods_for_element_analysis.rs:27-58)"""
    g = FEM(1e-12, 1e-12, 5)
    rng = np.random.default_rng(1)
    res = {"truss": rng.standard_normal((2, 1)), "beam": rng.standard_normal((1, 10)),
           "plate": rng.standard_normal((3, 8))}
    nums = {"truss": np.array([4, 1], np.uint32), "beam": np.array([9], np.uint32),
            "plate": np.array([3, 8, 2], np.uint32)}
    g.element_results = lambda displacements=None, out=None: res
    g.element_numbers = lambda kind: nums[kind]
    got = g.extract_elements_analysis_result()
    want = []
    for kind, names in (("truss", FEM.TRUSS_COMPONENTS), ("beam", FEM.BEAM_COMPONENTS),
                        ("plate", FEM.PLATE_COMPONENTS)):
        for number, row in zip(nums[kind], res[kind]):
            want.append((int(number), [(c, float(v)) for c, v in zip(names, row)]))
    assert got == want
    assert type(got[0][0]) is int and type(got[0][1][0][1]) is float


def test_size_checks_raise_before_the_c_call():
    """the sizes the C side trusts are checked on the host, as ValueError (not assert: they stay on under
    python -O), before anything is handed to the library"""
    from finite_element_method_gb300.fem import SeparatedStiffnessSparse

    g = FEM(1e-12, 1e-12, 3)
    ndof = 18
    with pytest.raises(ValueError, match="row_ptr needs 19"):
        g.assemble_to_host(np.zeros(ndof, np.int64), np.zeros(4, np.int32), np.zeros(4))
    with pytest.raises(ValueError, match="int64, int32, float64"):
        g.assemble_to_host(np.zeros(ndof + 1, np.int32), np.zeros(4, np.int32), np.zeros(4))
    with pytest.raises(ValueError, match=r"\(npairs, 18\)"):
        g.vjp(np.zeros((2, ndof)), np.zeros((2, ndof - 1)))
    with pytest.raises(ValueError, match="18 flags"):
        g.separate_stiffness_matrix_sparse_iterative(imposed=np.zeros(ndof - 6, np.uint8))
    sep = SeparatedStiffnessSparse(np.arange(12), np.arange(12, 18), {})
    with pytest.raises(ValueError, match="r_a must hold 12 values and u_b 6"):
        g.find_ua_vector_iterative_pcg_jacobi_sparse(sep, np.zeros(11), np.zeros(6), 10)
    with pytest.raises(ValueError, match="r_a must hold 12 values and u_b 6"):
        g.find_ua_vector_iterative_pcg_block_jacobi_sparse(sep, np.zeros(12), np.zeros(5), 10)
    g.forces_vector = lambda: np.zeros(ndof)
    with pytest.raises(ValueError, match="u_a must hold 12 values and u_b 6"):
        g.find_r_r_vector_sparse(sep, np.zeros(12), np.zeros(7))
    g.close()
