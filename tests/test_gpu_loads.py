"""GPU loads (fem_gpu_add_*_loads, fem_gpu_get_forces) against the CPU restatement (oracle/loads.py):
the forces vector bit for bit, in call order, with concentrated, line and surface loads interleaved;
the reference's messages for missing nodes and elements; the bulk form stopping at the first failure."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle.loads import forces_vector

pytestmark = pytest.mark.gpu


def mixed_model():
    m = meshes.adjoint_model(frame=(6, 6, 3), slab=(50, 50), seed=9)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    return m, g


def test_loads_in_call_order_bit_exact():
    m, g = mixed_model()
    rng = np.random.default_rng(3)
    nb, npl = len(m.beams["numbers"]), len(m.plates["numbers"])
    loads = []
    for step in range(3):  # interleaved bulk calls of each kind
        nodes = rng.integers(0, m.nodes_number, 500)
        dofs = rng.integers(0, 6, 500).astype(np.uint8)
        vals = rng.normal(size=500)
        g.add_concentrated_loads(m.node_numbers[nodes], dofs, vals)
        loads += [("node", int(i), int(d), v) for i, d, v in zip(nodes, dofs, vals)]
        beams = rng.integers(0, nb, 300)
        dofs = rng.integers(0, 6, 300).astype(np.uint8)
        vals = rng.normal(size=300) * 1e3
        g.add_uniformly_distributed_line_loads(m.beams["numbers"][beams], dofs, vals)
        loads += [("line", int(i), int(d), v) for i, d, v in zip(beams, dofs, vals)]
        plates = rng.integers(0, npl, 2000)
        dofs = rng.integers(0, 6, 2000).astype(np.uint8)
        vals = rng.normal(size=2000) * 5e3
        g.add_uniformly_distributed_surface_loads(m.plates["numbers"][plates], dofs, vals)
        loads += [("surface", int(i), int(d), v) for i, d, v in zip(plates, dofs, vals)]
    got = g.forces_vector()
    ref = forces_vector(m.nodes_number, m.xyz, loads, beam_nodes=m.beams["nodes"].astype(np.int64) - 1,
                        plate_nodes=m.plates["nodes"].astype(np.int64) - 1)
    np.testing.assert_array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_tilted_plates_and_single_calls():
    q, _ = np.linalg.qr(np.random.default_rng(5).normal(size=(3, 3)))
    m = meshes.plate_mesh(20, 20, size=3.0, rotation=q)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    g.add_uniformly_distributed_surface_load(7, "Z", -1500.0)
    g.add_uniformly_distributed_surface_load(8, 1, 250.0)
    g.add_concentrated_load(9, "ThX", 3.0)
    got = g.forces_vector()
    pn = m.plates["nodes"].astype(np.int64) - 1
    ref = forces_vector(m.nodes_number, m.xyz, [("surface", 6, 2, -1500.0), ("surface", 7, 1, 250.0),
                                                ("node", 8, 3, 3.0)], plate_nodes=pn)
    np.testing.assert_array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_errors_and_bulk_stop():
    m, g = mixed_model()
    with pytest.raises(FEMError, match="^Node with number 999999 does not exist!$"):
        g.add_concentrated_load(999999, "X", 1.0)
    with pytest.raises(FEMError, match="^Beam element with number 999999 does not exist!$"):
        g.add_uniformly_distributed_line_load(999999, "Z", 1.0)
    with pytest.raises(FEMError, match="^Plate element with number 999999 does not exist!$"):
        g.add_uniformly_distributed_surface_load(999999, "Z", 1.0)
    # a bulk call stops at its first failure, the earlier loads stay
    nums = np.array([1, 2, 999999, 3], np.uint32)
    with pytest.raises(FEMError):
        g.add_uniformly_distributed_surface_loads(nums, [2, 2, 2, 2], [1.0, 1.0, 1.0, 1.0])
    pn = m.plates["nodes"].astype(np.int64) - 1
    ref = forces_vector(m.nodes_number, m.xyz, [("surface", 0, 2, 1.0), ("surface", 1, 2, 1.0)], plate_nodes=pn)
    np.testing.assert_array_equal(g.forces_vector().view(np.uint64), ref.view(np.uint64))


def test_separation_vectors():
    """compose_r_a_vector / compose_u_b_vector from the separation's index lists"""
    m = meshes.beam_frame(5, 5, 3)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    for n in range(1, 26):  # base restrained, one imposed settlement
        for d in range(6):
            g.add_displacement(n, d, -0.01 if (n == 13 and d == 2) else 0.0)
    g.add_concentrated_loads(np.arange(51, 76), [0] * 25, np.linspace(1.0, 2.0, 25))
    sep = g.separate_stiffness_matrix_sparse_iterative()
    r_a = g.compose_r_a_vector(sep.k_aa_indexes)
    u_b = g.compose_u_b_vector(sep.k_bb_indexes)
    f = g.forces_vector()
    assert np.array_equal(r_a, f[sep.k_aa_indexes]) and r_a.sum() == pytest.approx(37.5)
    assert u_b.min() == -0.01 and np.count_nonzero(u_b) == 1
