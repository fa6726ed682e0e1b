"""FEM::reset (fem.rs:155-169) on the GPU model: after a reset nothing of the earlier model is left
(the next model's CSR equals a fresh oracle model's bit for bit, loads and imposed displacements are
gone), the stiffness and vectors take the new size, and the node limit stays the nodes_number given at
creation, as the crate's untouched props keep it."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle import fem_oracle as fo

pytestmark = pytest.mark.gpu


def test_reset_then_new_model_matches_fresh_oracle():
    frame = meshes.beam_frame(4, 4, 3)
    lattice = meshes.truss_lattice(4)
    n1 = max(frame.nodes_number, lattice.nodes_number)
    g = FEM(1e-12, 1e-12, n1)
    meshes.load(g, frame)
    g.assemble()
    g.add_displacement(int(frame.node_numbers[0]), "X", 0.0)
    g.add_concentrated_load(int(frame.node_numbers[-1]), "Z", -1e3)
    n2 = n1 + 7  # a reset to more nodes: vectors sized for them, limit unchanged
    g.reset(n2)
    assert g.node_count() == 0 and g.element_counts() == (0, 0, 0)
    meshes.load(g, lattice)
    g.assemble()
    o = fo.OracleFEM(1e-12, 1e-12, n2)
    meshes.load(o, lattice)
    rp, ci, va = g.stiffness_csr()
    rp_o, ci_o, va_o = o.csr()
    assert len(rp) == 6 * n2 + 1
    assert np.array_equal(rp, rp_o) and np.array_equal(ci, ci_o)
    assert np.array_equal(va.view(np.uint64), va_o.view(np.uint64))
    assert np.array_equal(g.forces_vector(), np.zeros(6 * n2))
    assert np.array_equal(g.displacements_vector(), np.zeros(6 * n2))
    g.close()


def test_reset_keeps_the_creation_node_limit():
    xyz = np.arange(18, dtype=np.float64).reshape(6, 3)
    g = FEM(1e-12, 1e-12, 4)
    g.add_nodes([1, 2], xyz[:2])
    g.reset(6)
    with pytest.raises(FEMError) as e:
        g.add_nodes([11, 12, 13, 14, 15], xyz[:5])
    # the crate's add_node checks the index against props.nodes_number, which reset leaves at 4
    assert str(e.value) == "Nodes number could not be greater than 4!"
    assert g.node_count() == 4
    assert list(g.index_node_numbers()) == [11, 12, 13, 14]
    g.close()


def test_reset_to_fewer_nodes_refuses_nodes_past_the_new_count():
    xyz = np.arange(12, dtype=np.float64).reshape(4, 3)
    g = FEM(1e-12, 1e-12, 4)
    g.reset(3)
    with pytest.raises(FEMError) as e:
        g.add_nodes([1, 2, 3, 4], xyz)
    assert str(e.value) == "Nodes number could not be greater than 3!"
    assert g.node_count() == 3
    g.close()
