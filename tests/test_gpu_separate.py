"""GPU sparse separation (fem_gpu_separate_sparse) against the CPU restatement of
separate_stiffness_matrix_sparse_iterative (oracle/separate.py) on the oracle's own stiffness:
index lists, block patterns and values bit-exact, and the reference's error messages."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle import fem_oracle as fo
from oracle.separate import BLOCKS, separate_sparse

pytestmark = pytest.mark.gpu


def build_pair(mesh):
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    o = fo.OracleFEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(o, mesh)
    return g, o


def imposed_for(mesh, nodes0, dofs):
    imp = np.zeros(6 * mesh.nodes_number, np.uint8)
    for d in dofs:
        imp[6 * np.asarray(nodes0) + d] = 1
    return imp


def check_same(g, o, imp):
    sep = g.separate_stiffness_matrix_sparse_iterative(imp)
    rp, ci, va = o.csr()
    aa, bb, blocks = separate_sparse(rp, ci, va, imp, o.index_node_numbers())
    np.testing.assert_array_equal(sep.k_aa_indexes, aa)
    np.testing.assert_array_equal(sep.k_bb_indexes, bb)
    for name in BLOCKS:
        r, c, v = sep.triplets(name)
        ro, co, vo = blocks[name]
        np.testing.assert_array_equal(r, ro)
        np.testing.assert_array_equal(c, co)
        np.testing.assert_array_equal(v.view(np.uint64), vo.view(np.uint64))
    return sep


def test_reference_truss_case():
    g = FEM(1e-4, 1e-12, 2)
    g.add_node(1, 0.0, 0.0, 0.0)
    g.add_node(2, 30.0, 0.0, 0.0)
    g.add_truss(1, 1, 2, 1e6, 2.0)
    g.assemble()
    g.add_displacement(1, "X", 0.0)
    sep = g.separate_stiffness_matrix_sparse_iterative()
    assert sep.k_aa_indexes.tolist() == [6] and sep.k_bb_indexes.tolist() == [0]
    assert sep.n_aa > 0 and sep.triplets("k_aa")[2].size == 1
    assert 100.0 / sep.triplets("k_aa")[2][0] == pytest.approx(0.0015, rel=1e-12)
    with pytest.raises(FEMError, match="^Displacement X already applied to node 1!$"):
        g.add_displacement(1, "X", 0.0)


def test_truss_lattice_base_fixed():
    """config 1: the 11 x 11 x 11 lattice with its z = 0 layer restrained in X, Y, Z; rotational DOFs
    carry no stiffness and are excluded.  Restraining them as well is the reference's error."""
    m = meshes.truss_lattice()
    g, o = build_pair(m)
    base = np.arange(11 * 11)
    sep = check_same(g, o, imposed_for(m, base, (0, 1, 2)))
    assert sep.n_bb == 3 * len(base) and sep.n_aa == 3 * (m.nodes_number - len(base))
    with pytest.raises(FEMError, match="^There are no stiffness to withstand displacement ThX applied to node 1!$"):
        g.separate_stiffness_matrix_sparse_iterative(imposed_for(m, base, range(6)))


def test_beam_frame_base_fixed():
    m = meshes.beam_frame(12, 10, 5)
    g, o = build_pair(m)
    check_same(g, o, imposed_for(m, np.arange(12 * 10), range(6)))


def test_plate_mesh_edge_fixed_and_tilted():
    m = meshes.plate_mesh(40, 30)
    g, o = build_pair(m)
    edge = np.flatnonzero(m.xyz[:, 0] == 0.0)
    check_same(g, o, imposed_for(m, edge, range(6)))
    q, _ = np.linalg.qr(np.random.default_rng(7).normal(size=(3, 3)))
    mt = meshes.plate_mesh(20, 20, size=3.0, rotation=q)
    gt, ot = build_pair(mt)
    check_same(gt, ot, imposed_for(mt, np.arange(0, 21 * 21, 21), range(6)))


def test_mixed_model_and_unused_node_slots():
    """frame + slab sharing nodes, with two node slots never added (their DOFs have no diagonal)"""
    m = meshes.adjoint_model(frame=(4, 4, 3), slab=(30, 30))
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number + 2)
    meshes.load(g, m)
    g.assemble()
    o = fo.OracleFEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number + 2)
    meshes.load(o, m)
    imp = np.zeros(6 * (m.nodes_number + 2), np.uint8)
    imp[:6 * 16] = 1  # the frame's base storey
    check_same(g, o, imp)


def test_errors_and_state():
    m = meshes.beam_frame(4, 4, 3)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    with pytest.raises(FEMError, match="assemble"):
        g.separate_stiffness_matrix_sparse_iterative(np.zeros(6 * m.nodes_number, np.uint8))
    g.assemble()
    with pytest.raises(FEMError, match="^No restraints$"):
        g.separate_stiffness_matrix_sparse_iterative(np.zeros(6 * m.nodes_number, np.uint8))
    with pytest.raises(FEMError, match="K_aa is empty"):
        g.separate_stiffness_matrix_sparse_iterative(np.ones(6 * m.nodes_number, np.uint8))
    # a numeric pass invalidates the previous separation's blocks
    imp = imposed_for(m, np.arange(16), range(6))
    g.separate_stiffness_matrix_sparse_iterative(imp)
    g.assemble_numeric_async()
    with pytest.raises(FEMError, match="separate"):
        g._check(g._L.fem_gpu_get_separation_sizes(g._h, None, None, None))


@pytest.mark.slow
def test_full_plate_mesh_edges_fixed():
    """config 3 at full size: 1,000,000 plates, all four edges restrained"""
    m = meshes.plate_mesh()
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    x, y = m.xyz[:, 0], m.xyz[:, 1]
    edge = np.flatnonzero((x == 0.0) | (y == 0.0) | (x == x.max()) | (y == y.max()))
    imp = imposed_for(m, edge, range(6))
    sep = g.separate_stiffness_matrix_sparse_iterative(imp)
    rp, ci, va = g.stiffness_csr()  # bit-identical to the oracle's (tests/test_gpu_parity.py)
    aa, bb, blocks = separate_sparse(rp, ci, va, imp, g.index_node_numbers())
    np.testing.assert_array_equal(sep.k_aa_indexes, aa)
    np.testing.assert_array_equal(sep.k_bb_indexes, bb)
    for name in BLOCKS:
        r, c, v = sep.triplets(name)
        np.testing.assert_array_equal(r, blocks[name][0])
        np.testing.assert_array_equal(c, blocks[name][1])
        np.testing.assert_array_equal(v.view(np.uint64), blocks[name][2].view(np.uint64))
