"""GPU solution path (fem_gpu_solve_pcg, fem_gpu_reactions) against the CPU restatement
(oracle/pcg.py on the oracle's separation): the reference's truss known answer, beam and plate models
with Jacobi and node-block Jacobi preconditioning, imposed settlements, and the no-convergence error."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle import fem_oracle as fo
from oracle.pcg import build_block_starts, find_b_sparse, find_r_r_sparse, pcg
from oracle.separate import separate_sparse

pytestmark = pytest.mark.gpu


def test_reference_truss():
    g = FEM(1e-4, 1e-12, 2)
    g.add_node(1, 0.0, 0.0, 0.0)
    g.add_node(2, 30.0, 0.0, 0.0)
    g.add_truss(1, 1, 2, 1e6, 2.0)
    g.assemble()
    g.add_displacement(1, "X", 0.0)
    g.add_concentrated_load(2, "X", 100.0)
    sep = g.separate_stiffness_matrix_sparse_iterative()
    r_a = g.compose_r_a_vector(sep.k_aa_indexes)
    u_b = g.compose_u_b_vector(sep.k_bb_indexes)
    for solve in (g.find_ua_vector_iterative_pcg_jacobi_sparse, g.find_ua_vector_iterative_pcg_block_jacobi_sparse):
        u_a, it = solve(sep, r_a, u_b, 1000)
        assert it == 1 and u_a[0] == pytest.approx(0.0015, rel=1e-12)
        r_r = g.find_r_r_vector_sparse(sep, u_a, u_b)
        assert r_r[0] == pytest.approx(-100.0, rel=1e-12)


def solve_both(m, imposed, disp, loads, block, rel_tol=1e-10, max_iter=5000):
    g = FEM(rel_tol, 1e-12, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    nodes0, dofs, vals = loads
    g.add_concentrated_loads(m.node_numbers[nodes0], dofs, vals)
    sep = g.separate_stiffness_matrix_sparse_iterative(imposed)
    f = g.forces_vector()
    r_a, u_b = f[sep.k_aa_indexes], disp[sep.k_bb_indexes]
    u_a, it = (g.find_ua_vector_iterative_pcg_block_jacobi_sparse if block
               else g.find_ua_vector_iterative_pcg_jacobi_sparse)(sep, r_a, u_b, max_iter)
    r_r = g.find_r_r_vector_sparse(sep, u_a, u_b)
    o = fo.OracleFEM(rel_tol, 1e-12, m.nodes_number)
    meshes.load(o, m)
    aa, bb, blocks = separate_sparse(*o.csr(), imposed, o.index_node_numbers())
    b = find_b_sparse(f[aa], blocks["k_ab"], disp[bb])
    x, it_ref, ok = pcg(blocks["k_aa"], b, rel_tol, 1e-12, max_iter, build_block_starts(aa) if block else None)
    assert ok
    rr_ref = find_r_r_sparse(blocks["k_ba"], x, blocks["k_bb"], disp[bb], f[bb])
    return u_a, it, r_r, x, it_ref, rr_ref, blocks, b


@pytest.mark.parametrize("block", [False, True])
def test_beam_frame_with_settlement(block):
    m = meshes.beam_frame(6, 5, 4)
    base = np.arange(30)
    imposed = np.zeros(6 * m.nodes_number, np.uint8)
    disp = np.zeros(6 * m.nodes_number)
    for d in range(6):
        imposed[6 * base + d] = 1
    disp[6 * 7 + 2] = -0.02  # a settlement under node 8
    top = np.arange(90, 120)
    loads = (top, np.zeros(30, np.uint8), np.linspace(1e3, 2e3, 30))
    u_a, it, r_r, x, it_ref, rr_ref, blocks, b = solve_both(m, imposed, disp, loads, block)
    assert abs(it - it_ref) <= 2 + it_ref // 10
    np.testing.assert_allclose(u_a, x, rtol=1e-7, atol=1e-9 * np.abs(x).max())
    np.testing.assert_allclose(r_r, rr_ref, rtol=1e-6, atol=1e-8 * np.abs(rr_ref).max())
    # equilibrium of the solution: K_aa u_a = b within the stopping tolerance
    n = len(b)
    rows, cols, vals = blocks["k_aa"]
    res = b - np.bincount(rows, weights=vals * u_a[cols], minlength=n)
    assert np.linalg.norm(res) <= 1e-9 * np.linalg.norm(b)


def test_plate_mesh_block_jacobi():
    m = meshes.plate_mesh(16, 12, size=2.0)
    x = m.xyz[:, 0]
    edge = np.flatnonzero((x == x.min()) | (x == x.max()))
    imposed = np.zeros(6 * m.nodes_number, np.uint8)
    for d in range(6):
        imposed[6 * edge + d] = 1
    mid = np.flatnonzero(np.abs(x - x.mean()) < 0.1)
    loads = (mid, np.full(len(mid), 2, np.uint8), np.full(len(mid), -500.0))
    u_a, it, r_r, xs, it_ref, rr_ref, blocks, b = solve_both(m, imposed, np.zeros(6 * m.nodes_number), loads, True)
    np.testing.assert_allclose(u_a, xs, rtol=1e-6, atol=1e-8 * np.abs(xs).max())
    # conjugate gradients on a plate (bending, ill-conditioned) are sensitive to summation order: the GPU's
    # products and dot products sum in another order than numpy, so the counts may differ a little
    assert abs(it - it_ref) <= 2 + it_ref // 10
    np.testing.assert_allclose(r_r, rr_ref, rtol=1e-6, atol=1e-8 * np.abs(rr_ref).max())


def test_no_convergence_error():
    m = meshes.plate_mesh(16, 12, size=2.0)
    g = FEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    x = m.xyz[:, 0]
    edge = np.flatnonzero(x == x.min())
    imposed = np.zeros(6 * m.nodes_number, np.uint8)
    for d in range(6):
        imposed[6 * edge + d] = 1
    g.add_concentrated_load(int(m.node_numbers[-1]), "Z", -1.0)
    sep = g.separate_stiffness_matrix_sparse_iterative(imposed)
    r_a = g.forces_vector()[sep.k_aa_indexes]
    with pytest.raises(FEMError, match="^find_ua_vector_iterative: PCG failed: no convergence in 3 iterations$"):
        g.find_ua_vector_iterative_pcg_jacobi_sparse(sep, r_a, None, 3)
