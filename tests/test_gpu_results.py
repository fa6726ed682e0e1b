"""GPU element results (fem_gpu_element_results) against the CPU restatement
(oracle/fem_oracle.c orc_*_results), bit for bit: the reference's integration
test end to end (src/tests/fem/test_fem.rs:83-225: u_2x = 0.0015, reaction -100,
ForceR = 100), truss / beam / tilted plate meshes with random displacements, a
mixed beam + plate model, the device-pointer entry point, and at the full
1000 x 1000 plate mesh a sample of elements against the oracle plus the
size-independent identities (linearity in the displacements, no stress under
rigid-body motion)."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle import fem_oracle as fo

pytestmark = pytest.mark.gpu


def _rot(seed):
    q, _ = np.linalg.qr(np.random.default_rng(seed).standard_normal((3, 3)))
    return q


@pytest.mark.parametrize("block", [False, True])
def test_reference_integration(block):
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
    solve = g.find_ua_vector_iterative_pcg_block_jacobi_sparse if block else g.find_ua_vector_iterative_pcg_jacobi_sparse
    u_a, it = solve(sep, r_a, u_b, 1000)
    r_r = g.find_r_r_vector_sparse(sep, u_a, u_b)
    g.compose_global_analysis_result(sep.k_aa_indexes, sep.k_bb_indexes, u_a, r_r)
    glob = sorted(g.extract_global_analysis_result(), key=lambda r: (r[0], g.DOF_PARAMETERS.index(r[1])))
    expected = [(1, "X", 0.0, -100.0)] + [(1, d, 0.0, 0.0) for d in g.DOF_PARAMETERS[1:]] + \
               [(2, "X", 0.0015, 100.0)] + [(2, d, 0.0, 0.0) for d in g.DOF_PARAMETERS[1:]]
    assert [(n, d) for n, d, _, _ in glob] == [(n, d) for n, d, _, _ in expected]
    for (_, _, u, f), (_, _, ue, fe) in zip(glob, expected):
        assert u == pytest.approx(ue, rel=1e-12, abs=0.0) and f == pytest.approx(fe, rel=1e-12, abs=0.0)
    elems = g.extract_elements_analysis_result()
    assert len(elems) == 1 and elems[0][0] == 1 and elems[0][1][0][0] == "ForceR"
    assert elems[0][1][0][1] == pytest.approx(100.0, rel=1e-12)
    assert it == 1


def _oracle_results(mesh, disp):
    out, _ = fo.element_results(mesh, disp, n_threads=4)
    return out


@pytest.mark.parametrize("case", ["truss", "beam", "plate_flat", "plate_tilted", "mixed"])
def test_results_match_oracle(case):
    if case == "truss":
        mesh = meshes.truss_lattice(n=7)
    elif case == "beam":
        mesh = meshes.beam_frame(nx=9, ny=7, nz=4)
    elif case == "plate_flat":
        mesh = meshes.plate_mesh(40, 30, size=10.0)
    elif case == "plate_tilted":
        mesh = meshes.plate_mesh(20, 20, size=3.0, rotation=_rot(9))
    else:
        mesh = meshes.adjoint_model(frame=(4, 4, 3), slab=(30, 30))
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    rng = np.random.default_rng(5)
    for scale in (1e-3, 1.0):
        disp = rng.standard_normal(6 * mesh.nodes_number) * scale
        got = g.element_results(disp)
        want = _oracle_results(mesh, disp)
        for k in ("truss", "beam", "plate"):
            assert got[k].shape == want[k].shape
            assert np.array_equal(got[k], want[k]), (k, np.max(np.abs(got[k] - want[k])))
    g.close()


def test_numbers_and_null_outputs():
    mesh = meshes.adjoint_model(frame=(2, 2, 2), slab=(10, 10))
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    assert np.array_equal(g.element_numbers("beam"), mesh.beams["numbers"])
    assert np.array_equal(g.element_numbers("plate"), mesh.plates["numbers"])
    disp = np.random.default_rng(1).standard_normal(6 * mesh.nodes_number) * 1e-3
    full = g.element_results(disp)
    import ctypes

    from finite_element_method_gb300._lib import ptr

    beam = np.full((len(mesh.beams["numbers"]), 10), -7.0)
    g._check(g._L.fem_gpu_element_results(g.handle, ptr(disp, ctypes.c_double), disp.size, None,
                                          ptr(beam, ctypes.c_double), None))
    assert np.array_equal(beam, full["beam"])
    with pytest.raises(FEMError):
        g.element_results(disp[:-1])
    g.compose_global_analysis_result(np.arange(disp.size), np.zeros(0, np.int64), disp, np.zeros(0))
    res = g.extract_elements_analysis_result()
    nb = len(mesh.beams["numbers"])
    assert len(res) == nb + len(mesh.plates["numbers"])
    assert [c for c, _ in res[0][1]] == list(g.BEAM_COMPONENTS)
    assert [c for c, _ in res[nb][1]] == list(g.PLATE_COMPONENTS)
    assert res[nb][1][3][1] == full["plate"][0, 3]
    g.close()


def test_device_entry_point():
    import torch

    mesh = meshes.plate_mesh(50, 40, size=5.0, rotation=_rot(3))
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    disp = np.random.default_rng(2).standard_normal(6 * mesh.nodes_number) * 1e-3
    host = g.element_results(disp)
    d = torch.from_numpy(disp).cuda()
    out = torch.empty((len(mesh.plates["numbers"]), 8), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    g.element_results_device(d.data_ptr(), 0, 0, out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), host["plate"])
    assert g.results_last_ms() > 0.0
    g.close()


@pytest.mark.slow
def test_full_plate_mesh_sample_and_identities():
    """1000 x 1000 plates: 3000 sampled elements bit-exact against the per-element oracle, linearity
    (results of a u1 + b u2 within 1e-12 of the magnitude scale) and rigid-body motion stress-free"""
    mesh = meshes.plate_mesh(1000, 1000)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    rng = np.random.default_rng(8)
    n = mesh.nodes_number
    u1 = rng.standard_normal(6 * n) * 1e-3
    u2 = rng.standard_normal(6 * n) * 1e-3
    r1 = g.element_results(u1)["plate"]
    r2 = g.element_results(u2)["plate"]
    r12 = g.element_results(2.0 * u1 - 0.5 * u2)["plate"]  # exact scalings of each vector
    scale = 2.0 * np.abs(r1) + 0.5 * np.abs(r2) + np.max(np.abs(r1), axis=0) * 1e-3
    assert np.all(np.abs(r12 - (2.0 * r1 - 0.5 * r2)) <= 1e-9 * scale)
    pl, X = mesh.plates, mesh.xyz
    for e in rng.choice(len(pl["numbers"]), 3000, replace=False):
        nd = pl["nodes"][e].astype(np.int64) - 1
        want = fo.plate_results(*(X[i] for i in nd), pl["young"][e], pl["poisson"][e], pl["thickness"][e],
                                pl["shear_factor"][e], np.concatenate([u1[6 * i:6 * i + 6] for i in nd]))
        assert np.array_equal(r1[e], want)
    # rigid-body motion: translation c and a small rotation w about the origin
    c, w = np.array([1e-3, -2e-3, 5e-4]), np.array([2e-5, -1e-5, 3e-5])
    u = np.zeros((n, 6))
    u[:, :3] = c + np.cross(w, X)
    u[:, 3:] = w
    rb = g.element_results(u.ravel())["plate"]
    assert np.max(np.abs(rb)) < 1e-6 * np.max(np.abs(r1))
    g.close()


def test_tapered_trusses_and_skew_beams_with_product_of_inertia():
    """element kinds and options the generated meshes do not exercise: tapered trusses (area_2), beams
    with I12 != 0 and equal I11 = I22, local axes along x, y and skew, vertical members"""
    rng = np.random.default_rng(21)
    n = 40
    xyz = rng.uniform(-3.0, 3.0, (n, 3))
    xyz[n - 2] = xyz[0] + [0.0, 0.0, 2.0]  # vertical members 0 -> n-2 and n-1 -> 1
    xyz[n - 1] = xyz[1] + [0.0, 0.0, -1.5]
    g = FEM(1e-12, 1e-12, n)
    g.add_nodes(np.arange(1, n + 1), xyz)
    trusses, beams = [], []
    pairs = [(a, b) for a in range(n - 2) for b in range(a + 1, n - 2)]
    order = rng.permutation(len(pairs))[:55]
    for e in range(25):
        a, b = pairs[order[e]]
        a2 = None if e % 3 == 0 else float(rng.uniform(1e-4, 5e-4))
        g.add_truss(e + 1, a + 1, b + 1, 200e9, 3e-4, a2)
        trusses.append((a, b, a2))
    for e in range(30):
        a, b = pairs[order[25 + e]]
        if e % 2:
            a, b = b, a
        d = xyz[b] - xyz[a]
        axis = [[0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.3, -0.4, 0.5]][e % 3]
        if abs(np.dot(d, axis)) > 0.99 * np.linalg.norm(d) * np.linalg.norm(axis):
            axis = [0.0, 1.0, 0.0]
        i11, i22 = (5e-5, 5e-5) if e % 4 == 0 else (8e-5, 3e-5)
        i12 = 0.0 if e % 2 else 1e-5
        g.add_beam(100 + e, a + 1, b + 1, 210e9, 0.3, 1.2e-2, i11, i22, i12, 2e-5, 5 / 6, axis)
        beams.append((a, b, i11, i22, i12, axis))
    for e, (a, b) in enumerate(((0, n - 2), (n - 1, 1))):
        g.add_beam(200 + e, a + 1, b + 1, 210e9, 0.3, 1.2e-2, 8e-5, 3e-5, 1e-5 * e, 2e-5, 5 / 6, [1.0, 0.0, 0.0])
        beams.append((a, b, 8e-5, 3e-5, 1e-5 * e, [1.0, 0.0, 0.0]))
    disp = rng.standard_normal(6 * n) * 1e-3
    got = g.element_results(disp)
    for e, (a, b, a2) in enumerate(trusses):
        want = fo.truss_results(xyz[a], xyz[b], 200e9, 3e-4, a2, np.r_[disp[6 * a:6 * a + 3], disp[6 * b:6 * b + 3]])
        assert got["truss"][e, 0] == want[0]
    for e, (a, b, i11, i22, i12, axis) in enumerate(beams):
        want = fo.beam_results(xyz[a], xyz[b], 210e9, 0.3, 1.2e-2, i11, i22, i12, 2e-5, 5 / 6, axis,
                               np.r_[disp[6 * a:6 * a + 6], disp[6 * b:6 * b + 6]])
        assert np.array_equal(got["beam"][e], want), (e, got["beam"][e] - want)
    g.close()
