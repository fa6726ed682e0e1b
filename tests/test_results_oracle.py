"""CPU tests of the element-results restatement (oracle/fem_oracle.c,
orc_*_results): pinned to the reference's integration-test known answer
(src/tests/fem/test_fem.rs:57-58, ForceR = 100), to 50-digit evaluations of the
reference's formulas (tests/golden/element_results.json, within 1e-12 of each
value's magnitude scale), and to size-independent identities: a two-node
element's results are components of R K_e u_e (the element's local end forces),
and a plate reproduces the closed-form membrane, bending and shear resultants of
constant-strain states."""
import json
import os

import numpy as np
import pytest

from finite_element_method_gb300 import meshes
from oracle import fem_oracle as fo
from oracle.pcg import find_b_sparse, find_r_r_sparse, pcg
from oracle.separate import separate_sparse

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "element_results.json")
TOL = 1e-12  # of the value's magnitude scale (sum of |terms|)


def test_reference_truss_known_answer():
    """test_integration_iterative_pcg_jacobi_sparse: u_2x from the solve, then ForceR = 100"""
    m = fo.OracleFEM(1e-4, 1e-12, 2)
    m.add_node(1, 0.0, 0.0, 0.0)
    m.add_node(2, 30.0, 0.0, 0.0)
    m.add_truss(1, 1, 2, 1e6, 2.0)
    imposed = np.zeros(12, np.uint8)
    imposed[0] = 1
    f = np.zeros(12)
    f[6] = 100.0
    aa, bb, blocks = separate_sparse(*m.csr(), imposed, m.index_node_numbers())
    x, it, ok = pcg(blocks["k_aa"], find_b_sparse(f[aa], blocks["k_ab"], np.zeros(len(bb))), 1e-4, 1e-12, 1000, None)
    assert ok
    disp = np.zeros(12)
    disp[aa] = x
    out = fo.truss_results([0, 0, 0], [30, 0, 0], 1e6, 2.0, None, np.r_[disp[0:3], disp[6:9]])
    assert out[0] == pytest.approx(100.0, rel=1e-12)


def _golden():
    with open(GOLDEN) as fh:
        return json.load(fh)["cases"]


def _run(case):
    a, u = case["args"], case["u"]
    if case["kind"] == "truss":
        return fo.truss_results(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"), u)
    if case["kind"] == "beam":
        return fo.beam_results(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"], a["i12"],
                               a["it"], a["shear_factor"], a["axis"], u)
    return fo.plate_results(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"], a["thickness"],
                            a["shear_factor"], u)


def test_golden_results():
    cases = _golden()
    assert {c["kind"] for c in cases} == {"truss", "beam", "plate"} and len(cases) == 29
    for case in cases:
        got = _run(case)
        want = np.array([float(v) for v in case["values"]])
        scale = np.array([float(v) for v in case["scale"]])
        err = np.abs(got - want)
        assert np.all(err <= TOL * np.maximum(scale, 1e-300)), (case["name"], err / scale)


def _beam_props(rng):
    return dict(young=210e9, poisson=rng.uniform(0.2, 0.4), area=rng.uniform(5e-3, 2e-2), i11=rng.uniform(1e-5, 1e-4),
                i22=rng.uniform(1e-5, 1e-4), i12=rng.uniform(-5e-6, 5e-6), it=rng.uniform(1e-6, 5e-5),
                shear_factor=5 / 6)


@pytest.mark.parametrize("seed", range(8))
def test_beam_results_are_local_end_forces(seed):
    """ForceR..MomentR = f_l[6..9], MomentS = (-f_l[4], avg, f_l[10]), MomentT = (-f_l[5], avg, f_l[11]) with
    f_l = T K_e u_e -- the reduced-integration element's end forces (beam.rs:495-605 with :803-993)"""
    rng = np.random.default_rng(seed)
    x1 = rng.uniform(-2, 2, 3)
    x2 = x1 + rng.uniform(-3, 3, 3)
    axis = [0.0, 0.0, 1.0] if abs(x2[0] - x1[0]) + abs(x2[1] - x1[1]) > 1e-3 else [1.0, 0.0, 0.0]
    p = _beam_props(rng)
    u = rng.standard_normal(12) * 1e-3
    args = (x1, x2, p["young"], p["poisson"], p["area"], p["i11"], p["i22"], p["i12"], p["it"], p["shear_factor"], axis)
    got = fo.beam_results(*args, u)
    K = fo.beam_global_matrix(*args)
    R, _, _ = fo.beam_rotation(x1, x2, p["i11"], p["i22"], p["i12"], axis)
    T = np.kron(np.eye(4), R)
    f = T @ (K @ u)
    want = np.array([f[6], f[7], f[8], f[9], -f[4], (f[10] - f[4]) / 2, f[10], -f[5], (f[11] - f[5]) / 2, f[11]])
    scale = np.abs(T) @ (np.abs(K) @ np.abs(u))
    assert np.max(np.abs(got - want)) <= 1e-12 * scale.max()


@pytest.mark.parametrize("tapered", [False, True])
def test_truss_result_is_local_end_force(tapered):
    rng = np.random.default_rng(7)
    for _ in range(5):
        x1 = rng.uniform(-2, 2, 3)
        x2 = x1 + rng.uniform(-3, 3, 3)
        a2 = 1e-4 if tapered else None
        u = rng.standard_normal(6) * 1e-3
        got = fo.truss_results(x1, x2, 200e9, 3e-4, a2, u)
        K = fo.truss_global_matrix(x1, x2, 200e9, 3e-4, a2)
        R = fo.truss_rotation(x1, x2)
        f = np.kron(np.eye(2), R) @ (K @ u)
        scale = np.abs(np.kron(np.eye(2), R)) @ (np.abs(K) @ np.abs(u))
        assert abs(got[0] - f[3]) <= 1e-12 * scale.max() and abs(got[0] + f[0]) <= 1e-12 * scale.max()


QUADS = {
    "distorted": ([0.12, 0.09, 0.0], [-0.02, 0.11, 0.0], [0.01, -0.015, 0.0], [0.105, 0.003, 0.0]),
    "rectangle": ([2.0, 1.5, 0.0], [0.0, 1.5, 0.0], [0.0, 0.0, 0.0], [2.0, 0.0, 0.0]),
}


@pytest.mark.parametrize("quad", sorted(QUADS))
def test_plate_constant_strain_states(quad):
    """membrane N = C_m e t, bending M = D k for linear u, v and theta fields on any quad; transverse shear
    Q = G k_s t gamma for w = gx x + gy y on an axis-aligned rectangle (r, s = x, y)"""
    E, nu, t, ks = 70e9, 0.3, 0.02, 5 / 6
    P = [np.array(p) for p in QUADS[quad]]
    ex, ey, gxy = 1e-4, -2e-4, 3e-4
    u = np.zeros(24)
    for i, p in enumerate(P):
        u[6 * i] = ex * p[0] + gxy * p[1]
        u[6 * i + 1] = ey * p[1]
    got = fo.plate_results(*P, E, nu, t, ks, u)
    C = E * t / (1 - nu ** 2)
    np.testing.assert_allclose(got[:3], [C * (ex + nu * ey), C * (nu * ex + ey), C * (1 - nu) / 2 * gxy], rtol=1e-12)
    np.testing.assert_allclose(got[3:], 0.0, atol=1e-9)
    kx, ky, kxy = 1e-3, -5e-4, 2e-4
    u = np.zeros(24)
    for i, p in enumerate(P):
        u[6 * i + 4] = -kx * p[0]  # kappa_x = -d thy / dx
        u[6 * i + 3] = ky * p[1] + kxy * p[0]  # kappa_y = d thx / dy, kappa_xy = d thx / dx - d thy / dy
    got = fo.plate_results(*P, E, nu, t, ks, u)
    D = E * t ** 3 / (12 * (1 - nu ** 2))
    np.testing.assert_allclose(got[3:6], [D * (nu * kx + ky), D * (kx + nu * ky), D * (1 - nu) / 2 * kxy], rtol=1e-12)
    np.testing.assert_allclose(got[:3], 0.0, atol=1e-9)
    if quad == "rectangle":
        gx, gy = 1e-3, 2e-3
        u = np.zeros(24)
        for i, p in enumerate(P):
            u[6 * i + 2] = gx * p[0] + gy * p[1]
        got = fo.plate_results(*P, E, nu, t, ks, u)
        Gk = E / (2 * (1 + nu)) * t * ks
        np.testing.assert_allclose(got[6:], [Gk * gx, Gk * gy], rtol=1e-12)


def test_plate_rigid_body_motion_is_stress_free():
    rng = np.random.default_rng(11)
    P = [np.array(p) for p in QUADS["distorted"]]
    w = rng.standard_normal(3) * 1e-3  # small rotation
    c = rng.standard_normal(3) * 1e-3
    u = np.zeros(24)
    for i, p in enumerate(P):
        u[6 * i:6 * i + 3] = c + np.cross(w, p)
        u[6 * i + 3:6 * i + 6] = w
    got = fo.plate_results(*P, 70e9, 0.3, 0.02, 5 / 6, u)
    assert np.max(np.abs(got)) < 1e-9 * 70e9 * 0.02 * 1e-3


def test_mesh_results_match_element_calls():
    """orc_element_results (threads over element ranges) equals the per-element calls bit for bit"""
    rng = np.random.default_rng(3)
    for mesh in (meshes.truss_lattice(n=4), meshes.beam_frame(nx=4, ny=3, nz=3), meshes.plate_mesh(nx=5, ny=4, size=2.0)):
        disp = rng.standard_normal(6 * mesh.nodes_number) * 1e-3
        out1, _ = fo.element_results(mesh, disp, n_threads=1)
        out3, _ = fo.element_results(mesh, disp, n_threads=3)
        for k in out1:
            assert np.array_equal(out1[k], out3[k])
        X = mesh.xyz
        if mesh.trusses is not None:
            t = mesh.trusses
            for e in range(len(t["numbers"])):
                a, b = np.asarray(t["nodes"][e]) - 1
                a2 = None if t.get("area_2") is None else t["area_2"][e]
                got = fo.truss_results(X[a], X[b], t["young"][e], t["area"][e], a2,
                                       np.r_[disp[6 * a:6 * a + 3], disp[6 * b:6 * b + 3]])
                assert got[0] == out1["truss"][e, 0]
        if mesh.beams is not None:
            bm = mesh.beams
            for e in range(0, len(bm["numbers"]), 7):
                a, b = np.asarray(bm["nodes"][e]) - 1
                got = fo.beam_results(X[a], X[b], bm["young"][e], bm["poisson"][e], bm["area"][e], bm["i11"][e],
                                      bm["i22"][e], bm["i12"][e], bm["it"][e], bm["shear_factor"][e], bm["axis"][e],
                                      np.r_[disp[6 * a:6 * a + 6], disp[6 * b:6 * b + 6]])
                assert np.array_equal(got, out1["beam"][e])
        if mesh.plates is not None:
            pl = mesh.plates
            for e in range(len(pl["numbers"])):
                nd = np.asarray(pl["nodes"][e]) - 1
                got = fo.plate_results(*(X[i] for i in nd), pl["young"][e], pl["poisson"][e], pl["thickness"][e],
                                       pl["shear_factor"][e], np.concatenate([disp[6 * i:6 * i + 6] for i in nd]))
                assert np.array_equal(got, out1["plate"][e])


@pytest.mark.parametrize("name", ["truss_tapered_1", "beam_i12_0", "plate_tilted_1"])
def test_golden_fixture_is_what_its_script_computes(name):
    """element_results.json holds what tests/golden/make_results_golden.py computes: the case is evaluated
    again from its recorded arguments and displacements in 50-digit arithmetic, values and scales digit for
    digit"""
    import importlib.util

    from oracle import literal

    spec = importlib.util.spec_from_file_location(
        "make_results_golden", os.path.join(os.path.dirname(GOLDEN), "make_results_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    with open(GOLDEN) as f:
        case = next(c for c in json.load(f)["cases"] if c["name"] == name)
    a, u = case["args"], case["u"]
    if case["kind"] == "truss":
        v, s = literal.truss_results(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"), u, bk=mg.BK)
    elif case["kind"] == "beam":
        v, s = literal.beam_results(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"],
                                    a["i12"], a["it"], a["shear_factor"], a["axis"], u, bk=mg.BK)
    else:
        v, s = literal.plate_results(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"], a["thickness"],
                                     a["shear_factor"], u, bk=mg.BK)
    assert mg.strs(v) == case["values"] and mg.strs(s) == case["scale"]
