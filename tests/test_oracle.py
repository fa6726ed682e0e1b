"""CPU tests of the oracle (oracle/fem_oracle.c): pinned to the reference's own
known answer, to a literal dense restatement of the reference formulas and to
high-precision golden element matrices; no GPU involved."""
import json
import math
import os

import numpy as np
import pytest

from oracle import literal

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel_err(a, b):
    """max |a - b| / max |b| (entries that cancel inside one element are measured against the element's scale)."""
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_reference_truss_known_answer(oracle):
    """src/tests/fem/test_fem.rs:5-64: truss 1-2 along x, E=1e6, A=2, L=30, node 1 fixed in X,
    100 N at node 2 X -> u2x = 0.0014999999 (f32), reaction -100."""
    m = oracle.OracleFEM(1e-4, 1e-12, 2)
    m.add_node(1, 0.0, 0.0, 0.0)
    m.add_node(2, 30.0, 0.0, 0.0)
    m.add_truss(1, 1, 2, 1e6, 2.0)
    rp, ci, va = m.csr()
    assert rp.shape == (13,)
    rows = np.repeat(np.arange(12), np.diff(rp))
    entries = {(int(r), int(c)): float(v) for r, c, v in zip(rows, ci, va)}
    k = 1e6 * 2.0 / 30.0
    assert set(entries) == {(0, 0), (0, 6), (6, 0), (6, 6)}
    assert entries[(0, 0)] == pytest.approx(k, rel=1e-15) and entries[(6, 6)] == entries[(0, 0)]
    assert entries[(0, 6)] == entries[(6, 0)] == -entries[(0, 0)]
    u2x = 100.0 / entries[(6, 6)]  # K_aa = [k] with the X DOF of node 2 the only free, loaded one
    # the reference test runs in f32: its 0.0014999999 is PL/EA to f32 rounding (1 ulp = 1.2e-10 here)
    assert abs(u2x - 0.0014999999) <= 2 * float(np.spacing(np.float32(0.0015)))
    assert u2x == pytest.approx(100.0 * 30.0 / (1e6 * 2.0), rel=1e-15)
    assert entries[(0, 6)] * u2x == pytest.approx(-100.0, rel=1e-14)


def _plate_nodes(rng, tilt=True):
    pts = np.array([[1, 1, 0], [-1, 1, 0], [-1, -1, 0], [1, -1, 0]], float)
    pts[:, :2] *= rng.uniform(0.2, 3.0, size=2)
    pts[:, :2] += rng.uniform(-0.25, 0.25, (4, 2)) * np.abs(pts[:, :2]).max()
    if tilt:
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        pts = pts @ q.T
    return pts + rng.normal(size=3)


def test_plate_matches_literal(oracle):
    rng = np.random.default_rng(11)
    worst = 0.0
    for t in range(300):
        P = _plate_nodes(rng, tilt=t % 3 != 0)
        E, nu, th = rng.uniform(1e9, 3e11), rng.uniform(0.05, 0.45), rng.uniform(1e-3, 0.3)
        a = oracle.plate_global_matrix(*P, E, nu, th, 5 / 6)
        b = literal.plate_global_matrix(*P, E, nu, th, 5 / 6)
        worst = max(worst, rel_err(a, b))
        np.testing.assert_array_equal(a, a.T)
    assert worst < 1e-12, worst


def test_beam_matches_literal(oracle):
    rng = np.random.default_rng(12)
    worst = 0.0
    for t in range(300):
        x1, x2 = rng.normal(size=3) * 3, rng.normal(size=3) * 3
        if t % 5 == 0:
            x2 = x1 + np.array([0.0, rng.uniform(1, 4), 0.0])  # vertical in y: the c_xz == 0 branch
        axis = rng.normal(size=3)
        i11, i22 = rng.uniform(1e-5, 1e-4, size=2)
        i12 = 0.0 if t % 2 else rng.uniform(-0.3, 0.3) * min(i11, i22)
        args = (x1, x2, 210e9, 0.3, rng.uniform(5e-3, 2e-2), i11, i22, i12, rng.uniform(1e-6, 5e-5), 5 / 6, axis)
        a = oracle.beam_global_matrix(*args)
        b = literal.beam_global_matrix(*args)
        worst = max(worst, rel_err(a, b))
        np.testing.assert_array_equal(a, a.T)
    assert worst < 1e-12, worst


def test_truss_matches_literal(oracle):
    rng = np.random.default_rng(13)
    worst = 0.0
    for t in range(300):
        x1, x2 = rng.normal(size=3), rng.normal(size=3)
        a2 = None if t % 2 else rng.uniform(1e-4, 5e-4)
        a = oracle.truss_global_matrix(x1, x2, 200e9, 3e-4, a2)
        b = literal.truss_global_matrix(x1, x2, 200e9, 3e-4, a2)
        worst = max(worst, rel_err(a, b))
    assert worst < 1e-13, worst


def test_beam_closed_form_x_axis(oracle):
    """x-aligned beam: k_uu = EA/L, k_vv = G A k/L, k_v,thz = G A k/2, k_thz,thz = E I11p/L + G A k L/4,
    k_thx,thx = G J/L (structs/beam.rs:495-563 at r = 0, alpha = 2, det J = L/2)."""
    L, E, nu, A, i11, i22, J, k = 4.0, 210e9, 0.3, 1e-2, 8e-5, 3e-5, 2e-5, 5 / 6
    Km = oracle.beam_global_matrix([0, 0, 0], [L, 0, 0], E, nu, A, i11, i22, 0.0, J, k, [0, 0, 1])
    G = E / (2 * (1 + nu))
    assert Km[0, 0] == pytest.approx(E * A / L, rel=1e-14)
    assert Km[0, 6] == pytest.approx(-E * A / L, rel=1e-14)
    assert Km[3, 3] == pytest.approx(G * J / L, rel=1e-14)
    assert Km[1, 1] == pytest.approx(G * A * k / L, rel=1e-14)
    assert Km[2, 2] == pytest.approx(G * A * k / L, rel=1e-14)
    # the bending pairs: one carries I11p, the other I22p (principal moments, I11p >= I22p)
    bend = sorted([Km[4, 4], Km[5, 5]])
    shear = G * A * k * L / 4
    assert bend[0] == pytest.approx(E * min(i11, i22) / L + shear, rel=1e-14)
    assert bend[1] == pytest.approx(E * max(i11, i22) / L + shear, rel=1e-14)
    assert abs(Km[1, 5]) == pytest.approx(G * A * k / 2, rel=1e-14)


def test_plate_rigid_body_modes(oracle):
    """translations and rotations of a tilted quad produce no force except on the drilling springs."""
    rng = np.random.default_rng(14)
    for _ in range(20):
        P = _plate_nodes(rng)
        K = oracle.plate_global_matrix(*P, 70e9, 0.3, 0.02, 5 / 6)
        scale = np.abs(K).max()
        for d in range(3):
            u = np.zeros(24)
            u[d::6] = 1.0
            assert np.abs(K @ u).max() < 1e-10 * scale
        R = oracle.plate_rotation(P[1], P[2], P[3])
        n = R[2]  # plate normal in global axes
        c = P.mean(0)
        for ax in (R[0], R[1]):  # rotations about in-plane axes (no drilling involved)
            u = np.zeros(24)
            for i in range(4):
                u[6 * i:6 * i + 3] = np.cross(ax, P[i] - c)
                u[6 * i + 3:6 * i + 6] = ax
            assert np.abs(K @ u).max() < 1e-9 * scale * np.abs(P - c).max()
        assert np.allclose(np.abs(n), np.abs(R[2]))


def test_plate_rotation_invariance(oracle):
    """K' = T^T K T when the whole quad is rotated: the local matrix does not change."""
    rng = np.random.default_rng(15)
    for _ in range(20):
        P = _plate_nodes(rng)
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(q) < 0:
            q[:, 0] *= -1
        K1 = oracle.plate_global_matrix(*P, 70e9, 0.3, 0.02, 5 / 6)
        K2 = oracle.plate_global_matrix(*(P @ q.T), 70e9, 0.3, 0.02, 5 / 6)
        R1 = oracle.plate_rotation(P[1], P[2], P[3])
        R2 = oracle.plate_rotation(*(P[1:] @ q.T))
        T1 = np.kron(np.eye(8), R1)
        T2 = np.kron(np.eye(8), R2)
        # local matrices agree up to the in-plane orientation of the local axes; compare invariants
        L1, L2 = T1 @ K1 @ T1.T, T2 @ K2 @ T2.T
        np.testing.assert_allclose(np.sort(np.linalg.eigvalsh(L1)), np.sort(np.linalg.eigvalsh(L2)),
                                   rtol=1e-9, atol=1e-9 * np.abs(L1).max())


@pytest.mark.parametrize("x", [0.0, 1e-300, 1e-8, 0.3, 0.7853981633974483, 1.0, 1.5, 2.5, 3.14159, 10.0, 100.0, -0.7,
                               -3.0, 1e3])
def test_transcendentals(oracle, x):
    ulp = lambda v: math.ulp(abs(v)) if v else 5e-324
    assert abs(oracle.sin(x) - math.sin(x)) <= 2 * ulp(math.sin(x)) + 1e-300
    assert abs(oracle.cos(x) - math.cos(x)) <= 2 * ulp(math.cos(x)) + 1e-300
    assert abs(oracle.atan(x) - math.atan(x)) <= 2 * ulp(math.atan(x)) + 1e-300
    c = math.tanh(x)
    assert abs(oracle.acos(c) - math.acos(c)) <= 4 * ulp(math.acos(c)) + 1e-300


def test_transcendentals_dense(oracle):
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-7, 7, 2000), rng.uniform(-1, 1, 2000)])
    worst = 0
    for x in xs:
        for f, g in ((oracle.sin, math.sin), (oracle.cos, math.cos), (oracle.atan, math.atan)):
            v = g(x)
            worst = max(worst, abs(f(x) - v) / math.ulp(abs(v)) if v else 0)
    assert worst <= 2.0, worst


# --- validation messages (the reference's Err strings) ----------------------------------------

def test_validation_messages(oracle):
    m = oracle.OracleFEM(1e-12, 1e-12, 6)
    m.add_node(1, 0, 0, 0)
    m.add_node(2, 1, 0, 0)
    m.add_node(3, 1, 1, 0)
    m.add_node(4, 0, 1, 0)
    with pytest.raises(oracle.OracleError, match=r"^Node with number 1 already exists!$"):
        m.add_node(1, 5, 5, 5)
    with pytest.raises(oracle.OracleError, match=r"^Node with coordinates x: 1.0, y: 1.0, z: 0.0 already exists!$"):
        m.add_node(9, 1.0, 1.0, 0.0)
    with pytest.raises(oracle.OracleError, match=r"^Node with number 7 does not exist!$"):
        m.add_truss(1, 1, 7, 1.0, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Young's modulus -1.0 is less or equal to zero!$"):
        m.add_truss(1, 1, 2, -1.0, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Area 0.0 is less or equal to zero!$"):
        m.add_truss(1, 1, 2, 1.0, 0.0)
    m.add_truss(1, 1, 2, 1.0, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Truss element with number 1 already exists!$"):
        m.add_truss(1, 3, 4, 1.0, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Truss element with node number 2 and 1 already exists!$"):
        m.add_truss(2, 2, 1, 1.0, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Local axis 1 direction \[1.0, 0.0, 0.0\] parallel to element 5!$"):
        m.add_beam(5, 1, 2, 1.0, 0.3, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0, [1.0, 0.0, 0.0])
    with pytest.raises(oracle.OracleError, match=r"^Element 3 non-convex!$"):
        m.add_node(5, 0.4, 0.6, 0.0)  # inside the triangle of nodes 3, 4, 1: a dart
        m.add_plate(3, 3, 4, 1, 5, 1.0, 0.3, 0.1, 1.0)
    m.add_node(6, 0.5, 0.5, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Not all nodes of element 4 lie on the plane!$"):
        m.add_plate(4, 6, 4, 1, 2, 1.0, 0.3, 0.1, 1.0)
    with pytest.raises(oracle.OracleError, match=r"^Nodes number could not be greater than 6!$"):
        m.add_node(10, 7, 7, 7)


# --- golden fixtures -----------------------------------------------------------------------------

def _golden():
    path = os.path.join(GOLDEN, "element_matrices.json")
    with open(path) as f:
        return json.load(f)


def test_golden_element_matrices(oracle):
    """high-precision (mpmath, 50 digits) evaluations of the reference's element formulas."""
    cases = _golden()["cases"]
    assert len(cases) >= 10
    for c in cases:
        ref = np.array([float(v) for v in c["matrix"]]).reshape(c["shape"])
        a = c["args"]
        if c["kind"] == "truss":
            got = oracle.truss_global_matrix(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"))
        elif c["kind"] == "beam":
            got = oracle.beam_global_matrix(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"],
                                            a["i12"], a["it"], a["shear_factor"], a["axis"])
        else:
            got = oracle.plate_global_matrix(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"],
                                             a["thickness"], a["shear_factor"])
        scale = np.abs(ref).max()
        err = np.abs(got - ref).max() / scale
        assert err < 1e-13, (c["name"], err)
        # entries that are exactly zero in the reference formulas are exactly zero in the oracle
        np.testing.assert_array_equal(got[ref == 0.0], 0.0, err_msg=c["name"])


@pytest.mark.parametrize("threads", [1, 3, 4])
def test_parallel_port_matches_the_eager_oracle(oracle, threads):
    """The reference arm's multi-threaded port (orc_assemble_parallel: CSR rows partitioned over threads,
    each row's entries summed in element call order) gives the eager oracle's CSR bit for bit: beams and
    plates sharing nodes, a truss lattice, a plate mesh."""
    from finite_element_method_gb300 import meshes

    for m in (meshes.adjoint_model(frame=(4, 4, 3), slab=(30, 30), seed=7), meshes.truss_lattice(5, seed=3),
              meshes.plate_mesh(20, 15, size=3.0, seed=11)):
        o = oracle.OracleFEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
        meshes.load(o, m)
        rp, ci, va = o.csr()
        _, nnz, (prp, pci, pva) = oracle.assemble_parallel(m, threads, meshes.REL_TOL, meshes.ABS_TOL)
        assert nnz == len(ci) > 0, m.name
        np.testing.assert_array_equal(prp, rp, err_msg=m.name)
        np.testing.assert_array_equal(pci, ci, err_msg=m.name)
        np.testing.assert_array_equal(pva.view(np.uint64), va.view(np.uint64), err_msg=m.name)


@pytest.mark.parametrize("name", ["truss_tapered", "beam_i12", "plate_tilted"])
def test_golden_fixture_is_what_its_script_computes(name):
    """element_matrices.json holds what tests/golden/make_golden.py computes: the case is evaluated again from
    its recorded arguments in 50-digit arithmetic and compared with the fixture digit for digit"""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    case = next(c for c in _golden()["cases"] if c["name"] == name)
    a = case["args"]
    if case["kind"] == "truss":
        M = literal.truss_global_matrix(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"), bk=mg.BK)
    elif case["kind"] == "beam":
        M = literal.beam_global_matrix(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"],
                                       a["i12"], a["it"], a["shear_factor"], a["axis"], bk=mg.BK)
    else:
        M = literal.plate_global_matrix(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"],
                                        a["thickness"], a["shear_factor"], bk=mg.BK)
    assert mg.mstr(M) == case["matrix"]
