"""GPU vector-Jacobian product against finite differences of the reference
assembly (the oracle's element matrices) and against a high-precision
derivative of the reference formulas (oracle/literal.py in 50-digit mpmath)."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, meshes
from oracle import fem_oracle as fo
from oracle import literal

pytestmark = pytest.mark.gpu

FD_REL = 1e-7  # GPU gradient vs central finite differences (step 1e-6 relative)


def element_dofs(nodes0, ndn):
    return np.concatenate([6 * n + np.arange(ndn) for n in nodes0])


def element_k(kind, mesh, e, xyz, props):
    """the oracle's element matrix (global axes) of element e of a kind, with its DOFs"""
    if kind == "plate":
        n0 = mesh.plates["nodes"][e].astype(np.int64) - 1
        K = fo.plate_global_matrix(*[xyz[n] for n in n0], props["young"], props["poisson"], props["thickness"],
                                   props["shear_factor"])
        return K, element_dofs(n0, 6)
    if kind == "beam":
        n0 = mesh.beams["nodes"][e].astype(np.int64) - 1
        K = fo.beam_global_matrix(xyz[n0[0]], xyz[n0[1]], props["young"], props["poisson"], props["area"],
                                  props["i11"], props["i22"], props["i12"], props["it"], props["shear_factor"],
                                  props["axis"])
        return K, element_dofs(n0, 6)
    n0 = mesh.trusses["nodes"][e].astype(np.int64) - 1
    a2 = props.get("area_2")
    K = fo.truss_global_matrix(xyz[n0[0]], xyz[n0[1]], props["young"], props["area"],
                               None if a2 is None or np.isnan(a2) else a2)
    return K, element_dofs(n0, 3)


def contract(dK, d, U, L):
    """-sum_p lam_p,e^T dK u_p,e"""
    return -float(np.einsum("pi,ij,pj->", L[:, d], dK, U[:, d]))


def props_of(mesh, kind, e):
    d = {"plate": mesh.plates, "beam": mesh.beams, "truss": mesh.trusses}[kind]
    return {k: (v[e] if v is not None else None) for k, v in d.items() if k not in ("numbers", "nodes")}


def touching(mesh, node0):
    out = []
    for kind, d in (("truss", mesh.trusses), ("beam", mesh.beams), ("plate", mesh.plates)):
        if d is None:
            continue
        hit = np.flatnonzero((d["nodes"].astype(np.int64) - 1 == node0).any(1))
        out += [(kind, int(e)) for e in hit]
    return out


# Central finite differences of the reference assembly: the element matrices at theta +- h are
# differenced entry by entry, then contracted with the pairs (so the cancellation inside
# sum_p lam_p^T K u_p does not swamp the difference).  The step is 1e-6 relative; the estimate is
# 2 D(h / 2) - D(h), which removes the O(h) error that central differences keep where the reference's
# section-angle parametrisation (acos of a cosine that reaches 1) has a kink.  Alongside the estimate
# comes its rounding bound: 8 eps sum |lam| |K| |u| / h.
EPS = np.finfo(np.float64).eps


def _central(ks_fn, h, U, L):
    kp, d = ks_fn(+h)
    km, _ = ks_fn(-h)
    return contract((kp - km) / (2 * h), d, U, L)


def _fd(ks_fn, h, U, L):
    K0, d = ks_fn(0.0)
    est = 2 * _central(ks_fn, h / 2, U, L) - _central(ks_fn, h, U, L)
    bound = 8 * EPS * float(np.einsum("pi,ij,pj->", np.abs(L[:, d]), np.abs(K0), np.abs(U[:, d]))) / h
    return est, bound


def fd_coord(mesh, node0, c, U, L, with_bound=False):
    x = mesh.xyz[node0, c]
    h = 1e-6 * max(abs(x), 1.0)
    tot, bnd = 0.0, 0.0
    for kind, e in touching(mesh, node0):
        def ks(dh, kind=kind, e=e):
            xyz = mesh.xyz.copy()
            xyz[node0, c] = x + dh
            return element_k(kind, mesh, e, xyz, props_of(mesh, kind, e))
        est, b = _fd(ks, h, U, L)
        tot += est
        bnd += b
    return (tot, bnd) if with_bound else tot


def fd_prop(mesh, kind, e, name, U, L, with_bound=False):
    p = props_of(mesh, kind, e)
    v = p[name]

    def ks(dh):
        q = dict(p)
        q[name] = v + dh
        return element_k(kind, mesh, e, mesh.xyz, q)
    est, b = _fd(ks, 1e-6 * abs(v), U, L)
    return (est, b) if with_bound else est


# The second reference: the reference formulas (oracle/literal.py) in 50-digit arithmetic, differenced
# centrally with step 1e-11 relative -- accurate to double precision even next to the kink of the
# section twist (acos of a cosine near 1), where the 1e-6 finite differences above carry an error of
# their own (up to ~1e-5 relative on beams whose twist is ~1e-6).  The step stays wide against the
# plateaus of the reference's tolerance clamps (compare_with_tolerance zeroes rotation entries below
# 1e-12, so a plate tilted by less than 1e-12 rad is not rotated at all): like the GPU and the 1e-6
# differences, it measures the slope of the formulas either side of such a plateau.
HP_REL = 1e-9  # GPU gradient vs the high-precision derivative, relative to the magnitude of its shares


def _hp():
    mp = pytest.importorskip("mpmath")
    return mp, literal.Backend.mp(50)


def _k_hp(kind, X, P, bk):
    if kind == "plate":
        return literal.plate_global_matrix(*X, P["young"], P["poisson"], P["thickness"], P["shear_factor"], bk=bk)
    if kind == "beam":
        return literal.beam_global_matrix(*X, P["young"], P["poisson"], P["area"], P["i11"], P["i22"], P["i12"],
                                          P["it"], P["shear_factor"], P["axis"], bk=bk)
    return literal.truss_global_matrix(*X, P["young"], P["area"], P.get("area_2"), bk=bk)


def hp_share(mesh, kind, e, U, L, node0=None, c=None, name=None):
    """element e's share of the gradient w.r.t. coordinate c of node0 (or property `name`), from the
    50-digit central difference (step 1e-11 relative) of the reference formulas, contracted with the pairs"""
    mp, bk = _hp()
    f = lambda v: mp.mpf(float(v))
    d = {"plate": mesh.plates, "beam": mesh.beams, "truss": mesh.trusses}[kind]
    n0 = d["nodes"][e].astype(np.int64) - 1
    P = {}
    for k, v in props_of(mesh, kind, e).items():
        if v is None or (np.ndim(v) == 0 and np.isnan(v)):
            P[k] = None
        else:
            P[k] = f(v) if np.ndim(v) == 0 else [f(x) for x in v]

    def k_at(s):
        X = [[f(v) for v in mesh.xyz[n]] for n in n0]
        Q = dict(P)
        if name is None:
            h = mp.mpf("1e-11") * max(abs(f(mesh.xyz[node0, c])), 1)
            for k, n in enumerate(n0):
                if n == node0:
                    X[k][c] += s * h
        else:
            h = mp.mpf("1e-11") * abs(P[name])
            Q[name] = P[name] + s * h
        return _k_hp(kind, X, Q, bk), h

    (kp, h), (km, _) = k_at(1), k_at(-1)
    n = kp.shape[0]
    dK = np.array([[float((kp[i, j] - km[i, j]) / (2 * h)) for j in range(n)] for i in range(n)])
    return contract(dK, element_dofs(n0, n // len(n0)), U, L)


def check_coord(mesh, node0, c, got, U, L):
    """(ok, fd_used, detail) for the gradient w.r.t. one nodal coordinate"""
    fd, bound = fd_coord(mesh, node0, c, U, L, with_bound=True)
    shares = [hp_share(mesh, kind, e, U, L, node0=node0, c=c) for kind, e in touching(mesh, node0)]
    return arbitrate(got, fd, bound, sum(shares), sum(abs(s) for s in shares))


def check_prop(mesh, kind, e, name, got, U, L):
    """(ok, fd_used, detail) for the gradient w.r.t. one element property"""
    fd, bound = fd_prop(mesh, kind, e, name, U, L, with_bound=True)
    hp = hp_share(mesh, kind, e, U, L, name=name)
    return arbitrate(got, fd, bound, hp, abs(hp))


def arbitrate(got, fd, bound, hp, mag):
    """The GPU gradient must lie within HP_REL * mag of the high-precision derivative (mag = the summed
    magnitude of the element shares, the scale of a sum that cancels), and within FD_REL of the
    finite-difference estimate (plus its rounding bound) wherever that estimate is itself within
    FD_REL / 2 of the high-precision derivative."""
    ok_hp = abs(got - hp) <= HP_REL * mag
    fd_used = abs(fd - hp) <= 0.5 * FD_REL * mag + bound
    ok_fd = not fd_used or abs(got - fd) <= FD_REL * max(abs(fd), mag) + bound
    return ok_hp and ok_fd, fd_used, (got, hp, fd, bound, mag)


def model_with_trusses(seed=3):
    m = meshes.adjoint_model(frame=(4, 4, 3), slab=(30, 30), seed=seed)
    rng = np.random.default_rng(seed)
    nx, ny, nz = 4, 4, 3
    node = lambda i, j, k: 1 + i + nx * (j + ny * k)
    pairs = [(node(i, j, k), node(i + 1, j + 1, k + 1)) for k in range(nz - 1) for j in range(ny - 1)
             for i in range(nx - 1)]
    t = len(pairs)
    m.trusses = dict(numbers=np.arange(1, t + 1, dtype=np.uint32), nodes=np.array(pairs, np.uint32),
                     young=np.full(t, 200e9), area=rng.uniform(1e-4, 5e-4, t),
                     area_2=np.where(np.arange(t) % 2 == 0, np.nan, rng.uniform(1e-4, 5e-4, t)))
    return m


@pytest.fixture(scope="module")
def case():
    m = model_with_trusses()
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    rng = np.random.default_rng(11)
    P = 4
    n = 6 * m.nodes_number
    U = rng.normal(size=(P, n))
    L = rng.normal(size=(P, n))
    return m, g, U, L, g.vjp(U, L)


def test_vjp_shapes_and_determinism(case):
    m, g, U, L, gr = case
    assert gr["plate"].shape == (m.counts()[2], 2) and gr["beam"].shape == (m.counts()[1], 5)
    assert gr["truss"].shape == (m.counts()[0], 3) and gr["xyz"].shape == (m.nodes_number, 3)
    again = g.vjp(U, L)
    for k in gr:
        np.testing.assert_array_equal(again[k].view(np.uint64), gr[k].view(np.uint64))


def test_vjp_property_gradients_vs_fd(case):
    m, g, U, L, gr = case
    rng = np.random.default_rng(1)
    checks = []
    for e in rng.choice(m.counts()[2], 12, replace=False):
        checks += [("plate", e, "young", gr["plate"][e, 0]), ("plate", e, "thickness", gr["plate"][e, 1])]
    for e in rng.choice(m.counts()[1], 10, replace=False):
        for j, name in enumerate(("young", "area", "i11", "i22", "it")):
            checks.append(("beam", e, name, gr["beam"][e, j]))
    for e in range(m.counts()[0]):
        checks += [("truss", e, "young", gr["truss"][e, 0]), ("truss", e, "area", gr["truss"][e, 1])]
        if not np.isnan(m.trusses["area_2"][e]):
            checks.append(("truss", e, "area_2", gr["truss"][e, 2]))
        else:
            assert gr["truss"][e, 2] == 0.0
    bad, n_fd = [], 0
    for kind, e, name, got in checks:
        ok, fd_used, detail = check_prop(m, kind, int(e), name, got, U, L)
        n_fd += fd_used
        if not ok:
            bad.append((kind, int(e), name) + detail)
    assert not bad, bad[:5]
    assert n_fd >= 0.9 * len(checks)


def test_vjp_coordinate_gradients_vs_fd(case):
    m, g, U, L, gr = case
    rng = np.random.default_rng(2)
    nodes = rng.choice(m.nodes_number, 40, replace=False)
    bad, n_fd = [], 0
    for n0 in nodes:
        for c in range(3):
            ok, fd_used, detail = check_coord(m, int(n0), c, gr["xyz"][n0, c], U, L)
            n_fd += fd_used
            if not ok:
                bad.append((int(n0), c) + detail)
    assert not bad, bad[:5]
    assert n_fd >= 0.9 * 3 * len(nodes)


def test_vjp_against_high_precision_reference():
    """one plate and one beam (tilted, general rotation): GPU gradients vs the derivative of the reference
    formulas evaluated in 50-digit arithmetic (central difference with step 1e-20)."""
    mp = pytest.importorskip("mpmath")
    bk = literal.Backend.mp(50)
    rng = np.random.default_rng(4)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    quad = np.array([[1.1, 0.9, 0.0], [-0.8, 1.2, 0.0], [-1.0, -1.0, 0.0], [0.9, -1.1, 0.0]]) @ q.T
    xyz = np.concatenate([quad, [[3.0, 2.0, 1.5]]])
    g = FEM(1e-12, 1e-12, 5)
    g.add_nodes([1, 2, 3, 4, 5], xyz)
    g.add_plate(1, 1, 2, 3, 4, 70e9, 0.3, 0.02, 5 / 6)
    g.add_beam(1, 1, 5, 210e9, 0.3, 1e-2, 8e-5, 3e-5, 0.0, 2e-5, 5 / 6, [0.0, 0.0, 1.0])
    g.assemble()
    U = rng.normal(size=(2, 30))
    Lm = rng.normal(size=(2, 30))
    gr = g.vjp(U, Lm)
    hp = mp.mpf("1e-20")

    def f_plate(P, E, t):
        K = literal.plate_global_matrix(*P, E, 0.3, t, 5 / 6, bk=bk)
        d = element_dofs(np.arange(4), 6)
        return -sum(mp.mpf(float(Lm[p, d[i]])) * K[i, j] * mp.mpf(float(U[p, d[j]]))
                    for p in range(2) for i in range(24) for j in range(24))

    def f_beam(x1, x2, E, A, i11, i22, it):
        K = literal.beam_global_matrix(x1, x2, E, 0.3, A, i11, i22, 0.0, it, 5 / 6, [0.0, 0.0, 1.0], bk=bk)
        d = element_dofs(np.array([0, 4]), 6)
        return -sum(mp.mpf(float(Lm[p, d[i]])) * K[i, j] * mp.mpf(float(U[p, d[j]]))
                    for p in range(2) for i in range(12) for j in range(12))

    P = [[mp.mpf(float(v)) for v in row] for row in quad]
    # plate thickness and one coordinate of node 2
    dt = (f_plate(P, mp.mpf(70e9), mp.mpf(0.02) + hp) - f_plate(P, mp.mpf(70e9), mp.mpf(0.02) - hp)) / (2 * hp)
    assert abs(gr["plate"][0, 1] - float(dt)) <= 1e-9 * abs(float(dt))
    Pp = [list(r) for r in P]
    Pm = [list(r) for r in P]
    Pp[1][2] += hp
    Pm[1][2] -= hp
    dz = (f_plate(Pp, mp.mpf(70e9), mp.mpf(0.02)) - f_plate(Pm, mp.mpf(70e9), mp.mpf(0.02))) / (2 * hp)
    # node 2's z gradient also has the beam's share only if the beam touches node 2 (it does not)
    assert abs(gr["xyz"][1, 2] - float(dz)) <= 1e-9 * max(abs(float(dz)), 1.0)
    # beam I11 and the z coordinate of its free node
    x1 = [mp.mpf(float(v)) for v in quad[0]]
    x2 = [mp.mpf(3.0), mp.mpf(2.0), mp.mpf(1.5)]
    base = dict(E=mp.mpf(210e9), A=mp.mpf(1e-2), i11=mp.mpf(8e-5), i22=mp.mpf(3e-5), it=mp.mpf(2e-5))
    bp, bm = dict(base), dict(base)
    bp["i11"] += hp
    bm["i11"] -= hp
    di = (f_beam(x1, x2, **bp) - f_beam(x1, x2, **bm)) / (2 * hp)
    assert abs(gr["beam"][0, 2] - float(di)) <= 1e-9 * abs(float(di))
    x2p, x2m = list(x2), list(x2)
    x2p[2] += hp
    x2m[2] -= hp
    dzb = (f_beam(x1, x2p, **base) - f_beam(x1, x2m, **base)) / (2 * hp)
    assert abs(gr["xyz"][4, 2] - float(dzb)) <= 1e-9 * abs(float(dzb))


@pytest.mark.slow
def test_vjp_full_adjoint_model_200_parameters():
    """the 51 x 51 x 11 frame + 500 x 500 slab with 64 pairs: 200 random parameters against central
    differences of the oracle's element matrices and the high-precision derivative of the reference
    formulas (the gradient is linear in the pairs: 8 of them are used)."""
    m = meshes.adjoint_model()
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    rng = np.random.default_rng(64)
    n = 6 * m.nodes_number
    U = rng.normal(size=(64, n))
    L = rng.normal(size=(64, n))
    full = g.vjp(U, L)
    part = g.vjp(U[:8], L[:8])
    # linearity in the pairs: the 64-pair gradient is the 8-pair one plus the other 56
    rest = g.vjp(U[8:], L[8:])
    for k in full:
        if full[k].size:
            np.testing.assert_allclose(full[k], part[k] + rest[k], rtol=1e-12, atol=1e-12 * np.abs(full[k]).max())
    U8, L8 = U[:8], L[:8]
    bad, n_checked, n_fd = [], 0, 0

    def record(key, res):
        nonlocal n_checked, n_fd
        ok, fd_used, detail = res
        n_checked += 1
        n_fd += fd_used
        if not ok:
            bad.append(key + detail)

    names_b = ("young", "area", "i11", "i22", "it")
    for e in rng.choice(len(m.beams["numbers"]), 60, replace=False):
        j = int(rng.integers(0, 5))
        record(("beam", int(e), names_b[j]), check_prop(m, "beam", int(e), names_b[j], part["beam"][e, j], U8, L8))
    for e in rng.choice(len(m.plates["numbers"]), 60, replace=False):
        j = int(rng.integers(0, 2))
        name = ("young", "thickness")[j]
        record(("plate", int(e), name), check_prop(m, "plate", int(e), name, part["plate"][e, j], U8, L8))
    for k, n0 in enumerate(rng.choice(m.nodes_number, 80, replace=False)):
        c = k % 3
        record(("node", int(n0), c), check_coord(m, int(n0), c, part["xyz"][n0, c], U8, L8))
    assert n_checked == 200
    assert not bad, bad[:5]
    assert n_fd >= 0.9 * n_checked
