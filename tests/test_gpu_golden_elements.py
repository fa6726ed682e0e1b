"""GPU stiffness on the reference's branch cases.

Every golden element of tests/golden/element_matrices.json (50-digit
evaluations of the reference formulas: the truss of src/tests/fem/test_fem.rs,
a tapered and an exactly anti-parallel truss, beams on both rotation branches
of structs/beam.rs:162-258, a section with I12 != 0 and one with I11 = I22,
flat, distorted, tilted and x-z plates) is assembled alone through the C ABI
(fem_gpu_assemble) and compared bit for bit with the oracle's assembly of the
same model, and with the golden matrix at 1e-13 of the element's scale.

Then frames that take the branches the generated workloads never take on the
device: sections with I12 != 0 (the arctangent and the principal-axes loop
of structs/beam.rs:119-160, :147-157), I11 = I22 with I12 != 0 (the
perturbation of :126-137), and members exactly anti-parallel to the local x
target of the rotation (the half-turn branch; structs/truss.rs:66-93,
structs/beam.rs:179)."""
import json
import os

import numpy as np
import pytest

from finite_element_method_gb300 import FEM, meshes
from oracle.fem_oracle import OracleFEM

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "element_matrices.json")
GOLDEN_REL = 1e-13  # of the element's largest entry, as the oracle's own golden test


def _cases():
    with open(GOLDEN) as f:
        return json.load(f)["cases"]


def _dense(rp, ci, va, n):
    K = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    K[rows, ci] = va
    return K


def _add_element(model, c):
    a = c["args"]
    if c["kind"] == "truss":
        pts = [a["x1"], a["x2"]]
    elif c["kind"] == "beam":
        pts = [a["x1"], a["x2"]]
    else:
        pts = [a["x1"], a["x2"], a["x3"], a["x4"]]
    for k, p in enumerate(pts):
        model.add_node(k + 1, *p)
    if c["kind"] == "truss":
        model.add_truss(1, 1, 2, a["young"], a["area"], a.get("area_2"))
    elif c["kind"] == "beam":
        model.add_beam(1, 1, 2, a["young"], a["poisson"], a["area"], a["i11"], a["i22"], a["i12"], a["it"],
                       a["shear_factor"], a["axis"])
    else:
        model.add_plate(1, 1, 2, 3, 4, a["young"], a["poisson"], a["thickness"], a["shear_factor"])
    return len(pts)


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_golden_element_on_gpu(case):
    n_nodes = 2 if case["kind"] in ("truss", "beam") else 4
    g = FEM(1e-12, 1e-12, n_nodes)
    o = OracleFEM(1e-12, 1e-12, n_nodes)
    _add_element(g, case)
    _add_element(o, case)
    g.assemble()
    rp, ci, va = g.stiffness_csr()
    rp_o, ci_o, va_o = o.csr()
    np.testing.assert_array_equal(rp, rp_o)
    np.testing.assert_array_equal(ci, ci_o)
    np.testing.assert_array_equal(va.view(np.uint64), va_o.view(np.uint64))
    K = _dense(rp, ci, va, 6 * n_nodes)
    if case["kind"] == "truss":  # the golden truss matrix is over the translations of its two nodes
        dofs = [0, 1, 2, 6, 7, 8]
        K = K[np.ix_(dofs, dofs)]
    ref = np.array([float(v) for v in case["matrix"]]).reshape(case["shape"])
    assert np.abs(K - ref).max() / np.abs(ref).max() < GOLDEN_REL, case["name"]
    # the reference's exact zeros are exact zeros (and absent from the pattern) on the GPU
    np.testing.assert_array_equal(K[ref == 0.0], 0.0)
    g.close()


def _compare(g, o):
    rp_g, ci_g, va_g = g.stiffness_csr()
    rp_o, ci_o, va_o = o.csr()
    np.testing.assert_array_equal(rp_g, rp_o)
    np.testing.assert_array_equal(ci_g, ci_o)
    np.testing.assert_array_equal(va_g.view(np.uint64), va_o.view(np.uint64))
    for a, b in zip(g.groups(), o.groups()):
        np.testing.assert_array_equal(a, b)
    return len(va_o)


def _branch_frame(nx, ny, nz, jitter, seed):
    """a beam frame whose sections cover every principal-axes case: I12 = 0 (the fast path), I12 != 0 with
    I11 > I22 and I11 < I22 (the axes loop turns), and I11 = I22 with I12 != 0 (the perturbation); with
    jitter = 0 every second x member runs from its +x node to its -x node, exactly anti-parallel to +x."""
    m = meshes.beam_frame(nx, ny, nz, jitter=jitter, seed=seed)
    b = m.beams
    rng = np.random.default_rng(seed + 100)
    k = len(b["numbers"])
    i12 = np.zeros(k)
    sel = np.arange(k) % 3 != 0
    i12[sel] = rng.uniform(-0.4, 0.4, sel.sum()) * np.minimum(b["i11"][sel], b["i22"][sel])
    b["i12"] = i12
    eq = np.arange(k) % 5 == 1
    b["i22"][eq] = b["i11"][eq]
    if jitter == 0.0:
        n_x = (nx - 1) * ny * nz
        flip = np.arange(k) < n_x
        flip &= np.arange(k) % 2 == 0
        b["nodes"][flip] = b["nodes"][flip][:, ::-1]
    return m


def test_beam_frame_branch_cases():
    m = _branch_frame(9, 8, 5, jitter=0.1, seed=61)
    g = FEM(1e-12, 1e-12, m.nodes_number)
    o = OracleFEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g, m)
    meshes.load(o, m)
    g.assemble()
    assert _compare(g, o) > 0
    g.close()


def test_beam_frame_antiparallel_members():
    m = _branch_frame(7, 6, 4, jitter=0.0, seed=62)
    d = m.xyz[m.beams["nodes"][:, 1] - 1] - m.xyz[m.beams["nodes"][:, 0] - 1]
    anti = (d[:, 0] < 0) & (d[:, 1] == 0) & (d[:, 2] == 0)
    assert anti.sum() > 50  # exactly anti-parallel to the rotation's target +x
    g = FEM(1e-12, 1e-12, m.nodes_number)
    o = OracleFEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g, m)
    meshes.load(o, m)
    g.assemble()
    _compare(g, o)
    # rotation getters on the half-turn branch
    for num in m.beams["numbers"][anti][:20]:
        from oracle import fem_oracle as fo

        k = int(num) - 1
        n1, n2 = m.beams["nodes"][k] - 1
        ref, _, _ = fo.beam_rotation(m.xyz[n1], m.xyz[n2], m.beams["i11"][k], m.beams["i22"][k],
                                     m.beams["i12"][k], m.beams["axis"][k])
        np.testing.assert_array_equal(g.get_beam_rotation_matrix_elements(int(num)), ref.ravel())
    g.close()


def test_truss_lattice_antiparallel_members():
    """an unjittered lattice whose x bars alternate direction (the half-turn of the truss rotation)."""
    m = meshes.truss_lattice(6, jitter=0.0, seed=63)
    t = m.trusses
    d = m.xyz[t["nodes"][:, 1] - 1] - m.xyz[t["nodes"][:, 0] - 1]
    xbar = (d[:, 1] == 0) & (d[:, 2] == 0)
    flip = xbar & (np.arange(len(d)) % 2 == 0)
    t["nodes"][flip] = t["nodes"][flip][:, ::-1]
    t["area_2"] = np.where(np.arange(len(d)) % 3 == 0, t["area"] * 0.5, np.nan)
    g = FEM(1e-12, 1e-12, m.nodes_number)
    o = OracleFEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g, m)
    meshes.load(o, m)
    g.assemble()
    _compare(g, o)
    from oracle import fem_oracle as fo

    for k in np.flatnonzero(flip)[:10]:
        n1, n2 = t["nodes"][k] - 1
        np.testing.assert_array_equal(g.get_truss_rotation_matrix_elements(int(t["numbers"][k])),
                                      fo.truss_rotation(m.xyz[n1], m.xyz[n2]).ravel())
    g.close()
