"""GPU parity: the CUDA assembly (through the C ABI) against the CPU oracle on
the same seeded meshes.  The CSR pattern, DOF map and stiffness groups must be
bit-exact; the values are compared at the 1e-12 relative bound and, because
both sides follow one evaluation order, are also expected bit-identical."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle.fem_oracle import OracleError, OracleFEM

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # values: max over nnz of |gpu - oracle| / |oracle|


def build_pair(mesh, rel_tol=1e-12, abs_tol=1e-12):
    g = FEM(rel_tol, abs_tol, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    o = OracleFEM(rel_tol, abs_tol, mesh.nodes_number)
    meshes.load(o, mesh)
    return g, o


def compare(g, o, groups=True):
    rp_g, ci_g, va_g = g.stiffness_csr()
    rp_o, ci_o, va_o = o.csr()
    np.testing.assert_array_equal(rp_g, rp_o)
    np.testing.assert_array_equal(ci_g, ci_o)
    nz = va_o != 0
    rel = np.abs(va_g - va_o)[nz] / np.abs(va_o[nz])
    assert (rel.max() if rel.size else 0.0) <= REL_TOL
    np.testing.assert_array_equal(va_g[~nz], va_o[~nz])
    # one evaluation order on both sides: bit-identical
    np.testing.assert_array_equal(va_g.view(np.uint64), va_o.view(np.uint64))
    np.testing.assert_array_equal(g.index_node_numbers(), o.index_node_numbers())
    if groups:
        for a, b in zip(g.groups(), o.groups()):
            np.testing.assert_array_equal(a, b)
    return len(va_o)


def test_truss_lattice_full_config():
    """11 x 11 x 11 lattice, 4630 bars (the CPU-runnable workload at full size)."""
    m = meshes.truss_lattice()
    assert m.counts() == (4630, 0, 0)
    g, o = build_pair(m)
    nnz = compare(g, o)
    assert nnz > 0


def test_beam_frame_small():
    m = meshes.beam_frame(9, 7, 5)
    g, o = build_pair(m)
    compare(g, o)


def test_plate_mesh_small():
    m = meshes.plate_mesh(37, 23)
    g, o = build_pair(m)
    compare(g, o)


def test_plate_mesh_tilted():
    """general rotation: the whole distorted mesh tilted out of z = 0."""
    q, _ = np.linalg.qr(np.random.default_rng(7).normal(size=(3, 3)))
    m = meshes.plate_mesh(20, 17, size=3.0, rotation=q)
    g, o = build_pair(m, abs_tol=1e-9)
    compare(g, o)


def test_adjoint_model_small():
    m = meshes.adjoint_model(frame=(6, 5, 3), slab=(50, 40))
    g, o = build_pair(m)
    compare(g, o)


def test_interleaved_kinds_and_call_order():
    """elements of all kinds added in several interleaved calls sharing nodes: the per-entry
    sums run in element call order across kinds, as the reference's eager accumulation."""
    rng = np.random.default_rng(21)
    fr = meshes.beam_frame(5, 5, 3, spacing=1.0, seed=9)
    n = fr.nodes_number
    b = fr.beams
    parts = np.array_split(np.arange(len(b["numbers"])), 3)
    # trusses on body diagonals of the first storey's cells
    tr_nodes = np.array([[1 + i + 5 * j, 1 + (i + 1) + 5 * (j + 1) + 25] for i in range(4) for j in range(4)],
                        np.uint32)
    areas = rng.uniform(1e-4, 5e-4, 8)
    # a planar plate patch on nine extra nodes, two of its quads sharing frame-free nodes only
    extra_xyz = np.array([[10.0 + x, 10.0 + y, 0.0] for y in range(3) for x in range(3)])
    pl_nodes = np.array([[n + 5, n + 4, n + 1, n + 2], [n + 6, n + 5, n + 2, n + 3], [n + 8, n + 7, n + 4, n + 5],
                         [n + 9, n + 8, n + 5, n + 6]], np.uint32)
    g, o = FEM(1e-12, 1e-12, n + 9), OracleFEM(1e-12, 1e-12, n + 9)

    def beams(model, sel):
        model.add_beams(b["numbers"][sel], b["nodes"][sel], b["young"][sel], b["poisson"][sel], b["area"][sel],
                        b["i11"][sel], b["i22"][sel], b["i12"][sel], b["it"][sel], b["shear_factor"][sel],
                        b["axis"][sel])

    for model in (g, o):
        model.add_nodes(fr.node_numbers, fr.xyz)
        model.add_nodes(np.arange(n + 1, n + 10), extra_xyz)
        beams(model, parts[0])
        model.add_trusses(np.arange(1, 9), tr_nodes[:8], 200e9, areas)
        model.add_plates([1, 2], pl_nodes[:2], 70e9, 0.3, [0.02, 0.03], 5 / 6)
        beams(model, parts[1])
        model.add_trusses(np.arange(9, 17), tr_nodes[8:], 200e9, areas, area_2=areas * 0.5)
        model.add_plates([3, 4], pl_nodes[2:], 70e9, 0.3, [0.025, 0.01], 5 / 6)
        beams(model, parts[2])
    g.assemble()
    compare(g, o)


def test_determinism_and_reassembly():
    m = meshes.plate_mesh(30, 30)
    g, o = build_pair(m)
    v1 = g.stiffness_values().copy()
    for _ in range(3):
        g.assemble_numeric_async()
    g.check_pattern()
    v2 = g.stiffness_values()
    np.testing.assert_array_equal(v1.view(np.uint64), v2.view(np.uint64))


def test_additions_after_assembly():
    """assemble, add more elements (a bulk call, a rejected call, single calls), assemble again: the numeric
    pass (replayed as a graph between symbolic phases) sees the new and moved arrays"""
    m = meshes.plate_mesh(40, 40, size=4.0)
    half = len(m.plates["numbers"]) // 2
    g = FEM(1e-12, 1e-12, m.nodes_number)
    o = OracleFEM(1e-12, 1e-12, m.nodes_number)
    p = m.plates
    for x in (g, o):
        x.add_nodes(m.node_numbers, m.xyz)
        x.add_plates(p["numbers"][:half], p["nodes"][:half], p["young"][:half], p["poisson"][:half],
                     p["thickness"][:half], p["shear_factor"][:half])
    g.assemble()
    for _ in range(2):
        g.assemble_numeric_async()
    g.check_pattern()
    for x in (g, o):
        x.add_plates(p["numbers"][half:], p["nodes"][half:], p["young"][half:], p["poisson"][half:],
                     p["thickness"][half:], p["shear_factor"][half:])
        with pytest.raises((FEMError, OracleError)):  # every plate rejected (numbers taken)
            x.add_plates(p["numbers"][:3], p["nodes"][:3], p["young"][:3], p["poisson"][:3], p["thickness"][:3],
                         p["shear_factor"][:3])
        x.add_truss(10 ** 6, 1, 41 * 41, 200e9, 3e-4)
    g.assemble()
    compare(g, o)
    g.assemble_numeric_async()
    g.check_pattern()
    compare(g, o)


def test_coordinate_update_reuses_or_rebuilds_pattern():
    """new coordinates (same topology): the next assemble equals a fresh oracle build on them."""
    m = meshes.beam_frame(6, 6, 4, seed=31)
    g = FEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    m2 = meshes.beam_frame(6, 6, 4, seed=32)
    g.set_node_coordinates(m2.xyz)
    g.assemble()
    o = OracleFEM(1e-12, 1e-12, m.nodes_number)
    m2.beams = m.beams
    meshes.load(o, m2)
    compare(g, o)


def test_rotation_getters_match_oracle():
    m = meshes.adjoint_model(frame=(4, 4, 3), slab=(30, 30))
    g, o = build_pair(m)
    from oracle import fem_oracle as fo

    xyz = m.xyz
    b = m.beams
    for k in range(0, len(b["numbers"]), 7):
        n1, n2 = b["nodes"][k] - 1
        ref, _, _ = fo.beam_rotation(xyz[n1], xyz[n2], b["i11"][k], b["i22"][k], b["i12"][k], b["axis"][k])
        np.testing.assert_array_equal(g.get_beam_rotation_matrix_elements(int(b["numbers"][k])), ref.ravel())
    p = m.plates
    for k in range(0, len(p["numbers"]), 97):
        i = p["nodes"][k] - 1
        ref = fo.plate_rotation(xyz[i[1]], xyz[i[2]], xyz[i[3]])
        np.testing.assert_array_equal(g.get_plate_rotation_matrix_elements(int(p["numbers"][k])), ref.ravel())
    with pytest.raises(FEMError):
        g.get_truss_rotation_matrix_elements(1)


def test_validation_matches_oracle():
    """the same inputs fail with the same code and message on both sides, and leave the model unchanged."""
    g, o = FEM(1e-12, 1e-12, 8), OracleFEM(1e-12, 1e-12, 8)
    calls = [
        ("add_node", (1, 0.0, 0.0, 0.0)), ("add_node", (2, 1.0, 0.0, 0.0)), ("add_node", (3, 1.0, 1.0, 0.0)),
        ("add_node", (4, 0.0, 1.0, 0.0)), ("add_node", (1, 5.0, 5.0, 5.0)), ("add_node", (9, 1.0, 1.0, 0.0)),
        ("add_truss", (1, 1, 7, 1.0, 1.0)), ("add_truss", (1, 1, 2, -1.0, 1.0)), ("add_truss", (1, 1, 2, 1.0, 0.0)),
        ("add_truss", (1, 1, 2, 200e9, 1e-4)), ("add_truss", (1, 3, 4, 1.0, 1.0)), ("add_truss", (2, 2, 1, 1.0, 1.0)),
        ("add_beam", (5, 1, 2, 1.0, 0.3, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0, [1.0, 0.0, 0.0])),
        ("add_beam", (5, 1, 3, 1.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0, 1.0, [0.0, 0.0, 1.0])),
        ("add_beam", (5, 1, 3, 210e9, 0.3, 1e-2, 1e-5, 2e-5, 0.0, 1e-6, 5 / 6, [0.0, 0.0, 1.0])),
        ("add_node", (5, 0.4, 0.6, 0.0)), ("add_plate", (3, 3, 4, 1, 5, 1.0, 0.3, 0.1, 1.0)),
        ("add_node", (6, 0.5, 0.5, 1.0)), ("add_plate", (4, 6, 4, 1, 2, 1.0, 0.3, 0.1, 1.0)),
        ("add_node", (7, 2.0, 2.0, 0.0)), ("add_plate", (4, 3, 7, 1, 2, 1.0, 0.3, 0.1, 1.0)),
        ("add_plate", (4, 3, 4, 1, 2, 1.0, 0.3, -0.1, 1.0)),
        ("add_plate", (4, 3, 4, 1, 2, 70e9, 0.3, 0.02, 5 / 6)), ("add_plate", (5, 2, 1, 4, 3, 70e9, 0.3, 0.02, 5 / 6)),
        ("add_node", (8, 3.0, 3.0, 3.0)), ("add_node", (10, 4.0, 3.0, 3.0)),
    ]
    for name, args in calls:
        errs = []
        for model, exc in ((g, FEMError), (o, OracleError)):
            try:
                getattr(model, name)(*args)
                errs.append(None)
            except exc as e:
                errs.append((e.code, str(e)))
        assert errs[0] == errs[1], (name, args, errs)
    g.assemble()
    compare(g, o)


def test_bulk_add_stops_at_first_failure():
    """a bulk call adds the elements before the first failing one, like repeated add_* calls."""
    m = meshes.plate_mesh(6, 5)
    p = m.plates
    th = p["thickness"].copy()
    th[17] = 0.0
    g, o = FEM(1e-12, 1e-12, m.nodes_number), OracleFEM(1e-12, 1e-12, m.nodes_number)
    res = []
    for model, exc in ((g, FEMError), (o, OracleError)):
        model.add_nodes(m.node_numbers, m.xyz)
        with pytest.raises(exc) as ei:
            model.add_plates(p["numbers"], p["nodes"], p["young"], p["poisson"], th, p["shear_factor"])
        res.append((ei.value.code, str(ei.value)))
    assert res[0] == res[1]
    assert g.element_counts() == (0, 0, 17)
    g.assemble()
    compare(g, o)


@pytest.mark.slow
def test_beam_frame_full_config():
    """101 x 101 x 21 frame, 628,220 beams, against the oracle at full size."""
    m = meshes.beam_frame()
    assert m.counts() == (0, 628220, 0)
    g, o = build_pair(m)
    nnz = compare(g, o, groups=False)
    assert nnz == 52943728


@pytest.mark.slow
def test_plate_mesh_full_config():
    """1000 x 1000 distorted plates, 1M elements, against the oracle at full size."""
    m = meshes.plate_mesh()
    g, o = build_pair(m)
    nnz = compare(g, o, groups=False)
    assert nnz == 118080014
    # size-independent property: the assembled matrix is exactly symmetric
    rp, ci, va = g.stiffness_csr()
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    order = np.lexsort((rows, ci))
    np.testing.assert_array_equal(ci[order], rows)
    np.testing.assert_array_equal(va[order].view(np.uint64), va.view(np.uint64))


def test_hub_node_many_contributions():
    """a hub node shared by 400 trusses and 300 beams: its diagonal block sums 700 contributions
    (a reduction tile too large to stage in shared memory takes the global-memory path)."""
    rng = np.random.default_rng(5)
    n_spokes = 700
    ang = rng.uniform(0, 2 * np.pi, n_spokes)
    el = rng.uniform(-1.2, 1.2, n_spokes)
    r = rng.uniform(1.0, 3.0, n_spokes)
    xyz = np.concatenate([[[0.0, 0.0, 0.0]], np.stack([r * np.cos(ang) * np.cos(el), r * np.sin(ang) * np.cos(el),
                                                        r * np.sin(el)], 1)])
    n = len(xyz)
    spokes = np.stack([np.ones(n_spokes, np.uint32), np.arange(2, n + 1, dtype=np.uint32)], 1)
    g, o = FEM(1e-12, 1e-12, n), OracleFEM(1e-12, 1e-12, n)
    areas = rng.uniform(1e-4, 5e-4, 400)
    m = n_spokes - 400
    for model in (g, o):
        model.add_nodes(np.arange(1, n + 1), xyz)
        model.add_trusses(np.arange(1, 401), spokes[:400], 200e9, areas)
        model.add_beams(np.arange(1, m + 1), spokes[400:], 210e9, 0.3, 1e-2, 5e-5, 3e-5, 0.0, 1e-5, 5 / 6,
                        [0.3, 0.2, 1.0])
    g.assemble()
    compare(g, o)


def test_batch_matches_each_model():
    """several structures of every kind assembled in one batch pass: each structure's values equal its own
    assembly bit for bit, for the default and for the autotuned launch configuration."""
    from finite_element_method_gb300 import Batch

    structures = meshes.batch_structures(9, lo=200, hi=3000, seed=8)
    models, refs = [], []
    for m in structures:
        g = FEM(meshes.REL_TOL, meshes.ABS_TOL, m.nodes_number)
        meshes.load(g, m)
        g.assemble()
        models.append(g)
        refs.append(g.stiffness_values().copy())
    b = Batch(models)
    b.assemble()
    for i, r in enumerate(refs):
        np.testing.assert_array_equal(b.values(i).view(np.uint64), r.view(np.uint64))
    table = b.autotune(reps=2)
    assert table["best_ms"] > 0 and len(table["candidates"]) >= 10
    b.assemble()
    for i, r in enumerate(refs):
        np.testing.assert_array_equal(b.values(i).view(np.uint64), r.view(np.uint64))
    # against the oracle for two of them
    for i in (0, len(structures) - 1):
        o = OracleFEM(meshes.REL_TOL, meshes.ABS_TOL, structures[i].nodes_number)
        meshes.load(o, structures[i])
        _, _, va = o.csr()
        np.testing.assert_array_equal(b.values(i).view(np.uint64), va.view(np.uint64))
    b.close()


@pytest.mark.parametrize("name", ["plate", "frame_slab", "truss", "tiny"])
def test_assemble_to_host_fresh_pattern(name):
    """A first assemble_to_host on a new model: row_ptr goes back once the rows are counted and the
    columns in node chunks as the row fill finishes each, during the symbolic phase; the host arrays
    hold the CSR of assemble() + stiffness_csr() and nothing past nnz is written."""
    m = {"plate": lambda: meshes.plate_mesh(60, 45, size=5.0),
         "frame_slab": lambda: meshes.adjoint_model(frame=(5, 4, 3), slab=(40, 30)),
         "truss": lambda: meshes.truss_lattice(5),
         "tiny": lambda: meshes.plate_mesh(1, 1, size=1.0)}[name]()
    g, _ = build_pair(m)
    rp0, ci0, va0 = g.stiffness_csr()
    g.close()
    g2 = FEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g2, m)
    rp = np.full(6 * m.nodes_number + 1, -1, np.int64)
    ci = np.full(len(ci0) + 3, -1, np.int32)
    va = np.full(len(va0) + 3, np.nan)
    nnz = g2.assemble_to_host(rp, ci, va)
    assert nnz == len(ci0)
    np.testing.assert_array_equal(rp, rp0)
    np.testing.assert_array_equal(ci[:nnz], ci0)
    np.testing.assert_array_equal(va[:nnz].view(np.uint64), va0.view(np.uint64))
    assert (ci[nnz:] == -1).all() and np.isnan(va[nnz:]).all()
    g2.close()


def test_assemble_to_host_after_pattern_change():
    """Nodes moved so that the exact-zero pattern changes (a flat mesh turned off the global planes): the
    kept pattern's pass finds it changed, the symbolic phase runs again inside the same call and sends
    the new pattern back while it runs; the host arrays hold the oracle's CSR of the moved mesh."""
    q, _ = np.linalg.qr(np.random.default_rng(11).normal(size=(3, 3)))
    flat = meshes.plate_mesh(30, 20, size=4.0)
    tilted = meshes.plate_mesh(30, 20, size=4.0, rotation=q)
    g = FEM(1e-12, 1e-12, flat.nodes_number)
    meshes.load(g, flat)
    o = OracleFEM(1e-12, 1e-12, tilted.nodes_number)
    meshes.load(o, tilted)
    rp0, ci0, va0 = o.csr()
    rp = np.zeros(6 * flat.nodes_number + 1, np.int64)
    ci = np.zeros(len(ci0) + 7, np.int32)
    va = np.zeros(len(va0) + 7, np.float64)
    nnz_flat = g.assemble_to_host(rp, ci, va)
    assert nnz_flat < len(ci0)  # packed blocks in the plane
    g.set_node_coordinates(tilted.xyz)
    nnz = g.assemble_to_host(rp, ci, va)
    assert nnz == len(ci0)
    np.testing.assert_array_equal(rp, rp0)
    np.testing.assert_array_equal(ci[:nnz], ci0)
    np.testing.assert_array_equal(va[:nnz].view(np.uint64), va0.view(np.uint64))
    g.close()


def test_assemble_to_host_matches_assemble():
    m = meshes.plate_mesh(50, 40, size=5.0)
    g, o = build_pair(m)
    rp0, ci0, va0 = g.stiffness_csr()
    g2 = FEM(1e-12, 1e-12, m.nodes_number)
    meshes.load(g2, m)
    rp = np.zeros(6 * m.nodes_number + 1, np.int64)
    ci = np.zeros(len(ci0) - 1, np.int32)
    va = np.zeros(len(va0) - 1, np.float64)
    with pytest.raises(FEMError, match="entries"):  # one entry short
        g2.assemble_to_host(rp, ci, va)
    ci = np.zeros(len(ci0) + 5, np.int32)
    va = np.full(len(va0) + 5, np.nan)
    for _ in range(2):  # fresh pattern, then the kept one
        nnz = g2.assemble_to_host(rp, ci, va)
        assert nnz == len(ci0)
        np.testing.assert_array_equal(rp, rp0)
        np.testing.assert_array_equal(ci[:nnz], ci0)
        np.testing.assert_array_equal(va[:nnz].view(np.uint64), va0.view(np.uint64))
    g2.close()
