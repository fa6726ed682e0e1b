"""The seeded synthetic workloads at their full sizes (CPU): element and node counts of the five
configurations, the value ranges of the properties, and the geometric conditions the reference's checks
impose on them (distinct node pairs, a beam local axis that is not along the member, flat, convex and
counter-clockwise plates with the node order of structs/plate.rs:1244-1249), so that every element of a
bench workload passes the reference's validation."""
import numpy as np
import pytest

from finite_element_method_gb300 import meshes


def _pairs_distinct(nodes):
    lo, hi = np.minimum(nodes[:, 0], nodes[:, 1]), np.maximum(nodes[:, 0], nodes[:, 1])
    assert np.all(lo != hi)
    key = lo.astype(np.uint64) << np.uint64(32) | hi.astype(np.uint64)
    assert len(np.unique(key)) == len(key)


def _numbering(mesh, kind):
    n = mesh.nodes_number
    assert np.array_equal(mesh.node_numbers, np.arange(1, n + 1, dtype=np.uint32))
    d = getattr(mesh, kind)
    assert np.array_equal(d["numbers"], np.arange(1, len(d["numbers"]) + 1, dtype=np.uint32))
    assert d["nodes"].min() >= 1 and d["nodes"].max() <= n


def test_truss_lattice_4630_bars():
    m = meshes.truss_lattice()
    assert (m.nodes_number, m.counts()) == (1331, (4630, 0, 0))
    _numbering(m, "trusses")
    _pairs_distinct(m.trusses["nodes"].astype(np.int64))
    a = m.trusses["area"]
    assert a.min() >= 1e-4 and a.max() <= 5e-4 and np.all(m.trusses["young"] == 200e9)
    kk, jj, ii = np.meshgrid(np.arange(11), np.arange(11), np.arange(11), indexing="ij")  # x fastest
    grid = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], -1) * 1.0
    assert np.abs(m.xyz - grid).max() <= 0.05 + 1e-12


def test_beam_frame_628220_beams():
    m = meshes.beam_frame()
    assert (m.nodes_number, m.counts()) == (214221, (0, 628220, 0))
    _numbering(m, "beams")
    b = m.beams
    nodes = b["nodes"].astype(np.int64) - 1
    _pairs_distinct(nodes)
    for k, lo, hi in (("area", 5e-3, 2e-2), ("i11", 1e-5, 1e-4), ("i22", 1e-5, 1e-4), ("it", 1e-6, 5e-5)):
        assert b[k].min() >= lo and b[k].max() <= hi
    assert np.all(b["i12"] == 0) and np.all(b["young"] == 210e9) and np.all(b["poisson"] == 0.3)
    # the local axis 1 is never along the member (the reference rejects a parallel axis)
    d = m.xyz[nodes[:, 1]] - m.xyz[nodes[:, 0]]
    d /= np.linalg.norm(d, axis=1)[:, None]
    assert np.abs(np.einsum("ij,ij->i", d, b["axis"])).max() < 0.2


def _plate_checks(xyz, quads):
    p = xyz[quads]  # (m, 4, 3)
    assert np.all(p[..., 2] == p[:, :1, 2])  # flat
    e = np.roll(p, -1, axis=1) - p
    cross_z = e[..., 0] * np.roll(e, -1, axis=1)[..., 1] - e[..., 1] * np.roll(e, -1, axis=1)[..., 0]
    assert cross_z.min() > 0  # every corner turns left: convex and counter-clockwise
    # node 1 at (+x, +y), 2 at (-x, +y), 3 at (-x, -y), 4 at (+x, -y) of the element
    assert np.all(p[:, 0, 0] > p[:, 1, 0]) and np.all(p[:, 3, 0] > p[:, 2, 0])
    assert np.all(p[:, 0, 1] > p[:, 3, 1]) and np.all(p[:, 1, 1] > p[:, 2, 1])


def test_plate_mesh_one_million_plates():
    m = meshes.plate_mesh()
    assert (m.nodes_number, m.counts()) == (1002001, (0, 0, 1000000))
    _numbering(m, "plates")
    _plate_checks(m.xyz, m.plates["nodes"].astype(np.int64) - 1)
    t = m.plates["thickness"]
    assert t.min() >= 0.01 and t.max() <= 0.03
    # boundary nodes stay on the 100 m square, interior ones move at most 20 % of the 0.1 m element
    grid = np.stack(np.meshgrid(np.arange(1001) * 0.1, np.arange(1001) * 0.1, indexing="xy"), -1).reshape(-1, 2)
    assert np.abs(m.xyz[:, :2] - grid).max() <= 0.2 * 0.1 + 1e-12
    edge = (grid[:, 0] == 0) | (grid[:, 1] == 0) | np.isclose(grid[:, 0], 100.0) | np.isclose(grid[:, 1], 100.0)
    assert np.array_equal(m.xyz[edge, :2], grid[edge])


def test_adjoint_model_frame_and_slab_share_the_top_storey():
    m = meshes.adjoint_model()
    assert m.counts() == (0, 82110, 250000)
    assert m.nodes_number == 28611 + 251001 - 51 * 51
    quads = m.plates["nodes"].astype(np.int64) - 1
    _plate_checks(m.xyz, quads)
    top = np.arange(51 * 51) + 51 * 51 * 10
    assert np.isin(top, quads).all()  # every top-storey frame node carries slab plates
    assert np.all(m.xyz[quads, 2] == 30.0)


def test_batch_512_structures_log_uniform():
    b = meshes.batch_structures()
    assert len(b) == 512
    sizes = np.array([s.n_elements for s in b])
    assert sizes.sum() == 21708538
    assert sizes.min() >= 1e3 * 0.9 and sizes.max() <= 2e5 * 1.1
    assert {s.name.split("_")[0] for s in b} == {"truss", "beam", "plate"}


@pytest.mark.parametrize("gen", [meshes.truss_lattice, lambda: meshes.plate_mesh(40, 30)])
def test_generators_are_deterministic(gen):
    a, b = gen(), gen()
    assert np.array_equal(a.xyz.view(np.uint64), b.xyz.view(np.uint64))
