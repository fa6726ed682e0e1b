"""Seeded synthetic meshes for the assembly workloads.

No public mesh set exists for this path; these generators produce the
workloads with their stated sizes and value distributions from numpy's PCG64
generator, so the same seed gives the same bits on every machine.

  truss_lattice  11 x 11 x 11 nodes at 1.0 m, jitter U[-0.05, 0.05] m, bars on
                 x/y/z grid neighbours + one body diagonal per cell (4630 bars),
                 A ~ U[1e-4, 5e-4] m^2, E = 200e9 Pa.
  beam_frame     101 x 101 x 21 nodes at 3.0 m, jitter U[-0.1, 0.1] m, beams on
                 x/y/z grid neighbours (628,220 beams), A ~ U[5e-3, 2e-2],
                 I11 (Iy), I22 (Iz) ~ U[1e-5, 1e-4], I12 = 0, It (J) ~ U[1e-6, 5e-5],
                 E = 210e9, nu = 0.3, shear factor 5/6; local axis 1 = +z, or
                 +x for vertical members.
  plate_mesh     1000 x 1000 quads on 100 m x 100 m in z = 0, interior nodes
                 jittered U[-0.2 h, 0.2 h] in x and y (h = element size),
                 t ~ U[0.01, 0.03] m, E = 70e9, nu = 0.3, shear factor 5/6; nodes
                 of each quad counter-clockwise from the (+x, +y) corner
                 (the order of structs/plate.rs:1244-1249).
  batch          512 independent structures, element counts log-uniform in
                 [1e3, 2e5], kind drawn per structure among the three above.
  adjoint_model  a 51 x 51 x 11 beam frame and a 500 x 500 plate slab whose
                 nodes coincide with the frame's top storey on every 10th slab
                 node.

Node numbers are 1..N in lexicographic order (x fastest); element numbers are
1..E in call order.  `load(model, mesh)` feeds a mesh to anything with the
reference's add_* API (the GPU `FEM` or the CPU oracle).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SHEAR_FACTOR = 5.0 / 6.0
REL_TOL = 1e-12
ABS_TOL = 1e-12


@dataclass
class Mesh:
    name: str
    node_numbers: np.ndarray  # uint32 [N]
    xyz: np.ndarray  # float64 [N, 3]
    trusses: dict | None = None  # numbers, nodes [m,2], young, area, area_2 (or None)
    beams: dict | None = None  # numbers, nodes [m,2], young, poisson, area, i11, i22, i12, it, shear_factor, axis [m,3]
    plates: dict | None = None  # numbers, nodes [m,4], young, poisson, thickness, shear_factor
    order: tuple = ("trusses", "beams", "plates")
    meta: dict = field(default_factory=dict)

    @property
    def nodes_number(self) -> int:
        return int(len(self.node_numbers))

    def counts(self):
        f = lambda d: 0 if d is None else int(len(d["numbers"]))
        return f(self.trusses), f(self.beams), f(self.plates)

    @property
    def n_elements(self) -> int:
        return sum(self.counts())


def _grid_nodes(nx, ny, nz, spacing, jitter, rng, jitter_z=True):
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # lexicographic with x fastest: index = i + nx * (j + ny * k)
    idx = (ii + nx * (jj + ny * kk)).ravel()
    xyz = np.zeros((nx * ny * nz, 3))
    xyz[idx, 0] = ii.ravel() * spacing
    xyz[idx, 1] = jj.ravel() * spacing
    xyz[idx, 2] = kk.ravel() * spacing
    j = rng.uniform(-jitter, jitter, size=xyz.shape)
    if not jitter_z:
        j[:, 2] = 0.0
    xyz += j
    return xyz


def _grid_edges(nx, ny, nz, diagonals=False):
    """node-index pairs of grid neighbours (x, then y, then z), then body diagonals."""
    node = lambda i, j, k: i + nx * (j + ny * k)
    out = []
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx - 1), indexing="ij")
    out.append(np.stack([node(i, j, k), node(i + 1, j, k)], -1).reshape(-1, 2))
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny - 1), np.arange(nx), indexing="ij")
    out.append(np.stack([node(i, j, k), node(i, j + 1, k)], -1).reshape(-1, 2))
    k, j, i = np.meshgrid(np.arange(nz - 1), np.arange(ny), np.arange(nx), indexing="ij")
    out.append(np.stack([node(i, j, k), node(i, j, k + 1)], -1).reshape(-1, 2))
    if diagonals:
        k, j, i = np.meshgrid(np.arange(nz - 1), np.arange(ny - 1), np.arange(nx - 1), indexing="ij")
        out.append(np.stack([node(i, j, k), node(i + 1, j + 1, k + 1)], -1).reshape(-1, 2))
    return np.concatenate(out).astype(np.int64)


def truss_lattice(n=11, spacing=1.0, jitter=0.05, seed=1, young=200e9, area_range=(1e-4, 5e-4)) -> Mesh:
    rng = np.random.default_rng(seed)
    xyz = _grid_nodes(n, n, n, spacing, jitter, rng)
    e = _grid_edges(n, n, n, diagonals=True)
    m = len(e)
    numbers = np.arange(1, len(xyz) + 1, dtype=np.uint32)
    trusses = dict(numbers=np.arange(1, m + 1, dtype=np.uint32), nodes=(e + 1).astype(np.uint32),
                   young=np.full(m, young), area=rng.uniform(*area_range, size=m), area_2=None)
    return Mesh("truss_lattice", numbers, xyz, trusses=trusses, meta=dict(n=n, seed=seed))


def beam_frame(nx=101, ny=101, nz=21, spacing=3.0, jitter=0.1, seed=2, young=210e9, poisson=0.3,
               jitter_top=True) -> Mesh:
    rng = np.random.default_rng(seed)
    xyz = _grid_nodes(nx, ny, nz, spacing, jitter, rng)
    if not jitter_top:  # keep the top storey exactly planar (a slab is attached there)
        top = np.arange(nx * ny) + nx * ny * (nz - 1)
        xyz[top, 2] = (nz - 1) * spacing
    e = _grid_edges(nx, ny, nz)
    m = len(e)
    n_vertical = nx * ny * (nz - 1)
    axis = np.zeros((m, 3))
    axis[:, 2] = 1.0
    axis[m - n_vertical:] = (1.0, 0.0, 0.0)
    beams = dict(numbers=np.arange(1, m + 1, dtype=np.uint32), nodes=(e + 1).astype(np.uint32),
                 young=np.full(m, young), poisson=np.full(m, poisson), area=rng.uniform(5e-3, 2e-2, size=m),
                 i11=rng.uniform(1e-5, 1e-4, size=m), i22=rng.uniform(1e-5, 1e-4, size=m), i12=np.zeros(m),
                 it=rng.uniform(1e-6, 5e-5, size=m), shear_factor=np.full(m, SHEAR_FACTOR), axis=axis)
    numbers = np.arange(1, len(xyz) + 1, dtype=np.uint32)
    return Mesh("beam_frame", numbers, xyz, beams=beams, meta=dict(nx=nx, ny=ny, nz=nz, seed=seed))


def _plate_grid(nx, ny, size_x, size_y, jitter_frac, rng):
    hx, hy = size_x / nx, size_y / ny
    ii, jj = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")  # rows: j, cols: i (x fastest)
    xyz = np.zeros(((nx + 1) * (ny + 1), 3))
    xyz[:, 0] = (ii * hx).ravel()
    xyz[:, 1] = (jj * hy).ravel()
    interior = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)).ravel()
    jit = np.stack([rng.uniform(-jitter_frac * hx, jitter_frac * hx, size=len(xyz)),
                    rng.uniform(-jitter_frac * hy, jitter_frac * hy, size=len(xyz))], -1)
    xyz[interior, :2] += jit[interior]
    node = lambda i, j: i + (nx + 1) * j
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    quads = np.stack([node(i + 1, j + 1), node(i, j + 1), node(i, j), node(i + 1, j)], -1).reshape(-1, 4)
    return xyz, quads.astype(np.int64)


def plate_mesh(nx=1000, ny=1000, size=100.0, jitter_frac=0.2, seed=3, young=70e9, poisson=0.3,
               t_range=(0.01, 0.03), rotation=None) -> Mesh:
    """Flat distorted-quad plate mesh; `rotation` (3x3) tilts the whole mesh out of z = 0."""
    rng = np.random.default_rng(seed)
    xyz, quads = _plate_grid(nx, ny, size, size, jitter_frac, rng)
    if rotation is not None:
        xyz = xyz @ np.asarray(rotation, float).T
    m = len(quads)
    plates = dict(numbers=np.arange(1, m + 1, dtype=np.uint32), nodes=(quads + 1).astype(np.uint32),
                  young=np.full(m, young), poisson=np.full(m, poisson), thickness=rng.uniform(*t_range, size=m),
                  shear_factor=np.full(m, SHEAR_FACTOR))
    numbers = np.arange(1, len(xyz) + 1, dtype=np.uint32)
    return Mesh("plate_mesh", numbers, xyz, plates=plates, meta=dict(nx=nx, ny=ny, seed=seed))


def adjoint_model(frame=(51, 51, 11), slab=(500, 500), spacing=3.0, seed=5) -> Mesh:
    """Beam frame plus a plate slab on its top storey.

    The slab spans the frame's top storey with slab element size spacing/10,
    so every 10th slab node (in x and y) is a frame node; the top storey is
    left unjittered in z (the slab must stay planar), and slab nodes are not
    jittered.  Beams are added first, then plates."""
    nx, ny, nz = frame
    fr = beam_frame(nx, ny, nz, spacing=spacing, seed=seed, jitter_top=False)
    sx, sy = slab
    step = 10
    assert sx == (nx - 1) * step and sy == (ny - 1) * step, "slab must span the frame's top storey"
    h = spacing / step
    ii, jj = np.meshgrid(np.arange(sx + 1), np.arange(sy + 1), indexing="xy")
    sxyz = np.zeros(((sx + 1) * (sy + 1), 3))
    sxyz[:, 0] = (ii * h).ravel()
    sxyz[:, 1] = (jj * h).ravel()
    sxyz[:, 2] = (nz - 1) * spacing
    # slab node -> model node index: shared with the frame where both indices are multiples of step
    n_frame = fr.nodes_number
    shared = ((ii % step == 0) & (jj % step == 0)).ravel()
    top0 = nx * ny * (nz - 1)
    frame_idx = top0 + (ii // step + nx * (jj // step)).ravel()
    # frame node positions (x, y jittered) are used for the shared slab nodes
    own = np.flatnonzero(~shared)
    slab_to_model = np.empty(len(sxyz), np.int64)
    slab_to_model[shared] = frame_idx[shared]
    slab_to_model[own] = n_frame + np.arange(len(own))
    xyz = np.concatenate([fr.xyz, sxyz[own]])
    node = lambda i, j: i + (sx + 1) * j
    j, i = np.meshgrid(np.arange(sy), np.arange(sx), indexing="ij")
    quads = np.stack([node(i + 1, j + 1), node(i, j + 1), node(i, j), node(i + 1, j)], -1).reshape(-1, 4)
    quads = slab_to_model[quads]
    rng = np.random.default_rng(seed + 100)
    m = len(quads)
    plates = dict(numbers=np.arange(1, m + 1, dtype=np.uint32), nodes=(quads + 1).astype(np.uint32),
                  young=np.full(m, 30e9), poisson=np.full(m, 0.2), thickness=rng.uniform(0.15, 0.25, size=m),
                  shear_factor=np.full(m, SHEAR_FACTOR))
    numbers = np.arange(1, len(xyz) + 1, dtype=np.uint32)
    return Mesh("adjoint_model", numbers, xyz, beams=fr.beams, plates=plates,
                meta=dict(frame=frame, slab=slab, seed=seed))


def batch_structures(n_structures=512, lo=1e3, hi=2e5, seed=4, kinds=("truss", "beam", "plate")):
    """512 independent structures of log-uniform size; kind drawn per structure."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_structures))
    kind_idx = rng.integers(0, len(kinds), size=n_structures)
    out = []
    for s, (target, k) in enumerate(zip(sizes, kind_idx)):
        kind = kinds[k]
        sub_seed = int(rng.integers(0, 2**31 - 1))
        if kind == "plate":
            a = max(2, int(round(np.sqrt(target))))
            b = max(2, int(round(target / a)))
            m = plate_mesh(a, b, size=0.1 * max(a, b), seed=sub_seed)
        elif kind == "beam":
            # an n x n x nz frame with nz ~ n / 4: 2 n (n - 1) nz + n^2 (nz - 1) beams closest to the target
            cand = [(abs(2 * n * (n - 1) * max(2, n // 4) + n * n * (max(2, n // 4) - 1) - target), n)
                    for n in range(2, 400)]
            n = min(cand)[1]
            m = beam_frame(n, n, max(2, n // 4), seed=sub_seed)
        else:
            # an n^3 lattice: 3 n^2 (n - 1) bars + (n - 1)^3 diagonals closest to the target
            n = min((abs(3 * n * n * (n - 1) + (n - 1) ** 3 - target), n) for n in range(2, 200))[1]
            m = truss_lattice(n, seed=sub_seed)
        m.name = f"{kind}_{s}"
        out.append(m)
    return out


def load(model, mesh: Mesh) -> None:
    """Add the mesh's nodes and elements to `model` (reference add_* API), in call order."""
    model.add_nodes(mesh.node_numbers, mesh.xyz)
    load_elements(model, mesh)


def load_elements(model, mesh: Mesh) -> None:
    """Add the mesh's elements (nodes already added), in call order."""
    for kind in mesh.order:
        d = getattr(mesh, kind)
        if d is None or len(d["numbers"]) == 0:
            continue
        if kind == "trusses":
            model.add_trusses(d["numbers"], d["nodes"], d["young"], d["area"], d.get("area_2"))
        elif kind == "beams":
            model.add_beams(d["numbers"], d["nodes"], d["young"], d["poisson"], d["area"], d["i11"], d["i22"],
                            d["i12"], d["it"], d["shear_factor"], d["axis"])
        else:
            model.add_plates(d["numbers"], d["nodes"], d["young"], d["poisson"], d["thickness"], d["shear_factor"])
