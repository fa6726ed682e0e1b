"""fem_gpu_assemble_dense_noalloc: the entry point for callers that cannot
allocate device memory (hosts that hand out every device byte from their own
pool, or must keep a fixed footprint).  It is called through the C ABI with
caller-owned device buffers and must reproduce, entry for entry, the global
stiffness that the regular handle-based path (fem_gpu_assemble) builds for the
same structure -- on two calls in a row, the second one on a different
structure, so that nothing left in the shared working array leaks into it.

This file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from finite_element_method_gb300 import FEM, _lib, meshes

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12
FEM_GPU_ERR_ARGUMENT = 30
FEM_GPU_ERR_NOALLOC_LIMIT = 43


def mixed_structure(frame, slab, seed):
    m = meshes.adjoint_model(frame=frame, slab=slab, seed=seed)
    nx, ny, nz = frame
    rng = np.random.default_rng(seed)
    # one body diagonal per frame cell as a truss
    node = lambda i, j, k: 1 + i + nx * (j + ny * k)
    pairs = [(node(i, j, k), node(i + 1, j + 1, k + 1)) for k in range(nz - 1) for j in range(ny - 1)
             for i in range(nx - 1)]
    t = len(pairs)
    m.trusses = dict(numbers=np.arange(1, t + 1, dtype=np.uint32), nodes=np.array(pairs, np.uint32),
                     young=np.full(t, 200e9), area=rng.uniform(1e-4, 5e-4, t),
                     area_2=np.where(np.arange(t) % 2 == 0, np.nan, rng.uniform(1e-4, 5e-4, t)))
    return m


def dense_from_handle(mesh):
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    rp, ci, va = g.stiffness_csr()
    g.close()
    n = 6 * mesh.nodes_number
    K = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    K[rows, ci] = va
    return K


def noalloc_inputs(mesh, torch):
    dev = torch.device("cuda:0")
    t, b, p = mesh.trusses, mesh.beams, mesh.plates
    xyz = torch.tensor(mesh.xyz, dtype=torch.float64, device=dev)
    tn = torch.tensor(t["nodes"].astype(np.int64) - 1, dtype=torch.int32, device=dev)
    tp = torch.tensor(np.stack([t["young"], t["area"], t["area_2"]], 1), dtype=torch.float64, device=dev)
    bn = torch.tensor(b["nodes"].astype(np.int64) - 1, dtype=torch.int32, device=dev)
    bp = torch.tensor(np.concatenate([np.stack([b["young"], b["poisson"], b["area"], b["i11"], b["i22"], b["i12"],
                                                b["it"], b["shear_factor"]], 1), b["axis"]], 1),
                      dtype=torch.float64, device=dev)
    pn = torch.tensor(p["nodes"].astype(np.int64) - 1, dtype=torch.int32, device=dev)
    pp = torch.tensor(np.stack([p["young"], p["poisson"], p["thickness"], p["shear_factor"]], 1),
                      dtype=torch.float64, device=dev)
    n = 6 * mesh.nodes_number
    K = torch.full((n, n), float("nan"), dtype=torch.float64, device=dev)  # every entry must be written
    return dict(n_nodes=mesh.nodes_number, xyz=xyz, tn=tn, tp=tp, bn=bn, bp=bp, pn=pn, pp=pp, K=K)


def call_noalloc(a, torch):
    stream = torch.cuda.current_stream(a["K"].device).cuda_stream
    return _lib.load().fem_gpu_assemble_dense_noalloc(
        a["n_nodes"], a["xyz"].data_ptr(), a["tn"].shape[0], a["tn"].data_ptr(), a["tp"].data_ptr(),
        a["bn"].shape[0], a["bn"].data_ptr(), a["bp"].data_ptr(), a["pn"].shape[0], a["pn"].data_ptr(),
        a["pp"].data_ptr(), meshes.REL_TOL, meshes.ABS_TOL, a["K"].data_ptr(), ctypes.c_void_p(stream))


def dense_noalloc(mesh, torch):
    a = noalloc_inputs(mesh, torch)
    st = call_noalloc(a, torch)
    assert st == 0, st
    return a["K"].cpu().numpy()


def check_equal(Kn, Kh):
    assert not np.isnan(Kn).any()
    nz = Kh != 0
    rel = np.abs(Kn[nz] - Kh[nz]) / np.abs(Kh[nz])
    assert rel.max() <= REL_TOL
    np.testing.assert_array_equal(Kn[~nz], 0.0)
    np.testing.assert_array_equal(Kn, Kh)  # same summation order on both paths


def test_noalloc_matches_handle_path_twice():
    torch = pytest.importorskip("torch")
    first = mixed_structure((3, 3, 3), (20, 20), seed=41)
    second = mixed_structure((4, 3, 2), (30, 20), seed=42)
    assert first.counts() != second.counts()
    for mesh in (first, second):
        check_equal(dense_noalloc(mesh, torch), dense_from_handle(mesh))


def test_noalloc_rejects_oversized_structure():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda:0")
    xyz = torch.zeros((4, 3), dtype=torch.float64, device=dev)
    nodes = torch.zeros((3277, 4), dtype=torch.int32, device=dev)  # 32770 node-pair blocks > 32768
    props = torch.zeros((3277, 4), dtype=torch.float64, device=dev)
    K = torch.zeros((24, 24), dtype=torch.float64, device=dev)
    st = L.fem_gpu_assemble_dense_noalloc(4, xyz.data_ptr(), 0, None, None, 0, None, None, 3277, nodes.data_ptr(),
                                          props.data_ptr(), 1e-12, 1e-12, K.data_ptr(), None)
    assert st == FEM_GPU_ERR_NOALLOC_LIMIT


def test_noalloc_second_call_allocates_nothing():
    """The property the entry point exists for: with its inputs and output in
    place, a call leaves the device's free memory exactly where it was."""
    torch = pytest.importorskip("torch")
    mesh = mixed_structure((3, 3, 2), (20, 20), seed=43)
    a = noalloc_inputs(mesh, torch)
    assert call_noalloc(a, torch) == 0  # first call on the device: loads the module, looks up the array
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert call_noalloc(a, torch) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    check_equal(a["K"].cpu().numpy(), dense_from_handle(mesh))


def test_noalloc_rejects_bad_elements_then_recovers():
    """Out-of-range node index, a zero-length truss, a plate with a repeated
    node and a plate off its plane each fail with FEM_GPU_ERR_ARGUMENT; a valid call afterwards still
    matches the handle path (the error flag is cleared per call)."""
    torch = pytest.importorskip("torch")
    mesh = mixed_structure((3, 3, 2), (20, 20), seed=44)
    cases = []
    a = noalloc_inputs(mesh, torch)
    a["tn"][1, 1] = mesh.nodes_number  # one past the last node
    cases.append(a)
    a = noalloc_inputs(mesh, torch)
    a["tn"][0, 1] = a["tn"][0, 0]  # both ends on one node: zero length
    cases.append(a)
    a = noalloc_inputs(mesh, torch)
    a["pn"][2, 3] = a["pn"][2, 0]  # plate nodes a, b, c, a
    cases.append(a)
    a = noalloc_inputs(mesh, torch)
    a["xyz"][int(a["pn"][3, 3]), 2] += 1.0  # one node of a plate lifted off the slab: not on one plane
    cases.append(a)
    for a in cases:
        assert call_noalloc(a, torch) == FEM_GPU_ERR_ARGUMENT
    check_equal(dense_noalloc(mesh, torch), dense_from_handle(mesh))
