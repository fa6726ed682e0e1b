"""Device memory: every model's arrays come from a pool that keeps freed memory; a later model reuses it,
results do not depend on what the pool held before, and fem_gpu_release_cached_memory hands the cache back."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, _lib, meshes

pytestmark = pytest.mark.gpu


def assembled_values(mesh):
    g = FEM(1e-12, 1e-12, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    v = g.stiffness_values().copy()
    g.close()
    return v


def test_pool_reuse_and_release():
    import torch

    L = _lib.load()
    m = meshes.plate_mesh(60, 60, size=6.0)
    first = assembled_values(m)
    # other models in between leave their arrays in the pool
    for nx in (80, 30):
        assembled_values(meshes.plate_mesh(nx, nx, size=6.0))
    assert np.array_equal(assembled_values(m).view(np.uint64), first.view(np.uint64))
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert L.fem_gpu_release_cached_memory() == 0
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after >= free_before
    assert np.array_equal(assembled_values(m).view(np.uint64), first.view(np.uint64))
