"""The index-checked build (libfem_gpu_debug.so, -DFEM_GPU_DEBUG): every node
index, packed-scratch position, block-sum source, CSR source and CSR /
stiffness-group position of the assembly kernels is range-checked on the
device, with no trap.  On models that exercise every element kind, both
rotation paths, several add calls and a batch, no check fires and the results
are the release build's bit for bit."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, _lib, meshes
from finite_element_method_gb300.fem import Batch

pytestmark = pytest.mark.gpu

TOL = (meshes.REL_TOL, meshes.ABS_TOL)


def debug_record(lib):
    import ctypes

    checked, site = ctypes.c_int(-1), ctypes.c_int(-1)
    index, bound = ctypes.c_int64(0), ctypes.c_int64(0)
    assert lib.fem_gpu_debug_check(ctypes.byref(checked), ctypes.byref(site), ctypes.byref(index),
                                   ctypes.byref(bound)) == 0
    return checked.value, site.value, index.value, bound.value


def csr_with(lib, mesh):
    g = FEM(*TOL, mesh.nodes_number, library=lib)
    meshes.load(g, mesh)
    g.assemble()
    g.assemble_numeric_async()
    g.check_pattern()
    out = g.stiffness_csr()
    g.close()
    return out


def test_index_checks_stay_clear_and_results_match_release():
    dbg, rel = _lib.load_debug(), _lib.load()
    assert debug_record(rel)[0] == 0  # the release build checks nothing
    checked, site, index, bound = debug_record(dbg)  # clears any earlier record
    assert checked == 1
    q, _ = np.linalg.qr(np.random.default_rng(7).normal(size=(3, 3)))
    models = [meshes.adjoint_model(frame=(5, 4, 3), slab=(40, 30)), meshes.truss_lattice(5),
              meshes.plate_mesh(25, 20, size=2.0, rotation=q)]
    for m in models:
        a, b = csr_with(dbg, m), csr_with(rel, m)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
        assert debug_record(dbg)[1:] == (0, 0, 0), m.name
    structures = meshes.batch_structures(5, lo=100, hi=800, seed=31)
    bd = Batch.from_meshes(structures, *TOL, library=dbg)
    bd.assemble()
    br = Batch.from_meshes(structures, *TOL)
    for i in range(len(structures)):
        for x, y in zip(bd.csr(i), br.csr(i)):
            np.testing.assert_array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
    assert debug_record(dbg)[1:] == (0, 0, 0)
    bd.close()
    br.close()
