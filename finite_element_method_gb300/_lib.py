"""ctypes binding of the C ABI declared in include/fem_gpu.h.

The shared library is the product: every call goes to CUDA kernels.  There
is no CPU path behind this module; when the library is missing it is built
with nvcc, and when no CUDA device is present the library's own calls fail
with FEM_GPU_ERR_CUDA.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32, c_void_p

from . import build as _build

dp, fp = POINTER(c_double), POINTER(c_float)
i32p, i64p, u32p, u8p, szp = POINTER(c_int32), POINTER(c_int64), POINTER(c_uint32), POINTER(c_uint8), POINTER(c_size_t)
hp = c_void_p

# name -> (restype, argtypes); the complete exported surface of include/fem_gpu.h
SIGNATURES = {
    "fem_gpu_create": (c_int, [c_double, c_double, c_uint32, POINTER(c_void_p)]),
    "fem_gpu_destroy": (c_int, [hp]),
    "fem_gpu_last_error": (c_char_p, [hp]),
    "fem_gpu_add_nodes": (c_int, [hp, u32p, dp, c_size_t, szp]),
    "fem_gpu_add_trusses": (c_int, [hp, u32p, u32p, dp, dp, dp, c_size_t, szp]),
    "fem_gpu_add_beams": (c_int, [hp, u32p, u32p] + [dp] * 9 + [c_size_t, szp]),
    "fem_gpu_add_plates": (c_int, [hp, u32p, u32p, dp, dp, dp, dp, c_size_t, szp]),
    "fem_gpu_assemble": (c_int, [hp]),
    "fem_gpu_assemble_numeric_async": (c_int, [hp]),
    "fem_gpu_check_pattern": (c_int, [hp]),
    "fem_gpu_set_node_coordinates": (c_int, [hp, dp, c_size_t]),
    "fem_gpu_set_plate_properties": (c_int, [hp, dp, dp, dp, dp, c_size_t]),
    "fem_gpu_get_csr_sizes": (c_int, [hp, i64p, i64p]),
    "fem_gpu_get_csr": (c_int, [hp, i64p, i32p, dp]),
    "fem_gpu_get_csr_values": (c_int, [hp, dp]),
    "fem_gpu_get_csr_device": (c_int, [hp, POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p)]),
    "fem_gpu_get_node_count": (c_int, [hp, i64p]),
    "fem_gpu_get_index_node_numbers": (c_int, [hp, u32p]),
    "fem_gpu_get_group_count": (c_int, [hp, i64p]),
    "fem_gpu_get_groups": (c_int, [hp, i32p, i32p, u8p, i32p]),
    "fem_gpu_get_truss_rotation": (c_int, [hp, c_uint32, dp]),
    "fem_gpu_get_beam_rotation": (c_int, [hp, c_uint32, dp]),
    "fem_gpu_get_plate_rotation": (c_int, [hp, c_uint32, dp]),
    "fem_gpu_get_element_counts": (c_int, [hp, i64p, i64p, i64p]),
    "fem_gpu_get_stream": (c_int, [hp, POINTER(c_void_p)]),
    "fem_gpu_numeric_launch_count": (c_int, [hp, POINTER(c_int)]),
    "fem_gpu_last_numeric_timing": (c_int, [hp, fp, fp]),
    "fem_gpu_get_pattern_stats": (c_int, [hp, i64p, i64p, i64p, i64p]),
    "fem_gpu_vjp": (c_int, [hp, dp, dp, c_int, dp, dp, dp, dp]),
    "fem_gpu_vjp_last_ms": (c_int, [hp, fp]),
    "fem_gpu_batch_create": (c_int, [POINTER(c_void_p), c_size_t, POINTER(c_void_p)]),
    "fem_gpu_batch_destroy": (c_int, [hp]),
    "fem_gpu_batch_last_error": (c_char_p, [hp]),
    "fem_gpu_batch_assemble": (c_int, [hp]),
    "fem_gpu_batch_assemble_async": (c_int, [hp]),
    "fem_gpu_batch_get_values": (c_int, [hp, c_size_t, dp]),
    "fem_gpu_batch_get_values_device": (c_int, [hp, c_size_t, POINTER(c_void_p)]),
    "fem_gpu_batch_get_stream": (c_int, [hp, POINTER(c_void_p)]),
    "fem_gpu_batch_last_ms": (c_int, [hp, fp]),
    "fem_gpu_batch_autotune": (c_int, [hp, c_int, c_char_p, c_char_p, c_size_t]),
    "fem_gpu_batch_configure": (c_int, [hp, c_int, c_int, c_int, c_int, c_int, c_int, c_int]),
    "fem_gpu_add_concentrated_loads": (c_int, [hp, u32p, u8p, dp, c_size_t, szp]),
    "fem_gpu_add_line_loads": (c_int, [hp, u32p, u8p, dp, c_size_t, szp]),
    "fem_gpu_add_surface_loads": (c_int, [hp, u32p, u8p, dp, c_size_t, szp]),
    "fem_gpu_get_forces": (c_int, [hp, dp]),
    "fem_gpu_get_forces_device": (c_int, [hp, POINTER(c_void_p)]),
    "fem_gpu_solve_pcg": (c_int, [hp, dp, dp, c_int, c_int, dp, POINTER(c_int)]),
    "fem_gpu_reactions": (c_int, [hp, dp, dp, dp, dp]),
    "fem_gpu_element_results": (c_int, [hp, dp, c_size_t, dp, dp, dp]),
    "fem_gpu_element_results_device": (c_int, [hp, c_void_p, c_void_p, c_void_p, c_void_p]),
    "fem_gpu_results_last_ms": (c_int, [hp, POINTER(c_float)]),
    "fem_gpu_get_element_numbers": (c_int, [hp, c_int, u32p]),
    "fem_gpu_release_cached_memory": (c_int, []),
    "fem_gpu_assemble_to_host": (c_int, [hp, i64p, i32p, dp, c_int64, i64p]),
    "fem_gpu_separate_sparse": (c_int, [hp, u8p]),
    "fem_gpu_get_separation_sizes": (c_int, [hp, i64p, i64p, i64p]),
    "fem_gpu_get_separation_indexes": (c_int, [hp, i64p, i64p]),
    "fem_gpu_get_separation_block": (c_int, [hp, c_int, i64p, i32p, dp]),
    "fem_gpu_get_separation_block_device": (c_int, [hp, c_int, POINTER(c_void_p), POINTER(c_void_p),
                                                    POINTER(c_void_p)]),
    "fem_gpu_batch_create_from_arrays": (c_int, [c_double, c_double, c_void_p, POINTER(c_void_p)]),
    "fem_gpu_batch_size": (c_int, [hp, szp]),
    "fem_gpu_batch_build_ms": (c_int, [hp, dp, c_size_t]),
    "fem_gpu_batch_get_csr_sizes": (c_int, [hp, c_size_t, i64p, i64p]),
    "fem_gpu_batch_get_csr": (c_int, [hp, c_size_t, i64p, i32p, dp]),
    "fem_gpu_debug_check": (c_int, [POINTER(c_int), POINTER(c_int), i64p, i64p]),
    "fem_gpu_assemble_dense_noalloc": (c_int, [c_uint32, c_void_p, c_size_t, c_void_p, c_void_p, c_size_t, c_void_p,
                                               c_void_p, c_size_t, c_void_p, c_void_p, c_double, c_double, c_void_p,
                                               c_void_p]),
}



class Structures(ctypes.Structure):
    """fem_gpu_structures_t: the host arrays of many structures, structure after structure."""
    _fields_ = [("n_structures", c_size_t), ("nodes_number", u32p), ("node_off", szp), ("node_numbers", u32p),
                ("xyz", dp),
                ("truss_off", szp), ("truss_numbers", u32p), ("truss_nodes", u32p), ("truss_young", dp),
                ("truss_area", dp), ("truss_area2", dp),
                ("beam_off", szp), ("beam_numbers", u32p), ("beam_nodes", u32p), ("beam_young", dp),
                ("beam_poisson", dp), ("beam_area", dp), ("beam_i11", dp), ("beam_i22", dp), ("beam_i12", dp),
                ("beam_it", dp), ("beam_shear_factor", dp), ("beam_local_axis", dp),
                ("plate_off", szp), ("plate_numbers", u32p), ("plate_nodes", u32p), ("plate_young", dp),
                ("plate_poisson", dp), ("plate_thickness", dp), ("plate_shear_factor", dp)]


_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def _bind(lib):
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_debug_lib = None


def load_debug(build_if_missing: bool = True) -> ctypes.CDLL:
    """libfem_gpu_debug.so: the same C ABI with the device-side index checks of the assembly path (its
    fem_gpu_debug_check reports the first out-of-range index).  Loaded beside the release library."""
    global _debug_lib
    if _debug_lib is None:
        if build_if_missing:
            _build.build()
        if not os.path.exists(_build.DEBUG_LIB_PATH):
            raise RuntimeError(f"index-checked library not found at {_build.DEBUG_LIB_PATH}")
        _debug_lib = _bind(ctypes.CDLL(_build.DEBUG_LIB_PATH))
    return _debug_lib


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libfem_gpu.so (building it first when absent or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA assembly library not found at {path}; build it with finite_element_method_gb300.build")
    _lib = _bind(ctypes.CDLL(path))
    return _lib


def ptr(a, ct):
    """ctypes pointer to a contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(POINTER(ct))
