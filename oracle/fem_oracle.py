"""ctypes loader for the CPU oracle (oracle/fem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU legs, never by the product package.

`OracleFEM` mirrors the reference's `FEM` API (src/fem/fem.rs:34,
methods_for_node_data_handle.rs:66, methods_for_truss_data_handle.rs:49,
methods_for_beam_data_handle.rs:49, methods_for_plate_data_handle.rs:62):
every add_* call validates and assembles eagerly, in call order, and raises
`OracleError` with the reference's message on failure.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32, c_void_p

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    src = os.path.join(_HERE, "fem_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-C", _HERE, "-B" if force else "all"], check=True, capture_output=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp, ip32, up32, i64p = POINTER(c_double), POINTER(c_int32), POINTER(c_uint32), POINTER(c_int64)
        L.orc_create.restype = c_void_p
        L.orc_create.argtypes = [c_double, c_double, c_uint32]
        L.orc_destroy.argtypes = [c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_last_error.argtypes = [c_void_p]
        L.orc_add_node.argtypes = [c_void_p, c_uint32, c_double, c_double, c_double]
        L.orc_add_truss.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32, c_double, c_double, c_int, c_double]
        L.orc_add_beam.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32] + [c_double] * 8 + [dp]
        L.orc_add_plate.argtypes = [c_void_p, c_uint32, c_uint32, c_uint32, c_uint32, c_uint32] + [c_double] * 4
        L.orc_add_nodes.argtypes = [c_void_p, up32, dp, c_size_t, POINTER(c_size_t)]
        L.orc_add_trusses.argtypes = [c_void_p, up32, up32, dp, dp, dp, c_size_t, POINTER(c_size_t)]
        L.orc_add_beams.argtypes = [c_void_p, up32, up32] + [dp] * 9 + [c_size_t, POINTER(c_size_t)]
        L.orc_add_plates.argtypes = [c_void_p, up32, up32, dp, dp, dp, dp, c_size_t, POINTER(c_size_t)]
        for f in ("orc_n_rows", "orc_nnz", "orc_n_nodes", "orc_n_groups"):
            getattr(L, f).restype = c_int64
            getattr(L, f).argtypes = [c_void_p]
        L.orc_get_csr.argtypes = [c_void_p, i64p, ip32, dp]
        L.orc_get_index_node_numbers.argtypes = [c_void_p, up32]
        L.orc_get_groups.argtypes = [c_void_p, ip32, ip32, POINTER(c_uint8), ip32]
        L.orc_truss_global_matrix.argtypes = [dp, dp, c_double, c_double, c_int, c_double, c_double, c_double, dp]
        L.orc_beam_global_matrix.argtypes = [dp, dp] + [c_double] * 8 + [dp, c_double, c_double, dp]
        L.orc_plate_global_matrix.argtypes = [dp, dp, dp, dp] + [c_double] * 6 + [dp]
        L.orc_truss_rotation.argtypes = [dp, dp, c_double, c_double, dp]
        L.orc_beam_rotation.argtypes = [dp, dp, c_double, c_double, c_double, dp, c_double, c_double, dp, dp, dp]
        L.orc_plate_rotation.argtypes = [dp, dp, dp, c_double, c_double, dp]
        L.orc_beam_line_load.argtypes = [dp, dp, c_double, dp]
        L.orc_plate_surface_load.argtypes = [dp, dp, dp, dp, c_double, c_double, c_double, dp]
        for f in ("orc_sin", "orc_cos", "orc_atan", "orc_acos"):
            getattr(L, f).restype = c_double
            getattr(L, f).argtypes = [c_double]
        L.orc_assemble_parallel.argtypes = [ctypes.POINTER(OrcMesh), c_double, c_double, c_int, i64p, ip32, dp,
                                            c_int64, i64p, dp]
        L.orc_truss_results.argtypes = [dp, dp, c_double, c_double, c_int, c_double, c_double, c_double, dp, dp]
        L.orc_beam_results.argtypes = [dp, dp] + [c_double] * 8 + [dp, c_double, c_double, dp, dp]
        L.orc_plate_results.argtypes = [dp, dp, dp, dp] + [c_double] * 6 + [dp, dp]
        L.orc_element_results.argtypes = [ctypes.POINTER(OrcMesh), dp, c_double, c_double, c_int, dp, dp, dp, dp]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(POINTER(ct))


class OracleError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class OracleFEM:
    def __init__(self, rel_tol: float, abs_tol: float, nodes_number: int):
        self._L = lib()
        self._h = self._L.orc_create(rel_tol, abs_tol, nodes_number)
        self.rel_tol, self.abs_tol, self.nodes_number = rel_tol, abs_tol, nodes_number

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_destroy(h)
            self._h = None

    def _check(self, st: int):
        if st:
            raise OracleError(st, self._L.orc_last_error(self._h).decode())

    # single-element API, as the reference
    def add_node(self, number, x, y, z):
        self._check(self._L.orc_add_node(self._h, number, x, y, z))

    def add_truss(self, number, n1, n2, young, area, area2=None):
        self._check(self._L.orc_add_truss(self._h, number, n1, n2, young, area, int(area2 is not None),
                                          0.0 if area2 is None else area2))

    def add_beam(self, number, n1, n2, young, poisson, area, i11, i22, i12, it, shear_factor, axis):
        ax = np.ascontiguousarray(axis, dtype=np.float64)
        self._check(self._L.orc_add_beam(self._h, number, n1, n2, young, poisson, area, i11, i22, i12, it,
                                         shear_factor, _p(ax, c_double)))

    def add_plate(self, number, n1, n2, n3, n4, young, poisson, thickness, shear_factor):
        self._check(self._L.orc_add_plate(self._h, number, n1, n2, n3, n4, young, poisson, thickness, shear_factor))

    # batched API: stops at the first failure (elements before it stay added)
    def add_nodes(self, numbers, xyz):
        numbers = np.ascontiguousarray(numbers, dtype=np.uint32)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = c_size_t(0)
        self._check(self._L.orc_add_nodes(self._h, _p(numbers, c_uint32), _p(xyz, c_double), len(numbers),
                                          ctypes.byref(n)))
        return n.value

    def add_trusses(self, numbers, nodes, young, area, area_2=None):
        m = len(numbers)
        numbers = np.ascontiguousarray(numbers, dtype=np.uint32)
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(m, 2)
        young = np.ascontiguousarray(np.broadcast_to(young, (m,)), dtype=np.float64)
        area = np.ascontiguousarray(np.broadcast_to(area, (m,)), dtype=np.float64)
        a2 = np.full(m, np.nan) if area_2 is None else np.ascontiguousarray(np.broadcast_to(area_2, (m,)),
                                                                          dtype=np.float64)
        n = c_size_t(0)
        self._check(self._L.orc_add_trusses(self._h, _p(numbers, c_uint32), _p(nodes, c_uint32), _p(young, c_double),
                                            _p(area, c_double), _p(a2, c_double), m, ctypes.byref(n)))
        return n.value

    def add_beams(self, numbers, nodes, young, poisson, area, i11, i22, i12, it, shear_factor, axis):
        m = len(numbers)
        numbers = np.ascontiguousarray(numbers, dtype=np.uint32)
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(m, 2)
        arrs = [np.ascontiguousarray(np.broadcast_to(v, (m,)), dtype=np.float64)
                for v in (young, poisson, area, i11, i22, i12, it, shear_factor)]
        ax = np.ascontiguousarray(np.broadcast_to(axis, (m, 3)), dtype=np.float64)
        n = c_size_t(0)
        self._check(self._L.orc_add_beams(self._h, _p(numbers, c_uint32), _p(nodes, c_uint32),
                                          *[_p(a, c_double) for a in arrs], _p(ax, c_double), m, ctypes.byref(n)))
        return n.value

    def add_plates(self, numbers, nodes, young, poisson, thickness, shear_factor):
        m = len(numbers)
        numbers = np.ascontiguousarray(numbers, dtype=np.uint32)
        nodes = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(m, 4)
        arrs = [np.ascontiguousarray(np.broadcast_to(v, (m,)), dtype=np.float64)
                for v in (young, poisson, thickness, shear_factor)]
        n = c_size_t(0)
        self._check(self._L.orc_add_plates(self._h, _p(numbers, c_uint32), _p(nodes, c_uint32),
                                           *[_p(a, c_double) for a in arrs], m, ctypes.byref(n)))
        return n.value

    # read-out
    def csr(self):
        nr, nnz = self._L.orc_n_rows(self._h), self._L.orc_nnz(self._h)
        rp = np.zeros(nr + 1, np.int64)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        self._L.orc_get_csr(self._h, _p(rp, c_int64), _p(ci, c_int32), _p(va, c_double))
        return rp, ci[:nnz], va[:nnz]

    def index_node_numbers(self):
        n = self._L.orc_n_nodes(self._h)
        out = np.zeros(max(n, 1), np.uint32)
        self._L.orc_get_index_node_numbers(self._h, _p(out, c_uint32))
        return out[:n]

    def groups(self):
        ng, nnz = self._L.orc_n_groups(self._h), self._L.orc_nnz(self._h)
        rn = np.zeros(max(ng, 1), np.int32)
        cn = np.zeros(max(ng, 1), np.int32)
        kd = np.zeros(max(ng, 1), np.uint8)
        gi = np.zeros(max(nnz, 1), np.int32)
        self._L.orc_get_groups(self._h, _p(rn, c_int32), _p(cn, c_int32), _p(kd, c_uint8), _p(gi, c_int32))
        return rn[:ng], cn[:ng], kd[:ng], gi[:nnz]


# element-level helpers -------------------------------------------------------

def _v3(x):
    return np.ascontiguousarray(x, dtype=np.float64).reshape(3)


def truss_global_matrix(x1, x2, young, area, area2=None, rel_tol=1e-12, abs_tol=1e-12):
    L = lib()
    out = np.zeros(36)
    a, b = _v3(x1), _v3(x2)
    st = L.orc_truss_global_matrix(_p(a, c_double), _p(b, c_double), young, area, int(area2 is not None),
                                   0.0 if area2 is None else area2, rel_tol, abs_tol, _p(out, c_double))
    if st:
        raise OracleError(st, "truss matrix failed")
    return out.reshape(6, 6)


def beam_global_matrix(x1, x2, young, poisson, area, i11, i22, i12, it, shear_factor, axis, rel_tol=1e-12,
                       abs_tol=1e-12):
    L = lib()
    out = np.zeros(144)
    a, b, ax = _v3(x1), _v3(x2), _v3(axis)
    st = L.orc_beam_global_matrix(_p(a, c_double), _p(b, c_double), young, poisson, area, i11, i22, i12, it,
                                  shear_factor, _p(ax, c_double), rel_tol, abs_tol, _p(out, c_double))
    if st:
        raise OracleError(st, "beam matrix failed")
    return out.reshape(12, 12)


def plate_global_matrix(x1, x2, x3, x4, young, poisson, thickness, shear_factor, rel_tol=1e-12, abs_tol=1e-12):
    L = lib()
    out = np.zeros(576)
    p = [_v3(x) for x in (x1, x2, x3, x4)]
    st = L.orc_plate_global_matrix(*[_p(x, c_double) for x in p], young, poisson, thickness, shear_factor, rel_tol,
                                   abs_tol, _p(out, c_double))
    if st:
        raise OracleError(st, "plate matrix failed")
    return out.reshape(24, 24)


def beam_line_load(x1, x2, q):
    """equivalent nodal loads of a uniformly distributed line load (beam.rs:775-797)"""
    out = np.zeros(2)
    a, b = _v3(x1), _v3(x2)
    lib().orc_beam_line_load(_p(a, c_double), _p(b, c_double), q, _p(out, c_double))
    return out


def plate_surface_load(x1, x2, x3, x4, q, rel_tol=1e-12, abs_tol=1e-12):
    """equivalent nodal loads of a uniformly distributed surface load (plate.rs:1145-1185)"""
    out = np.zeros(4)
    p = [_v3(x) for x in (x1, x2, x3, x4)]
    st = lib().orc_plate_surface_load(*[_p(x, c_double) for x in p], q, rel_tol, abs_tol, _p(out, c_double))
    if st:
        raise OracleError(st, "plate load failed")
    return out


def beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol=1e-12, abs_tol=1e-12):
    L = lib()
    r = np.zeros(9)
    a, b = c_double(0), c_double(0)
    x1, x2, ax = _v3(x1), _v3(x2), _v3(axis)
    L.orc_beam_rotation(_p(x1, c_double), _p(x2, c_double), i11, i22, i12, _p(ax, c_double), rel_tol, abs_tol,
                        _p(r, c_double), ctypes.byref(a), ctypes.byref(b))
    return r.reshape(3, 3), a.value, b.value


def plate_rotation(x2, x3, x4, rel_tol=1e-12, abs_tol=1e-12):
    L = lib()
    r = np.zeros(9)
    p = [_v3(x) for x in (x2, x3, x4)]
    L.orc_plate_rotation(*[_p(x, c_double) for x in p], rel_tol, abs_tol, _p(r, c_double))
    return r.reshape(3, 3)


def truss_rotation(x1, x2, rel_tol=1e-12, abs_tol=1e-12):
    L = lib()
    r = np.zeros(9)
    a, b = _v3(x1), _v3(x2)
    L.orc_truss_rotation(_p(a, c_double), _p(b, c_double), rel_tol, abs_tol, _p(r, c_double))
    return r.reshape(3, 3)


class OrcMesh(ctypes.Structure):
    _fields_ = [("nodes_number", c_uint32), ("xyz", POINTER(c_double)),
                ("n_truss", c_size_t), ("t_nodes", POINTER(c_int32)), ("t_young", POINTER(c_double)),
                ("t_area", POINTER(c_double)), ("t_area2", POINTER(c_double)),
                ("n_beam", c_size_t), ("b_nodes", POINTER(c_int32))]
    _fields_ += [(f"b_{k}", POINTER(c_double)) for k in ("young", "poisson", "area", "i11", "i22", "i12", "it",
                                                             "shear", "axis")]
    _fields_ += [("n_plate", c_size_t), ("p_nodes", POINTER(c_int32))]
    _fields_ += [(f"p_{k}", POINTER(c_double)) for k in ("young", "poisson", "thickness", "shear")]


def mesh_struct(mesh):
    """OrcMesh view of a finite_element_method_gb300.meshes.Mesh (node numbers 1..N in index order)."""
    keep = []

    def d(a, shape=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return _p(a, c_double)

    def i(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.int64) - 1, dtype=np.int32)
        keep.append(a)
        return _p(a, c_int32)

    assert np.array_equal(mesh.node_numbers, np.arange(1, mesh.nodes_number + 1))
    s = OrcMesh()
    s.nodes_number = mesh.nodes_number
    s.xyz = d(mesh.xyz)
    t, b, p = mesh.trusses, mesh.beams, mesh.plates
    if t is not None:
        s.n_truss, s.t_nodes, s.t_young, s.t_area = len(t["numbers"]), i(t["nodes"]), d(t["young"]), d(t["area"])
        s.t_area2 = d(t["area_2"]) if t.get("area_2") is not None else None
    if b is not None:
        s.n_beam, s.b_nodes = len(b["numbers"]), i(b["nodes"])
        for k, src in (("young", "young"), ("poisson", "poisson"), ("area", "area"), ("i11", "i11"), ("i22", "i22"),
                       ("i12", "i12"), ("it", "it"), ("shear", "shear_factor"), ("axis", "axis")):
            setattr(s, f"b_{k}", d(b[src]))
    if p is not None:
        s.n_plate, s.p_nodes = len(p["numbers"]), i(p["nodes"])
        for k, src in (("young", "young"), ("poisson", "poisson"), ("thickness", "thickness"),
                       ("shear", "shear_factor")):
            setattr(s, f"p_{k}", d(p[src]))
    s._keep = keep
    return s


def assemble_parallel(mesh, n_threads, rel_tol=1e-12, abs_tol=1e-12, want_csr=True):
    """Multi-threaded port of the eager assembly; returns (seconds, nnz, (row_ptr, col_idx, values) or None)."""
    L = lib()
    s = mesh_struct(mesh)
    nnz = c_int64(0)
    sec = c_double(0)
    if not want_csr:
        st = L.orc_assemble_parallel(ctypes.byref(s), rel_tol, abs_tol, n_threads, None, None, None, 0,
                                     ctypes.byref(nnz), ctypes.byref(sec))
        if st:
            raise OracleError(st, "parallel assembly failed")
        return sec.value, nnz.value, None
    # size first with a cheap upper bound: every element entry distinct
    cap = sum(len(d["numbers"]) * w for d, w in ((mesh.trusses, 36), (mesh.beams, 144), (mesh.plates, 576))
              if d is not None)
    rp = np.zeros(mesh.nodes_number * 6 + 1, np.int64)
    ci = np.zeros(max(cap, 1), np.int32)
    va = np.zeros(max(cap, 1), np.float64)
    st = L.orc_assemble_parallel(ctypes.byref(s), rel_tol, abs_tol, n_threads, _p(rp, c_int64), _p(ci, c_int32),
                                 _p(va, c_double), cap, ctypes.byref(nnz), ctypes.byref(sec))
    if st:
        raise OracleError(st, "parallel assembly failed")
    n = nnz.value
    return sec.value, n, (rp, ci[:n], va[:n])


def truss_results(x1, x2, young, area, area2, u6, rel_tol=1e-12, abs_tol=1e-12):
    """[ForceR] of one truss from its nodes' global displacements (3 per node), truss.rs:281-333"""
    out = np.zeros(1)
    a, b = _v3(x1), _v3(x2)
    u = np.ascontiguousarray(u6, dtype=np.float64).reshape(6)
    st = lib().orc_truss_results(_p(a, c_double), _p(b, c_double), young, area, int(area2 is not None),
                                 0.0 if area2 is None else area2, rel_tol, abs_tol, _p(u, c_double), _p(out, c_double))
    if st:
        raise OracleError(st, "truss results failed")
    return out


def beam_results(x1, x2, young, poisson, area, i11, i22, i12, it, shear_factor, axis, u12, rel_tol=1e-12,
                 abs_tol=1e-12):
    """the 10 beam results (beam.rs:803-993) from its nodes' global displacements (6 per node)"""
    out = np.zeros(10)
    a, b, ax = _v3(x1), _v3(x2), _v3(axis)
    u = np.ascontiguousarray(u12, dtype=np.float64).reshape(12)
    st = lib().orc_beam_results(_p(a, c_double), _p(b, c_double), young, poisson, area, i11, i22, i12, it,
                                shear_factor, _p(ax, c_double), rel_tol, abs_tol, _p(u, c_double), _p(out, c_double))
    if st:
        raise OracleError(st, "beam results failed")
    return out


def plate_results(x1, x2, x3, x4, young, poisson, thickness, shear_factor, u24, rel_tol=1e-12, abs_tol=1e-12):
    """the 8 plate results (plate.rs:1196-1409) from its nodes' global displacements (6 per node)"""
    out = np.zeros(8)
    p = [_v3(x) for x in (x1, x2, x3, x4)]
    u = np.ascontiguousarray(u24, dtype=np.float64).reshape(24)
    st = lib().orc_plate_results(*[_p(x, c_double) for x in p], young, poisson, thickness, shear_factor, rel_tol,
                                 abs_tol, _p(u, c_double), _p(out, c_double))
    if st:
        raise OracleError(st, "plate results failed")
    return out


def element_results(mesh, displacements, n_threads=1, rel_tol=1e-12, abs_tol=1e-12):
    """Every element's results of a meshes.Mesh from its displacements vector (6 per node, index order):
    ({"truss": (n, 1), "beam": (n, 10), "plate": (n, 8)}, seconds)."""
    s = mesh_struct(mesh)
    disp = np.ascontiguousarray(displacements, dtype=np.float64)
    assert disp.shape == (6 * mesh.nodes_number,)
    out = {"truss": np.zeros((s.n_truss, 1)), "beam": np.zeros((s.n_beam, 10)), "plate": np.zeros((s.n_plate, 8))}
    sec = c_double(0)
    st = lib().orc_element_results(ctypes.byref(s), _p(disp, c_double), rel_tol, abs_tol, n_threads,
                                   _p(out["truss"], c_double), _p(out["beam"], c_double), _p(out["plate"], c_double),
                                   ctypes.byref(sec))
    if st:
        raise OracleError(st, "element results failed")
    return out, sec.value


def sin(x):
    return lib().orc_sin(x)


def cos(x):
    return lib().orc_cos(x)


def atan(x):
    return lib().orc_atan(x)


def acos(x):
    return lib().orc_acos(x)
