"""Host-side mirror of the reference crate's `FEM` assembly API over the C ABI.

Reference interface (Rust crate finite_element_method 0.9.12):
  FEM::create(rel_tol, abs_tol, nodes_number)          src/fem/fem.rs:34
  FEM::add_node(number, x, y, z)                        src/fem/methods_for_node_data_handle.rs:66
  FEM::add_truss(number, n1, n2, E, A, Option<A2>)      src/fem/methods_for_truss_data_handle.rs:49
  FEM::add_beam(number, n1, n2, E, nu, A, I11, I22, I12, It, k, axis)
                                                        src/fem/methods_for_beam_data_handle.rs:49
  FEM::add_plate(number, n1, n2, n3, n4, E, nu, t, k)   src/fem/methods_for_plate_data_handle.rs:62
  FEM::get_{truss,beam,plate}_rotation_matrix_elements  src/fem/fem.rs:171-202
  FEM.stiffness_matrix (SquareMatrix, read by the separation step, fem.rs:71)

Each add_* raises `FEMError` with the reference's message where the reference
returns Err(String); the failing element leaves the model unchanged.  The
reference assembles eagerly inside add_*; here the stiffness is built by
`assemble()` (one symbolic + numeric pass on the GPU), after which
`stiffness_csr()` returns the same matrix as CSR (row = 6 * node index + DOF,
DOFParameter order X, Y, Z, ThX, ThY, ThZ).  The bulk forms add many elements
of one kind in one call, in array order, stopping at the first failure.
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32, c_void_p

import numpy as np

from . import _lib
from ._lib import ptr

FEM_GPU_ERR_NODE_LIMIT = 1
FEM_GPU_ERR_NODE_NOT_EXIST = 5
FEM_GPU_ERR_ARGUMENT = 30
FEM_GPU_ERR_CUDA = 40


class FEMError(RuntimeError):
    """A failed C-ABI call: `code` is the FEM_GPU_* status, the message the reference's."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def _require(ok, what):
    """argument check that stays on under python -O: the C side trusts the sizes it is given"""
    if not ok:
        raise ValueError(what)


def _f64(v, m):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (m,)))


def _u32(v, shape):
    return np.ascontiguousarray(np.asarray(v, dtype=np.uint32).reshape(shape))


class FEM:
    """FEM::create(rel_tol, abs_tol, nodes_number) with the GPU assembly behind it."""

    def __init__(self, rel_tol: float, abs_tol: float, nodes_number: int, library=None):
        """`library`: the loaded C library to use (default the release build; `_lib.load_debug()` gives the
        build with device-side index checks)."""
        self._L = library if library is not None else _lib.load()
        h = c_void_p()
        self._check(self._L.fem_gpu_create(rel_tol, abs_tol, nodes_number, ctypes.byref(h)), None)
        self._h = h
        self.rel_tol, self.abs_tol, self.nodes_number = rel_tol, abs_tol, nodes_number
        self._node_limit = nodes_number  # the crate's props keep the nodes_number of create, reset or not

    def reset(self, nodes_number: int) -> None:
        """FEM::reset (fem.rs:155-169): drop every node, element, load and imposed displacement and size the
        stiffness, forces and displacements for `nodes_number` nodes.  As in the crate, the tolerances and
        the node limit stay those of create (reset leaves the crate's props untouched): add_node refuses the
        node past the nodes_number given at creation, with the crate's message, even after a reset to more.
        After a reset to fewer nodes the handle refuses the node past the new count; the crate would accept
        it although its DOFs lie outside the matrix and the vectors it has just sized."""
        h = c_void_p()
        self._check(self._L.fem_gpu_create(self.rel_tol, self.abs_tol, nodes_number, ctypes.byref(h)), None)
        self.close()
        self._h = h
        self.nodes_number = nodes_number
        self._imposed_arr = self._displacements = self._result_forces = self._lookup = None

    # -- plumbing ---------------------------------------------------------
    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.fem_gpu_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, st: int, h=-1):
        if st:
            hh = self._h if h == -1 else h
            msg = self._L.fem_gpu_last_error(hh).decode() if hh else f"status {st}"
            raise FEMError(st, msg)

    # -- node / element API (reference names) ------------------------------
    def add_node(self, number: int, x: float, y: float, z: float) -> None:
        self.add_nodes([number], [[x, y, z]])

    def add_nodes(self, numbers, xyz) -> int:
        numbers = _u32(numbers, (-1,))
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(len(numbers), 3))
        m = len(numbers)
        if self._node_limit < self.nodes_number:  # reset to more nodes than at creation: the old limit holds
            m = min(m, max(self._node_limit - self.node_count(), 0))
        n = c_size_t(0)
        if m:
            st = self._L.fem_gpu_add_nodes(self._h, ptr(numbers, c_uint32), ptr(xyz, c_double), m, ctypes.byref(n))
            self._check(st)
        if m < len(numbers):
            raise FEMError(FEM_GPU_ERR_NODE_LIMIT, f"Nodes number could not be greater than {self._node_limit}!")
        return n.value

    def add_truss(self, number, node_1_number, node_2_number, young_modulus, area, area_2=None) -> None:
        self.add_trusses([number], [[node_1_number, node_2_number]], young_modulus, area,
                         None if area_2 is None else [area_2])

    def add_trusses(self, numbers, nodes, young_modulus, area, area_2=None) -> int:
        m = len(numbers)
        numbers, nodes = _u32(numbers, (m,)), _u32(nodes, (m, 2))
        E, A = _f64(young_modulus, m), _f64(area, m)
        A2 = None if area_2 is None else _f64(area_2, m)
        n = c_size_t(0)
        st = self._L.fem_gpu_add_trusses(self._h, ptr(numbers, c_uint32), ptr(nodes, c_uint32), ptr(E, c_double),
                                         ptr(A, c_double), ptr(A2, c_double), m, ctypes.byref(n))
        self._check(st)
        return n.value

    def add_beam(self, number, node_1_number, node_2_number, young_modulus, poisson_ratio, area, i11, i22, i12, it,
                 shear_factor, local_axis_1_direction) -> None:
        self.add_beams([number], [[node_1_number, node_2_number]], young_modulus, poisson_ratio, area, i11, i22, i12,
                       it, shear_factor, [local_axis_1_direction])

    def add_beams(self, numbers, nodes, young_modulus, poisson_ratio, area, i11, i22, i12, it, shear_factor,
                  local_axis_1_direction) -> int:
        m = len(numbers)
        numbers, nodes = _u32(numbers, (m,)), _u32(nodes, (m, 2))
        arrs = [_f64(v, m) for v in (young_modulus, poisson_ratio, area, i11, i22, i12, it, shear_factor)]
        axis = np.ascontiguousarray(np.broadcast_to(np.asarray(local_axis_1_direction, dtype=np.float64), (m, 3)))
        n = c_size_t(0)
        st = self._L.fem_gpu_add_beams(self._h, ptr(numbers, c_uint32), ptr(nodes, c_uint32),
                                       *[ptr(a, c_double) for a in arrs], ptr(axis, c_double), m, ctypes.byref(n))
        self._check(st)
        return n.value

    def add_plate(self, number, node_1_number, node_2_number, node_3_number, node_4_number, young_modulus,
                  poisson_ratio, thickness, shear_factor) -> None:
        self.add_plates([number], [[node_1_number, node_2_number, node_3_number, node_4_number]], young_modulus,
                        poisson_ratio, thickness, shear_factor)

    def add_plates(self, numbers, nodes, young_modulus, poisson_ratio, thickness, shear_factor) -> int:
        m = len(numbers)
        numbers, nodes = _u32(numbers, (m,)), _u32(nodes, (m, 4))
        arrs = [_f64(v, m) for v in (young_modulus, poisson_ratio, thickness, shear_factor)]
        n = c_size_t(0)
        st = self._L.fem_gpu_add_plates(self._h, ptr(numbers, c_uint32), ptr(nodes, c_uint32),
                                        *[ptr(a, c_double) for a in arrs], m, ctypes.byref(n))
        self._check(st)
        return n.value

    # -- assembly ----------------------------------------------------------
    def assemble(self) -> None:
        self._check(self._L.fem_gpu_assemble(self._h))

    def assemble_numeric_async(self) -> None:
        self._check(self._L.fem_gpu_assemble_numeric_async(self._h))

    def check_pattern(self) -> None:
        self._check(self._L.fem_gpu_check_pattern(self._h))

    def set_node_coordinates(self, xyz) -> None:
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
        self._check(self._L.fem_gpu_set_node_coordinates(self._h, ptr(xyz, c_double), len(xyz)))

    def set_plate_properties(self, young_modulus, poisson_ratio, thickness, shear_factor) -> None:
        m = self.element_counts()[2]
        arrs = [_f64(v, m) for v in (young_modulus, poisson_ratio, thickness, shear_factor)]
        self._check(self._L.fem_gpu_set_plate_properties(self._h, *[ptr(a, c_double) for a in arrs], m))

    # -- read-out ----------------------------------------------------------
    def csr_sizes(self):
        nr, nnz = c_int64(0), c_int64(0)
        self._check(self._L.fem_gpu_get_csr_sizes(self._h, ctypes.byref(nr), ctypes.byref(nnz)))
        return nr.value, nnz.value

    def stiffness_csr(self):
        """(row_ptr int64[n_rows+1], col_idx int32[nnz], values float64[nnz]) of the global stiffness."""
        nr, nnz = self.csr_sizes()
        rp = np.zeros(nr + 1, np.int64)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        self._check(self._L.fem_gpu_get_csr(self._h, ptr(rp, c_int64), ptr(ci, c_int32), ptr(va, c_double)))
        return rp, ci[:nnz], va[:nnz]

    def assemble_to_host(self, row_ptr, col_idx, values) -> int:
        """assemble() with the CSR read back into the given host arrays (row_ptr of 6 * nodes_number + 1
        int64, col_idx int32 and values float64 with room for the entries; page-locked arrays copy fastest):
        during a symbolic phase row_ptr travels back once the rows are counted and col_idx as the rows are
        filled, otherwise the pattern travels back while the numeric pass runs; the values follow the pass.
        Returns nnz."""
        rp = np.asarray(row_ptr)
        ci = np.asarray(col_idx)
        va = np.asarray(values)
        _require(rp.dtype == np.int64 and ci.dtype == np.int32 and va.dtype == np.float64,
                 "row_ptr, col_idx, values must be int64, int32, float64")
        _require(rp.flags.c_contiguous and ci.flags.c_contiguous and va.flags.c_contiguous,
                 "row_ptr, col_idx, values must be C-contiguous")
        _require(rp.size >= 6 * self.nodes_number + 1, f"row_ptr needs {6 * self.nodes_number + 1} entries")
        cap = min(ci.size, va.size)
        nnz = c_int64(0)
        self._check(self._L.fem_gpu_assemble_to_host(self._h, ptr(rp, c_int64), ptr(ci, c_int32), ptr(va, c_double),
                                                     cap, ctypes.byref(nnz)))
        return nnz.value

    def stiffness_values(self, out=None):
        _, nnz = self.csr_sizes()
        if out is None:
            out = np.zeros(max(nnz, 1), np.float64)
        self._check(self._L.fem_gpu_get_csr_values(self._h, ptr(out, c_double)))
        return out[:nnz]

    def stiffness_device_pointers(self):
        a, b, c = c_void_p(), c_void_p(), c_void_p()
        self._check(self._L.fem_gpu_get_csr_device(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def node_count(self) -> int:
        n = c_int64(0)
        self._check(self._L.fem_gpu_get_node_count(self._h, ctypes.byref(n)))
        return n.value

    def index_node_numbers(self):
        """DOF map: node index (insertion order) -> node number; DOF = 6 * index + DOFParameter."""
        n = self.node_count()
        out = np.zeros(max(n, 1), np.uint32)
        self._check(self._L.fem_gpu_get_index_node_numbers(self._h, ptr(out, c_uint32)))
        return out[:n]

    def groups(self):
        """Stiffness groups: (row_node, col_node, kind, nnz_group); kind 0 Kuu, 1 Kuth, 2 Kthu, 3 Kthth."""
        ng = c_int64(0)
        self._check(self._L.fem_gpu_get_group_count(self._h, ctypes.byref(ng)))
        ng = ng.value
        _, nnz = self.csr_sizes()
        rn, cn = np.zeros(max(ng, 1), np.int32), np.zeros(max(ng, 1), np.int32)
        kd, gi = np.zeros(max(ng, 1), np.uint8), np.zeros(max(nnz, 1), np.int32)
        self._check(self._L.fem_gpu_get_groups(self._h, ptr(rn, c_int32), ptr(cn, c_int32), ptr(kd, c_uint8),
                                               ptr(gi, c_int32)))
        return rn[:ng], cn[:ng], kd[:ng], gi[:nnz]

    def _rotation(self, fn, number):
        r = np.zeros(9)
        self._check(fn(self._h, number, ptr(r, c_double)))
        return r

    def get_truss_rotation_matrix_elements(self, number):
        return self._rotation(self._L.fem_gpu_get_truss_rotation, number)

    def get_beam_rotation_matrix_elements(self, number):
        return self._rotation(self._L.fem_gpu_get_beam_rotation, number)

    def get_plate_rotation_matrix_elements(self, number):
        return self._rotation(self._L.fem_gpu_get_plate_rotation, number)

    def element_counts(self):
        a, b, c = c_int64(0), c_int64(0), c_int64(0)
        self._check(self._L.fem_gpu_get_element_counts(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def stream(self) -> int:
        s = c_void_p()
        self._check(self._L.fem_gpu_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def numeric_launch_count(self) -> int:
        n = c_int(0)
        self._check(self._L.fem_gpu_numeric_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def pattern_stats(self):
        """(global node-pair blocks, element node-pair contributions, packed scratch doubles, block-sum slots)."""
        a, b, c, d = c_int64(0), c_int64(0), c_int64(0), c_int64(0)
        self._check(self._L.fem_gpu_get_pattern_stats(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                      ctypes.byref(d)))
        return a.value, b.value, c.value, d.value

    def vjp(self, u, lam):
        """Gradient of F = -sum_p lam_p^T K u_p for u, lam of shape (npairs, 6 * nodes_number):
        returns dict(truss (n_truss, 3: E, A, A2), beam (n_beam, 5: E, A, I11, I22, It),
        plate (n_plate, 2: E, t), xyz (n_nodes, 3))."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        if u.ndim == 1:
            u, lam = u[None], lam[None]
        _require(u.ndim == 2 and u.shape == lam.shape and u.shape[1] == 6 * self.nodes_number,
                 f"u and lam must both be (npairs, {6 * self.nodes_number})")
        nt, nb, npl = self.element_counts()
        out = dict(truss=np.zeros((nt, 3)), beam=np.zeros((nb, 5)), plate=np.zeros((npl, 2)),
                   xyz=np.zeros((self.node_count(), 3)))
        self._check(self._L.fem_gpu_vjp(self._h, ptr(u, c_double), ptr(lam, c_double), u.shape[0],
                                        ptr(out["truss"], c_double), ptr(out["beam"], c_double),
                                        ptr(out["plate"], c_double), ptr(out["xyz"], c_double)))
        return out

    # -- boundary conditions and sparse separation ---------------------------------
    DOF_PARAMETERS = ("X", "Y", "Z", "ThX", "ThY", "ThZ")

    def add_displacement(self, node_number: int, dof_parameter, value: float = 0.0) -> None:
        """add_displacement (methods_for_bc_data_handle.rs:176-203): impose a displacement on one DOF."""
        self.add_displacements([node_number], [self._dof(dof_parameter)], [value])

    def add_displacements(self, node_numbers, dofs, values=0.0) -> int:
        """add_displacement for every (node, DOF, value) in call order, stopping at the first failure like a
        loop of single calls: a node that does not exist, or a DOF already imposed (by an earlier call or
        earlier in this one).  The items before the failure stay imposed; returns how many were imposed."""
        numbers = np.atleast_1d(np.asarray(node_numbers, dtype=np.int64))
        m = len(numbers)
        d = np.atleast_1d(np.asarray(dofs))
        d = np.array([self._dof(x) for x in d], np.int64) if d.dtype.kind in "OU" else d.astype(np.int64)
        d = np.broadcast_to(d, (m,))
        if m and (d.min() < 0 or d.max() > 5):
            raise FEMError(FEM_GPU_ERR_ARGUMENT, "DOF parameter out of range (0 X .. 5 ThZ)")
        v = np.broadcast_to(np.asarray(values, dtype=np.float64), (m,))
        imp = self._imposed()
        idx = self._node_indexes(numbers)
        k = np.where(idx >= 0, 6 * idx + d, -1 - np.arange(m))  # (missing nodes get keys of their own)
        bad = idx < 0
        bad[idx >= 0] |= imp[k[idx >= 0]] != 0
        _, first = np.unique(k, return_index=True)
        repeat = np.ones(m, bool)
        repeat[first] = False
        bad |= repeat
        f = int(np.argmax(bad)) if bad.any() else m
        imp[k[:f]] = 1
        self._displacements[k[:f]] = v[:f]
        if f == m:
            return m
        if idx[f] < 0:
            raise FEMError(FEM_GPU_ERR_NODE_NOT_EXIST, f"Node with number {numbers[f]} does not exist!")
        raise FEMError(FEM_GPU_ERR_ARGUMENT,
                       f"Displacement {self.DOF_PARAMETERS[d[f]]} already applied to node {numbers[f]}!")

    def _dof(self, dof_parameter):
        return dof_parameter if isinstance(dof_parameter, (int, np.integer)) else self.DOF_PARAMETERS.index(dof_parameter)

    def _loads(self, fn, numbers, dofs, values) -> int:
        numbers = _u32(numbers, (-1,))
        m = len(numbers)
        d = np.ascontiguousarray(np.broadcast_to(np.asarray([self._dof(x) for x in np.atleast_1d(dofs)]
                                                            if np.asarray(dofs).dtype.kind in "OU"
                                                            else np.asarray(dofs), dtype=np.uint8), (m,)))
        v = _f64(values, m)
        n = c_size_t(0)
        self._check(fn(self._h, ptr(numbers, c_uint32), ptr(d, c_uint8), ptr(v, c_double), m, ctypes.byref(n)))
        return n.value

    def add_concentrated_load(self, node_number: int, dof_parameter, value: float) -> None:
        """add_concentrated_load (methods_for_bc_data_handle.rs:30-56)"""
        self.add_concentrated_loads([node_number], [self._dof(dof_parameter)], [value])

    def add_concentrated_loads(self, node_numbers, dofs, values) -> int:
        return self._loads(self._L.fem_gpu_add_concentrated_loads, node_numbers, dofs, values)

    def add_uniformly_distributed_line_load(self, beam_number: int, dof_parameter, value: float) -> None:
        """add_uniformly_distributed_line_load (methods_for_bc_data_handle.rs:58-101)"""
        self.add_uniformly_distributed_line_loads([beam_number], [self._dof(dof_parameter)], [value])

    def add_uniformly_distributed_line_loads(self, beam_numbers, dofs, values) -> int:
        return self._loads(self._L.fem_gpu_add_line_loads, beam_numbers, dofs, values)

    def add_uniformly_distributed_surface_load(self, plate_number: int, dof_parameter, value: float) -> None:
        """add_uniformly_distributed_surface_load (methods_for_bc_data_handle.rs:103-175)"""
        self.add_uniformly_distributed_surface_loads([plate_number], [self._dof(dof_parameter)], [value])

    def add_uniformly_distributed_surface_loads(self, plate_numbers, dofs, values) -> int:
        return self._loads(self._L.fem_gpu_add_surface_loads, plate_numbers, dofs, values)

    def forces_vector(self):
        """the forces vector (6 * nodes_number, DOF order): every load's nodal contributions summed in call order"""
        f = np.zeros(6 * self.nodes_number)
        self._check(self._L.fem_gpu_get_forces(self._h, ptr(f, c_double)))
        return f

    def compose_r_a_vector(self, k_aa_indexes):
        """compose_r_a_vector (methods_for_separate_stiffness_matrix.rs:322-331): forces at the free DOFs"""
        return self.forces_vector()[np.asarray(k_aa_indexes, np.int64)]

    def compose_u_b_vector(self, k_bb_indexes):
        """compose_u_b_vector (methods_for_separate_stiffness_matrix.rs:333-342): imposed displacements"""
        self._imposed()
        return self._displacements[np.asarray(k_bb_indexes, np.int64)].copy()

    def _imposed(self):
        if getattr(self, "_imposed_arr", None) is None:
            self._imposed_arr = np.zeros(6 * self.nodes_number, np.uint8)
            self._displacements = np.zeros(6 * self.nodes_number)
        return self._imposed_arr

    def _node_indexes(self, numbers):
        """the node index of each node number (-1 where no node has it).  Node numbers are unique and nodes
        are only appended, so the lookup keeps the numbers sorted up to some node count and scans the few
        nodes added after it, sorting again once those are more than an eighth of the sorted ones."""
        count = self.node_count()
        lk = getattr(self, "_lookup", None)
        if lk is None or lk[0] > count or 8 * (count - lk[0]) > max(lk[0], 8192):
            all_numbers = self.index_node_numbers().astype(np.int64)
            order = np.argsort(all_numbers, kind="stable")
            self._lookup = lk = (count, all_numbers[order], order)
        c0, srt, order = lk
        numbers = np.asarray(numbers, dtype=np.int64)
        out = np.full(numbers.shape, -1, np.int64)
        if c0:
            pos = np.minimum(np.searchsorted(srt, numbers), c0 - 1)
            hit = srt[pos] == numbers
            out[hit] = order[pos[hit]]
        if count > c0:
            tail = self.index_node_numbers()[c0:].astype(np.int64)
            t_order = np.argsort(tail, kind="stable")
            t_srt = tail[t_order]
            miss = np.flatnonzero(out < 0)
            pos = np.minimum(np.searchsorted(t_srt, numbers[miss]), len(t_srt) - 1)
            hit = t_srt[pos] == numbers[miss]
            out[miss[hit]] = c0 + t_order[pos[hit]]
        return out

    def separate_stiffness_matrix_sparse_iterative(self, imposed=None) -> "SeparatedStiffnessSparse":
        """separate_stiffness_matrix_sparse_iterative (methods_for_separate_stiffness_matrix.rs:217-320) on the
        GPU: the imposed displacements (from add_displacement, or `imposed`, 6 * nodes_number flags) split the
        assembled stiffness into K_aa, K_ab, K_ba, K_bb, each a CSR matrix sorted by (row, column)."""
        imp = self._imposed() if imposed is None else np.ascontiguousarray(imposed, dtype=np.uint8)
        _require(imp.shape == (6 * self.nodes_number,), f"imposed must hold {6 * self.nodes_number} flags")
        self._check(self._L.fem_gpu_separate_sparse(self._h, ptr(imp, c_uint8)))
        n_aa, n_bb, nnz = c_int64(0), c_int64(0), (c_int64 * 4)()
        self._check(self._L.fem_gpu_get_separation_sizes(self._h, ctypes.byref(n_aa), ctypes.byref(n_bb), nnz))
        aa = np.zeros(n_aa.value, np.int64)
        bb = np.zeros(n_bb.value, np.int64)
        self._check(self._L.fem_gpu_get_separation_indexes(self._h, ptr(aa, c_int64), ptr(bb, c_int64)))
        blocks = {}
        for which, name in enumerate(SeparatedStiffnessSparse.BLOCKS):
            rows = n_aa.value if which < 2 else n_bb.value
            rp = np.zeros(rows + 1, np.int64)
            ci = np.zeros(nnz[which], np.int32)
            va = np.zeros(nnz[which], np.float64)
            self._check(self._L.fem_gpu_get_separation_block(self._h, which, ptr(rp, c_int64), ptr(ci, c_int32),
                                                             ptr(va, c_double)))
            blocks[name] = (rp, ci, va)
        return SeparatedStiffnessSparse(aa, bb, blocks)

    def _pcg(self, sep, r_a_vector, u_b_vector, max_iter, block):
        r_a = np.ascontiguousarray(r_a_vector, dtype=np.float64)
        u_b = None if u_b_vector is None else np.ascontiguousarray(u_b_vector, dtype=np.float64)
        _require(r_a.shape == (sep.n_aa,) and (u_b is None or u_b.shape == (sep.n_bb,)),
                 f"r_a must hold {sep.n_aa} values and u_b {sep.n_bb}")
        u_a = np.zeros(sep.n_aa)
        it = c_int(0)
        self._check(self._L.fem_gpu_solve_pcg(self._h, ptr(r_a, c_double), None if u_b is None else ptr(u_b, c_double),
                                              int(block), int(max_iter), ptr(u_a, c_double), ctypes.byref(it)))
        return u_a, it.value

    def find_ua_vector_iterative_pcg_jacobi_sparse(self, sep, r_a_vector, u_b_vector, max_iter):
        """find_ua_vector_iterative_pcg_jacobi_sparse (methods_for_global_analysis.rs:189-233) on the GPU, for the
        separation `sep` of this model's last separate_stiffness_matrix_sparse_iterative: (u_a, iterations)"""
        return self._pcg(sep, r_a_vector, u_b_vector, max_iter, False)

    def find_ua_vector_iterative_pcg_block_jacobi_sparse(self, sep, r_a_vector, u_b_vector, max_iter):
        """find_ua_vector_iterative_pcg_block_jacobi_sparse (methods_for_global_analysis.rs:235-275): node blocks"""
        return self._pcg(sep, r_a_vector, u_b_vector, max_iter, True)

    def find_r_r_vector_sparse(self, sep, u_a_vector, u_b_vector):
        """find_r_r_vector_sparse (methods_for_global_analysis.rs:293-330): reactions K_ba u_a + K_bb u_b - r_b"""
        u_a = np.ascontiguousarray(u_a_vector, dtype=np.float64)
        u_b = np.ascontiguousarray(u_b_vector, dtype=np.float64)
        _require(u_a.shape == (sep.n_aa,) and u_b.shape == (sep.n_bb,),
                 f"u_a must hold {sep.n_aa} values and u_b {sep.n_bb}")
        r_b = np.ascontiguousarray(self.forces_vector()[np.asarray(sep.k_bb_indexes, np.int64)])
        r_r = np.zeros(sep.n_bb)
        self._check(self._L.fem_gpu_reactions(self._h, ptr(u_a, c_double), ptr(u_b, c_double), ptr(r_b, c_double),
                                              ptr(r_r, c_double)))
        return r_r

    # -- global and element results ------------------------------------------------
    TRUSS_COMPONENTS = ("ForceR",)
    BEAM_COMPONENTS = ("ForceR", "ForceS", "ForceT", "MomentR", "MomentS", "MomentS", "MomentS", "MomentT", "MomentT",
                       "MomentT")
    PLATE_COMPONENTS = ("MembraneForceR", "MembraneForceS", "MembraneForceRS", "BendingMomentR", "BendingMomentS",
                        "BendingMomentRS", "ShearForceRT", "ShearForceST")

    def compose_global_analysis_result(self, k_aa_indexes, k_bb_indexes, u_a_vector, r_r_vector) -> None:
        """compose_global_analysis_result (methods_for_global_analysis.rs:334-359): the free DOFs' displacements
        into the displacements vector, the reactions into the forces vector at the restrained DOFs"""
        self._imposed()
        forces = self.forces_vector()
        self._displacements[np.asarray(k_aa_indexes, np.int64)] = np.asarray(u_a_vector, dtype=np.float64)
        forces[np.asarray(k_bb_indexes, np.int64)] = np.asarray(r_r_vector, dtype=np.float64)
        self._result_forces = forces

    def displacements_vector(self):
        """the displacements vector (6 * nodes_number): imposed values, then the solution once composed"""
        self._imposed()
        return self._displacements.copy()

    def extract_global_analysis_result(self):
        """extract_global_analysis_result (methods_for_global_analysis.rs:361-387): (node number, DOF, displacement,
        load) for every DOF of every node, in node index order"""
        self._imposed()
        forces = getattr(self, "_result_forces", None)
        if forces is None:
            forces = self.forces_vector()
        numbers = self.index_node_numbers().astype(np.int64)
        n = 6 * len(numbers)
        return list(zip(np.repeat(numbers, 6).tolist(), list(self.DOF_PARAMETERS) * len(numbers),
                        self._displacements[:n].tolist(), np.asarray(forces[:n], np.float64).tolist()))

    def element_results(self, displacements=None, out=None):
        """Every element's results on the GPU (fem_gpu_element_results) from `displacements` (default: this
        model's displacements vector): {"truss": (n, 1), "beam": (n, 10), "plate": (n, 8)} in call order, the
        components in the order of TRUSS_COMPONENTS, BEAM_COMPONENTS (MomentS and MomentT at node 1, average, node
        2) and PLATE_COMPONENTS.  `out` may supply the three C-contiguous float64 arrays (e.g. in pinned memory)."""
        if displacements is None:
            self._imposed()
            displacements = self._displacements
        disp = np.ascontiguousarray(displacements, dtype=np.float64).ravel()
        nt, nb, np_ = self.element_counts()
        if out is None:
            out = {"truss": np.zeros((nt, 1)), "beam": np.zeros((nb, 10)), "plate": np.zeros((np_, 8))}
        for k, shape in (("truss", (nt, 1)), ("beam", (nb, 10)), ("plate", (np_, 8))):
            a = out[k]
            if a.shape != shape or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"out[{k!r}] must be a C-contiguous float64 array of shape {shape}")
        self._check(self._L.fem_gpu_element_results(self._h, ptr(disp, c_double), disp.size,
                                                    ptr(out["truss"], c_double), ptr(out["beam"], c_double),
                                                    ptr(out["plate"], c_double)))
        return out

    def element_results_device(self, displacements, truss_out, beam_out, plate_out) -> None:
        """fem_gpu_element_results_device on device pointers (ints), asynchronous on the model's stream"""
        self._check(self._L.fem_gpu_element_results_device(self._h, displacements, truss_out, beam_out, plate_out))

    def results_last_ms(self) -> float:
        x = c_float(0)
        self._check(self._L.fem_gpu_results_last_ms(self._h, ctypes.byref(x)))
        return x.value

    def element_numbers(self, kind: str):
        """element numbers of one kind ("truss", "beam", "plate") in call order"""
        k = ("truss", "beam", "plate").index(kind)
        out = np.zeros(self.element_counts()[k], np.uint32)
        self._check(self._L.fem_gpu_get_element_numbers(self._h, k, ptr(out, c_uint32)))
        return out

    def extract_elements_analysis_result(self):
        """extract_elements_analysis_result (methods_for_element_analysis.rs:27-58): (element number,
        [(component, value), ...]) for the trusses, then the beams, then the plates, each in call order"""
        res = self.element_results()
        out = []
        for kind, names in (("truss", self.TRUSS_COMPONENTS), ("beam", self.BEAM_COMPONENTS),
                            ("plate", self.PLATE_COMPONENTS)):
            rows = np.asarray(res[kind], np.float64).reshape(-1, len(names)).tolist()
            out.extend((number, list(zip(names, row)))
                       for number, row in zip(np.asarray(self.element_numbers(kind), np.int64).tolist(), rows))
        return out

    def vjp_last_ms(self) -> float:
        x = c_float(0)
        self._check(self._L.fem_gpu_vjp_last_ms(self._h, ctypes.byref(x)))
        return x.value

    def last_numeric_timing(self):
        """(element kernels ms, reduction ms) of the last numeric pass, CUDA events on the handle's stream."""
        a, b = c_float(0), c_float(0)
        self._check(self._L.fem_gpu_last_numeric_timing(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value


class SeparatedStiffnessSparse:
    """SeparatedStiffnessMatrixSparse (structs/separated_stiffness_matrix_sparse.rs): the free (a) and restrained (b)
    DOF index lists and the four blocks as CSR (row_ptr, col_idx, values) with local indices."""
    BLOCKS = ("k_aa", "k_ab", "k_ba", "k_bb")

    def __init__(self, k_aa_indexes, k_bb_indexes, blocks):
        self.k_aa_indexes, self.k_bb_indexes, self.blocks = k_aa_indexes, k_bb_indexes, blocks
        self.n_aa, self.n_bb = len(k_aa_indexes), len(k_bb_indexes)

    def triplets(self, name):
        """the block as (row, column, value) arrays, row-major order"""
        rp, ci, va = self.blocks[name]
        return np.repeat(np.arange(len(rp) - 1), np.diff(rp)), ci.astype(np.int64), va


class Batch:
    """Many independent, assembled `FEM` models assembled together in one numeric pass (one CUDA graph launch).

    The models must stay alive and keep their topology; model i's CSR pattern is its own
    (`models[i].stiffness_csr()`), the batch supplies its values (`values(i)`)."""

    def __init__(self, models):
        self._L = _lib.load()
        self.models = list(models)
        arr = (c_void_p * len(self.models))(*[m.handle for m in self.models])
        h = c_void_p()
        st = self._L.fem_gpu_batch_create(arr, len(self.models), ctypes.byref(h))
        self._h = h
        if st:
            msg = self._L.fem_gpu_batch_last_error(h).decode() if h else f"status {st}"
            self.close()
            raise FEMError(st, msg)

    @classmethod
    def from_meshes(cls, meshes, rel_tol: float, abs_tol: float, nodes_number=None, library=None) -> "Batch":
        """One batch standing for `FEM(rel_tol, abs_tol, n)` + add_nodes + add_trusses + add_beams +
        add_plates + assemble per mesh (fem_gpu_batch_create_from_arrays): the checks of every mesh run in
        bulk on the GPU, one symbolic phase covers all meshes and one graph launch assembles them.
        `nodes_number` (per mesh, or one value for all) defaults to each mesh's node count.  A failing mesh raises its first
        failing call's error, the message prefixed by "structure i: "."""
        return cls.from_structures(cls.structures(meshes, nodes_number), rel_tol, abs_tol, library)

    @classmethod
    def from_structures(cls, structures, rel_tol: float, abs_tol: float, library=None) -> "Batch":
        """The batch of `Batch.structures(...)` (the arrays of many meshes laid out one after another)."""
        st, _keep = structures
        self = cls.__new__(cls)
        self._L = library if library is not None else _lib.load()
        self.models = None
        h = c_void_p()
        code = self._L.fem_gpu_batch_create_from_arrays(rel_tol, abs_tol, ctypes.byref(st), ctypes.byref(h))
        self._h = h
        if code:
            msg = self._L.fem_gpu_batch_last_error(h).decode() if h else f"status {code}"
            self.close()
            raise FEMError(code, msg)
        return self

    @staticmethod
    def structures(meshes, nodes_number=None):
        """The host arrays of many meshes laid out one after another, as fem_gpu_structures_t: returns the
        ctypes structure and the arrays it points into (keep both alive while it is used)."""
        S = len(meshes)
        keep = []

        def arr(a, dt, shape=None):
            a = np.ascontiguousarray(a, dtype=dt)
            if shape is not None:
                a = a.reshape(shape)
            keep.append(a)
            return a

        def cat(parts, dt, width=None):
            parts = [np.asarray(x, dtype=dt).reshape(-1) for x in parts]
            return arr(np.concatenate(parts) if parts else np.zeros(0, dt), dt)

        def offsets(counts):
            return arr(np.concatenate([[0], np.cumsum(counts)]), np.uintp)

        for m in meshes:
            if tuple(k for k in m.order if getattr(m, k) is not None) != tuple(
                    k for k in ("trusses", "beams", "plates") if getattr(m, k) is not None):
                raise ValueError("a batch adds each mesh's trusses, then beams, then plates")
        nn = [m.nodes_number for m in meshes]
        room = np.asarray(nn if nodes_number is None else nodes_number)
        if room.ndim == 0:
            room = np.full(S, room)
        if room.shape != (S,):
            raise ValueError(f"nodes_number: one value or one per mesh ({S}), got shape {room.shape}")
        cap = arr(room, np.uint32)
        st = _lib.Structures()
        st.n_structures = S
        st.nodes_number = ptr(cap, c_uint32)
        st.node_off = ptr(offsets(nn), ctypes.c_size_t)
        st.node_numbers = ptr(cat([m.node_numbers for m in meshes], np.uint32), c_uint32)
        st.xyz = ptr(cat([m.xyz for m in meshes], np.float64), c_double)

        def part(m, kind):
            d = getattr(m, kind)
            return d if d is not None and len(d["numbers"]) else None

        def count(m, kind):
            d = part(m, kind)
            return 0 if d is None else len(d["numbers"])

        def col(kind, key, width=1, fill=None):
            out = []
            for m in meshes:
                d = part(m, kind)
                if d is None:
                    continue
                v = d.get(key)
                if v is None:
                    v = np.full(len(d["numbers"]) * width, fill)
                out.append(np.broadcast_to(np.asarray(v, np.float64), (len(d["numbers"]),) if width == 1 else
                                           (len(d["numbers"]), width)).reshape(-1))
            return cat(out, np.float64)

        if any(count(m, "trusses") for m in meshes):
            st.truss_off = ptr(offsets([count(m, "trusses") for m in meshes]), ctypes.c_size_t)
            st.truss_numbers = ptr(cat([part(m, "trusses")["numbers"] for m in meshes if part(m, "trusses")],
                                       np.uint32), c_uint32)
            st.truss_nodes = ptr(cat([part(m, "trusses")["nodes"] for m in meshes if part(m, "trusses")], np.uint32),
                                 c_uint32)
            st.truss_young = ptr(col("trusses", "young"), c_double)
            st.truss_area = ptr(col("trusses", "area"), c_double)
            st.truss_area2 = ptr(col("trusses", "area_2", fill=np.nan), c_double)
        if any(count(m, "beams") for m in meshes):
            st.beam_off = ptr(offsets([count(m, "beams") for m in meshes]), ctypes.c_size_t)
            st.beam_numbers = ptr(cat([part(m, "beams")["numbers"] for m in meshes if part(m, "beams")], np.uint32),
                                  c_uint32)
            st.beam_nodes = ptr(cat([part(m, "beams")["nodes"] for m in meshes if part(m, "beams")], np.uint32),
                                c_uint32)
            for field, key in (("beam_young", "young"), ("beam_poisson", "poisson"), ("beam_area", "area"),
                               ("beam_i11", "i11"), ("beam_i22", "i22"), ("beam_i12", "i12"), ("beam_it", "it"),
                               ("beam_shear_factor", "shear_factor")):
                setattr(st, field, ptr(col("beams", key), c_double))
            st.beam_local_axis = ptr(col("beams", "axis", width=3), c_double)
        if any(count(m, "plates") for m in meshes):
            st.plate_off = ptr(offsets([count(m, "plates") for m in meshes]), ctypes.c_size_t)
            st.plate_numbers = ptr(cat([part(m, "plates")["numbers"] for m in meshes if part(m, "plates")],
                                       np.uint32), c_uint32)
            st.plate_nodes = ptr(cat([part(m, "plates")["nodes"] for m in meshes if part(m, "plates")], np.uint32),
                                 c_uint32)
            for field, key in (("plate_young", "young"), ("plate_poisson", "poisson"),
                               ("plate_thickness", "thickness"), ("plate_shear_factor", "shear_factor")):
                setattr(st, field, ptr(col("plates", key), c_double))
        return st, keep

    def build_ms(self):
        """host times (ms from the start) at the end of the phases of a batch built from arrays: nodes,
        trusses, beams, plates uploaded and checked, checks read, symbolic + first numeric pass,
        per-structure CSR offsets, graph captured"""
        out = np.zeros(8)
        self._check(self._L.fem_gpu_batch_build_ms(self._h, ptr(out, c_double), 8))
        return out

    def __len__(self) -> int:
        n = ctypes.c_size_t(0)
        self._check(self._L.fem_gpu_batch_size(self._h, ctypes.byref(n)))
        return n.value

    def csr_sizes(self, i):
        rows, nnz = c_int64(0), c_int64(0)
        self._check(self._L.fem_gpu_batch_get_csr_sizes(self._h, i, ctypes.byref(rows), ctypes.byref(nnz)))
        return rows.value, nnz.value

    def csr(self, i, row_ptr=None, col_idx=None, values=None):
        """Structure i's CSR (row_ptr, col_idx, values) as its own plain assembly gives it; pass
        arrays (for instance pinned ones) to receive it in place."""
        rows, nnz = self.csr_sizes(i)
        rp = np.zeros(rows + 1, np.int64) if row_ptr is None else row_ptr
        ci = np.zeros(max(nnz, 1), np.int32) if col_idx is None else col_idx
        va = np.zeros(max(nnz, 1), np.float64) if values is None else values
        self._check(self._L.fem_gpu_batch_get_csr(self._h, i, ptr(rp, c_int64), ptr(ci, c_int32),
                                                  ptr(va, c_double)))
        return rp, ci[:nnz], va[:nnz]

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.fem_gpu_batch_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st:
            raise FEMError(st, self._L.fem_gpu_batch_last_error(self._h).decode())

    def assemble(self):
        self._check(self._L.fem_gpu_batch_assemble(self._h))

    def assemble_async(self):
        self._check(self._L.fem_gpu_batch_assemble_async(self._h))

    def values(self, i):
        _, nnz = self.csr_sizes(i)
        out = np.zeros(max(nnz, 1), np.float64)
        self._check(self._L.fem_gpu_batch_get_values(self._h, i, ptr(out, c_double)))
        return out[:nnz]

    def stream(self) -> int:
        s = c_void_p()
        self._check(self._L.fem_gpu_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def last_ms(self) -> float:
        x = c_float(0)
        self._check(self._L.fem_gpu_batch_last_ms(self._h, ctypes.byref(x)))
        return x.value

    def autotune(self, reps=5, cache_path=None):
        """Time the candidate launch configurations, keep the fastest; returns the JSON table (dict)."""
        import json

        buf = ctypes.create_string_buffer(1 << 16)
        self._check(self._L.fem_gpu_batch_autotune(self._h, reps, cache_path.encode() if cache_path else None, buf,
                                                   len(buf)))
        return json.loads(buf.value.decode())

    def configure(self, persistent, block, ctas_per_sm, tile_truss, tile_beam, tile_plate, sum_block):
        self._check(self._L.fem_gpu_batch_configure(self._h, int(persistent), block, ctas_per_sm, tile_truss,
                                                    tile_beam, tile_plate, sum_block))
