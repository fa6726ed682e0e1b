//! finite_element_method_gb300 -- the `FEM` element/assembly API of the crate
//! `finite_element_method` 0.9.12, backed by the GB300 (sm_103a) CUDA library
//! `libfem_gpu.so` through its C ABI (`include/fem_gpu.h`, raw declarations in
//! [`ffi`]).
//!
//! Method names, argument order and `Result<_, String>` errors follow the
//! reference:
//!
//! | here | reference |
//! |---|---|
//! | [`FEM::create`] | `FEM::create` (src/fem/fem.rs:34) |
//! | [`FEM::add_node`] | `add_node` (src/fem/methods_for_node_data_handle.rs:66) |
//! | [`FEM::add_truss`] | `add_truss` (src/fem/methods_for_truss_data_handle.rs:49) |
//! | [`FEM::add_beam`] | `add_beam` (src/fem/methods_for_beam_data_handle.rs:49) |
//! | [`FEM::add_plate`] | `add_plate` (src/fem/methods_for_plate_data_handle.rs:62) |
//! | [`FEM::get_truss_rotation_matrix_elements`] and the beam / plate forms | src/fem/fem.rs:171-202 |
//!
//! The reference assembles eagerly inside every `add_*`; here `add_*` checks the
//! element exactly as the reference does (same checks, same order, same
//! messages; a failing element leaves the model unchanged) and records it, and
//! [`FEM::assemble`] builds the global stiffness on the GPU in one pass.  The
//! stiffness is returned as CSR (`row_ptr`, `col_idx`, `values`), the pattern
//! being the reference's key set and the values its per-key sums in element
//! call order.  Everything is `f64`; there is no CPU fallback: without a CUDA
//! device the calls that need one fail with the library's message.
//!
//! Beyond the reference: bulk `add_*s` forms (arrays in call order, stopping at
//! the first failing item like a loop of single calls), [`FEM::vjp`], the
//! adjoint vector-Jacobian product in the role of a `torch.autograd.Function`
//! backward, and [`Batch`], many structures assembled together.

pub mod ffi;

use std::ffi::CStr;
use std::os::raw::c_int;
use std::ptr;

/// The global stiffness in CSR form (`n_rows` = 6 * nodes_number).
#[derive(Debug, Clone, PartialEq)]
pub struct Csr {
    pub row_ptr: Vec<i64>,
    pub col_idx: Vec<i32>,
    pub values: Vec<f64>,
}

/// Gradients of F = -sum_p lambda_p^T K u_p (see [`FEM::vjp`]).
#[derive(Debug, Clone, PartialEq)]
pub struct Vjp {
    /// per truss in call order: dF/dE, dF/dA, dF/dA2
    pub truss: Vec<[f64; 3]>,
    /// per beam: dF/dE, dF/dA, dF/dI11, dF/dI22, dF/dIt
    pub beam: Vec<[f64; 5]>,
    /// per plate: dF/dE, dF/dthickness
    pub plate: Vec<[f64; 2]>,
    /// per node in index (insertion) order: dF/dx, dF/dy, dF/dz
    pub xyz: Vec<[f64; 3]>,
}

/// One model: nodes, elements and their global stiffness on the GPU.
pub struct FEM {
    h: *mut ffi::FemGpu,
    nodes_number: u32,
}

// The handle owns its device memory and one CUDA stream; it may move between
// threads but is not shared (&mut self on every mutating call, as the reference).
unsafe impl Send for FEM {}

impl FEM {
    /// `FEM::create(rel_tol, abs_tol, nodes_number)`.  Allocates nothing on the
    /// device until the first `add_*`.
    pub fn create(rel_tol: f64, abs_tol: f64, nodes_number: u32) -> Self {
        let mut h = ptr::null_mut();
        let st = unsafe { ffi::fem_gpu_create(rel_tol, abs_tol, nodes_number, &mut h) };
        assert!(st == 0 && !h.is_null(), "fem_gpu_create failed with status {st}");
        FEM { h, nodes_number }
    }

    fn check(&self, st: c_int) -> Result<(), String> {
        if st == 0 {
            return Ok(());
        }
        let msg = unsafe { CStr::from_ptr(ffi::fem_gpu_last_error(self.h)) };
        Err(msg.to_string_lossy().into_owned())
    }

    pub fn nodes_number(&self) -> u32 {
        self.nodes_number
    }

    /// `add_node(number, x, y, z)`: node index = insertion order, DOFs 6 * index + {X..ThZ}.
    pub fn add_node(&mut self, number: u32, x: f64, y: f64, z: f64) -> Result<(), String> {
        self.add_nodes(&[number], &[[x, y, z]]).map(|_| ())
    }

    /// Bulk `add_node` in call order; stops at the first failure (earlier nodes stay added).
    pub fn add_nodes(&mut self, numbers: &[u32], xyz: &[[f64; 3]]) -> Result<usize, String> {
        assert_eq!(numbers.len(), xyz.len());
        let mut n = 0usize;
        let st = unsafe {
            ffi::fem_gpu_add_nodes(self.h, numbers.as_ptr(), xyz.as_ptr() as *const f64, numbers.len(), &mut n)
        };
        self.check(st).map(|_| n)
    }

    /// `add_truss(number, node_1_number, node_2_number, young_modulus, area, optional_area_2)`.
    pub fn add_truss(
        &mut self,
        number: u32,
        node_1_number: u32,
        node_2_number: u32,
        young_modulus: f64,
        area: f64,
        optional_area_2: Option<f64>,
    ) -> Result<(), String> {
        let a2 = optional_area_2.map(|a| vec![a]);
        self.add_trusses(&[number], &[[node_1_number, node_2_number]], &[young_modulus], &[area], a2.as_deref())
            .map(|_| ())
    }

    /// Bulk `add_truss`; `area_2` None means no second area for every truss (a NaN entry means none for that one).
    pub fn add_trusses(
        &mut self,
        numbers: &[u32],
        nodes: &[[u32; 2]],
        young_modulus: &[f64],
        area: &[f64],
        area_2: Option<&[f64]>,
    ) -> Result<usize, String> {
        let m = numbers.len();
        assert!(nodes.len() == m && young_modulus.len() == m && area.len() == m);
        let a2 = area_2.map_or(ptr::null(), |a| {
            assert_eq!(a.len(), m);
            a.as_ptr()
        });
        let mut n = 0usize;
        let st = unsafe {
            ffi::fem_gpu_add_trusses(
                self.h,
                numbers.as_ptr(),
                nodes.as_ptr() as *const u32,
                young_modulus.as_ptr(),
                area.as_ptr(),
                a2,
                m,
                &mut n,
            )
        };
        self.check(st).map(|_| n)
    }

    /// `add_beam(number, node_1_number, node_2_number, young_modulus, poisson_ratio, area, i11, i22, i12, it,
    /// shear_factor, local_axis_1_direction)`.
    #[allow(clippy::too_many_arguments)]
    pub fn add_beam(
        &mut self,
        number: u32,
        node_1_number: u32,
        node_2_number: u32,
        young_modulus: f64,
        poisson_ratio: f64,
        area: f64,
        i11: f64,
        i22: f64,
        i12: f64,
        it: f64,
        shear_factor: f64,
        local_axis_1_direction: [f64; 3],
    ) -> Result<(), String> {
        let b = BeamSection { young_modulus, poisson_ratio, area, i11, i22, i12, it, shear_factor, local_axis_1_direction };
        self.add_beams(&[number], &[[node_1_number, node_2_number]], &[b]).map(|_| ())
    }

    /// Bulk `add_beam` in call order.
    pub fn add_beams(&mut self, numbers: &[u32], nodes: &[[u32; 2]], sections: &[BeamSection]) -> Result<usize, String> {
        let m = numbers.len();
        assert!(nodes.len() == m && sections.len() == m);
        let col = |f: fn(&BeamSection) -> f64| sections.iter().map(f).collect::<Vec<f64>>();
        let (e, nu, a) = (col(|s| s.young_modulus), col(|s| s.poisson_ratio), col(|s| s.area));
        let (i11, i22, i12, it, k) = (col(|s| s.i11), col(|s| s.i22), col(|s| s.i12), col(|s| s.it), col(|s| s.shear_factor));
        let axis: Vec<f64> = sections.iter().flat_map(|s| s.local_axis_1_direction).collect();
        let mut n = 0usize;
        let st = unsafe {
            ffi::fem_gpu_add_beams(
                self.h,
                numbers.as_ptr(),
                nodes.as_ptr() as *const u32,
                e.as_ptr(),
                nu.as_ptr(),
                a.as_ptr(),
                i11.as_ptr(),
                i22.as_ptr(),
                i12.as_ptr(),
                it.as_ptr(),
                k.as_ptr(),
                axis.as_ptr(),
                m,
                &mut n,
            )
        };
        self.check(st).map(|_| n)
    }

    /// `add_plate(number, node_1_number, .., node_4_number, young_modulus, poisson_ratio, thickness, shear_factor)`.
    #[allow(clippy::too_many_arguments)]
    pub fn add_plate(
        &mut self,
        number: u32,
        node_1_number: u32,
        node_2_number: u32,
        node_3_number: u32,
        node_4_number: u32,
        young_modulus: f64,
        poisson_ratio: f64,
        thickness: f64,
        shear_factor: f64,
    ) -> Result<(), String> {
        self.add_plates(
            &[number],
            &[[node_1_number, node_2_number, node_3_number, node_4_number]],
            &[young_modulus],
            &[poisson_ratio],
            &[thickness],
            &[shear_factor],
        )
        .map(|_| ())
    }

    /// Bulk `add_plate` in call order.
    pub fn add_plates(
        &mut self,
        numbers: &[u32],
        nodes: &[[u32; 4]],
        young_modulus: &[f64],
        poisson_ratio: &[f64],
        thickness: &[f64],
        shear_factor: &[f64],
    ) -> Result<usize, String> {
        let m = numbers.len();
        assert!(nodes.len() == m && young_modulus.len() == m && poisson_ratio.len() == m);
        assert!(thickness.len() == m && shear_factor.len() == m);
        let mut n = 0usize;
        let st = unsafe {
            ffi::fem_gpu_add_plates(
                self.h,
                numbers.as_ptr(),
                nodes.as_ptr() as *const u32,
                young_modulus.as_ptr(),
                poisson_ratio.as_ptr(),
                thickness.as_ptr(),
                shear_factor.as_ptr(),
                m,
                &mut n,
            )
        };
        self.check(st).map(|_| n)
    }

    /// Builds the global stiffness on the GPU (pattern once per topology, then the values).
    pub fn assemble(&mut self) -> Result<(), String> {
        let st = unsafe { ffi::fem_gpu_assemble(self.h) };
        self.check(st)
    }

    /// The assembled stiffness, read back to host memory.
    pub fn stiffness_csr(&self) -> Result<Csr, String> {
        let (mut rows, mut nnz) = (0i64, 0i64);
        self.check(unsafe { ffi::fem_gpu_get_csr_sizes(self.h, &mut rows, &mut nnz) })?;
        let mut csr = Csr {
            row_ptr: vec![0; rows as usize + 1],
            col_idx: vec![0; nnz as usize],
            values: vec![0.0; nnz as usize],
        };
        let st = unsafe {
            ffi::fem_gpu_get_csr(self.h, csr.row_ptr.as_mut_ptr(), csr.col_idx.as_mut_ptr(), csr.values.as_mut_ptr())
        };
        self.check(st).map(|_| csr)
    }

    fn rotation(
        &self,
        f: unsafe extern "C" fn(*mut ffi::FemGpu, u32, *mut f64) -> c_int,
        number: u32,
    ) -> Result<[f64; 9], String> {
        let mut r = [0.0f64; 9];
        let st = unsafe { f(self.h, number, r.as_mut_ptr()) };
        self.check(st).map(|_| r)
    }

    /// `get_truss_rotation_matrix_elements(number)` (fem.rs:171).
    pub fn get_truss_rotation_matrix_elements(&self, number: u32) -> Result<[f64; 9], String> {
        self.rotation(ffi::fem_gpu_get_truss_rotation, number)
    }

    /// `get_beam_rotation_matrix_elements(number)` (fem.rs:182).
    pub fn get_beam_rotation_matrix_elements(&self, number: u32) -> Result<[f64; 9], String> {
        self.rotation(ffi::fem_gpu_get_beam_rotation, number)
    }

    /// `get_plate_rotation_matrix_elements(number)` (fem.rs:193).
    pub fn get_plate_rotation_matrix_elements(&self, number: u32) -> Result<[f64; 9], String> {
        self.rotation(ffi::fem_gpu_get_plate_rotation, number)
    }

    /// Adjoint sensitivities dF/dtheta of F = -sum_p lambda_p^T K u_p for `u`, `lam` of npairs rows of
    /// 6 * nodes_number, in the role of a `torch.autograd.Function` backward (element matrices are
    /// recomputed in forward-mode dual arithmetic, never stored).  Requires a prior [`FEM::assemble`].
    pub fn vjp(&mut self, u: &[f64], lam: &[f64], npairs: usize) -> Result<Vjp, String> {
        let ndof = 6 * self.nodes_number as usize;
        assert!(u.len() == npairs * ndof && lam.len() == npairs * ndof);
        let (mut t, mut b, mut p, mut nn) = (0i64, 0i64, 0i64, 0i64);
        self.check(unsafe { ffi::fem_gpu_get_element_counts(self.h, &mut t, &mut b, &mut p) })?;
        self.check(unsafe { ffi::fem_gpu_get_node_count(self.h, &mut nn) })?;
        let mut out = Vjp {
            truss: vec![[0.0; 3]; t as usize],
            beam: vec![[0.0; 5]; b as usize],
            plate: vec![[0.0; 2]; p as usize],
            xyz: vec![[0.0; 3]; nn as usize],
        };
        let st = unsafe {
            ffi::fem_gpu_vjp(
                self.h,
                u.as_ptr(),
                lam.as_ptr(),
                npairs as c_int,
                out.truss.as_mut_ptr() as *mut f64,
                out.beam.as_mut_ptr() as *mut f64,
                out.plate.as_mut_ptr() as *mut f64,
                out.xyz.as_mut_ptr() as *mut f64,
            )
        };
        self.check(st).map(|_| out)
    }
}

impl Drop for FEM {
    fn drop(&mut self) {
        unsafe {
            ffi::fem_gpu_destroy(self.h);
        }
    }
}

/// Many independent structures assembled together (no counterpart in the reference): built from
/// their host arrays, it stands for one `FEM::create` + `add_*` + assemble sequence per structure, with
/// the checks of all structures run in bulk on the GPU, one symbolic phase and one CUDA-graph numeric
/// pass.  Structure i's [`Csr`] is bit-identical to its plain assembly.
pub struct Batch {
    b: *mut ffi::FemGpuBatch,
}

unsafe impl Send for Batch {}

impl Batch {
    /// `structures` lays the structures out one after another (see `fem_gpu_structures_t` in
    /// include/fem_gpu.h); every pointer in it must stay valid for the call.  A failing structure
    /// returns its first failing call's message, prefixed by "structure i: ".
    pub fn from_structures(rel_tol: f64, abs_tol: f64, structures: &ffi::FemGpuStructures) -> Result<Batch, String> {
        let mut b = ptr::null_mut();
        let st = unsafe { ffi::fem_gpu_batch_create_from_arrays(rel_tol, abs_tol, structures, &mut b) };
        let batch = Batch { b };
        if st != 0 {
            return Err(batch.message());
        }
        Ok(batch)
    }

    fn message(&self) -> String {
        if self.b.is_null() {
            return "batch creation failed".to_string();
        }
        unsafe { CStr::from_ptr(ffi::fem_gpu_batch_last_error(self.b)) }.to_string_lossy().into_owned()
    }

    fn check(&self, st: c_int) -> Result<(), String> {
        if st == 0 { Ok(()) } else { Err(self.message()) }
    }

    pub fn len(&self) -> usize {
        let mut n = 0usize;
        unsafe { ffi::fem_gpu_batch_size(self.b, &mut n) };
        n
    }

    pub fn is_empty(&self) -> bool {
        self.len() == 0
    }

    /// One more numeric pass of every structure (after changed coordinates or properties are not
    /// supported: rebuild the batch).
    pub fn assemble(&mut self) -> Result<(), String> {
        let st = unsafe { ffi::fem_gpu_batch_assemble(self.b) };
        self.check(st)
    }

    /// Structure i's global stiffness, exactly as its own `FEM` would give it.
    pub fn csr(&self, i: usize) -> Result<Csr, String> {
        let (mut rows, mut nnz) = (0i64, 0i64);
        self.check(unsafe { ffi::fem_gpu_batch_get_csr_sizes(self.b, i, &mut rows, &mut nnz) })?;
        let mut csr = Csr {
            row_ptr: vec![0; rows as usize + 1],
            col_idx: vec![0; nnz as usize],
            values: vec![0.0; nnz as usize],
        };
        let st = unsafe {
            ffi::fem_gpu_batch_get_csr(self.b, i, csr.row_ptr.as_mut_ptr(), csr.col_idx.as_mut_ptr(), csr.values.as_mut_ptr())
        };
        self.check(st).map(|_| csr)
    }
}

impl Drop for Batch {
    fn drop(&mut self) {
        unsafe {
            ffi::fem_gpu_batch_destroy(self.b);
        }
    }
}

/// The section and material arguments of one `add_beam` call.
#[derive(Debug, Clone, Copy, PartialEq)]
pub struct BeamSection {
    pub young_modulus: f64,
    pub poisson_ratio: f64,
    pub area: f64,
    pub i11: f64,
    pub i22: f64,
    pub i12: f64,
    pub it: f64,
    pub shear_factor: f64,
    pub local_axis_1_direction: [f64; 3],
}
