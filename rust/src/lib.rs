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
//! | [`FEM::reset`] | `reset` (src/fem/fem.rs:154-168) |
//! | [`FEM::add_node`] | `add_node` (src/fem/methods_for_node_data_handle.rs:66) |
//! | [`FEM::add_truss`] | `add_truss` (src/fem/methods_for_truss_data_handle.rs:49) |
//! | [`FEM::add_beam`] | `add_beam` (src/fem/methods_for_beam_data_handle.rs:49) |
//! | [`FEM::add_plate`] | `add_plate` (src/fem/methods_for_plate_data_handle.rs:62) |
//! | [`FEM::get_truss_rotation_matrix_elements`] and the beam / plate forms | src/fem/fem.rs:171-202 |
//! | [`FEM::add_displacement`], [`FEM::add_concentrated_load`], [`FEM::add_uniformly_distributed_line_load`], [`FEM::add_uniformly_distributed_surface_load`] | src/fem/methods_for_bc_data_handle.rs:34-203 |
//! | [`FEM::separate_stiffness_matrix_sparse_iterative`], [`FEM::compose_r_a_vector`], [`FEM::compose_u_b_vector`] | src/fem/methods_for_separate_stiffness_matrix.rs:217-342 |
//! | [`FEM::find_ua_vector_iterative_pcg_jacobi_sparse`], [`FEM::find_ua_vector_iterative_pcg_block_jacobi_sparse`], [`FEM::find_r_r_vector_sparse`], [`FEM::compose_global_analysis_result`], [`FEM::extract_global_analysis_result`] | src/fem/methods_for_global_analysis.rs:189-387 |
//! | [`FEM::extract_elements_analysis_result`] | src/fem/methods_for_element_analysis.rs:27-58 |
//!
//! The separation, the solution, the reactions and the element results run on the GPU; the crate's
//! `Vector<V>` is a `Vec<f64>` here.  Where the crate walks a `HashMap` (the nodes in
//! `extract_global_analysis_result`, the elements in `extract_elements_analysis_result`) the order here
//! is insertion order.
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
//! backward, and [`Batch`], many structures assembled together (their calls
//! recorded in a [`Structures`]: one `create` + `add_*` sequence each).

pub mod ffi;

use std::collections::HashMap;
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
    rel_tol: f64,
    abs_tol: f64,
    /// the nodes_number of create: the crate's props keep it through a reset
    node_limit: u32,
    /// the reference's imposed_constraints: one flag per DOF (6 * nodes_number)
    imposed: Vec<u8>,
    /// the reference's displacements_vector: imposed values, then the solution once composed
    displacements: Vec<f64>,
    /// the forces vector with the reactions at the restrained DOFs, after compose_global_analysis_result
    result_forces: Option<Vec<f64>>,
    /// node number -> node index, for the nodes looked up so far (nodes are only ever appended)
    node_index: HashMap<u32, usize>,
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
        let ndof = 6 * nodes_number as usize;
        FEM {
            h,
            nodes_number,
            rel_tol,
            abs_tol,
            node_limit: nodes_number,
            imposed: vec![0; ndof],
            displacements: vec![0.0; ndof],
            result_forces: None,
            node_index: HashMap::new(),
        }
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

    /// `reset(nodes_number)` (fem.rs:154-168): drops every node, element, load and imposed displacement and
    /// sizes the stiffness, forces and displacements for `nodes_number` nodes (a new handle).  As in the
    /// crate, the tolerances and the node limit stay those of create: `add_node` refuses the node past the
    /// nodes_number given at creation even after a reset to more.  After a reset to fewer nodes the node
    /// past the new count is refused; the crate would accept it with its DOFs outside the matrix.
    pub fn reset(&mut self, nodes_number: u32) {
        let mut h = ptr::null_mut();
        let st = unsafe { ffi::fem_gpu_create(self.rel_tol, self.abs_tol, nodes_number, &mut h) };
        assert!(st == 0 && !h.is_null(), "fem_gpu_create failed with status {st}");
        unsafe {
            ffi::fem_gpu_destroy(self.h);
        }
        let ndof = 6 * nodes_number as usize;
        self.h = h;
        self.nodes_number = nodes_number;
        self.imposed = vec![0; ndof];
        self.displacements = vec![0.0; ndof];
        self.result_forces = None;
        self.node_index.clear();
    }

    /// `add_node(number, x, y, z)`: node index = insertion order, DOFs 6 * index + {X..ThZ}.
    pub fn add_node(&mut self, number: u32, x: f64, y: f64, z: f64) -> Result<(), String> {
        self.add_nodes(&[number], &[[x, y, z]]).map(|_| ())
    }

    /// Bulk `add_node` in call order; stops at the first failure (earlier nodes stay added).
    pub fn add_nodes(&mut self, numbers: &[u32], xyz: &[[f64; 3]]) -> Result<usize, String> {
        assert_eq!(numbers.len(), xyz.len());
        let mut m = numbers.len();
        if self.node_limit < self.nodes_number {
            // reset to more nodes than at creation: the limit of create holds
            let mut count = 0i64;
            self.check(unsafe { ffi::fem_gpu_get_node_count(self.h, &mut count) })?;
            m = m.min((self.node_limit as i64 - count).max(0) as usize);
        }
        let mut n = 0usize;
        if m > 0 {
            let st = unsafe { ffi::fem_gpu_add_nodes(self.h, numbers.as_ptr(), xyz.as_ptr() as *const f64, m, &mut n) };
            self.check(st)?;
        }
        if m < numbers.len() {
            return Err(format!("Nodes number could not be greater than {}!", self.node_limit));
        }
        Ok(n)
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

    /// [`FEM::assemble`] with the stiffness read back into `csr`: on a new topology the pattern travels back
    /// while the symbolic phase finishes and the values are computed, then the values follow.  `csr`'s
    /// vectors are resized to fit (a call whose buffers turn out too small is repeated once with room, the
    /// pattern being kept).  Returns nnz.
    pub fn assemble_to_host(&mut self, csr: &mut Csr) -> Result<usize, String> {
        csr.row_ptr.resize(6 * self.nodes_number as usize + 1, 0);
        for _ in 0..2 {
            let cap = csr.col_idx.len().min(csr.values.len());
            let mut nnz = 0i64;
            let st = unsafe {
                ffi::fem_gpu_assemble_to_host(
                    self.h,
                    csr.row_ptr.as_mut_ptr(),
                    csr.col_idx.as_mut_ptr(),
                    csr.values.as_mut_ptr(),
                    cap as i64,
                    &mut nnz,
                )
            };
            let nnz = nnz as usize;
            if st == 0 {
                csr.col_idx.truncate(nnz);
                csr.values.truncate(nnz);
                return Ok(nnz);
            }
            if nnz <= cap {
                return Err(self.check(st).unwrap_err());
            }
            csr.col_idx.resize(nnz, 0);
            csr.values.resize(nnz, 0.0);
        }
        Err("the stiffness did not fit the buffers twice".to_string())
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

    // -- boundary conditions, loads, solution and results (the callers either side of the assembly) --

    /// The node index of a node number (None: no such node).  Nodes are only appended, so the map is
    /// extended with the nodes added since the last lookup.
    fn node_index_of(&mut self, number: u32) -> Result<Option<usize>, String> {
        let mut count = 0i64;
        self.check(unsafe { ffi::fem_gpu_get_node_count(self.h, &mut count) })?;
        let count = count as usize;
        if self.node_index.len() < count {
            let mut numbers = vec![0u32; count];
            self.check(unsafe { ffi::fem_gpu_get_index_node_numbers(self.h, numbers.as_mut_ptr()) })?;
            let known = self.node_index.len();
            for (i, n) in numbers.iter().enumerate().skip(known) {
                self.node_index.insert(*n, i);
            }
        }
        Ok(self.node_index.get(&number).copied())
    }

    /// `add_displacement(node_number, dof_parameter, value)` (methods_for_bc_data_handle.rs:176-203):
    /// imposes a displacement on one DOF; a DOF takes one imposed displacement.
    pub fn add_displacement(&mut self, node_number: u32, dof_parameter: DOFParameter, value: f64) -> Result<(), String> {
        let index = match self.node_index_of(node_number)? {
            Some(i) => 6 * i + dof_parameter as usize,
            None => return Err(format!("Node with number {node_number} does not exist!")),
        };
        if self.imposed[index] != 0 {
            return Err(format!("Displacement {dof_parameter:?} already applied to node {node_number}!"));
        }
        self.imposed[index] = 1;
        self.displacements[index] = value;
        Ok(())
    }

    fn load(
        &mut self,
        f: unsafe extern "C" fn(*mut ffi::FemGpu, *const u32, *const u8, *const f64, usize, *mut usize) -> c_int,
        number: u32,
        dof_parameter: DOFParameter,
        value: f64,
    ) -> Result<(), String> {
        let (dof, mut n) = (dof_parameter as u8, 0usize);
        let st = unsafe { f(self.h, &number, &dof, &value, 1, &mut n) };
        self.check(st)
    }

    /// `add_concentrated_load(node_number, dof_parameter, value)` (methods_for_bc_data_handle.rs:34-56).
    pub fn add_concentrated_load(&mut self, node_number: u32, dof_parameter: DOFParameter, value: f64) -> Result<(), String> {
        self.load(ffi::fem_gpu_add_concentrated_loads, node_number, dof_parameter, value)
    }

    /// `add_uniformly_distributed_line_load(beam_element_number, dof_parameter, value)`
    /// (methods_for_bc_data_handle.rs:58-101): the beam's equivalent nodal loads, from its geometry now.
    pub fn add_uniformly_distributed_line_load(
        &mut self,
        beam_element_number: u32,
        dof_parameter: DOFParameter,
        value: f64,
    ) -> Result<(), String> {
        self.load(ffi::fem_gpu_add_line_loads, beam_element_number, dof_parameter, value)
    }

    /// `add_uniformly_distributed_surface_load(plate_element_number, dof_parameter, value)`
    /// (methods_for_bc_data_handle.rs:103-175).
    pub fn add_uniformly_distributed_surface_load(
        &mut self,
        plate_element_number: u32,
        dof_parameter: DOFParameter,
        value: f64,
    ) -> Result<(), String> {
        self.load(ffi::fem_gpu_add_surface_loads, plate_element_number, dof_parameter, value)
    }

    /// The forces vector (6 * nodes_number, DOF order): every load's nodal contributions in call order.
    pub fn forces_vector(&self) -> Result<Vec<f64>, String> {
        let mut f = vec![0.0f64; 6 * self.nodes_number as usize];
        self.check(unsafe { ffi::fem_gpu_get_forces(self.h, f.as_mut_ptr()) })?;
        Ok(f)
    }

    /// `separate_stiffness_matrix_sparse_iterative()` (methods_for_separate_stiffness_matrix.rs:217-320) of
    /// the assembled stiffness, on the GPU: K_aa, K_ab, K_ba, K_bb as triplets in (row, column) order.  The
    /// blocks also stay with the model for the solution calls below, until its next assembly.
    pub fn separate_stiffness_matrix_sparse_iterative(&self) -> Result<SeparatedStiffnessMatrixSparse, String> {
        self.check(unsafe { ffi::fem_gpu_separate_sparse(self.h, self.imposed.as_ptr()) })?;
        let (mut n_aa, mut n_bb, mut nnz) = (0i64, 0i64, [0i64; 4]);
        self.check(unsafe { ffi::fem_gpu_get_separation_sizes(self.h, &mut n_aa, &mut n_bb, nnz.as_mut_ptr()) })?;
        let (n_aa, n_bb) = (n_aa as usize, n_bb as usize);
        let (mut aa, mut bb) = (vec![0i64; n_aa], vec![0i64; n_bb]);
        self.check(unsafe { ffi::fem_gpu_get_separation_indexes(self.h, aa.as_mut_ptr(), bb.as_mut_ptr()) })?;
        let mut blocks: Vec<Vec<(usize, usize, f64)>> = Vec::with_capacity(4);
        for which in 0..4usize {
            let rows = if which < 2 { n_aa } else { n_bb };
            let mut row_ptr = vec![0i64; rows + 1];
            let mut col_idx = vec![0i32; nnz[which] as usize];
            let mut values = vec![0.0f64; nnz[which] as usize];
            let st = unsafe {
                ffi::fem_gpu_get_separation_block(
                    self.h,
                    which as c_int,
                    row_ptr.as_mut_ptr(),
                    col_idx.as_mut_ptr(),
                    values.as_mut_ptr(),
                )
            };
            self.check(st)?;
            let mut t = Vec::with_capacity(values.len());
            for r in 0..rows {
                for k in row_ptr[r] as usize..row_ptr[r + 1] as usize {
                    t.push((r, col_idx[k] as usize, values[k]));
                }
            }
            blocks.push(t);
        }
        let k_bb_triplets = blocks.pop().unwrap_or_default();
        let k_ba_triplets = blocks.pop().unwrap_or_default();
        let k_ab_triplets = blocks.pop().unwrap_or_default();
        let k_aa_triplets = blocks.pop().unwrap_or_default();
        Ok(SeparatedStiffnessMatrixSparse {
            k_aa_indexes: aa.iter().map(|&i| i as usize).collect(),
            k_bb_indexes: bb.iter().map(|&i| i as usize).collect(),
            k_aa_triplets,
            k_ab_triplets,
            k_ba_triplets,
            k_bb_triplets,
            n_aa,
            n_bb,
        })
    }

    /// `compose_r_a_vector(k_aa_indexes)` (methods_for_separate_stiffness_matrix.rs:322-331): the forces at
    /// the free DOFs.
    pub fn compose_r_a_vector(&self, k_aa_indexes: &Vec<usize>) -> Result<Vec<f64>, String> {
        let f = self.forces_vector()?;
        Ok(k_aa_indexes.iter().map(|&i| f[i]).collect())
    }

    /// `compose_u_b_vector(k_bb_indexes)` (methods_for_separate_stiffness_matrix.rs:333-342): the imposed
    /// displacements at the restrained DOFs.
    pub fn compose_u_b_vector(&self, k_bb_indexes: &Vec<usize>) -> Result<Vec<f64>, String> {
        Ok(k_bb_indexes.iter().map(|&i| self.displacements[i]).collect())
    }

    fn pcg(
        &self,
        sep: &SeparatedStiffnessMatrixSparse,
        r_a_vector: &Vec<f64>,
        u_b_vector: &Vec<f64>,
        max_iter: usize,
        block_jacobi: bool,
    ) -> Result<(Vec<f64>, usize), String> {
        if r_a_vector.len() != sep.n_aa || u_b_vector.len() != sep.n_bb {
            return Err("r_a / u_b vector sizes do not match the separation".to_string());
        }
        let mut u_a = vec![0.0f64; sep.n_aa];
        let mut iterations: c_int = 0;
        let st = unsafe {
            ffi::fem_gpu_solve_pcg(
                self.h,
                r_a_vector.as_ptr(),
                u_b_vector.as_ptr(),
                block_jacobi as c_int,
                max_iter.min(c_int::MAX as usize) as c_int,
                u_a.as_mut_ptr(),
                &mut iterations,
            )
        };
        self.check(st).map(|_| (u_a, iterations as usize))
    }

    /// `find_ua_vector_iterative_pcg_jacobi_sparse(separated_stiffness_matrix_sparse, r_a_vector,
    /// u_b_vector, max_iter)` (methods_for_global_analysis.rs:189-233) on the GPU: (u_a, iterations).  The
    /// separation must be this model's latest.
    pub fn find_ua_vector_iterative_pcg_jacobi_sparse(
        &self,
        separated_stiffness_matrix_sparse: &SeparatedStiffnessMatrixSparse,
        r_a_vector: &Vec<f64>,
        u_b_vector: &Vec<f64>,
        max_iter: usize,
    ) -> Result<(Vec<f64>, usize), String> {
        self.pcg(separated_stiffness_matrix_sparse, r_a_vector, u_b_vector, max_iter, false)
    }

    /// `find_ua_vector_iterative_pcg_block_jacobi_sparse(...)` (methods_for_global_analysis.rs:235-275): the
    /// node blocks of K_aa as preconditioner.
    pub fn find_ua_vector_iterative_pcg_block_jacobi_sparse(
        &self,
        separated_stiffness_matrix_sparse: &SeparatedStiffnessMatrixSparse,
        r_a_vector: &Vec<f64>,
        u_b_vector: &Vec<f64>,
        max_iter: usize,
    ) -> Result<(Vec<f64>, usize), String> {
        self.pcg(separated_stiffness_matrix_sparse, r_a_vector, u_b_vector, max_iter, true)
    }

    /// `find_r_r_vector_sparse(sep, u_a_vector, u_b_vector)` (methods_for_global_analysis.rs:306-330): the
    /// reactions K_ba u_a + K_bb u_b - r_b at the restrained DOFs.
    pub fn find_r_r_vector_sparse(
        &self,
        sep: &SeparatedStiffnessMatrixSparse,
        u_a_vector: &Vec<f64>,
        u_b_vector: &Vec<f64>,
    ) -> Result<Vec<f64>, String> {
        if u_a_vector.len() != sep.n_aa || u_b_vector.len() != sep.n_bb {
            return Err("u_a / u_b vector sizes do not match the separation".to_string());
        }
        let f = self.forces_vector()?;
        let r_b: Vec<f64> = sep.k_bb_indexes.iter().map(|&i| f[i]).collect();
        let mut r_r = vec![0.0f64; sep.n_bb];
        let st = unsafe {
            ffi::fem_gpu_reactions(self.h, u_a_vector.as_ptr(), u_b_vector.as_ptr(), r_b.as_ptr(), r_r.as_mut_ptr())
        };
        self.check(st).map(|_| r_r)
    }

    /// `compose_global_analysis_result(k_aa_indexes, k_bb_indexes, u_a_vector, r_r_vector)`
    /// (methods_for_global_analysis.rs:335-359): the free DOFs' displacements into the displacements
    /// vector, the reactions into the forces vector at the restrained DOFs.
    pub fn compose_global_analysis_result(
        &mut self,
        k_aa_indexes: &[usize],
        k_bb_indexes: &[usize],
        u_a_vector: &Vec<f64>,
        r_r_vector: &Vec<f64>,
    ) -> Result<(), String> {
        if u_a_vector.len() != k_aa_indexes.len() || r_r_vector.len() != k_bb_indexes.len() {
            return Err("u_a / r_r vector sizes do not match the index lists".to_string());
        }
        let mut forces = self.forces_vector()?;
        for (k, &i) in k_aa_indexes.iter().enumerate() {
            self.displacements[i] = u_a_vector[k];
        }
        for (k, &i) in k_bb_indexes.iter().enumerate() {
            forces[i] = r_r_vector[k];
        }
        self.result_forces = Some(forces);
        Ok(())
    }

    /// `extract_global_analysis_result()` (methods_for_global_analysis.rs:361-387): (node number, DOF,
    /// displacement, load) for every DOF of every node, in node index (insertion) order.
    pub fn extract_global_analysis_result(&self) -> Result<Vec<(u32, DOFParameter, f64, f64)>, String> {
        let forces = match &self.result_forces {
            Some(f) => f.clone(),
            None => self.forces_vector()?,
        };
        let mut count = 0i64;
        self.check(unsafe { ffi::fem_gpu_get_node_count(self.h, &mut count) })?;
        let mut numbers = vec![0u32; count as usize];
        self.check(unsafe { ffi::fem_gpu_get_index_node_numbers(self.h, numbers.as_mut_ptr()) })?;
        let mut out = Vec::with_capacity(6 * numbers.len());
        for (i, &number) in numbers.iter().enumerate() {
            for p in 0..6usize {
                out.push((number, DOFParameter::from_usize(p), self.displacements[6 * i + p], forces[6 * i + p]));
            }
        }
        Ok(out)
    }

    /// `extract_elements_analysis_result()` (methods_for_element_analysis.rs:27-58) on the GPU, from the
    /// displacements vector: (element number, [(component, value), ...]) for the trusses, then the beams,
    /// then the plates, each in call order.
    pub fn extract_elements_analysis_result(&self) -> Result<Vec<(u32, Vec<(ElementForceComponent, f64)>)>, String> {
        use ElementForceComponent::*;
        let (mut t, mut b, mut p) = (0i64, 0i64, 0i64);
        self.check(unsafe { ffi::fem_gpu_get_element_counts(self.h, &mut t, &mut b, &mut p) })?;
        let (t, b, p) = (t as usize, b as usize, p as usize);
        let (mut truss, mut beam, mut plate) = (vec![0.0f64; t], vec![0.0f64; 10 * b], vec![0.0f64; 8 * p]);
        let st = unsafe {
            ffi::fem_gpu_element_results(
                self.h,
                self.displacements.as_ptr(),
                self.displacements.len(),
                truss.as_mut_ptr(),
                beam.as_mut_ptr(),
                plate.as_mut_ptr(),
            )
        };
        self.check(st)?;
        let kinds: [(usize, &[ElementForceComponent], &Vec<f64>); 3] = [
            (t, &[ForceR], &truss),
            (b, &[ForceR, ForceS, ForceT, MomentR, MomentS, MomentS, MomentS, MomentT, MomentT, MomentT], &beam),
            (
                p,
                &[MembraneForceR, MembraneForceS, MembraneForceRS, BendingMomentR, BendingMomentS, BendingMomentRS,
                  ShearForceRT, ShearForceST],
                &plate,
            ),
        ];
        let mut out = Vec::with_capacity(t + b + p);
        for (kind, (n, names, values)) in kinds.iter().enumerate() {
            let mut numbers = vec![0u32; *n];
            self.check(unsafe { ffi::fem_gpu_get_element_numbers(self.h, kind as c_int, numbers.as_mut_ptr()) })?;
            let w = names.len();
            for (e, &number) in numbers.iter().enumerate() {
                out.push((number, names.iter().copied().zip(values[w * e..w * (e + 1)].iter().copied()).collect()));
            }
        }
        Ok(out)
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

    /// The batch of the structures whose calls `structures` recorded (see [`Structures`]).  The call is
    /// synchronous: nothing reads the recorded arrays after it returns.
    pub fn from_calls(rel_tol: f64, abs_tol: f64, structures: &mut Structures) -> Result<Batch, String> {
        let layout = structures.layout();
        Batch::from_structures(rel_tol, abs_tol, &layout)
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

    /// One more numeric pass of every structure.  The structures' coordinates and properties are those
    /// recorded at creation; for changed ones, build a new batch.
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

/// `DOFParameter` (methods_for_bc_data_handle.rs:7-29): a node's six degrees of freedom in DOF order.
#[derive(Debug, Clone, Copy, PartialEq, Eq, PartialOrd, Ord, Hash)]
#[repr(u8)]
pub enum DOFParameter {
    X = 0,
    Y = 1,
    Z = 2,
    ThX = 3,
    ThY = 4,
    ThZ = 5,
}

impl DOFParameter {
    pub fn from_usize(number: usize) -> Self {
        match number {
            0 => DOFParameter::X,
            1 => DOFParameter::Y,
            2 => DOFParameter::Z,
            3 => DOFParameter::ThX,
            4 => DOFParameter::ThY,
            5 => DOFParameter::ThZ,
            _ => panic!("Incorrect dof parameter number!"),
        }
    }
}

/// `ElementForceComponent` (methods_for_element_analysis.rs:6-21).
#[derive(Debug, Clone, Copy, PartialEq, Eq, PartialOrd, Ord, Hash)]
pub enum ElementForceComponent {
    ForceR,
    ForceS,
    ForceT,
    MembraneForceR,
    MembraneForceS,
    MembraneForceRS,
    ShearForceRT,
    ShearForceST,
    MomentR,
    MomentS,
    MomentT,
    BendingMomentR,
    BendingMomentS,
    BendingMomentRS,
}

/// `SeparatedStiffnessMatrixSparse` (structs/separated_stiffness_matrix_sparse.rs): the free (a) and
/// restrained (b) DOF lists and the four blocks as (local row, local column, value) triplets.
#[derive(Debug, Clone, PartialEq)]
pub struct SeparatedStiffnessMatrixSparse {
    k_aa_indexes: Vec<usize>,
    k_bb_indexes: Vec<usize>,
    k_aa_triplets: Vec<(usize, usize, f64)>,
    k_ab_triplets: Vec<(usize, usize, f64)>,
    k_ba_triplets: Vec<(usize, usize, f64)>,
    k_bb_triplets: Vec<(usize, usize, f64)>,
    n_aa: usize,
    n_bb: usize,
}

impl SeparatedStiffnessMatrixSparse {
    pub fn get_k_aa_indexes(&self) -> &Vec<usize> {
        &self.k_aa_indexes
    }

    pub fn get_k_bb_indexes(&self) -> &Vec<usize> {
        &self.k_bb_indexes
    }

    pub fn get_k_aa_triplets(&self) -> &Vec<(usize, usize, f64)> {
        &self.k_aa_triplets
    }

    pub fn get_k_ab_triplets(&self) -> &Vec<(usize, usize, f64)> {
        &self.k_ab_triplets
    }

    pub fn get_k_ba_triplets(&self) -> &Vec<(usize, usize, f64)> {
        &self.k_ba_triplets
    }

    pub fn get_k_bb_triplets(&self) -> &Vec<(usize, usize, f64)> {
        &self.k_bb_triplets
    }

    pub fn get_n_aa(&self) -> usize {
        self.n_aa
    }

    pub fn get_n_bb(&self) -> usize {
        self.n_bb
    }
}

/// The calls of many plain sequences, recorded for one [`Batch`]: [`Structures::create`] starts a
/// structure (the `FEM::create(rel_tol, abs_tol, nodes_number)` of its sequence), then its `add_node`,
/// `add_truss`, `add_beam` and `add_plate` calls follow with the reference's arguments.  The batch applies
/// each structure's calls as its sequence would, kind by kind: nodes, trusses, beams, plates, each kind in
/// call order.
#[derive(Debug, Clone, Default)]
pub struct Structures {
    nodes_number: Vec<u32>,
    /// per structure: nodes, trusses, beams, plates
    counts: Vec<[usize; 4]>,
    node_numbers: Vec<u32>,
    xyz: Vec<f64>,
    truss_numbers: Vec<u32>,
    truss_nodes: Vec<u32>,
    truss_young: Vec<f64>,
    truss_area: Vec<f64>,
    /// NaN: no second area
    truss_area2: Vec<f64>,
    beam_numbers: Vec<u32>,
    beam_nodes: Vec<u32>,
    /// young, poisson, area, i11, i22, i12, it, shear_factor
    beam_props: [Vec<f64>; 8],
    beam_axis: Vec<f64>,
    plate_numbers: Vec<u32>,
    plate_nodes: Vec<u32>,
    /// young, poisson, thickness, shear_factor
    plate_props: [Vec<f64>; 4],
    /// per kind, the structures' offsets (made by `layout`)
    offsets: [Vec<usize>; 4],
}

impl Structures {
    pub fn new() -> Self {
        Self::default()
    }

    /// Starts the next structure: the `FEM::create(rel_tol, abs_tol, nodes_number)` of its sequence.
    pub fn create(&mut self, nodes_number: u32) {
        self.nodes_number.push(nodes_number);
        self.counts.push([0; 4]);
    }

    fn count(&mut self, kind: usize) -> &mut usize {
        let c = self.counts.last_mut().expect("Structures::create starts a structure");
        &mut c[kind]
    }

    pub fn add_node(&mut self, number: u32, x: f64, y: f64, z: f64) {
        *self.count(0) += 1;
        self.node_numbers.push(number);
        self.xyz.extend_from_slice(&[x, y, z]);
    }

    pub fn add_truss(
        &mut self,
        number: u32,
        node_1_number: u32,
        node_2_number: u32,
        young_modulus: f64,
        area: f64,
        optional_area_2: Option<f64>,
    ) {
        *self.count(1) += 1;
        self.truss_numbers.push(number);
        self.truss_nodes.extend_from_slice(&[node_1_number, node_2_number]);
        self.truss_young.push(young_modulus);
        self.truss_area.push(area);
        self.truss_area2.push(optional_area_2.unwrap_or(f64::NAN));
    }

    pub fn add_beam(&mut self, number: u32, node_1_number: u32, node_2_number: u32, section: &BeamSection) {
        *self.count(2) += 1;
        self.beam_numbers.push(number);
        self.beam_nodes.extend_from_slice(&[node_1_number, node_2_number]);
        let s = section;
        let values = [s.young_modulus, s.poisson_ratio, s.area, s.i11, s.i22, s.i12, s.it, s.shear_factor];
        for (column, v) in self.beam_props.iter_mut().zip(values) {
            column.push(v);
        }
        self.beam_axis.extend_from_slice(&s.local_axis_1_direction);
    }

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
    ) {
        *self.count(3) += 1;
        self.plate_numbers.push(number);
        self.plate_nodes.extend_from_slice(&[node_1_number, node_2_number, node_3_number, node_4_number]);
        for (column, v) in self.plate_props.iter_mut().zip([young_modulus, poisson_ratio, thickness, shear_factor]) {
            column.push(v);
        }
    }

    /// Structures recorded so far.
    pub fn len(&self) -> usize {
        self.counts.len()
    }

    pub fn is_empty(&self) -> bool {
        self.counts.is_empty()
    }

    /// The C layout (`fem_gpu_structures_t`): offsets from the per-structure counts, pointers into this
    /// builder's arrays, valid while the builder is neither changed nor dropped; kinds without elements
    /// are NULL.
    fn layout(&mut self) -> ffi::FemGpuStructures {
        for kind in 0..4 {
            let mut off = Vec::with_capacity(self.counts.len() + 1);
            let mut run = 0usize;
            off.push(run);
            for c in &self.counts {
                run += c[kind];
                off.push(run);
            }
            self.offsets[kind] = off;
        }
        fn p<T>(v: &[T]) -> *const T {
            if v.is_empty() { ptr::null() } else { v.as_ptr() }
        }
        let has = |n: &Vec<u32>, off: &Vec<usize>| if n.is_empty() { ptr::null() } else { off.as_ptr() };
        ffi::FemGpuStructures {
            n_structures: self.counts.len(),
            nodes_number: p(&self.nodes_number),
            node_off: self.offsets[0].as_ptr(),
            node_numbers: p(&self.node_numbers),
            xyz: p(&self.xyz),
            truss_off: has(&self.truss_numbers, &self.offsets[1]),
            truss_numbers: p(&self.truss_numbers),
            truss_nodes: p(&self.truss_nodes),
            truss_young: p(&self.truss_young),
            truss_area: p(&self.truss_area),
            truss_area2: p(&self.truss_area2),
            beam_off: has(&self.beam_numbers, &self.offsets[2]),
            beam_numbers: p(&self.beam_numbers),
            beam_nodes: p(&self.beam_nodes),
            beam_young: p(&self.beam_props[0]),
            beam_poisson: p(&self.beam_props[1]),
            beam_area: p(&self.beam_props[2]),
            beam_i11: p(&self.beam_props[3]),
            beam_i22: p(&self.beam_props[4]),
            beam_i12: p(&self.beam_props[5]),
            beam_it: p(&self.beam_props[6]),
            beam_shear_factor: p(&self.beam_props[7]),
            beam_local_axis: p(&self.beam_axis),
            plate_off: has(&self.plate_numbers, &self.offsets[3]),
            plate_numbers: p(&self.plate_numbers),
            plate_nodes: p(&self.plate_nodes),
            plate_young: p(&self.plate_props[0]),
            plate_poisson: p(&self.plate_props[1]),
            plate_thickness: p(&self.plate_props[2]),
            plate_shear_factor: p(&self.plate_props[3]),
        }
    }
}
