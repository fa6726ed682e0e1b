// ffi.rs -- raw declarations of the C ABI in include/fem_gpu.h (libfem_gpu.so).
// Generated by rust/gen_ffi.py from the header; do not edit by hand.
#![allow(non_camel_case_types, dead_code)]

use std::os::raw::{c_char, c_int, c_void};

/// The library's model handle (`fem_gpu_t`): opaque, owned through `FEM`.
#[repr(C)]
pub struct FemGpu {
    _opaque: [u8; 0],
}

/// A batch of structures (`fem_gpu_batch_t`): opaque.
#[repr(C)]
pub struct FemGpuBatch {
    _opaque: [u8; 0],
}

/// `fem_gpu_structures_t`: plain data, laid out as the C struct.
#[repr(C)]
pub struct FemGpuStructures {
    pub n_structures: usize,
    pub nodes_number: *const u32,
    pub node_off: *const usize,
    pub node_numbers: *const u32,
    pub xyz: *const f64,
    pub truss_off: *const usize,
    pub truss_numbers: *const u32,
    pub truss_nodes: *const u32,
    pub truss_young: *const f64,
    pub truss_area: *const f64,
    pub truss_area2: *const f64,
    pub beam_off: *const usize,
    pub beam_numbers: *const u32,
    pub beam_nodes: *const u32,
    pub beam_young: *const f64,
    pub beam_poisson: *const f64,
    pub beam_area: *const f64,
    pub beam_i11: *const f64,
    pub beam_i22: *const f64,
    pub beam_i12: *const f64,
    pub beam_it: *const f64,
    pub beam_shear_factor: *const f64,
    pub beam_local_axis: *const f64,
    pub plate_off: *const usize,
    pub plate_numbers: *const u32,
    pub plate_nodes: *const u32,
    pub plate_young: *const f64,
    pub plate_poisson: *const f64,
    pub plate_thickness: *const f64,
    pub plate_shear_factor: *const f64,
}

unsafe extern "C" {
    pub fn fem_gpu_create(rel_tol: f64, abs_tol: f64, nodes_number: u32, out: *mut *mut FemGpu) -> c_int;
    pub fn fem_gpu_destroy(h: *mut FemGpu) -> c_int;
    pub fn fem_gpu_last_error(h: *const FemGpu) -> *const c_char;
    pub fn fem_gpu_add_nodes(h: *mut FemGpu, numbers: *const u32, xyz: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_add_trusses(h: *mut FemGpu, numbers: *const u32, nodes: *const u32, young: *const f64, area: *const f64, area2: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_add_beams(h: *mut FemGpu, numbers: *const u32, nodes: *const u32, young: *const f64, poisson: *const f64, area: *const f64, i11: *const f64, i22: *const f64, i12: *const f64, it: *const f64, shear_factor: *const f64, local_axis: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_add_plates(h: *mut FemGpu, numbers: *const u32, nodes: *const u32, young: *const f64, poisson: *const f64, thickness: *const f64, shear_factor: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_assemble(h: *mut FemGpu) -> c_int;
    pub fn fem_gpu_assemble_to_host(h: *mut FemGpu, row_ptr: *mut i64, col_idx: *mut i32, values: *mut f64, nnz_capacity: i64, nnz: *mut i64) -> c_int;
    pub fn fem_gpu_assemble_numeric_async(h: *mut FemGpu) -> c_int;
    pub fn fem_gpu_check_pattern(h: *mut FemGpu) -> c_int;
    pub fn fem_gpu_set_node_coordinates(h: *mut FemGpu, xyz: *const f64, n_nodes: usize) -> c_int;
    pub fn fem_gpu_set_plate_properties(h: *mut FemGpu, young: *const f64, poisson: *const f64, thickness: *const f64, shear_factor: *const f64, n: usize) -> c_int;
    pub fn fem_gpu_get_csr_sizes(h: *mut FemGpu, n_rows: *mut i64, nnz: *mut i64) -> c_int;
    pub fn fem_gpu_get_csr(h: *mut FemGpu, row_ptr: *mut i64, col_idx: *mut i32, values: *mut f64) -> c_int;
    pub fn fem_gpu_get_csr_values(h: *mut FemGpu, values: *mut f64) -> c_int;
    pub fn fem_gpu_get_csr_device(h: *mut FemGpu, row_ptr: *mut *const i64, col_idx: *mut *const i32, values: *mut *const f64) -> c_int;
    pub fn fem_gpu_get_node_count(h: *mut FemGpu, n_nodes: *mut i64) -> c_int;
    pub fn fem_gpu_get_index_node_numbers(h: *mut FemGpu, numbers: *mut u32) -> c_int;
    pub fn fem_gpu_get_group_count(h: *mut FemGpu, n_groups: *mut i64) -> c_int;
    pub fn fem_gpu_get_groups(h: *mut FemGpu, row_node: *mut i32, col_node: *mut i32, kind: *mut u8, nnz_group: *mut i32) -> c_int;
    pub fn fem_gpu_get_truss_rotation(h: *mut FemGpu, number: u32, r9: *mut f64) -> c_int;
    pub fn fem_gpu_get_beam_rotation(h: *mut FemGpu, number: u32, r9: *mut f64) -> c_int;
    pub fn fem_gpu_get_plate_rotation(h: *mut FemGpu, number: u32, r9: *mut f64) -> c_int;
    pub fn fem_gpu_get_element_counts(h: *mut FemGpu, n_truss: *mut i64, n_beam: *mut i64, n_plate: *mut i64) -> c_int;
    pub fn fem_gpu_get_stream(h: *mut FemGpu, stream: *mut *mut c_void) -> c_int;
    pub fn fem_gpu_numeric_launch_count(h: *mut FemGpu, n_launches: *mut c_int) -> c_int;
    pub fn fem_gpu_debug_check(checked: *mut c_int, site: *mut c_int, index: *mut i64, bound: *mut i64) -> c_int;
    pub fn fem_gpu_get_pattern_stats(h: *mut FemGpu, n_blocks: *mut i64, n_contributions: *mut i64, scratch_doubles: *mut i64, sum_slots: *mut i64) -> c_int;
    pub fn fem_gpu_last_numeric_timing(h: *mut FemGpu, element_ms: *mut f32, reduce_ms: *mut f32) -> c_int;
    pub fn fem_gpu_vjp(h: *mut FemGpu, u: *const f64, lam: *const f64, npairs: c_int, g_truss: *mut f64, g_beam: *mut f64, g_plate: *mut f64, g_xyz: *mut f64) -> c_int;
    pub fn fem_gpu_vjp_last_ms(h: *mut FemGpu, ms: *mut f32) -> c_int;
    pub fn fem_gpu_batch_create(models: *const *mut FemGpu, n_models: usize, out: *mut *mut FemGpuBatch) -> c_int;
    pub fn fem_gpu_batch_destroy(b: *mut FemGpuBatch) -> c_int;
    pub fn fem_gpu_batch_last_error(b: *const FemGpuBatch) -> *const c_char;
    pub fn fem_gpu_batch_assemble(b: *mut FemGpuBatch) -> c_int;
    pub fn fem_gpu_batch_assemble_async(b: *mut FemGpuBatch) -> c_int;
    pub fn fem_gpu_batch_get_values(b: *mut FemGpuBatch, i: usize, values: *mut f64) -> c_int;
    pub fn fem_gpu_batch_get_values_device(b: *mut FemGpuBatch, i: usize, values: *mut *const f64) -> c_int;
    pub fn fem_gpu_batch_get_stream(b: *mut FemGpuBatch, stream: *mut *mut c_void) -> c_int;
    pub fn fem_gpu_batch_last_ms(b: *mut FemGpuBatch, ms: *mut f32) -> c_int;
    pub fn fem_gpu_batch_autotune(b: *mut FemGpuBatch, reps: c_int, cache_path: *const c_char, summary: *mut c_char, cap: usize) -> c_int;
    pub fn fem_gpu_batch_create_from_arrays(rel_tol: f64, abs_tol: f64, structures: *const FemGpuStructures, out: *mut *mut FemGpuBatch) -> c_int;
    pub fn fem_gpu_batch_build_ms(b: *const FemGpuBatch, ms: *mut f64, n: usize) -> c_int;
    pub fn fem_gpu_batch_size(b: *const FemGpuBatch, n_structures: *mut usize) -> c_int;
    pub fn fem_gpu_batch_get_csr_sizes(b: *mut FemGpuBatch, i: usize, n_rows: *mut i64, nnz: *mut i64) -> c_int;
    pub fn fem_gpu_batch_get_csr(b: *mut FemGpuBatch, i: usize, row_ptr: *mut i64, col_idx: *mut i32, values: *mut f64) -> c_int;
    pub fn fem_gpu_batch_configure(b: *mut FemGpuBatch, persistent: c_int, block: c_int, ctas_per_sm: c_int, tile_truss: c_int, tile_beam: c_int, tile_plate: c_int, sum_block: c_int) -> c_int;
    pub fn fem_gpu_add_concentrated_loads(h: *mut FemGpu, node_numbers: *const u32, dofs: *const u8, values: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_add_line_loads(h: *mut FemGpu, beam_numbers: *const u32, dofs: *const u8, values: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_add_surface_loads(h: *mut FemGpu, plate_numbers: *const u32, dofs: *const u8, values: *const f64, n: usize, n_added: *mut usize) -> c_int;
    pub fn fem_gpu_get_forces(h: *mut FemGpu, forces: *mut f64) -> c_int;
    pub fn fem_gpu_get_forces_device(h: *mut FemGpu, forces: *mut *const f64) -> c_int;
    pub fn fem_gpu_separate_sparse(h: *mut FemGpu, imposed: *const u8) -> c_int;
    pub fn fem_gpu_get_separation_sizes(h: *mut FemGpu, n_aa: *mut i64, n_bb: *mut i64, nnz4: *mut i64) -> c_int;
    pub fn fem_gpu_get_separation_indexes(h: *mut FemGpu, aa_indexes: *mut i64, bb_indexes: *mut i64) -> c_int;
    pub fn fem_gpu_get_separation_block(h: *mut FemGpu, which: c_int, row_ptr: *mut i64, col_idx: *mut i32, values: *mut f64) -> c_int;
    pub fn fem_gpu_get_separation_block_device(h: *mut FemGpu, which: c_int, row_ptr: *mut *const i64, col_idx: *mut *const i32, values: *mut *const f64) -> c_int;
    pub fn fem_gpu_solve_pcg(h: *mut FemGpu, r_a: *const f64, u_b: *const f64, block_jacobi: c_int, max_iter: c_int, u_a: *mut f64, iterations: *mut c_int) -> c_int;
    pub fn fem_gpu_reactions(h: *mut FemGpu, u_a: *const f64, u_b: *const f64, r_b: *const f64, r_r: *mut f64) -> c_int;
    pub fn fem_gpu_element_results(h: *mut FemGpu, displacements: *const f64, n_displacements: usize, truss_out: *mut f64, beam_out: *mut f64, plate_out: *mut f64) -> c_int;
    pub fn fem_gpu_element_results_device(h: *mut FemGpu, displacements: *const f64, truss_out: *mut f64, beam_out: *mut f64, plate_out: *mut f64) -> c_int;
    pub fn fem_gpu_results_last_ms(h: *mut FemGpu, ms: *mut f32) -> c_int;
    pub fn fem_gpu_get_element_numbers(h: *mut FemGpu, kind: c_int, numbers: *mut u32) -> c_int;
    pub fn fem_gpu_release_cached_memory() -> c_int;
    pub fn fem_gpu_assemble_dense_noalloc(n_nodes: u32, xyz: *const f64, n_truss: usize, truss_nodes: *const i32, truss_props: *const f64, n_beam: usize, beam_nodes: *const i32, beam_props: *const f64, n_plate: usize, plate_nodes: *const i32, plate_props: *const f64, rel_tol: f64, abs_tol: f64, K: *mut f64, stream: *mut c_void) -> c_int;
}
