/*
 * fem_gpu.h -- C ABI of the GB300 (sm_103a) element-stiffness-and-assembly
 * library.  Drop-in for the eager assembly path of the Rust crate
 * `finite_element_method` 0.9.12:
 *
 *   FEM::create(rel_tol, abs_tol, nodes_number)   src/fem/fem.rs:34-65
 *   FEM::add_node                                  src/fem/methods_for_node_data_handle.rs:66-79
 *   FEM::add_truss                                 src/fem/methods_for_truss_data_handle.rs:49-128
 *   FEM::add_beam                                  src/fem/methods_for_beam_data_handle.rs:49-142
 *   FEM::add_plate                                 src/fem/methods_for_plate_data_handle.rs:62-217
 *   FEM.stiffness_matrix (read by the separation)  src/fem/fem.rs:17, :71-73
 *   get_{truss,beam,plate}_rotation_matrix_elements src/fem/fem.rs:171-202
 *
 * The reference assembles eagerly inside each add_*; here add_* validates the
 * element on the GPU (same checks, same messages, same "first failure wins,
 * model unchanged by the failing element" behaviour) and records it, and
 * fem_gpu_assemble() builds the CSR global stiffness in one pass.  Results are
 * the reference's: the CSR pattern is the set of (row, col) that received a
 * non-zero element contribution, values are summed per entry in element call
 * order.  Everything is FP64.
 *
 * Conventions: every function returns 0 on success or a FEM_GPU_* code; the
 * message of the last failure is fem_gpu_last_error(h).  A handle owns its
 * device buffers and one CUDA stream; it is not thread-safe.  Host pointers are
 * plain host memory (pinned or pageable); *_device getters return device
 * pointers owned by the handle, valid until the next call that changes the
 * model.  No CPU fallback exists: without a CUDA device every call that needs
 * one returns FEM_GPU_ERR_CUDA.
 */
#ifndef FEM_GPU_H
#define FEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fem_gpu fem_gpu_t;

enum {
  FEM_GPU_OK = 0,
  FEM_GPU_ERR_NODE_LIMIT = 1,      /* "Nodes number could not be greater than N!" */
  FEM_GPU_ERR_NODE_NUMBER = 2,     /* "Node with number N already exists!" */
  FEM_GPU_ERR_NODE_INDEX = 3,
  FEM_GPU_ERR_NODE_COORDS = 4,     /* "Node with coordinates x: .., y: .., z: .. already exists!" */
  FEM_GPU_ERR_NODE_NOT_EXIST = 5,  /* "Node with number N does not exist!" */
  FEM_GPU_ERR_ELEM_NUMBER = 6,     /* "<Kind> element with number N already exists!" */
  FEM_GPU_ERR_ELEM_SAME_NODES = 7,
  FEM_GPU_ERR_YOUNG = 8,
  FEM_GPU_ERR_POISSON = 9,
  FEM_GPU_ERR_AREA = 10,
  FEM_GPU_ERR_AREA2 = 11,
  FEM_GPU_ERR_I11 = 12,
  FEM_GPU_ERR_I22 = 13,
  FEM_GPU_ERR_IT = 14,
  FEM_GPU_ERR_SHEAR_FACTOR = 15,
  FEM_GPU_ERR_PARALLEL_AXIS = 16,
  FEM_GPU_ERR_THICKNESS = 17,
  FEM_GPU_ERR_NODES_ON_LINE = 18,
  FEM_GPU_ERR_NOT_ON_PLANE = 19,
  FEM_GPU_ERR_NOT_CONVEX = 20,
  FEM_GPU_ERR_ZERO_LENGTH = 21,    /* two-node element whose nodes coincide */
  FEM_GPU_ERR_SEP_DISPLACEMENT = 22, /* "There are no stiffness to withstand displacement D applied to node N!" */
  FEM_GPU_ERR_SEP_NO_RESTRAINTS = 23, /* "No restraints" */
  FEM_GPU_ERR_SEP_EMPTY_KAA = 24,  /* "Sparse separation: K_aa is empty (structure has no free stiffness?)" */
  FEM_GPU_ERR_ELEM_NOT_EXIST = 25, /* "<Kind> element with number N does not exist!" */
  FEM_GPU_ERR_NOT_CONVERGED = 26,  /* fem_gpu_solve_pcg: "find_ua_vector_iterative: PCG failed: ..." */
  FEM_GPU_ERR_ARGUMENT = 30,       /* null pointer / size out of range */
  FEM_GPU_ERR_STATE = 31,          /* e.g. CSR requested before fem_gpu_assemble */
  FEM_GPU_ERR_CUDA = 40,           /* CUDA runtime failure or no device */
  FEM_GPU_ERR_OUT_OF_MEMORY = 41,
  FEM_GPU_ERR_PATTERN_CHANGED = 42, /* numeric pass saw a non-zero outside the stored pattern */
  FEM_GPU_ERR_NOALLOC_LIMIT = 43    /* fem_gpu_assemble_dense_noalloc: structure above its fixed maximum */
};

/* FEM::create (fem.rs:34).  Allocates nothing on the device until the first add. */
int fem_gpu_create(double rel_tol, double abs_tol, uint32_t nodes_number, fem_gpu_t** out);
int fem_gpu_destroy(fem_gpu_t* h);
const char* fem_gpu_last_error(const fem_gpu_t* h);

/* FEM::add_node (methods_for_node_data_handle.rs:66), n of them in order.
 * xyz is n x 3 row-major.  Stops at the first failure; *n_added (optional)
 * receives how many were added before it. */
int fem_gpu_add_nodes(fem_gpu_t* h, const uint32_t* numbers, const double* xyz, size_t n, size_t* n_added);

/* FEM::add_truss (methods_for_truss_data_handle.rs:49).  nodes is n x 2 node
 * numbers; area2 may be NULL, or hold NaN for "None" per element. */
int fem_gpu_add_trusses(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                        const double* area, const double* area2, size_t n, size_t* n_added);

/* FEM::add_beam (methods_for_beam_data_handle.rs:49); local_axis is n x 3. */
int fem_gpu_add_beams(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                      const double* poisson, const double* area, const double* i11, const double* i22,
                      const double* i12, const double* it, const double* shear_factor, const double* local_axis,
                      size_t n, size_t* n_added);

/* FEM::add_plate (methods_for_plate_data_handle.rs:62); nodes is n x 4. */
int fem_gpu_add_plates(fem_gpu_t* h, const uint32_t* numbers, const uint32_t* nodes, const double* young,
                       const double* poisson, const double* thickness, const double* shear_factor, size_t n,
                       size_t* n_added);

/* Build the global stiffness: the symbolic phase (pattern, DOF map, groups and
 * the destination map) when the element set changed, then the numeric phase.
 * Synchronous; returns after the CSR is complete on the device. */
int fem_gpu_assemble(fem_gpu_t* h);
/* fem_gpu_assemble with the CSR read back into host arrays (row_ptr 6 * nodes_number + 1, col_idx and
 * values room for nnz_capacity entries; page-locked arrays copy fastest).  The pattern goes back on a
 * second stream -- during a symbolic phase row_ptr as soon as the rows are counted and col_idx in node
 * chunks as they are filled, otherwise while the numeric pass runs -- and the values after the pass.
 * Every copy has landed when the call returns.  *nnz gets the entry count; FEM_GPU_ERR_ARGUMENT when it
 * exceeds nnz_capacity (fem_gpu_get_csr_sizes tells it after a fem_gpu_assemble). */
int fem_gpu_assemble_to_host(fem_gpu_t* h, int64_t* row_ptr, int32_t* col_idx, double* values,
                             int64_t nnz_capacity, int64_t* nnz);

/* Numeric phase only, enqueued on the handle's stream without synchronising
 * (requires a prior fem_gpu_assemble).  For timing loops and graph capture.
 * fem_gpu_check_pattern() synchronises and reports whether the last numeric
 * pass found the stored pattern still exact (0) or changed (PATTERN_CHANGED). */
int fem_gpu_assemble_numeric_async(fem_gpu_t* h);
int fem_gpu_check_pattern(fem_gpu_t* h);

/* Replace all node coordinates (index order, n_nodes x 3) / plate properties
 * (element order) without changing the topology; the next assemble reuses the
 * pattern.  Host pointers. */
int fem_gpu_set_node_coordinates(fem_gpu_t* h, const double* xyz, size_t n_nodes);
int fem_gpu_set_plate_properties(fem_gpu_t* h, const double* young, const double* poisson, const double* thickness,
                                 const double* shear_factor, size_t n);

/* CSR read-out.  n_rows = 6 * nodes_number (the reference's SquareMatrix size). */
int fem_gpu_get_csr_sizes(fem_gpu_t* h, int64_t* n_rows, int64_t* nnz);
int fem_gpu_get_csr(fem_gpu_t* h, int64_t* row_ptr, int32_t* col_idx, double* values);
int fem_gpu_get_csr_values(fem_gpu_t* h, double* values);
int fem_gpu_get_csr_device(fem_gpu_t* h, const int64_t** row_ptr, const int32_t** col_idx, const double** values);

/* DOF map: node index (insertion order) -> node number; global DOF of
 * (node, DOFParameter p) is 6 * index + p (methods_for_bc_data_handle.rs:7-14). */
int fem_gpu_get_node_count(fem_gpu_t* h, int64_t* n_nodes);
int fem_gpu_get_index_node_numbers(fem_gpu_t* h, uint32_t* numbers);

/* Stiffness groups (docs/Stiffness_groups.md): every non-empty 3x3 region
 * (kind 0 Kuu, 1 Kuth, 2 Kthu, 3 Kthth) of every node-pair block, sorted by
 * (row node, col node, kind); nnz_group[k] is the group of CSR entry k. */
int fem_gpu_get_group_count(fem_gpu_t* h, int64_t* n_groups);
int fem_gpu_get_groups(fem_gpu_t* h, int32_t* row_node, int32_t* col_node, uint8_t* kind, int32_t* nnz_group);

/* get_{truss,beam,plate}_rotation_matrix_elements (fem.rs:171-202): the 3x3
 * rotation (row-major) of element `number` of that kind. */
int fem_gpu_get_truss_rotation(fem_gpu_t* h, uint32_t number, double* r9);
int fem_gpu_get_beam_rotation(fem_gpu_t* h, uint32_t number, double* r9);
int fem_gpu_get_plate_rotation(fem_gpu_t* h, uint32_t number, double* r9);

/* Element counts, the handle's CUDA stream (cudaStream_t) and the number of
 * kernels one numeric pass launches. */
int fem_gpu_get_element_counts(fem_gpu_t* h, int64_t* n_truss, int64_t* n_beam, int64_t* n_plate);
int fem_gpu_get_stream(fem_gpu_t* h, void** stream);
int fem_gpu_numeric_launch_count(fem_gpu_t* h, int* n_launches);

/* Device-side index checks (no counterpart in the reference).  The library
 * built with -DFEM_GPU_DEBUG (lib/libfem_gpu_debug.so) checks every node
 * index, packed-scratch position, block-sum source, CSR source and CSR /
 * stiffness-group position of the assembly kernels against its array's length
 * and skips an out-of-range access instead of making it.  This waits for the
 * current device, sets *checked (1 in that build, 0 in the release build) and
 * the first failing access since the last call: *site 0 when none, else 1 node
 * index, 2 scratch write, 3 block-sum read, 4 gather read, 5 CSR entry,
 * 6 stiffness group, 7 CSR value source; *index and *bound the offending index
 * and its array's length.  Reading clears the record.  Any pointer may be NULL. */
int fem_gpu_debug_check(int* checked, int* site, int64_t* index, int64_t* bound);

/* Sizes of the stored pattern: global node-pair blocks, element node-pair
 * contributions, packed element-block entries one numeric pass writes and reads
 * (the scratch also holds one padding word per contribution of a 13-entry
 * block, written with it and never read), and packed block-sum slots the CSR
 * values are gathered from. */
int fem_gpu_get_pattern_stats(fem_gpu_t* h, int64_t* n_blocks, int64_t* n_contributions, int64_t* scratch_doubles,
                              int64_t* sum_slots);

/* Per-kernel timing of the last numeric pass, measured with CUDA events on the
 * handle's stream (milliseconds): element kernels (all types) and the reduction. */
int fem_gpu_last_numeric_timing(fem_gpu_t* h, float* element_ms, float* reduce_ms);

/* ---- vector-Jacobian product --------------------------------------------------
 * No counterpart in the reference (it has no derivatives).  For npairs (u, lambda)
 * pairs -- host arrays of npairs x (6 * nodes_number) doubles, pair-major, DOFs
 * in the stiffness's row order -- the gradient of F = -sum_p lambda_p^T K u_p:
 *   g_truss  n_truss x 3  (E, A, A2; A2 is 0 without a taper)
 *   g_beam   n_beam x 5   (E, A, I11, I22, It)
 *   g_plate  n_plate x 2  (E, thickness)
 *   g_xyz    n_nodes x 3  (node coordinates, index order)
 * i.e. dF/dtheta = -sum_p lambda_p^T (dK/dtheta) u_p, the adjoint sensitivity of
 * a compliance-type objective.  Element matrices are recomputed in forward-mode
 * dual arithmetic, one parameter per thread, and never stored.  Any output may be
 * NULL.  1 <= npairs <= 512.  Requires a prior fem_gpu_assemble. */
int fem_gpu_vjp(fem_gpu_t* h, const double* u, const double* lam, int npairs, double* g_truss, double* g_beam,
                double* g_plate, double* g_xyz);
/* device time of the last fem_gpu_vjp (transposes, element products, node sums), ms */
int fem_gpu_vjp_last_ms(fem_gpu_t* h, float* ms);

/* ---- batched assembly -------------------------------------------------------
 * No counterpart in the reference (it assembles one model per FEM value): a
 * batch assembles many independent, already assembled models in one numeric
 * pass -- one CUDA graph launch -- instead of one pass per model.  The models
 * must outlive the batch and keep their topology; their CSR patterns stay
 * theirs (fem_gpu_get_csr on model i gives row_ptr / col_idx), the batch
 * supplies the values.  Results are bit-identical to each model's own pass. */
typedef struct fem_gpu_batch fem_gpu_batch_t;
int fem_gpu_batch_create(fem_gpu_t* const* models, size_t n_models, fem_gpu_batch_t** out);
int fem_gpu_batch_destroy(fem_gpu_batch_t* b);
const char* fem_gpu_batch_last_error(const fem_gpu_batch_t* b);
/* one numeric pass of every model: synchronous (checks the exact-zero patterns) or enqueued */
int fem_gpu_batch_assemble(fem_gpu_batch_t* b);
int fem_gpu_batch_assemble_async(fem_gpu_batch_t* b);
/* CSR values of model i (its own pattern order), to host or as a device pointer */
int fem_gpu_batch_get_values(fem_gpu_batch_t* b, size_t i, double* values);
int fem_gpu_batch_get_values_device(fem_gpu_batch_t* b, size_t i, const double** values);
int fem_gpu_batch_get_stream(fem_gpu_batch_t* b, void** stream);
/* device time of the last synchronous fem_gpu_batch_assemble (CUDA events), ms */
int fem_gpu_batch_last_ms(fem_gpu_batch_t* b, float* ms);
/* Measure the candidate launch configurations (plain element launches of 64,
 * 128 or 256 threads; one persistent launch with 1 or 2 CTAs per SM and four
 * tile-size sets; reduction blocks of 128, 256, 512 threads) with `reps` graph
 * replays each, keep the fastest, write the table as JSON to cache_path (if
 * not NULL) and into summary (if not NULL, at most cap bytes). */
int fem_gpu_batch_autotune(fem_gpu_batch_t* b, int reps, const char* cache_path, char* summary, size_t cap);
/* A batch built from the host arrays of many independent structures, laid
 * out structure after structure (offset arrays of n_structures + 1 entries
 * starting at 0; element nodes are node NUMBERS of the element's structure).
 * It stands for one plain call sequence per structure --
 * fem_gpu_create(rel_tol, abs_tol, nodes_number[i]), fem_gpu_add_nodes,
 * fem_gpu_add_trusses, fem_gpu_add_beams, fem_gpu_add_plates, fem_gpu_assemble
 * -- with every check of those calls run in bulk on the GPU, one symbolic
 * phase over all structures and one CUDA-graph numeric pass.  On failure the
 * status and message are those of the structure's first failing call, the
 * message prefixed by "structure i: ".  Structure i's CSR (fem_gpu_batch_get_csr)
 * is bit-identical to its plain assembly.  truss_area2 may be NULL (no second
 * area); a NULL offset array means no element of that kind.  The call is
 * synchronous, failures included: no array is read after it returns. */
typedef struct fem_gpu_structures {
  size_t n_structures;
  const uint32_t* nodes_number; /* per structure: the nodes_number of its fem_gpu_create */
  const size_t* node_off;
  const uint32_t* node_numbers;
  const double* xyz; /* 3 per node */
  const size_t* truss_off;
  const uint32_t* truss_numbers;
  const uint32_t* truss_nodes; /* 2 per truss */
  const double* truss_young;
  const double* truss_area;
  const double* truss_area2;
  const size_t* beam_off;
  const uint32_t* beam_numbers;
  const uint32_t* beam_nodes; /* 2 per beam */
  const double* beam_young;
  const double* beam_poisson;
  const double* beam_area;
  const double* beam_i11;
  const double* beam_i22;
  const double* beam_i12;
  const double* beam_it;
  const double* beam_shear_factor;
  const double* beam_local_axis; /* 3 per beam */
  const size_t* plate_off;
  const uint32_t* plate_numbers;
  const uint32_t* plate_nodes; /* 4 per plate */
  const double* plate_young;
  const double* plate_poisson;
  const double* plate_thickness;
  const double* plate_shear_factor;
} fem_gpu_structures_t;
int fem_gpu_batch_create_from_arrays(double rel_tol, double abs_tol, const fem_gpu_structures_t* structures,
                                     fem_gpu_batch_t** out);
/* Host times of the phases of fem_gpu_batch_create_from_arrays, ms from its start at the end of each:
 * [0] nodes uploaded and checked, [1] trusses, [2] beams, [3] plates uploaded and checked, [4] the checks'
 * result read, [5] the union's symbolic phase and first numeric pass, [6] per-structure columns and row
 * starts, [7] the numeric pass captured as a graph (all 0 for a batch of models).  At most n values. */
int fem_gpu_batch_build_ms(const fem_gpu_batch_t* b, double* ms, size_t n);
/* structures (or models) in the batch, and structure i's CSR: sizes, then host copies (any may be NULL) */
int fem_gpu_batch_size(const fem_gpu_batch_t* b, size_t* n_structures);
int fem_gpu_batch_get_csr_sizes(fem_gpu_batch_t* b, size_t i, int64_t* n_rows, int64_t* nnz);
int fem_gpu_batch_get_csr(fem_gpu_batch_t* b, size_t i, int64_t* row_ptr, int32_t* col_idx, double* values);
/* apply a configuration read back from that table */
int fem_gpu_batch_configure(fem_gpu_batch_t* b, int persistent, int block, int ctas_per_sm, int tile_truss,
                            int tile_beam, int tile_plate, int sum_block);

/* ---- loads ----------------------------------------------------------------
 * add_concentrated_load, add_uniformly_distributed_line_load and
 * add_uniformly_distributed_surface_load (methods_for_bc_data_handle.rs:20-175),
 * bulk: loads in call order, stopping at the first whose node or element does
 * not exist (FEM_GPU_ERR_NODE_NOT_EXIST / FEM_GPU_ERR_ELEM_NOT_EXIST with the
 * reference's messages).  dofs[k] is the DOFParameter (0 X, 1 Y, 2 Z, 3 ThX,
 * 4 ThY, 5 ThZ).  Element loads are converted to nodal loads with the element's
 * geometry at the time of the call (beam.rs:775-797, plate.rs:1145-1185) and
 * added, like the reference's `+=`, in call order. */
int fem_gpu_add_concentrated_loads(fem_gpu_t* h, const uint32_t* node_numbers, const uint8_t* dofs,
                                   const double* values, size_t n, size_t* n_added);
int fem_gpu_add_line_loads(fem_gpu_t* h, const uint32_t* beam_numbers, const uint8_t* dofs, const double* values,
                           size_t n, size_t* n_added);
int fem_gpu_add_surface_loads(fem_gpu_t* h, const uint32_t* plate_numbers, const uint8_t* dofs, const double* values,
                              size_t n, size_t* n_added);
/* the forces vector (6 * nodes_number doubles, DOF order), to host or as a device pointer */
int fem_gpu_get_forces(fem_gpu_t* h, double* forces);
int fem_gpu_get_forces_device(fem_gpu_t* h, const double** forces);

/* ---- sparse separation ----------------------------------------------------
 * separate_stiffness_matrix_sparse_iterative (methods_for_separate_stiffness_
 * matrix.rs:217-320) of the assembled stiffness.  imposed: 6 * nodes_number
 * bytes, non-zero where a displacement is imposed (the reference's
 * imposed_constraints, set by add_displacement).  DOFs in ascending order:
 * diagonal 0 -> excluded (FEM_GPU_ERR_SEP_DISPLACEMENT if a displacement is
 * imposed on it), else restrained (b, imposed) or free (a).  Every non-zero
 * K(i, j) with both DOFs kept goes to K_aa, K_ab, K_ba or K_bb (which = 0..3)
 * with local row / column indices; each block is CSR sorted by (row, column),
 * the reference's triplets in a fixed order.  FEM_GPU_ERR_SEP_NO_RESTRAINTS
 * without restrained DOFs, FEM_GPU_ERR_SEP_EMPTY_KAA when K_aa has no entry.
 * The blocks stay on the device with the handle until the next numeric pass. */
int fem_gpu_separate_sparse(fem_gpu_t* h, const uint8_t* imposed);
/* number of free and restrained DOFs, and nnz of K_aa, K_ab, K_ba, K_bb (nnz4[4]) */
int fem_gpu_get_separation_sizes(fem_gpu_t* h, int64_t* n_aa, int64_t* n_bb, int64_t* nnz4);
/* the DOF indexes of the a and b lists (host arrays of n_aa and n_bb) */
int fem_gpu_get_separation_indexes(fem_gpu_t* h, int64_t* aa_indexes, int64_t* bb_indexes);
/* block `which` (0 K_aa, 1 K_ab, 2 K_ba, 3 K_bb) to host arrays (rows + 1, nnz, nnz) or as device pointers */
int fem_gpu_get_separation_block(fem_gpu_t* h, int which, int64_t* row_ptr, int32_t* col_idx, double* values);
int fem_gpu_get_separation_block_device(fem_gpu_t* h, int which, const int64_t** row_ptr, const int32_t** col_idx,
                                        const double** values);

/* ---- solution -------------------------------------------------------------
 * find_ua_vector_iterative_pcg_jacobi_sparse / ..._block_jacobi_sparse
 * (methods_for_global_analysis.rs:189-275) on the separation of the last
 * fem_gpu_separate_sparse: b = r_a - K_ab u_b, then K_aa u_a = b by
 * preconditioned conjugate gradients from u_a = 0 with the diagonal of K_aa
 * (block_jacobi = 0) or its node blocks (1) as preconditioner, stopping when
 * ||r||_2 <= max(rel_tol ||b||_2, abs_tol) (the handle's tolerances) or after
 * max_iter iterations (FEM_GPU_ERR_NOT_CONVERGED).  r_a: n_aa host doubles (the
 * forces at the free DOFs), u_b: n_bb (imposed displacements; NULL = 0), u_a:
 * n_aa out; *iterations: the iterations run. */
int fem_gpu_solve_pcg(fem_gpu_t* h, const double* r_a, const double* u_b, int block_jacobi, int max_iter,
                      double* u_a, int* iterations);
/* find_r_r_vector_sparse (methods_for_global_analysis.rs:100-133, :293-330): the reactions at the restrained
 * DOFs, r_r = K_ba u_a + K_bb u_b - r_b (host arrays; u_b, r_b NULL = 0) */
int fem_gpu_reactions(fem_gpu_t* h, const double* u_a, const double* u_b, const double* r_b, double* r_r);

/* ---- element results ------------------------------------------------------
 * extract_elements_analysis_result (methods_for_element_analysis.rs:27-58;
 * truss.rs:281-333, beam.rs:803-993, plate.rs:1196-1409): every element's
 * forces and moments from the displacements vector (6 per node in node index
 * order, DOF order X, Y, Z, ThX, ThY, ThZ -- the reference's
 * displacements_vector after compose_global_analysis_result).  Elements in
 * call order per kind; components in the reference's order:
 *   truss_out  n_truss x 1   ForceR
 *   beam_out   n_beam x 10   ForceR, ForceS, ForceT, MomentR, MomentS at node 1,
 *                            MomentS average, MomentS at node 2, MomentT at node 1,
 *                            MomentT average, MomentT at node 2
 *   plate_out  n_plate x 8   MembraneForceR, MembraneForceS, MembraneForceRS,
 *                            BendingMomentR, BendingMomentS, BendingMomentRS,
 *                            ShearForceRT, ShearForceST
 * A NULL output skips that kind.  Host arrays; n_displacements >= 6 * nodes
 * added.  Values are those of the reference's formulas within 1e-12 of each
 * value's magnitude scale (the sum of the absolute terms). */
int fem_gpu_element_results(fem_gpu_t* h, const double* displacements, size_t n_displacements, double* truss_out,
                            double* beam_out, double* plate_out);
/* the same on DEVICE arrays (displacements, beam_out and plate_out 16-byte aligned), launched on the handle's
 * stream without synchronising */
int fem_gpu_element_results_device(fem_gpu_t* h, const double* displacements, double* truss_out, double* beam_out,
                                   double* plate_out);
/* device time (CUDA events on the handle's stream) of the last element-results launch */
int fem_gpu_results_last_ms(fem_gpu_t* h, float* ms);
/* element numbers of one kind (0 truss, 1 beam, 2 plate) in call order (n of that kind, host array) */
int fem_gpu_get_element_numbers(fem_gpu_t* h, int kind, uint32_t* numbers);

/* Device arrays of every model and batch come from one stream-ordered memory pool per device that keeps
 * freed memory for reuse (no cudaMalloc / cudaFree on the assembly path after the first model).  This hands
 * the cached memory of the current device back to the driver (after a device synchronisation). */
int fem_gpu_release_cached_memory(void);

/* Dense assembly of one small structure without any device allocation.
 * No counterpart in the reference: it serves callers that cannot call
 * cudaMalloc -- hosts that own all device memory through their own pool or
 * arena, or that must keep a fixed memory footprint after set-up.  Every
 * pointer except `stream` is DEVICE memory owned by the caller:
 *   xyz          n_nodes x 3 coordinates, node index order
 *   truss_nodes  n_truss x 2 node indices (0-based); truss_props n_truss x 3 (E, A, A2 or NaN)
 *   beam_nodes   n_beam x 2; beam_props n_beam x 11 (E, nu, A, I11, I22, I12, It, shear factor,
 *                local axis 1 x, y, z)
 *   plate_nodes  n_plate x 4; plate_props n_plate x 4 (E, nu, thickness, shear factor)
 *   K            (6 n_nodes) x (6 n_nodes) row-major, fully overwritten
 * Elements are taken in the call order trusses, beams, plates, and every
 * entry of K is the sum of its element contributions in that order -- the
 * values fem_gpu_assemble puts in the CSR for the same model, with zeros
 * where the CSR has no entry.  No validation beyond index range, n_nodes
 * below 2^24, and degenerate geometry -- coincident nodes of a truss or beam;
 * a plate with a repeated node, nodes on a line, off one plane or not convex
 * (FEM_GPU_ERR_ARGUMENT).  Working memory is one fixed device array of 32768
 * node-pair blocks (3 per truss or beam, 10 per plate; about 10 MB on every
 * GPU where the library's device code is loaded -- with CUDA's default lazy
 * loading, from the first use of its kernels on that GPU -- until the
 * process exits): larger structures return FEM_GPU_ERR_NOALLOC_LIMIT.  The
 * call allocates no device memory.  The array's address is
 * looked up on the first call on each device (make it before any stream
 * capture); all calls share it, so calls that overlap on the GPU race and
 * must be serialised by the caller.  Synchronises `stream` (a cudaStream_t,
 * NULL = legacy default stream) before returning. */
int fem_gpu_assemble_dense_noalloc(uint32_t n_nodes, const double* xyz, size_t n_truss, const int32_t* truss_nodes,
                                   const double* truss_props, size_t n_beam, const int32_t* beam_nodes,
                                   const double* beam_props, size_t n_plate, const int32_t* plate_nodes,
                                   const double* plate_props, double rel_tol, double abs_tol, double* K,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif
