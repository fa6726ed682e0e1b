/*
 * fem_oracle.h -- CPU oracle for the element-stiffness-and-assembly path of the
 * Rust crate `finite_element_method` (v0.9.12).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker and the timed
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * may load it; the product (finite_element_method_gb300/) never does.
 *
 * It restates, in FP64 C, the reference's eager assembly:
 *   FEM::create                 src/fem/fem.rs:34-65
 *   FEM::add_node               src/fem/methods_for_node_data_handle.rs:66-79
 *   FEM::add_truss              src/fem/methods_for_truss_data_handle.rs:49-128
 *   FEM::add_beam               src/fem/methods_for_beam_data_handle.rs:49-142
 *   FEM::add_plate              src/fem/methods_for_plate_data_handle.rs:62-217
 * with the element routines of src/fem/structs/{truss,beam,plate}.rs,
 * src/fem/bar_2n_element_functions.rs and
 * src/fem/quadrilateral_4n_element_functions.rs.  The global stiffness is kept,
 * like the reference's SquareMatrix, as a (row, col) -> value hash map filled
 * in element call order with exact zeros skipped; it is read out as CSR.
 *
 * Parity status: the truss path is pinned by the reference's own known answer
 * (src/tests/fem/test_fem.rs:5-64: 2-node truss, E=1e6, A=2, L=30).  Beam and
 * plate values are pinned only by closed-form answers derived from the
 * reference formulas and by a literal dense restatement (oracle/literal.py);
 * the reference's own tests hold no golden data for them.
 */
#ifndef FEM_ORACLE_H
#define FEM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_fem orc_fem_t;

/* status codes, shared meaning with the GPU library's FEM_GPU_* codes */
enum {
  ORC_OK = 0,
  ORC_ERR_NODE_LIMIT = 1,        /* methods_for_node_data_handle.rs:47-51 */
  ORC_ERR_NODE_NUMBER = 2,       /* :53-55 */
  ORC_ERR_NODE_INDEX = 3,        /* :56-58 */
  ORC_ERR_NODE_COORDS = 4,       /* :59-61 */
  ORC_ERR_NODE_NOT_EXIST = 5,    /* :81-86 */
  ORC_ERR_ELEM_NUMBER = 6,       /* e.g. methods_for_truss_data_handle.rs:39-41 */
  ORC_ERR_ELEM_SAME_NODES = 7,   /* e.g. methods_for_truss_data_handle.rs:42-44 */
  ORC_ERR_YOUNG = 8,
  ORC_ERR_POISSON = 9,
  ORC_ERR_AREA = 10,
  ORC_ERR_AREA2 = 11,
  ORC_ERR_I11 = 12,
  ORC_ERR_I22 = 13,
  ORC_ERR_IT = 14,
  ORC_ERR_SHEAR_FACTOR = 15,
  ORC_ERR_PARALLEL_AXIS = 16,    /* structs/beam.rs:104-114 */
  ORC_ERR_THICKNESS = 17,
  ORC_ERR_NODES_ON_LINE = 18,    /* structs/plate.rs:87-106 */
  ORC_ERR_NOT_ON_PLANE = 19,     /* structs/plate.rs:107-127 */
  ORC_ERR_NOT_CONVEX = 20,       /* structs/plate.rs:128-155 */
  ORC_ERR_ZERO_LENGTH = 21,      /* two-node element whose nodes coincide */
  ORC_ERR_INTERNAL = 99
};

orc_fem_t* orc_create(double rel_tol, double abs_tol, uint32_t nodes_number);
void orc_destroy(orc_fem_t* h);
const char* orc_last_error(const orc_fem_t* h);

int orc_add_node(orc_fem_t* h, uint32_t number, double x, double y, double z);
int orc_add_truss(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, double young, double area,
                  int has_area2, double area2);
int orc_add_beam(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, double young, double poisson,
                 double area, double i11, double i22, double i12, double it, double shear_factor,
                 const double local_axis_1_direction[3]);
int orc_add_plate(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, uint32_t n3, uint32_t n4,
                  double young, double poisson, double thickness, double shear_factor);

/* Batched forms: loop over add_* in array order; stop at the first failure.
 * *n_added receives the number of elements accepted before it. */
int orc_add_nodes(orc_fem_t* h, const uint32_t* numbers, const double* xyz, size_t n, size_t* n_added);
int orc_add_trusses(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes2, const double* young,
                    const double* area, const double* area2_or_nan, size_t n, size_t* n_added);
int orc_add_beams(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes2, const double* young,
                  const double* poisson, const double* area, const double* i11, const double* i22,
                  const double* i12, const double* it, const double* shear_factor, const double* axis3,
                  size_t n, size_t* n_added);
int orc_add_plates(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes4, const double* young,
                   const double* poisson, const double* thickness, const double* shear_factor, size_t n,
                   size_t* n_added);

/* Global stiffness as CSR (rows = 6 * nodes_number). */
int64_t orc_n_rows(const orc_fem_t* h);
int64_t orc_nnz(const orc_fem_t* h);
int orc_get_csr(const orc_fem_t* h, int64_t* row_ptr, int32_t* col_idx, double* values);
/* DOF map: index -> node number (insertion order), length = nodes added. */
int64_t orc_n_nodes(const orc_fem_t* h);
int orc_get_index_node_numbers(const orc_fem_t* h, uint32_t* numbers);
/* Stiffness groups (docs/Stiffness_groups.md): every non-empty 3x3 region
 * (Kuu, Kuth, Kthu, Kthth) of every node-pair block, sorted by (row node, col
 * node, kind); and per CSR entry the index of its group. */
int64_t orc_n_groups(const orc_fem_t* h);
int orc_get_groups(const orc_fem_t* h, int32_t* row_node, int32_t* col_node, uint8_t* kind,
                   int32_t* nnz_group);

/* Element-level matrices in global axes (exactly what add_* scatters).
 * truss: 6x6 (3 DOF per node), beam: 12x12, plate: 24x24, row-major.
 * Return a status code (validation is NOT run here, only the arithmetic). */
int orc_truss_global_matrix(const double x1[3], const double x2[3], double young, double area,
                            int has_area2, double area2, double rel_tol, double abs_tol, double* out36);
int orc_beam_global_matrix(const double x1[3], const double x2[3], double young, double poisson,
                           double area, double i11, double i22, double i12, double it, double shear_factor,
                           const double axis[3], double rel_tol, double abs_tol, double* out144);
/* equivalent nodal loads (beam.rs:775-797, plate.rs:1145-1185) */
int orc_beam_line_load(const double x1[3], const double x2[3], double q, double* out2);
int orc_plate_surface_load(const double x1[3], const double x2[3], const double x3[3], const double x4[3], double q,
                           double rel_tol, double abs_tol, double* out4);
int orc_plate_global_matrix(const double x1[3], const double x2[3], const double x3[3], const double x4[3],
                            double young, double poisson, double thickness, double shear_factor,
                            double rel_tol, double abs_tol, double* out576);
/* rotation matrices as stored by Truss/Beam/Plate::create (row-major 3x3) */
int orc_truss_rotation(const double x1[3], const double x2[3], double rel_tol, double abs_tol, double* r9);
int orc_beam_rotation(const double x1[3], const double x2[3], double i11, double i22, double i12,
                      const double axis[3], double rel_tol, double abs_tol, double* r9,
                      double* i11_p, double* i22_p);
int orc_plate_rotation(const double x2[3], const double x3[3], const double x4[3], double rel_tol,
                       double abs_tol, double* r9);

/* element results from local displacements of the element's nodes in global
 * axes (truss: 3 per node, beam and plate: 6 per node), in the reference's
 * component order: truss [ForceR]; beam [ForceR, ForceS, ForceT, MomentR,
 * MomentS x3 (node 1, average, node 2), MomentT x3]; plate [MembraneForceR,
 * MembraneForceS, MembraneForceRS, BendingMomentR, BendingMomentS,
 * BendingMomentRS, ShearForceRT, ShearForceST] (truss.rs:281-333,
 * beam.rs:803-993, plate.rs:1196-1409) */
int orc_truss_results(const double x1[3], const double x2[3], double young, double area, int has_area2,
                      double area2, double rel_tol, double abs_tol, const double* u6, double* out1);
int orc_beam_results(const double x1[3], const double x2[3], double young, double poisson, double area, double i11,
                     double i22, double i12, double it, double shear_factor, const double axis[3], double rel_tol,
                     double abs_tol, const double* u12, double* out10);
int orc_plate_results(const double x1[3], const double x2[3], const double x3[3], const double x4[3], double young,
                      double poisson, double thickness, double shear_factor, double rel_tol, double abs_tol,
                      const double* u24, double* out8);

/* the transcendental kernels shared (by algorithm, not by code) with the GPU */
double orc_sin(double x);
double orc_cos(double x);
double orc_atan(double x);
double orc_acos(double x);

/* A whole mesh by node index (0-based), elements in call order per kind:
 * trusses, then beams, then plates.  t_area2 may be NULL (NaN = no taper). */
typedef struct {
  uint32_t nodes_number;
  const double* xyz; /* nodes_number x 3 */
  size_t n_truss;
  const int32_t* t_nodes;
  const double *t_young, *t_area, *t_area2;
  size_t n_beam;
  const int32_t* b_nodes;
  const double *b_young, *b_poisson, *b_area, *b_i11, *b_i22, *b_i12, *b_it, *b_shear, *b_axis;
  size_t n_plate;
  const int32_t* p_nodes;
  const double *p_young, *p_poisson, *p_thickness, *p_shear;
} orc_mesh_t;

/* Multi-threaded port of the eager assembly (no validation): n_threads
 * threads own contiguous node ranges and sum their rows' entries in element
 * call order, so the result is bit-identical to orc_add_* in that order.
 * Writes the CSR when row_ptr is given and nnz <= values_cap; *nnz_out gets
 * nnz, *seconds the wall time of assembly + CSR conversion. */
int orc_assemble_parallel(const orc_mesh_t* mesh, double rel_tol, double abs_tol, int n_threads, int64_t* row_ptr,
                          int32_t* col_idx, double* values, int64_t values_cap, int64_t* nnz_out, double* seconds);

/* Every element's results of a mesh from the displacements vector (6 per
 * node, node index order), n_threads threads over contiguous element ranges;
 * outputs in element call order (NULL skips a kind), *seconds: wall time. */
int orc_element_results(const orc_mesh_t* mesh, const double* displacements, double rel_tol, double abs_tol,
                        int n_threads, double* truss_out, double* beam_out, double* plate_out, double* seconds);

#ifdef __cplusplus
}
#endif
#endif
