/*
 * fem_oracle.c -- CPU oracle (FP64) for the element-stiffness-and-assembly path
 * of the Rust crate `finite_element_method` v0.9.12.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker and the timed CPU baseline.
 * The product never links this file.
 *
 * Arithmetic contract.  The reference's matrix arithmetic lives in the
 * unvendored crate `extended_matrix` 0.9.9 (Matrix::multiply, SquareMatrix::
 * inverse/determinant, Vector3::rotation_matrix_to_align_with_vector, ...), so
 * its floating-point evaluation order cannot be reproduced.  This file fixes
 * one evaluation order for every quantity ("the formula spec"), written from
 * the reference's equations; the GPU kernels follow the same order operation
 * by operation, which is what makes GPU-vs-oracle parity bit-exact.  Every
 * restructuring below is an algebraic identity of the reference's formulas
 * (symmetry of B^T C B, the bending/membrane shared sums, grouping of the
 * assumed-strain shear rows by tying line); oracle/literal.py checks the
 * result against a literal dense restatement at 1e-12.
 *
 * Rules of the spec: IEEE binary64, round to nearest; `fma` means one fused
 * multiply-add; nothing else is contracted (build with -ffp-contract=off).
 * Transcendentals are this file's own (Cody-Waite reduction + Taylor series,
 * a table-based arctangent), because libm and CUDA's libdevice differ in the
 * last bit; both sides implement the same algorithm with the same constants.
 *
 * Pinning.  The reference's own tests hold known answers for the truss only
 * (src/tests/fem/test_fem.rs:5-225), and tests/test_oracle.py reproduces them.
 * For beams and plates there is no reference-held vector and the reference
 * cannot be built here (Rust, with extended_matrix unvendored): beam and plate
 * parity is unpinned by the reference.  It is bounded instead by a 50-digit
 * evaluation of a literal dense transcription of the reference's formulas
 * (oracle/literal.py, tests/golden/make_golden.py), which this file matches to
 * 1e-13 of each element's scale.
 */
#include "fem_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ------------------------------------------------------------------------ */
/* transcendentals (own implementations; identical algorithm on the GPU)     */
/* ------------------------------------------------------------------------ */

/* pi/2 split in three doubles (Cody & Waite 1980 style reduction constants),
 * from a 300-bit value of pi. */
static const double PIO2_1 = 0x1.921fb54442d18p+0;
static const double PIO2_2 = 0x1.1a62633145c07p-54;
static const double PIO2_3 = -0x1.f1976b7ed8fbcp-110;
static const double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
/* 1/n! rounded to nearest */
static const double INV_FACT[23] = {
    1.0, 1.0, 0x1.0000000000000p-1, 0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
    0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19,
    0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26, 0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33,
    0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-41, 0x1.ae7f3e733b81fp-45, 0x1.952c77030ad4ap-49,
    0x1.6827863b97d97p-53, 0x1.2f49b46814157p-57, 0x1.e542ba4020225p-62, 0x1.71b8ef6dcf572p-66,
    0x1.0ce396db7f853p-70};
/* atan(k/8), k = 0..8, rounded to nearest */
static const double ATAN_K8[9] = {0.0,
                                  0x1.fd5ba9aac2f6ep-4,
                                  0x1.f5b75f92c80ddp-3,
                                  0x1.6f61941e4def1p-2,
                                  0x1.dac670561bb4fp-2,
                                  0x1.1e00babdefeb4p-1,
                                  0x1.4978fa3269ee1p-1,
                                  0x1.700a7c5784634p-1,
                                  0x1.921fb54442d18p-1};
/* 1/(2k+1) rounded to nearest, k = 1..8 */
static const double INV_ODD[9] = {1.0,
                                  0x1.5555555555555p-2,
                                  0x1.999999999999ap-3,
                                  0x1.2492492492492p-3,
                                  0x1.c71c71c71c71cp-4,
                                  0x1.745d1745d1746p-4,
                                  0x1.3b13b13b13b14p-4,
                                  0x1.1111111111111p-4,
                                  0x1.e1e1e1e1e1e1ep-5};

/* sin and cos of the reduced argument r, |r| <= pi/4 (Taylor to r^21 / r^22) */
static void sincos_reduced(double r, double* s, double* c) {
  double r2 = r * r;
  double ps = INV_FACT[21];
  ps = fma(ps, r2, -INV_FACT[19]);
  ps = fma(ps, r2, INV_FACT[17]);
  ps = fma(ps, r2, -INV_FACT[15]);
  ps = fma(ps, r2, INV_FACT[13]);
  ps = fma(ps, r2, -INV_FACT[11]);
  ps = fma(ps, r2, INV_FACT[9]);
  ps = fma(ps, r2, -INV_FACT[7]);
  ps = fma(ps, r2, INV_FACT[5]);
  ps = fma(ps, r2, -INV_FACT[3]);
  *s = fma(r * r2, ps, r);
  double pc = -INV_FACT[22];
  pc = fma(pc, r2, INV_FACT[20]);
  pc = fma(pc, r2, -INV_FACT[18]);
  pc = fma(pc, r2, INV_FACT[16]);
  pc = fma(pc, r2, -INV_FACT[14]);
  pc = fma(pc, r2, INV_FACT[12]);
  pc = fma(pc, r2, -INV_FACT[10]);
  pc = fma(pc, r2, INV_FACT[8]);
  pc = fma(pc, r2, -INV_FACT[6]);
  pc = fma(pc, r2, INV_FACT[4]);
  pc = fma(pc, r2, -INV_FACT[2]);
  *c = fma(r2, pc, 1.0);
}

static int reduce_pio2(double x, double* r) {
  double k = nearbyint(x * TWO_OVER_PI);
  double t = fma(-k, PIO2_1, x);
  t = fma(-k, PIO2_2, t);
  t = fma(-k, PIO2_3, t);
  *r = t;
  return ((int)k) & 3;
}

double orc_sin(double x) {
  double r, s, c;
  int q = reduce_pio2(x, &r);
  sincos_reduced(r, &s, &c);
  switch (q) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
  }
}

double orc_cos(double x) {
  double r, s, c;
  int q = reduce_pio2(x, &r);
  sincos_reduced(r, &s, &c);
  switch (q) {
    case 0: return c;
    case 1: return -s;
    case 2: return -c;
    default: return s;
  }
}

/* atan: |t| > 1 folded by atan(t) = pi/2 - atan(1/t); then
 * atan(a) = atan(k/8) + atan((a - k/8) / (1 + a k/8)), |reduced| <= 1/16,
 * odd Taylor series to u^17. */
double orc_atan(double t) {
  if (t != t) return t;
  int neg = t < 0.0;
  double a = neg ? -t : t;
  int inv = a > 1.0;
  if (inv) a = 1.0 / a;
  double kf = nearbyint(a * 8.0);
  int k = (int)kf;
  double c = kf * 0.125;
  double u = (a - c) / fma(a, c, 1.0);
  double u2 = u * u;
  double p = INV_ODD[8];
  p = fma(p, u2, -INV_ODD[7]);
  p = fma(p, u2, INV_ODD[6]);
  p = fma(p, u2, -INV_ODD[5]);
  p = fma(p, u2, INV_ODD[4]);
  p = fma(p, u2, -INV_ODD[3]);
  p = fma(p, u2, INV_ODD[2]);
  p = fma(p, u2, -INV_ODD[1]);
  double res = ATAN_K8[k] + fma(u * u2, p, u);
  if (inv) res = (PIO2_1 - res) + PIO2_2;
  return neg ? -res : res;
}

/* acos(x) = 2 atan(sqrt((1 - x) / (1 + x))), x in [-1, 1] */
double orc_acos(double x) { return 2.0 * orc_atan(sqrt((1.0 - x) / (1.0 + x))); }

/* ------------------------------------------------------------------------ */
/* small vector helpers (plain, left-to-right, as the reference's formulas)  */
/* ------------------------------------------------------------------------ */

static inline double dot3(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static inline double norm3(const double a[3]) { return sqrt(dot3(a, a)); }
static inline void sub3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
static inline void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
/* compare_with_tolerance, src/fem/math_functions.rs:3-12 */
static inline double cwt(double v, double abs_tol) { return fabs(v) < abs_tol ? 0.0 : v; }

/* rotation taking direction a onto direction b.
 * Restates extended_matrix's Vector3::rotation_matrix_to_align_with_vector
 * (called at structs/truss.rs:80, structs/beam.rs:179,
 * quadrilateral_4n_element_functions.rs:158) as the Rodrigues rotation about
 * a x b, in its trig-free form R = c I + [v]x + v v^T / (1 + c) with v = a^ x b^,
 * c = a^ . b^.  Exactly parallel: identity; exactly anti-parallel: the half
 * turn about the unit axis a x e_z (or a x e_x when that vanishes).  Entries
 * below abs_tol are set to zero (compare_with_tolerance). */
static void align_rotation(const double a[3], const double b[3], double abs_tol, double R[9]) {
  double ia = 1.0 / norm3(a), ib = 1.0 / norm3(b);
  double ua[3] = {a[0] * ia, a[1] * ia, a[2] * ia};
  double ub[3] = {b[0] * ib, b[1] * ib, b[2] * ib};
  double v[3];
  cross3(ua, ub, v);
  double c = dot3(ua, ub);
  if (v[0] == 0.0 && v[1] == 0.0 && v[2] == 0.0) {
    if (c > 0.0) {
      R[0] = 1.0; R[1] = 0.0; R[2] = 0.0;
      R[3] = 0.0; R[4] = 1.0; R[5] = 0.0;
      R[6] = 0.0; R[7] = 0.0; R[8] = 1.0;
      return;
    }
    double ez[3] = {0.0, 0.0, 1.0}, ex[3] = {1.0, 0.0, 0.0}, n[3];
    cross3(ua, ez, n);
    if (n[0] == 0.0 && n[1] == 0.0 && n[2] == 0.0) cross3(ua, ex, n);
    double in = 1.0 / norm3(n);
    n[0] *= in; n[1] *= in; n[2] *= in;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double tn = 2.0 * n[i];
        R[3 * i + j] = cwt(i == j ? fma(tn, n[j], -1.0) : tn * n[j], abs_tol);
      }
    return;
  }
  double h = 1.0 / (1.0 + c);
  double hv0 = h * v[0], hv1 = h * v[1], hv2 = h * v[2];
  R[0] = cwt(fma(hv0, v[0], c), abs_tol);
  R[1] = cwt(fma(hv0, v[1], -v[2]), abs_tol);
  R[2] = cwt(fma(hv0, v[2], v[1]), abs_tol);
  R[3] = cwt(fma(hv0, v[1], v[2]), abs_tol);
  R[4] = cwt(fma(hv1, v[1], c), abs_tol);
  R[5] = cwt(fma(hv1, v[2], -v[0]), abs_tol);
  R[6] = cwt(fma(hv0, v[2], -v[1]), abs_tol);
  R[7] = cwt(fma(hv1, v[2], v[0]), abs_tol);
  R[8] = cwt(fma(hv2, v[2], c), abs_tol);
}

/* symmetric 3x3 block R^T D R for D = diag(d): lower entries mirrored */
static void rt_diag_r(const double R[9], const double d[3], double out[9]) {
  double t[9];
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i) t[3 * k + i] = R[3 * k + i] * d[k];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      double s = fma(t[6 + i], R[6 + j], fma(t[3 + i], R[3 + j], t[i] * R[j]));
      out[3 * i + j] = s;
      out[3 * j + i] = s;
    }
}

/* ------------------------------------------------------------------------ */
/* truss (structs/truss.rs, bar_2n_element_functions.rs)                     */
/* ------------------------------------------------------------------------ */

int orc_truss_rotation(const double x1[3], const double x2[3], double rel_tol, double abs_tol, double* r9) {
  (void)rel_tol;
  double d[3];
  sub3(x2, x1, d); /* find_2n_element_vector: node_2 - node_1 (bar_2n_element_functions.rs:23-28) */
  double L = norm3(d);
  if (!(L > 0.0)) return ORC_ERR_ZERO_LENGTH;
  double target[3] = {L, 0.0, 0.0}; /* truss.rs:78 */
  align_rotation(d, target, abs_tol, r9);
  return ORC_OK;
}

/* 6x6 (3 DOF per node) truss matrix in global axes, truss.rs:95-214 and
 * methods_for_truss_data_handle.rs:75-81. */
int orc_truss_global_matrix(const double x1[3], const double x2[3], double young, double area, int has_area2,
                            double area2, double rel_tol, double abs_tol, double* out36) {
  double R[9];
  int st = orc_truss_rotation(x1, x2, rel_tol, abs_tol, R);
  if (st) return st;
  double d[3];
  sub3(x2, x1, d);
  double L = norm3(d);
  double jac = L * 0.5;      /* dx_dr with x1=-L/2, x2=L/2 (bar_2n_element_functions.rs:35-59) */
  double inv = 1.0 / jac;    /* inverse_jacobian_at_r */
  double b = 0.5 * inv;      /* B = [dh1_dr, 0, 0, dh2_dr, 0, 0] * inv, dh = -+0.5 (truss.rs:95-118) */
  double a_r = area;         /* area_at_r at r = 0 (truss.rs:120-130) */
  if (has_area2) {
    double hh = (area2 - area) * 0.5;
    a_r = area + hh;
  }
  double scalar = ((a_r * young) * jac) * 2.0; /* c_at_r * det * alpha, alpha = 2 (truss.rs:147-153, :244) */
  double q = (b * b) * scalar;                 /* (B^T B)_00 * scalar; _03 = -q */
  /* T = diag(R, R) (truss.rs:191-214); (T^T k T) = +-q r0 r0^T, r0 = first row of R */
  double m[3] = {R[0] * q, R[1] * q, R[2] * q};
  double g[9];
  for (int i = 0; i < 3; ++i)
    for (int j = i; j < 3; ++j) {
      double s = m[i] * R[j];
      g[3 * i + j] = s;
      g[3 * j + i] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = g[3 * i + j];
      out36[6 * i + j] = s;
      out36[6 * i + 3 + j] = -s;
      out36[6 * (3 + i) + j] = -s;
      out36[6 * (3 + i) + 3 + j] = s;
    }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* beam (structs/beam.rs)                                                    */
/* ------------------------------------------------------------------------ */

static const double PI_F32 = 3.1415927410125732; /* f32 PI widened, beam.rs:7, :149 */

/* find_principal_moments_of_inertia, beam.rs:119-160 (loop capped at 8 turns;
 * in exact arithmetic one half-turn swap always suffices) */
static void principal_moments(double i11, double i22, double i12, double rel_tol, double* i11p, double* i22p,
                              double* angle_out) {
  double angle;
  if (i11 != i22) {
    angle = orc_atan((2.0 * i12) / (i22 - i11)) / 2.0;
  } else {
    double i11m, i22m;
    if (i22 < i11) {
      i11m = i11;
      i22m = ((fabs(i22) - fabs(i22) * rel_tol) * i22) / fabs(i22);
    } else {
      i11m = ((fabs(i11) - fabs(i11) * rel_tol) * i11) / fabs(i11);
      i22m = i22;
    }
    angle = orc_atan((2.0 * i12) / (i22m - i11m)) / 2.0;
  }
  double c = orc_cos(angle), s = orc_sin(angle), s2 = orc_sin(2.0 * angle);
  double a = (i11 * (c * c) + i22 * (s * s)) - i12 * s2;
  double bb = (i11 * (s * s) + i22 * (c * c)) + i12 * s2;
  int it = 1;
  while (a < bb && it <= 8) {
    angle = (orc_atan((2.0 * i12) / (i22 - i11)) + PI_F32 * (double)it) / 2.0;
    c = orc_cos(angle);
    s = orc_sin(angle);
    s2 = orc_sin(2.0 * angle);
    a = (i11 * (c * c) + i22 * (s * s)) - i12 * s2;
    bb = (i11 * (s * s) + i22 * (c * c)) + i12 * s2;
    ++it;
  }
  *i11p = a;
  *i22p = bb;
  *angle_out = angle;
}

/* projection_perpendicular_to_vector (extended_matrix, not vendored; used at
 * beam.rs:104-105 and :186-187), restated as p = a - ((a.b)/(b.b)) b */
static void project_perp(const double a[3], const double b[3], double p[3]) {
  double s = dot3(a, b) / dot3(b, b);
  p[0] = a[0] - s * b[0];
  p[1] = a[1] - s * b[1];
  p[2] = a[2] - s * b[2];
}

int orc_beam_rotation(const double x1[3], const double x2[3], double i11, double i22, double i12,
                      const double axis[3], double rel_tol, double abs_tol, double* r9, double* i11_p,
                      double* i22_p) {
  double angle;
  principal_moments(i11, i22, i12, rel_tol, i11_p, i22_p, &angle);
  /* find_rotation_matrix_elements, beam.rs:162-258 */
  double d[3];
  sub3(x2, x1, d);
  double L = norm3(d);
  if (!(L > 0.0)) return ORC_ERR_ZERO_LENGTH;
  double target[3] = {L, 0.0, 0.0};
  double Ri[9];
  align_rotation(d, target, abs_tol, Ri);
  double p[3];
  project_perp(axis, d, p);
  double tp[3];
  for (int i = 0; i < 3; ++i) tp[i] = (Ri[3 * i] * p[0] + Ri[3 * i + 1] * p[1]) + Ri[3 * i + 2] * p[2];
  /* cosine between (0,0,1) and tp: dot / (|e_z| |tp|) = tp_z / |tp| */
  double cosang = tp[2] / norm3(tp);
  if (cosang > 1.0) cosang = 1.0;
  if (cosang < -1.0) cosang = -1.0;
  double total = angle + orc_acos(cosang);
  double cx = cwt(d[0] / L, abs_tol), cy = cwt(d[1] / L, abs_tol), cz = cwt(d[2] / L, abs_tol);
  double cxz = cwt(sqrt(cx * cx + cz * cz), abs_tol);
  double c = cwt(orc_cos(total), abs_tol), s = cwt(orc_sin(total), abs_tol);
  if (cxz != 0.0) {
    r9[0] = cx;
    r9[1] = cy;
    r9[2] = cz;
    r9[3] = ((((-1.0 * cx) * cy) * c) - cz * s) / cxz;
    r9[4] = cxz * c;
    r9[5] = ((((-1.0 * cy) * cz) * c) + cx * s) / cxz;
    r9[6] = (((cx * cy) * s) - cz * c) / cxz;
    r9[7] = (-1.0 * cxz) * s;
    r9[8] = (((cy * cz) * s) + cx * c) / cxz;
  } else {
    r9[0] = 0.0;
    r9[1] = cy;
    r9[2] = 0.0;
    r9[3] = (-1.0 * cy) * c;
    r9[4] = 0.0;
    r9[5] = s;
    r9[6] = cy * s;
    r9[7] = 0.0;
    r9[8] = c;
  }
  return ORC_OK;
}

/* 12x12 beam matrix in global axes: local Timoshenko k at r = 0, alpha = 2
 * (beam.rs:260-605) and T^T k T with T = diag(R, R, R, R) (beam.rs:607-667,
 * methods_for_beam_data_handle.rs:88-95).  Local DOF order per node:
 * u, v, w, thx, thy, thz. */
int orc_beam_global_matrix(const double x1[3], const double x2[3], double young, double poisson, double area,
                           double i11, double i22, double i12, double it, double shear_factor,
                           const double axis[3], double rel_tol, double abs_tol, double* out144) {
  double R[9], i11p, i22p;
  int st = orc_beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol, R, &i11p, &i22p);
  if (st) return st;
  double d[3];
  sub3(x2, x1, d);
  double L = norm3(d);
  double jac = L * 0.5, inv = 1.0 / jac;
  double b = 0.5 * inv;   /* |dh_dr * inv| */
  double hb = 0.5 * b;    /* h(0) * |dh_dr * inv| = 0.5 b */
  double b2 = b * b;
  double G = young / (2.0 * (1.0 + poisson)); /* beam.rs:519 */
  double su = ((area * young) * jac) * 2.0;
  double sv = ((((G * area) * shear_factor)) * jac) * 2.0;
  double sw = ((((G * area) * shear_factor)) * jac) * 2.0;
  double stu = ((G * it) * jac) * 2.0;
  double stv = ((young * i22p) * jac) * 2.0;
  double stw = ((young * i11p) * jac) * 2.0;
  double A1 = b2 * su, V1 = b2 * sv, W1 = b2 * sw, T1 = b2 * stu, Y1 = b2 * stv, Z1 = b2 * stw;
  double HV = hb * sv, HW = hb * sw, QV = 0.25 * sv, QW = 0.25 * sw;

  double uu[9], th[9], thth2[9];
  double du[3] = {A1, V1, W1};
  double dth[3] = {T1, QW + Y1, QV + Z1};
  double dth2[3] = {-T1, QW + (-Y1), QV + (-Z1)};
  rt_diag_r(R, du, uu);
  rt_diag_r(R, dth, th);
  rt_diag_r(R, dth2, thth2);
  /* blocks with local entries only at (1,2) = alpha and (2,1) = beta:
   * (R^T M R)_ij = beta * P_ji + alpha * P_ij with P_ij = R_1i R_2j */
  double P[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[3 * i + j] = R[3 + i] * R[6 + j];
  double ut[9], tu[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      ut[3 * i + j] = fma(HW, P[3 * j + i], HV * P[3 * i + j]);       /* u1-th1: alpha=HV, beta=HW */
      tu[3 * i + j] = fma(-HV, P[3 * j + i], (-HW) * P[3 * i + j]);   /* th1-u2: alpha=-HW, beta=-HV */
    }
  /* upper blocks, block order [u1, th1, u2, th2] */
  const double* blk[4][4] = {{0}};
  double neg_uu[9], neg_ut[9];
  for (int i = 0; i < 9; ++i) {
    neg_uu[i] = -uu[i];
    neg_ut[i] = -ut[i];
  }
  blk[0][0] = uu; blk[0][1] = ut; blk[0][2] = neg_uu; blk[0][3] = ut;
  blk[1][1] = th; blk[1][2] = tu; blk[1][3] = thth2;
  blk[2][2] = uu; blk[2][3] = neg_ut;
  blk[3][3] = th;
  for (int P_ = 0; P_ < 4; ++P_)
    for (int Q_ = P_; Q_ < 4; ++Q_) {
      const double* m = blk[P_][Q_];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          out144[12 * (3 * P_ + i) + 3 * Q_ + j] = m[3 * i + j];
          out144[12 * (3 * Q_ + j) + 3 * P_ + i] = m[3 * i + j];
        }
    }
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* plate (structs/plate.rs, quadrilateral_4n_element_functions.rs)           */
/* ------------------------------------------------------------------------ */

int orc_plate_rotation(const double x2[3], const double x3[3], const double x4[3], double rel_tol, double abs_tol,
                       double* r9) {
  (void)rel_tol;
  /* find_rotation_matrix_elements_of_quadrilateral, quad.rs:131-171 */
  double e34[3], e32[3], n[3];
  sub3(x4, x3, e34);
  sub3(x2, x3, e32);
  cross3(e34, e32, n);
  if (n[0] == 0.0 && n[1] == 0.0 && n[2] > 0.0) {
    /* normal already along +z: the rotation is exactly the identity */
    r9[0] = 1.0; r9[1] = 0.0; r9[2] = 0.0;
    r9[3] = 0.0; r9[4] = 1.0; r9[5] = 0.0;
    r9[6] = 0.0; r9[7] = 0.0; r9[8] = 1.0;
    return ORC_OK;
  }
  double ln = norm3(n);
  if (!(ln > 0.0)) return ORC_ERR_NODES_ON_LINE;
  double target[3] = {0.0, 0.0, ln};
  align_rotation(n, target, abs_tol, r9);
  return ORC_OK;
}

static int is_identity(const double R[9]) {
  return R[0] == 1.0 && R[1] == 0.0 && R[2] == 0.0 && R[3] == 0.0 && R[4] == 1.0 && R[5] == 0.0 && R[6] == 0.0 &&
         R[7] == 0.0 && R[8] == 1.0;
}

/* Gauss point coordinate sqrt(f64(1f32/3f32)) (plate.rs:1066-1091) */
static double plate_gauss_g(void) { return sqrt((double)(1.0f / 3.0f)); }

/* local 24x24 stiffness (plate.rs:513-724), written row-major into K (zeroed
 * by the caller); DOF order per node u, v, w, thx, thy, thz.
 *
 * Scaled quantities (exact powers of two aside, identical to the reference's):
 *   Jh = 4 J(r,s) = [[ax + s bx, ay + s by], [cx + r bx, cy + r by]]
 *       (quad.rs:252-338 and 380-446; ax.. are the sums of plate.rs:424-429)
 *   D  = det Jh = 16 det J,  q = 1 / D
 *   gx_i = D dh_i/dx,  gy_i = D dh_i/dy    (quad.rs:613-653)
 *   S..  = sum over IPs of (cm/16) q g_i g_j   ->  K_mem = T, K_bend = (t^2 / 12) T
 *       (the membrane factor rides on the integration-point weights)
 *   shear: m^2 det w = Q / (4 D) with Q = |Jh row|^2 (plate.rs:443-447); the
 *   four rank-1 rows of each IP are grouped by tying line (rows at s = +-g share
 *   a direction, rows at r = +-g share a direction), coefficient c_s / 64.
 * One reciprocal serves the four determinants and one the material constants. */
static void plate_local_matrix(const double xl[4], const double yl[4], double young, double poisson,
                               double thickness, double shear_factor, double* K) {
  const double g = plate_gauss_g();
  const double ipr[4] = {g * 1.0, g * -1.0, g * -1.0, g * 1.0};
  const double ips[4] = {g * 1.0, g * 1.0, g * -1.0, g * -1.0};
  const double al = 1.0 + g, be = 1.0 - g;
  double x1 = xl[0], x2 = xl[1], x4 = xl[3];
  double y1 = yl[0], y2 = yl[1], y4 = yl[3];
  /* plate.rs:415-429 with x3 = y3 = 0 */
  double d12x = x1 - x2, d12y = y1 - y2;
  double ax = d12x + x4, bx = d12x - x4, cx = (x1 + x2) - x4;
  double ay = d12y + y4, by = d12y - y4, cy = (y1 + y2) - y4;

  double J00[4], J01[4], J10[4], J11[4], D[4], q[4];
  for (int ip = 0; ip < 4; ++ip) {
    J00[ip] = fma(ips[ip], bx, ax);
    J01[ip] = fma(ips[ip], by, ay);
    J10[ip] = fma(ipr[ip], bx, cx);
    J11[ip] = fma(ipr[ip], by, cy);
    D[ip] = fma(J00[ip], J11[ip], -(J01[ip] * J10[ip]));
  }
  {
    double D01 = D[0] * D[1], D23 = D[2] * D[3];
    double inv = 1.0 / (D01 * D23);
    q[0] = (D[1] * D23) * inv;
    q[1] = (D[0] * D23) * inv;
    q[2] = (D[3] * D01) * inv;
    q[3] = (D[2] * D01) * inv;
  }
  /* material (plate.rs:532-548, :580-597, :629-636), one reciprocal: cm/16 = E t / (16 (1 - nu^2)) scales
   * the membrane sums through the integration-point weights, bending = (t^2 / 12) x membrane, shear
   * c_s/64 = E t k (1 - nu) / (128 (1 - nu^2)) */
  double dinv = 1.0 / (1.0 - poisson * poisson);
  double Et = young * thickness;
  double cmq = (Et * dinv) * 0.0625;
  double tb = (thickness * thickness) * 0x1.5555555555555p-4;
  double omn = 1.0 - poisson;
  double cq = ((Et * shear_factor) * omn) * (dinv * 0x1p-7);
  double gam = omn * 0.5;
  double Sxx[16] = {0}, Syy[16] = {0}, Sxy[16] = {0};
  double Wr[4], Ws[4];
  for (int ip = 0; ip < 4; ++ip) {
    double sp = 1.0 + ips[ip], sm = 1.0 - ips[ip], rp = 1.0 + ipr[ip], rm = 1.0 - ipr[ip];
    /* gx = [J11 sp - J01 rp, -J11 sp - J01 rm, J01 rm - J11 sm, J11 sm + J01 rp],
     * gy = [J00 rp - J10 sp, J00 rm + J10 sp, J10 sm - J00 rm, -J00 rp - J10 sm]: one product and one fma each */
    double P3 = J01[ip] * rp, P4 = J01[ip] * rm, Q1 = J00[ip] * rp, Q2 = J00[ip] * rm;
    double gx[4] = {fma(J11[ip], sp, -P3), fma(-J11[ip], sp, -P4), fma(-J11[ip], sm, P4), fma(J11[ip], sm, P3)};
    double gy[4] = {fma(-J10[ip], sp, Q1), fma(J10[ip], sp, Q2), fma(J10[ip], sm, -Q2), fma(-J10[ip], sm, -Q1)};
    double qm = cmq * q[ip];
    double a[4], bq[4];
    for (int i = 0; i < 4; ++i) {
      a[i] = qm * gx[i];
      bq[i] = qm * gy[i];
    }
    for (int i = 0; i < 4; ++i)
      for (int j = i; j < 4; ++j) {
        Sxx[4 * i + j] = fma(a[i], gx[j], Sxx[4 * i + j]);
        Syy[4 * i + j] = fma(bq[i], gy[j], Syy[4 * i + j]);
      }
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) Sxy[4 * i + j] = fma(a[i], gy[j], Sxy[4 * i + j]);
    Wr[ip] = fma(J11[ip], J11[ip], J10[ip] * J10[ip]) * q[ip];
    Ws[ip] = fma(J01[ip], J01[ip], J00[ip] * J00[ip]) * q[ip];
  }

  /* membrane: (u_i,u_j) = T_uu, (v_i,v_j) = T_vv, (u_i,v_j) = T_uv(i,j) (the sums carry cm/16) */
  double Tuu[16], Tvv[16], Tuv[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      int lo = i < j ? i : j, hi = i < j ? j : i;
      Tuu[4 * i + j] = fma(gam, Syy[4 * lo + hi], Sxx[4 * lo + hi]);
      Tvv[4 * i + j] = fma(gam, Sxx[4 * lo + hi], Syy[4 * lo + hi]);
      Tuv[4 * i + j] = fma(gam, Sxy[4 * j + i], poisson * Sxy[4 * i + j]);
    }
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j) {
      int ri = 6 * i, cj = 6 * j;
      double uu = Tuu[4 * i + j], vv = Tvv[4 * i + j];
      K[24 * (ri + 0) + cj + 0] = uu;
      K[24 * (cj + 0) + ri + 0] = uu;
      K[24 * (ri + 1) + cj + 1] = vv;
      K[24 * (cj + 1) + ri + 1] = vv;
      double uv = Tuv[4 * i + j];
      K[24 * (ri + 0) + cj + 1] = uv;
      K[24 * (cj + 1) + ri + 0] = uv;
      if (i != j) {
        double vu = Tuv[4 * j + i]; /* (v_i, u_j) = (u_j, v_i) */
        K[24 * (ri + 1) + cj + 0] = vu;
        K[24 * (cj + 0) + ri + 1] = vu;
      }
    }
  /* transverse shear (assumed strain, plate.rs:392-511) grouped by tying line */
  const double al2 = al * al, be2 = be * be, ab = al * be;
  double W0p = Wr[0] + Wr[1], W0m = Wr[2] + Wr[3];
  double W1p = Ws[0] + Ws[3], W1m = Ws[1] + Ws[2];
  double A12 = cq * fma(W0p, al2, W0m * be2);
  double A1243 = cq * ((W0p + W0m) * ab);
  double A43 = cq * fma(W0p, be2, W0m * al2);
  double B14 = cq * fma(W1p, al2, W1m * be2);
  double B1423 = cq * ((W1p + W1m) * ab);
  double B23 = cq * fma(W1p, be2, W1m * al2);
  /* tying vectors over (w, thx, thy) */
  double E12[3] = {2.0, -d12y, d12x};
  double E43[3] = {2.0, -y4, x4};
  double E14[3] = {2.0, -(y1 - y4), x1 - x4};
  double E23[3] = {2.0, -y2, x2};
  double F12[3], G12[3], F43[3], F14[3], H14[3], F23[3];
  for (int a_ = 0; a_ < 3; ++a_) {
    F12[a_] = A12 * E12[a_];
    G12[a_] = A1243 * E12[a_];
    F43[a_] = A43 * E43[a_];
    F14[a_] = B14 * E14[a_];
    H14[a_] = B1423 * E14[a_];
    F23[a_] = B23 * E23[a_];
  }
  /* gamma_sz products (symmetric ones for a <= b only) */
  double P14[9], P23[9], P1423[9];
  for (int a_ = 0; a_ < 3; ++a_)
    for (int b_ = 0; b_ < 3; ++b_) {
      if (b_ >= a_) {
        P14[3 * a_ + b_] = P14[3 * b_ + a_] = F14[a_] * E14[b_];
        P23[3 * a_ + b_] = P23[3 * b_ + a_] = F23[a_] * E23[b_];
      }
      P1423[3 * a_ + b_] = H14[a_] * E23[b_];
    }
  /* node groups: gamma_rz pairs (1,2)/(4,3), gamma_sz pairs (1,4)/(2,3); w-sign per node */
  static const int g0[4] = {0, 0, 1, 1};
  static const double s0[4] = {1.0, -1.0, -1.0, 1.0};
  static const int g1[4] = {0, 1, 1, 0};
  static const double s1[4] = {1.0, 1.0, -1.0, -1.0};
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      for (int a_ = 0; a_ < 3; ++a_)
        for (int b_ = (i == j ? a_ : 0); b_ < 3; ++b_) {
          int lo = a_ < b_ ? a_ : b_, hi = a_ < b_ ? b_ : a_;
          /* gamma_sz term */
          double t1;
          if (g1[i] == 0 && g1[j] == 0) t1 = P14[3 * lo + hi];
          else if (g1[i] == 1 && g1[j] == 1) t1 = P23[3 * lo + hi];
          else if (g1[i] == 0) t1 = P1423[3 * a_ + b_];
          else t1 = P1423[3 * b_ + a_];
          double sg1 = (a_ == 0 ? s1[i] : 1.0) * (b_ == 0 ? s1[j] : 1.0);
          if (sg1 < 0) t1 = -t1;
          /* gamma_rz term, fused: sh = f * e + t1 */
          double f, e;
          if (g0[i] == 0 && g0[j] == 0) { f = F12[lo]; e = E12[hi]; }
          else if (g0[i] == 1 && g0[j] == 1) { f = F43[lo]; e = E43[hi]; }
          else if (g0[i] == 0) { f = G12[a_]; e = E43[b_]; }
          else { f = G12[b_]; e = E43[a_]; }
          double sg0 = (a_ == 0 ? s0[i] : 1.0) * (b_ == 0 ? s0[j] : 1.0);
          if (sg0 < 0) f = -f;
          double sh = fma(f, e, t1);
          double v = sh;
          if (a_ >= 1 && b_ >= 1) {
            /* bending on (thx, thy): (thy,thy) = tb T_uu, (thx,thx) = tb T_vv,
             * (thy_i, thx_j) = -tb T_uv(i,j), (thx_i, thy_j) = -tb T_uv(j,i) */
            if (a_ == 2 && b_ == 2) v = fma(tb, Tuu[4 * i + j], sh);
            else if (a_ == 1 && b_ == 1) v = fma(tb, Tvv[4 * i + j], sh);
            else if (a_ == 2 && b_ == 1) v = fma(-tb, Tuv[4 * i + j], sh);
            else v = fma(-tb, Tuv[4 * j + i], sh);
          }
          int r_ = 6 * i + 2 + a_, c_ = 6 * j + 2 + b_;
          K[24 * r_ + c_] = v;
          K[24 * c_ + r_] = v;
        }
  /* drilling spring KROT6 = 1.0 on the local thz diagonals (plate.rs:25, :716-721) */
  for (int i = 0; i < 4; ++i) K[24 * (6 * i + 5) + 6 * i + 5] = 0.0 + 1.0;
}

/* R^T M R for one 3x3 block (dense, left-to-right fma chains); sym: only i <= j, mirrored */
static void rt_m_r(const double R[9], const double M[9], double out[9], int sym) {
  double Y[9];
  for (int k = 0; k < 3; ++k)
    for (int b_ = 0; b_ < 3; ++b_)
      Y[3 * k + b_] = fma(M[3 * k + 2], R[6 + b_], fma(M[3 * k + 1], R[3 + b_], M[3 * k] * R[b_]));
  for (int a_ = 0; a_ < 3; ++a_)
    for (int b_ = (sym ? a_ : 0); b_ < 3; ++b_) {
      double s = fma(R[6 + a_], Y[6 + b_], fma(R[3 + a_], Y[3 + b_], R[a_] * Y[b_]));
      out[3 * a_ + b_] = s;
      if (sym) out[3 * b_ + a_] = s;
    }
}

/* equivalent nodal loads of a uniformly distributed line load q on a two-node
 * element (beam.rs:775-797): one Gauss point r = 0, alpha = 2, h1 = h2 = 0.5,
 * det J = L / 2 (bar_2n_element_functions.rs:35-83); out[i] = 0 + (h_i q) (detJ alpha) */
int orc_beam_line_load(const double x1[3], const double x2[3], double q, double* out2) {
  double d[3];
  sub3(x2, x1, d);
  const double L = norm3(d);
  const double jac = L * 0.5;
  const double h1 = 0.5 * (1.0 - 0.0), h2 = 0.5 * (1.0 + 0.0);
  out2[0] = 0.0 + (h1 * q) * (jac * 2.0);
  out2[1] = 0.0 + (h2 * q) * (jac * 2.0);
  return ORC_OK;
}

/* equivalent nodal loads of a uniformly distributed surface load q on a plate
 * (plate.rs:1145-1185): 2 x 2 Gauss points in the order of plate.rs:1066-1091,
 * alpha_r = alpha_s = 1, h_i(r, s) = (0.25 (1 +- r)) (1 +- s)
 * (quadrilateral_4n_element_functions.rs:585-611), det J(r, s) from the local
 * coordinates (quad.rs:380-505) as det(4 J) / 16 -- the same determinant the
 * stiffness uses; out[i] = sum over the points, in order, from 0. */
int orc_plate_surface_load(const double x1[3], const double x2[3], const double x3[3], const double x4[3], double q,
                           double rel_tol, double abs_tol, double* out4) {
  double R[9];
  int st = orc_plate_rotation(x2, x3, x4, rel_tol, abs_tol, R);
  if (st) return st;
  const double* X[4] = {x1, x2, x3, x4};
  double xl[4] = {0, 0, 0, 0}, yl[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    double dd[3];
    sub3(X[i], x3, dd);
    xl[i] = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    yl[i] = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  const double g = plate_gauss_g();
  const double ipr[4] = {g * 1.0, g * -1.0, g * -1.0, g * 1.0};
  const double ips[4] = {g * 1.0, g * 1.0, g * -1.0, g * -1.0};
  double x1l = xl[0], x2l = xl[1], x4l = xl[3];
  double y1l = yl[0], y2l = yl[1], y4l = yl[3];
  double d12x = x1l - x2l, d12y = y1l - y2l;
  double ax = d12x + x4l, bx = d12x - x4l, cx = (x1l + x2l) - x4l;
  double ay = d12y + y4l, by = d12y - y4l, cy = (y1l + y2l) - y4l;
  for (int i = 0; i < 4; ++i) out4[i] = 0.0;
  for (int ip = 0; ip < 4; ++ip) {
    const double r = ipr[ip], s = ips[ip];
    const double J00 = fma(s, bx, ax), J01 = fma(s, by, ay), J10 = fma(r, bx, cx), J11 = fma(r, by, cy);
    const double detj = fma(J00, J11, -(J01 * J10)) * 0.0625;
    const double w = (detj * 1.0) * 1.0;
    const double h[4] = {(0.25 * (1.0 + r)) * (1.0 + s), (0.25 * (1.0 - r)) * (1.0 + s),
                         (0.25 * (1.0 - r)) * (1.0 - s), (0.25 * (1.0 + r)) * (1.0 - s)};
    for (int i = 0; i < 4; ++i) out4[i] = out4[i] + (h[i] * q) * w;
  }
  return ORC_OK;
}

int orc_plate_global_matrix(const double x1[3], const double x2[3], const double x3[3], const double x4[3],
                            double young, double poisson, double thickness, double shear_factor, double rel_tol,
                            double abs_tol, double* out576) {
  double R[9];
  int st = orc_plate_rotation(x2, x3, x4, rel_tol, abs_tol, R);
  if (st) return st;
  /* node directions relative to node 3, rotated (quad.rs:340-378): the differences themselves when R is
   * exactly the identity, else one product and two fused multiply-adds per coordinate */
  const double* X[4] = {x1, x2, x3, x4};
  const int ident = is_identity(R);
  double xl[4] = {0, 0, 0, 0}, yl[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    if (ident) {
      xl[i] = X[i][0] - x3[0];
      yl[i] = X[i][1] - x3[1];
      continue;
    }
    double dd[3];
    sub3(X[i], x3, dd);
    xl[i] = fma(R[2], dd[2], fma(R[1], dd[1], R[0] * dd[0]));
    yl[i] = fma(R[5], dd[2], fma(R[4], dd[1], R[3] * dd[0]));
  }
  double* K = out576;
  memset(K, 0, sizeof(double) * 576);
  plate_local_matrix(xl, yl, young, poisson, thickness, shear_factor, K);
  if (ident) return ORC_OK; /* T^T K T == K bit for bit when T == I */
  /* T^T K T with T = diag(R x 8) (plate.rs:726-1002, methods_for_plate_data_handle.rs:109-112),
   * node-pair blocks i <= j, 3x3 sub-blocks, lower triangle mirrored */
  double Kg[576];
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      for (int p = 0; p < 2; ++p)
        for (int q = 0; q < 2; ++q) {
          if (i == j && p == 1 && q == 0) continue; /* mirror of (0,1) */
          double M[9], o[9];
          for (int a_ = 0; a_ < 3; ++a_)
            for (int b_ = 0; b_ < 3; ++b_) M[3 * a_ + b_] = K[24 * (6 * i + 3 * p + a_) + 6 * j + 3 * q + b_];
          rt_m_r(R, M, o, i == j && p == q);
          for (int a_ = 0; a_ < 3; ++a_)
            for (int b_ = 0; b_ < 3; ++b_) {
              int r_ = 6 * i + 3 * p + a_, c_ = 6 * j + 3 * q + b_;
              Kg[24 * r_ + c_] = o[3 * a_ + b_];
              Kg[24 * c_ + r_] = o[3 * a_ + b_];
            }
        }
  memcpy(out576, Kg, sizeof(Kg));
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* validation (element checks of structs/truss.rs, beam.rs, plate.rs)         */
/* ------------------------------------------------------------------------ */

/* is_points_of_quadrilateral_on_the_same_line, quad.rs:14-86 */
static int quad_on_line(const double* p1, const double* p2, const double* p3, const double* p4) {
  const double* P[4] = {p1, p2, p3, p4};
  static const int pairs[4][3] = {{0, 1, 3}, {1, 0, 2}, {2, 1, 3}, {3, 2, 0}};
  for (int k = 0; k < 4; ++k) {
    double u[3], v[3], c[3];
    sub3(P[pairs[k][1]], P[pairs[k][0]], u);
    sub3(P[pairs[k][2]], P[pairs[k][0]], v);
    cross3(u, v, c);
    if (norm3(c) == 0.0) return 1;
  }
  return 0;
}

/* is_points_of_quadrilateral_on_the_same_plane, quad.rs:88-129 */
static int quad_on_plane(const double* p1, const double* p2, const double* p3, const double* p4, double abs_tol) {
  double v32[3], v34[3], n[3];
  sub3(p2, p3, v32);
  sub3(p4, p3, v34);
  cross3(v32, v34, n);
  double d = -1.0 * ((n[0] * p3[0] + n[1] * p3[1]) + n[2] * p3[2]);
  double val = ((n[0] * p1[0] + n[1] * p1[1]) + n[2] * p1[2]) + d;
  (void)p4;
  return cwt(val, abs_tol) == 0.0;
}

/* point on the plane with its sort key (angle from +x, degrees) */
typedef struct {
  double x, y, key;
} hpt;

static double hull_key(double x, double y) {
  /* Point::partial_cmp (convex_hull_on_plane.rs:84-103): angle between (1,0) and (x,y),
   * acos(x / sqrt(x^2 + y^2)) in degrees (f64::to_degrees = v * (180/pi)) */
  double len = sqrt((0.0 - x) * (0.0 - x) + (0.0 - y) * (0.0 - y));
  double sp = (0.0 - 1.0) * (0.0 - x) + (0.0 - 0.0) * (0.0 - y);
  double c = sp / (1.0 * len);
  return orc_acos(c) * 0x1.ca5dc1a63c1f8p+5;
}

/* quick_sort / partition of convex_hull_on_plane.rs:14-58 on keys */
static long hull_partition(hpt* a, long low, long high) {
  long pivot = high, store = low - 1, last = high;
  for (;;) {
    store += 1;
    while (a[store].key < a[pivot].key) store += 1;
    last -= 1;
    while (last >= 0 && a[last].key > a[pivot].key) last -= 1;
    if (store >= last) break;
    hpt t = a[store];
    a[store] = a[last];
    a[last] = t;
  }
  hpt t = a[store];
  a[store] = a[pivot];
  a[pivot] = t;
  return store;
}
static void hull_qsort(hpt* a, long low, long high) {
  if (low < high) {
    long p = hull_partition(a, low, high);
    hull_qsort(a, low, p - 1);
    hull_qsort(a, p + 1, high);
  }
}

/* convex_hull_on_four_points_on_plane (quad.rs:173-250) + convex_hull_on_plane
 * (convex_hull_on_plane.rs:178-214): returns the hull size */
static int quad_hull_size(const double* p1, const double* p2, const double* p3, const double* p4, double rel_tol,
                          double abs_tol, int* status) {
  double R[9];
  *status = orc_plate_rotation(p2, p3, p4, rel_tol, abs_tol, R);
  if (*status) return 0;
  const double* P[4] = {p1, p2, p3, p4};
  hpt pts[4];
  for (int i = 0; i < 4; ++i) {
    if (i == 2) {
      pts[i].x = 0.0;
      pts[i].y = 0.0;
      continue;
    }
    double dd[3];
    sub3(P[i], p3, dd);
    pts[i].x = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    pts[i].y = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  double shift_x = pts[0].x, min_y = pts[0].y;
  int pos = 0;
  for (int i = 0; i < 4; ++i)
    if (pts[i].y < min_y) {
      shift_x = pts[i].x;
      min_y = pts[i].y;
      pos = i;
    }
  hpt t = pts[0];
  pts[0] = pts[pos];
  pts[pos] = t;
  for (int i = 0; i < 4; ++i) {
    pts[i].x -= shift_x;
    pts[i].y -= min_y;
  }
  for (int i = 1; i < 4; ++i) pts[i].key = hull_key(pts[i].x, pts[i].y);
  hull_qsort(pts + 1, 0, 2);
  int len = 4;
  int i = 0;
  while (i + 2 < len) {
    const hpt *a = &pts[i], *b = &pts[i + 1], *c = &pts[i + 2];
    double area2 = (b->x - a->x) * (c->y - a->y) - (b->y - a->y) * (c->x - a->x);
    if (area2 <= 0.0) {
      for (int k = i + 1; k + 1 < len; ++k) pts[k] = pts[k + 1];
      len -= 1;
    } else {
      i += 1;
    }
  }
  return len;
}

/* ------------------------------------------------------------------------ */
/* Rust-Debug-style float formatting for the reference's error messages      */
/* ------------------------------------------------------------------------ */

static void rust_f64(double v, char* out, size_t n) {
  if (v != v) { snprintf(out, n, "NaN"); return; }
  if (isinf(v)) { snprintf(out, n, v > 0 ? "inf" : "-inf"); return; }
  if (v == 0.0) { snprintf(out, n, signbit(v) ? "-0.0" : "0.0"); return; }
  char buf[64];
  int prec;
  for (prec = 1; prec <= 17; ++prec) {
    snprintf(buf, sizeof buf, "%.*e", prec - 1, v);
    if (strtod(buf, NULL) == v) break;
  }
  /* buf = d.ddde[+-]XX ; decide notation like Rust's Debug (1e-4 <= |v| < 1e16 -> plain) */
  double av = fabs(v);
  char mant[64];
  char* e = strchr(buf, 'e');
  int ex = atoi(e + 1);
  size_t ml = (size_t)(e - buf);
  memcpy(mant, buf, ml);
  mant[ml] = 0;
  if (av >= 1e-4 && av < 1e16) {
    /* digits without dot */
    char digs[64];
    int nd = 0, neg = mant[0] == '-';
    for (const char* c = mant + neg; *c; ++c)
      if (*c >= '0' && *c <= '9') digs[nd++] = *c;
    digs[nd] = 0;
    char res[96];
    int k = 0;
    if (neg) res[k++] = '-';
    if (ex >= 0) {
      for (int i = 0; i <= ex; ++i) res[k++] = i < nd ? digs[i] : '0';
      res[k++] = '.';
      if (ex + 1 < nd)
        for (int i = ex + 1; i < nd; ++i) res[k++] = digs[i];
      else
        res[k++] = '0';
    } else {
      res[k++] = '0';
      res[k++] = '.';
      for (int i = 0; i < -ex - 1; ++i) res[k++] = '0';
      for (int i = 0; i < nd; ++i) res[k++] = digs[i];
    }
    res[k] = 0;
    snprintf(out, n, "%s", res);
  } else {
    /* strip trailing zeros of mantissa; Rust prints e.g. 1e-5, 1.5e20 */
    size_t L = strlen(mant);
    if (strchr(mant, '.')) {
      while (L > 0 && mant[L - 1] == '0') mant[--L] = 0;
      if (L > 0 && mant[L - 1] == '.') mant[--L] = 0;
    }
    snprintf(out, n, "%se%d", mant, ex);
  }
}

/* ------------------------------------------------------------------------ */
/* hash containers                                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
  uint64_t* keys; /* key+1, 0 = empty */
  int64_t* vals;
  size_t cap, len;
} u64map;

static uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

static void u64map_init(u64map* m, size_t cap) {
  size_t c = 16;
  while (c < cap * 2) c <<= 1;
  m->cap = c;
  m->len = 0;
  m->keys = (uint64_t*)calloc(c, sizeof(uint64_t));
  m->vals = (int64_t*)calloc(c, sizeof(int64_t));
}
static void u64map_free(u64map* m) {
  free(m->keys);
  free(m->vals);
  memset(m, 0, sizeof *m);
}
static int64_t* u64map_find(const u64map* m, uint64_t key) {
  size_t mask = m->cap - 1, i = mix64(key) & mask;
  while (m->keys[i]) {
    if (m->keys[i] == key + 1) return &m->vals[i];
    i = (i + 1) & mask;
  }
  return NULL;
}
static void u64map_grow(u64map* m);
static int64_t* u64map_insert(u64map* m, uint64_t key, int64_t val, int* inserted) {
  if ((m->len + 1) * 2 > m->cap) u64map_grow(m);
  size_t mask = m->cap - 1, i = mix64(key) & mask;
  while (m->keys[i]) {
    if (m->keys[i] == key + 1) {
      if (inserted) *inserted = 0;
      return &m->vals[i];
    }
    i = (i + 1) & mask;
  }
  m->keys[i] = key + 1;
  m->vals[i] = val;
  m->len++;
  if (inserted) *inserted = 1;
  return &m->vals[i];
}
static void u64map_grow(u64map* m) {
  u64map n;
  u64map_init(&n, m->cap);
  for (size_t i = 0; i < m->cap; ++i)
    if (m->keys[i]) u64map_insert(&n, m->keys[i] - 1, m->vals[i], NULL);
  u64map_free(m);
  *m = n;
}

/* stiffness map: (row, col) -> double, kept as u64map with bit-cast values */
static void kadd(u64map* K, uint64_t key, double v) {
  int ins;
  int64_t bits;
  memcpy(&bits, &v, 8);
  int64_t* slot = u64map_insert(K, key, bits, &ins);
  if (!ins) {
    double cur;
    memcpy(&cur, slot, 8);
    cur = cur + v;
    memcpy(slot, &cur, 8);
  }
}

/* ------------------------------------------------------------------------ */
/* the model                                                                 */
/* ------------------------------------------------------------------------ */

struct orc_fem {
  double rel_tol, abs_tol;
  uint32_t nodes_number;
  size_t n_nodes;
  double* xyz;          /* by index */
  uint32_t* idx_number; /* index -> number */
  u64map node_by_number;
  u64map node_by_coords; /* hash of coordinate bits -> chain via linear scan fallback */
  u64map truss_numbers, beam_numbers, plate_numbers;
  u64map truss_pairs, beam_pairs, plate_sets;
  uint32_t* plate_nodes; /* all plate node numbers for the rare subset scan */
  size_t n_plates, cap_plates;
  u64map K;
  char err[512];
};

static int set_err(orc_fem_t* h, int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(h->err, sizeof h->err, fmt, ap);
  va_end(ap);
  return code;
}

orc_fem_t* orc_create(double rel_tol, double abs_tol, uint32_t nodes_number) {
  orc_fem_t* h = (orc_fem_t*)calloc(1, sizeof(orc_fem_t));
  h->rel_tol = rel_tol;
  h->abs_tol = abs_tol;
  h->nodes_number = nodes_number;
  h->xyz = (double*)malloc(sizeof(double) * 3 * (nodes_number ? nodes_number : 1));
  h->idx_number = (uint32_t*)malloc(sizeof(uint32_t) * (nodes_number ? nodes_number : 1));
  u64map_init(&h->node_by_number, 1024);
  u64map_init(&h->node_by_coords, 1024);
  u64map_init(&h->truss_numbers, 1024);
  u64map_init(&h->beam_numbers, 1024);
  u64map_init(&h->plate_numbers, 1024);
  u64map_init(&h->truss_pairs, 1024);
  u64map_init(&h->beam_pairs, 1024);
  u64map_init(&h->plate_sets, 1024);
  u64map_init(&h->K, 4096);
  return h;
}

void orc_destroy(orc_fem_t* h) {
  if (!h) return;
  free(h->xyz);
  free(h->idx_number);
  free(h->plate_nodes);
  u64map_free(&h->node_by_number);
  u64map_free(&h->node_by_coords);
  u64map_free(&h->truss_numbers);
  u64map_free(&h->beam_numbers);
  u64map_free(&h->plate_numbers);
  u64map_free(&h->truss_pairs);
  u64map_free(&h->beam_pairs);
  u64map_free(&h->plate_sets);
  u64map_free(&h->K);
  free(h);
}

const char* orc_last_error(const orc_fem_t* h) { return h->err; }

static uint64_t coord_hash(double x, double y, double z) {
  uint64_t a, b, c;
  /* -0.0 == 0.0 for the reference's coordinate comparison */
  if (x == 0.0) x = 0.0;
  if (y == 0.0) y = 0.0;
  if (z == 0.0) z = 0.0;
  memcpy(&a, &x, 8);
  memcpy(&b, &y, 8);
  memcpy(&c, &z, 8);
  return mix64(a ^ mix64(b ^ mix64(c)));
}

/* add_node, methods_for_node_data_handle.rs:39-79 */
int orc_add_node(orc_fem_t* h, uint32_t number, double x, double y, double z) {
  char bx[40], by[40], bz[40];
  size_t index = h->n_nodes;
  if (h->nodes_number == 0 || index > (size_t)h->nodes_number - 1)
    return set_err(h, ORC_ERR_NODE_LIMIT, "Nodes number could not be greater than %u!", h->nodes_number);
  if (u64map_find(&h->node_by_number, number))
    return set_err(h, ORC_ERR_NODE_NUMBER, "Node with number %u already exists!", number);
  /* exact coordinate duplicate: bucket by hash, confirm by comparison */
  if (x == x && y == y && z == z) {
    uint64_t hk = coord_hash(x, y, z);
    int64_t* hit = u64map_find(&h->node_by_coords, hk);
    if (hit) {
      /* the bucket stores the first index with this hash; scan all on a collision */
      for (size_t i = 0; i < h->n_nodes; ++i)
        if (h->xyz[3 * i] == x && h->xyz[3 * i + 1] == y && h->xyz[3 * i + 2] == z) {
          rust_f64(x, bx, sizeof bx);
          rust_f64(y, by, sizeof by);
          rust_f64(z, bz, sizeof bz);
          return set_err(h, ORC_ERR_NODE_COORDS, "Node with coordinates x: %s, y: %s, z: %s already exists!", bx, by, bz);
        }
    }
    u64map_insert(&h->node_by_coords, hk, (int64_t)index, NULL);
  }
  u64map_insert(&h->node_by_number, number, (int64_t)index, NULL);
  h->xyz[3 * index] = x;
  h->xyz[3 * index + 1] = y;
  h->xyz[3 * index + 2] = z;
  h->idx_number[index] = number;
  h->n_nodes++;
  return ORC_OK;
}

static int node_index(orc_fem_t* h, uint32_t number, size_t* idx) {
  int64_t* v = u64map_find(&h->node_by_number, number);
  if (!v) return set_err(h, ORC_ERR_NODE_NOT_EXIST, "Node with number %u does not exist!", number);
  *idx = (size_t)*v;
  return ORC_OK;
}

static uint64_t pair_key(uint32_t a, uint32_t b) {
  uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
  return ((uint64_t)lo << 32) | hi;
}

/* scatter an element's global matrix: node-pair blocks in the reference's
 * start_positions order, exact zeros skipped, accumulated in call order */
static void scatter(orc_fem_t* h, const size_t* idx, int nn, int ndof, const double* kg) {
  int w = nn * ndof;
  uint64_t nrows = (uint64_t)h->nodes_number * 6u;
  for (int bi = 0; bi < nn; ++bi)
    for (int bj = 0; bj < nn; ++bj)
      for (int a = 0; a < ndof; ++a)
        for (int b = 0; b < ndof; ++b) {
          double v = kg[w * (bi * ndof + a) + bj * ndof + b];
          if (v != 0.0) {
            uint64_t row = (uint64_t)idx[bi] * 6u + (uint64_t)a, col = (uint64_t)idx[bj] * 6u + (uint64_t)b;
            kadd(&h->K, row * nrows + col, v);
          }
        }
}

/* Truss::create checks (truss.rs:44-64) */
static int truss_props(orc_fem_t* h, double young, double area, int has_a2, double area2) {
  char b[40];
  if (young <= 0.0) {
    rust_f64(young, b, sizeof b);
    return set_err(h, ORC_ERR_YOUNG, "Young's modulus %s is less or equal to zero!", b);
  }
  if (area <= 0.0) {
    rust_f64(area, b, sizeof b);
    return set_err(h, ORC_ERR_AREA, "Area %s is less or equal to zero!", b);
  }
  if (has_a2 && area2 <= 0.0) {
    rust_f64(area2, b, sizeof b);
    return set_err(h, ORC_ERR_AREA2, "Area2 %s is less or equal to zero!", b);
  }
  return ORC_OK;
}

int orc_add_truss(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, double young, double area, int has_area2,
                  double area2) {
  size_t idx[2];
  int st;
  if ((st = node_index(h, n1, &idx[0]))) return st;
  if ((st = node_index(h, n2, &idx[1]))) return st;
  if (u64map_find(&h->truss_numbers, number))
    return set_err(h, ORC_ERR_ELEM_NUMBER, "Truss element with number %u already exists!", number);
  if (u64map_find(&h->truss_pairs, pair_key(n1, n2)))
    return set_err(h, ORC_ERR_ELEM_SAME_NODES, "Truss element with node number %u and %u already exists!", n1, n2);
  if ((st = truss_props(h, young, area, has_area2, area2))) return st;
  double kg[36];
  st = orc_truss_global_matrix(h->xyz + 3 * idx[0], h->xyz + 3 * idx[1], young, area, has_area2, area2, h->rel_tol,
                               h->abs_tol, kg);
  if (st) return set_err(h, st, "Truss element %u has coincident nodes %u and %u!", number, n1, n2);
  scatter(h, idx, 2, 3, kg);
  u64map_insert(&h->truss_numbers, number, 0, NULL);
  u64map_insert(&h->truss_pairs, pair_key(n1, n2), 0, NULL);
  return ORC_OK;
}

/* Beam::create checks (beam.rs:63-117) */
static int beam_checks(orc_fem_t* h, uint32_t number, const double* x1, const double* x2, double young,
                       double poisson, double area, double i11, double i22, double it, double shear_factor,
                       const double axis[3]) {
  char b[40], c[40], d[40];
  if (young <= 0.0) {
    rust_f64(young, b, sizeof b);
    return set_err(h, ORC_ERR_YOUNG, "Young's modulus %s is less or equal to zero!", b);
  }
  if (poisson <= 0.0) {
    rust_f64(young, b, sizeof b); /* the reference reports the Young's modulus value here (beam.rs:84) */
    return set_err(h, ORC_ERR_POISSON, "Poisson's ratio %s is less or equal to zero!", b);
  }
  if (area <= 0.0) {
    rust_f64(area, b, sizeof b);
    return set_err(h, ORC_ERR_AREA, "Area %s is less or equal to zero!", b);
  }
  if (i11 <= 0.0) {
    rust_f64(i11, b, sizeof b);
    return set_err(h, ORC_ERR_I11, "I11 %s is less or equal to zero!", b);
  }
  if (i22 <= 0.0) {
    rust_f64(i22, b, sizeof b);
    return set_err(h, ORC_ERR_I22, "I22 %s is less or equal to zero!", b);
  }
  if (it <= 0.0) {
    rust_f64(it, b, sizeof b);
    return set_err(h, ORC_ERR_IT, "It %s is less or equal to zero!", b);
  }
  if (shear_factor <= 0.0) {
    rust_f64(shear_factor, b, sizeof b);
    return set_err(h, ORC_ERR_SHEAR_FACTOR, "Shear factor %s is less or equal to zero!", b);
  }
  double dv[3], p[3];
  sub3(x2, x1, dv);
  project_perp(axis, dv, p);
  if (norm3(p) == 0.0) {
    rust_f64(axis[0], b, sizeof b);
    rust_f64(axis[1], c, sizeof c);
    rust_f64(axis[2], d, sizeof d);
    return set_err(h, ORC_ERR_PARALLEL_AXIS, "Local axis 1 direction [%s, %s, %s] parallel to element %u!", b, c, d,
                   number);
  }
  return ORC_OK;
}

int orc_add_beam(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, double young, double poisson, double area,
                 double i11, double i22, double i12, double it, double shear_factor,
                 const double local_axis_1_direction[3]) {
  size_t idx[2];
  int st;
  if ((st = node_index(h, n1, &idx[0]))) return st;
  if ((st = node_index(h, n2, &idx[1]))) return st;
  if (u64map_find(&h->beam_numbers, number))
    return set_err(h, ORC_ERR_ELEM_NUMBER, "Beam element with number %u already exists!", number);
  if (u64map_find(&h->beam_pairs, pair_key(n1, n2)))
    return set_err(h, ORC_ERR_ELEM_SAME_NODES, "Beam element with node number %u and %u already exists!", n1, n2);
  const double* x1 = h->xyz + 3 * idx[0];
  const double* x2 = h->xyz + 3 * idx[1];
  if (idx[0] == idx[1]) return set_err(h, ORC_ERR_ZERO_LENGTH, "Beam element %u has coincident nodes %u and %u!", number, n1, n2);
  if ((st = beam_checks(h, number, x1, x2, young, poisson, area, i11, i22, it, shear_factor, local_axis_1_direction)))
    return st;
  double kg[144];
  st = orc_beam_global_matrix(x1, x2, young, poisson, area, i11, i22, i12, it, shear_factor, local_axis_1_direction,
                              h->rel_tol, h->abs_tol, kg);
  if (st) return set_err(h, st, "Beam element %u has coincident nodes %u and %u!", number, n1, n2);
  scatter(h, idx, 2, 6, kg);
  u64map_insert(&h->beam_numbers, number, 0, NULL);
  u64map_insert(&h->beam_pairs, pair_key(n1, n2), 0, NULL);
  return ORC_OK;
}

static uint64_t set4_key(const uint32_t n[4]) {
  uint32_t s[4] = {n[0], n[1], n[2], n[3]};
  for (int i = 1; i < 4; ++i)
    for (int j = i; j > 0 && s[j - 1] > s[j]; --j) {
      uint32_t t = s[j];
      s[j] = s[j - 1];
      s[j - 1] = t;
    }
  return mix64(((uint64_t)s[0] << 32 | s[1]) ^ mix64((uint64_t)s[2] << 32 | s[3]));
}

/* check_plate_data (methods_for_plate_data_handle.rs:33-60): same node set */
static int plate_same_nodes(orc_fem_t* h, const uint32_t n[4]) {
  int distinct = n[0] != n[1] && n[0] != n[2] && n[0] != n[3] && n[1] != n[2] && n[1] != n[3] && n[2] != n[3];
  if (distinct) {
    int64_t* hit = u64map_find(&h->plate_sets, set4_key(n));
    if (!hit) return 0;
  }
  /* confirm (or, with repeated numbers, decide) by the reference's predicate
   * Plate::is_nodes_numbers_same (plate.rs:1107-1118) */
  for (size_t e = 0; e < h->n_plates; ++e) {
    const uint32_t* m = h->plate_nodes + 4 * e;
    int all = 1;
    for (int k = 0; k < 4 && all; ++k) all = (n[k] == m[0] || n[k] == m[1] || n[k] == m[2] || n[k] == m[3]);
    if (all) return 1;
  }
  return 0;
}

static int plate_checks(orc_fem_t* h, uint32_t number, const double* p1, const double* p2, const double* p3,
                        const double* p4, double young, double poisson, double thickness, double shear_factor) {
  char b[40];
  if (young <= 0.0) {
    rust_f64(young, b, sizeof b);
    return set_err(h, ORC_ERR_YOUNG, "Young's modulus %s is less or equal to zero!", b);
  }
  if (poisson <= 0.0) {
    rust_f64(young, b, sizeof b); /* plate.rs:79 reports the Young's modulus */
    return set_err(h, ORC_ERR_POISSON, "Poisson's ratio %s is less or equal to zero!", b);
  }
  if (thickness <= 0.0) {
    rust_f64(young, b, sizeof b); /* plate.rs:82 reports the Young's modulus */
    return set_err(h, ORC_ERR_THICKNESS, "Thickness %s is less or equal to zero!", b);
  }
  if (shear_factor <= 0.0) {
    rust_f64(shear_factor, b, sizeof b);
    return set_err(h, ORC_ERR_SHEAR_FACTOR, "Shear factor %s is less or equal to zero!", b);
  }
  if (quad_on_line(p1, p2, p3, p4))
    return set_err(h, ORC_ERR_NODES_ON_LINE, "Some nodes of %u element lie on the line!", number);
  if (!quad_on_plane(p1, p2, p3, p4, h->abs_tol))
    return set_err(h, ORC_ERR_NOT_ON_PLANE, "Not all nodes of element %u lie on the plane!", number);
  int st;
  int hs = quad_hull_size(p1, p2, p3, p4, h->rel_tol, h->abs_tol, &st);
  if (st) return set_err(h, ORC_ERR_NODES_ON_LINE, "Some nodes of %u element lie on the line!", number);
  if (hs != 4) return set_err(h, ORC_ERR_NOT_CONVEX, "Element %u non-convex!", number);
  return ORC_OK;
}

int orc_add_plate(orc_fem_t* h, uint32_t number, uint32_t n1, uint32_t n2, uint32_t n3, uint32_t n4, double young,
                  double poisson, double thickness, double shear_factor) {
  uint32_t nn[4] = {n1, n2, n3, n4};
  size_t idx[4];
  int st;
  for (int k = 0; k < 4; ++k)
    if ((st = node_index(h, nn[k], &idx[k]))) return st;
  if (u64map_find(&h->plate_numbers, number))
    return set_err(h, ORC_ERR_ELEM_NUMBER, "Plate element with number %u already exists!", number);
  if (plate_same_nodes(h, nn))
    return set_err(h, ORC_ERR_ELEM_SAME_NODES, "Plate element with nodes numbers [%u, %u, %u, %u] already exists!",
                   n1, n2, n3, n4);
  const double *p1 = h->xyz + 3 * idx[0], *p2 = h->xyz + 3 * idx[1], *p3 = h->xyz + 3 * idx[2],
               *p4 = h->xyz + 3 * idx[3];
  if ((st = plate_checks(h, number, p1, p2, p3, p4, young, poisson, thickness, shear_factor))) return st;
  double kg[576];
  st = orc_plate_global_matrix(p1, p2, p3, p4, young, poisson, thickness, shear_factor, h->rel_tol, h->abs_tol, kg);
  if (st) return set_err(h, ORC_ERR_NODES_ON_LINE, "Some nodes of %u element lie on the line!", number);
  scatter(h, idx, 4, 6, kg);
  u64map_insert(&h->plate_numbers, number, 0, NULL);
  u64map_insert(&h->plate_sets, set4_key(nn), 0, NULL);
  if (h->n_plates == h->cap_plates) {
    h->cap_plates = h->cap_plates ? 2 * h->cap_plates : 1024;
    h->plate_nodes = (uint32_t*)realloc(h->plate_nodes, sizeof(uint32_t) * 4 * h->cap_plates);
  }
  memcpy(h->plate_nodes + 4 * h->n_plates, nn, sizeof nn);
  h->n_plates++;
  return ORC_OK;
}

/* batched forms */
int orc_add_nodes(orc_fem_t* h, const uint32_t* numbers, const double* xyz, size_t n, size_t* n_added) {
  size_t i;
  int st = ORC_OK;
  for (i = 0; i < n; ++i)
    if ((st = orc_add_node(h, numbers[i], xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]))) break;
  if (n_added) *n_added = i;
  return st;
}
int orc_add_trusses(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes2, const double* young,
                    const double* area, const double* area2_or_nan, size_t n, size_t* n_added) {
  size_t i;
  int st = ORC_OK;
  for (i = 0; i < n; ++i) {
    double a2 = area2_or_nan ? area2_or_nan[i] : NAN;
    int has = a2 == a2;
    if ((st = orc_add_truss(h, numbers[i], nodes2[2 * i], nodes2[2 * i + 1], young[i], area[i], has, has ? a2 : 0.0)))
      break;
  }
  if (n_added) *n_added = i;
  return st;
}
int orc_add_beams(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes2, const double* young,
                  const double* poisson, const double* area, const double* i11, const double* i22, const double* i12,
                  const double* it, const double* shear_factor, const double* axis3, size_t n, size_t* n_added) {
  size_t i;
  int st = ORC_OK;
  for (i = 0; i < n; ++i)
    if ((st = orc_add_beam(h, numbers[i], nodes2[2 * i], nodes2[2 * i + 1], young[i], poisson[i], area[i], i11[i],
                           i22[i], i12[i], it[i], shear_factor[i], axis3 + 3 * i)))
      break;
  if (n_added) *n_added = i;
  return st;
}
int orc_add_plates(orc_fem_t* h, const uint32_t* numbers, const uint32_t* nodes4, const double* young,
                   const double* poisson, const double* thickness, const double* shear_factor, size_t n,
                   size_t* n_added) {
  size_t i;
  int st = ORC_OK;
  for (i = 0; i < n; ++i)
    if ((st = orc_add_plate(h, numbers[i], nodes4[4 * i], nodes4[4 * i + 1], nodes4[4 * i + 2], nodes4[4 * i + 3],
                            young[i], poisson[i], thickness[i], shear_factor[i])))
      break;
  if (n_added) *n_added = i;
  return st;
}

/* ------------------------------------------------------------------------ */
/* read-out                                                                  */
/* ------------------------------------------------------------------------ */

int64_t orc_n_rows(const orc_fem_t* h) { return (int64_t)h->nodes_number * 6; }
int64_t orc_nnz(const orc_fem_t* h) { return (int64_t)h->K.len; }
int64_t orc_n_nodes(const orc_fem_t* h) { return (int64_t)h->n_nodes; }

int orc_get_index_node_numbers(const orc_fem_t* h, uint32_t* numbers) {
  memcpy(numbers, h->idx_number, sizeof(uint32_t) * h->n_nodes);
  return ORC_OK;
}

typedef struct {
  uint64_t key;
  double val;
} kv;

static int kv_cmp(const void* a, const void* b) {
  uint64_t x = ((const kv*)a)->key, y = ((const kv*)b)->key;
  return x < y ? -1 : x > y ? 1 : 0;
}

/* entries sorted by (row, col): counting sort by row, then a small sort per row */
static kv* sorted_entries(const orc_fem_t* h) {
  uint64_t nrows = (uint64_t)h->nodes_number * 6u;
  size_t n = h->K.len;
  kv* e = (kv*)malloc(sizeof(kv) * (n ? n : 1));
  int64_t* off = (int64_t*)calloc(nrows + 2, sizeof(int64_t));
  for (size_t i = 0; i < h->K.cap; ++i)
    if (h->K.keys[i]) off[(h->K.keys[i] - 1) / nrows + 2]++;
  for (uint64_t r = 0; r < nrows; ++r) off[r + 2] += off[r + 1];
  for (size_t i = 0; i < h->K.cap; ++i)
    if (h->K.keys[i]) {
      uint64_t key = h->K.keys[i] - 1;
      int64_t at = off[key / nrows + 1]++;
      e[at].key = key;
      memcpy(&e[at].val, &h->K.vals[i], 8);
    }
  for (uint64_t r = 0; r < nrows; ++r) {
    int64_t b = off[r], m = off[r + 1] - off[r];
    if (m > 1) qsort(e + b, (size_t)m, sizeof(kv), kv_cmp);
  }
  free(off);
  return e;
}

static int u64_cmp(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return x < y ? -1 : x > y ? 1 : 0;
}

int orc_get_csr(const orc_fem_t* h, int64_t* row_ptr, int32_t* col_idx, double* values) {
  uint64_t nrows = (uint64_t)h->nodes_number * 6u;
  kv* e = sorted_entries(h);
  size_t n = h->K.len;
  for (uint64_t r = 0; r <= nrows; ++r) row_ptr[r] = 0;
  for (size_t i = 0; i < n; ++i) {
    uint64_t r = e[i].key / nrows;
    row_ptr[r + 1]++;
    col_idx[i] = (int32_t)(e[i].key % nrows);
    values[i] = e[i].val;
  }
  for (uint64_t r = 0; r < nrows; ++r) row_ptr[r + 1] += row_ptr[r];
  free(e);
  return ORC_OK;
}

/* groups = distinct (row node, col node, kind) over the pattern, in sorted
 * order (docs/Stiffness_groups.md: every node-pair 6x6 block splits into the
 * 3x3 groups Kuu, Kuth, Kthu, Kthth) */
static int64_t groups_impl(const orc_fem_t* h, int32_t* row_node, int32_t* col_node, uint8_t* kind,
                           int32_t* nnz_group) {
  uint64_t nrows = (uint64_t)h->nodes_number * 6u;
  kv* e = sorted_entries(h);
  size_t n = h->K.len;
  uint64_t* gk = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  for (size_t i = 0; i < n; ++i) {
    uint64_t r = e[i].key / nrows, c = e[i].key % nrows;
    uint64_t kd = 2u * ((r % 6u) / 3u) + (c % 6u) / 3u;
    gk[i] = ((r / 6u) << 34) | ((c / 6u) << 2) | kd; /* node indices < 2^30 */
  }
  /* entries are sorted by row, so each row node's entries are contiguous:
   * sort and unique its group keys locally */
  uint64_t* sk = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  size_t ng = 0, i = 0;
  while (i < n) {
    uint64_t rn = gk[i] >> 34;
    size_t j = i;
    while (j < n && (gk[j] >> 34) == rn) ++j;
    size_t g0 = ng;
    memcpy(sk + ng, gk + i, sizeof(uint64_t) * (j - i));
    qsort(sk + ng, j - i, sizeof(uint64_t), u64_cmp);
    size_t w = g0;
    for (size_t k = g0; k < g0 + (j - i); ++k)
      if (k == g0 || sk[k] != sk[k - 1]) sk[w++] = sk[k];
    if (nnz_group)
      for (size_t k = i; k < j; ++k) {
        size_t lo = g0, hi = w;
        while (lo < hi) {
          size_t mid = (lo + hi) / 2;
          if (sk[mid] < gk[k]) lo = mid + 1;
          else hi = mid;
        }
        nnz_group[k] = (int32_t)lo;
      }
    ng = w;
    i = j;
  }
  if (row_node) {
    for (size_t g = 0; g < ng; ++g) {
      row_node[g] = (int32_t)(sk[g] >> 34);
      col_node[g] = (int32_t)((sk[g] >> 2) & ((1ull << 32) - 1));
      kind[g] = (uint8_t)(sk[g] & 3u);
    }
  }
  free(gk);
  free(sk);
  free(e);
  return (int64_t)ng;
}

int64_t orc_n_groups(const orc_fem_t* h) { return groups_impl(h, NULL, NULL, NULL, NULL); }
int orc_get_groups(const orc_fem_t* h, int32_t* row_node, int32_t* col_node, uint8_t* kind, int32_t* nnz_group) {
  groups_impl(h, row_node, col_node, kind, nnz_group);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* multi-threaded assembly of a whole mesh (the timed CPU reference arm)     */
/* ------------------------------------------------------------------------ */

/* Row-partitioned port of the eager assembly: thread t owns the node range
 * [n0, n1) and walks every element in call order, forming the element matrix
 * (element routines above) whenever the element touches its range and adding
 * the non-zero entries of its own rows to a private hash map.  Each entry is
 * therefore summed in element call order exactly as in orc_add_* (results
 * are bit-identical), and threads share nothing but the read-only inputs. */
typedef struct {
  const orc_mesh_t* m;
  double rel_tol, abs_tol;
  size_t n0, n1;
  u64map K;
  int status;
} asm_job;

static int touches(const int32_t* nd, int k, size_t n0, size_t n1) {
  for (int i = 0; i < k; ++i)
    if ((size_t)nd[i] >= n0 && (size_t)nd[i] < n1) return 1;
  return 0;
}

static void scatter_rows(u64map* K, uint64_t nrows, const int32_t* idx, int nn, int ndof, const double* kg, size_t n0,
                         size_t n1) {
  int w = nn * ndof;
  for (int bi = 0; bi < nn; ++bi) {
    if ((size_t)idx[bi] < n0 || (size_t)idx[bi] >= n1) continue;
    for (int bj = 0; bj < nn; ++bj)
      for (int a = 0; a < ndof; ++a)
        for (int b = 0; b < ndof; ++b) {
          double v = kg[w * (bi * ndof + a) + bj * ndof + b];
          if (v != 0.0) {
            uint64_t row = (uint64_t)idx[bi] * 6u + (uint64_t)a, col = (uint64_t)idx[bj] * 6u + (uint64_t)b;
            kadd(K, row * nrows + col, v);
          }
        }
  }
}

static void* asm_worker(void* p) {
  asm_job* j = (asm_job*)p;
  const orc_mesh_t* m = j->m;
  uint64_t nrows = (uint64_t)m->nodes_number * 6u;
  double kg[576];
  const double* X = m->xyz;
  for (size_t e = 0; e < m->n_truss; ++e) {
    const int32_t* nd = m->t_nodes + 2 * e;
    if (!touches(nd, 2, j->n0, j->n1)) continue;
    double a2 = m->t_area2 ? m->t_area2[e] : NAN;
    if (orc_truss_global_matrix(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], m->t_young[e], m->t_area[e], a2 == a2,
                                a2 == a2 ? a2 : 0.0, j->rel_tol, j->abs_tol, kg)) {
      j->status = ORC_ERR_ZERO_LENGTH;
      continue;
    }
    scatter_rows(&j->K, nrows, nd, 2, 3, kg, j->n0, j->n1);
  }
  for (size_t e = 0; e < m->n_beam; ++e) {
    const int32_t* nd = m->b_nodes + 2 * e;
    if (!touches(nd, 2, j->n0, j->n1)) continue;
    if (orc_beam_global_matrix(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], m->b_young[e], m->b_poisson[e],
                               m->b_area[e], m->b_i11[e], m->b_i22[e], m->b_i12[e], m->b_it[e], m->b_shear[e],
                               m->b_axis + 3 * e, j->rel_tol, j->abs_tol, kg)) {
      j->status = ORC_ERR_ZERO_LENGTH;
      continue;
    }
    scatter_rows(&j->K, nrows, nd, 2, 6, kg, j->n0, j->n1);
  }
  for (size_t e = 0; e < m->n_plate; ++e) {
    const int32_t* nd = m->p_nodes + 4 * e;
    if (!touches(nd, 4, j->n0, j->n1)) continue;
    if (orc_plate_global_matrix(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], X + 3 * (size_t)nd[2],
                                X + 3 * (size_t)nd[3], m->p_young[e], m->p_poisson[e], m->p_thickness[e],
                                m->p_shear[e], j->rel_tol, j->abs_tol, kg)) {
      j->status = ORC_ERR_NODES_ON_LINE;
      continue;
    }
    scatter_rows(&j->K, nrows, nd, 4, 6, kg, j->n0, j->n1);
  }
  return NULL;
}

int orc_assemble_parallel(const orc_mesh_t* mesh, double rel_tol, double abs_tol, int n_threads, int64_t* row_ptr,
                          int32_t* col_idx, double* values, int64_t values_cap, int64_t* nnz_out, double* seconds) {
  if (n_threads < 1) n_threads = 1;
  uint64_t nrows = (uint64_t)mesh->nodes_number * 6u;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
  asm_job* jobs = (asm_job*)calloc((size_t)n_threads, sizeof(asm_job));
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < n_threads; ++t) {
    jobs[t].m = mesh;
    jobs[t].rel_tol = rel_tol;
    jobs[t].abs_tol = abs_tol;
    jobs[t].n0 = (size_t)mesh->nodes_number * (size_t)t / (size_t)n_threads;
    jobs[t].n1 = (size_t)mesh->nodes_number * (size_t)(t + 1) / (size_t)n_threads;
    u64map_init(&jobs[t].K, 4096);
    pthread_create(&th[t], NULL, asm_worker, &jobs[t]);
  }
  int st = ORC_OK;
  for (int t = 0; t < n_threads; ++t) {
    pthread_join(th[t], NULL);
    if (jobs[t].status) st = jobs[t].status;
  }
  /* CSR: each thread's rows are a contiguous row range; count, then fill */
  int64_t nnz = 0;
  for (int t = 0; t < n_threads; ++t) nnz += (int64_t)jobs[t].K.len;
  if (nnz_out) *nnz_out = nnz;
  if (row_ptr && nnz <= values_cap) {
    for (uint64_t r = 0; r <= nrows; ++r) row_ptr[r] = 0;
    for (int t = 0; t < n_threads; ++t) {
      u64map* K = &jobs[t].K;
      for (size_t i = 0; i < K->cap; ++i)
        if (K->keys[i]) row_ptr[(K->keys[i] - 1) / nrows + 1]++;
    }
    for (uint64_t r = 0; r < nrows; ++r) row_ptr[r + 1] += row_ptr[r];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (nrows + 1));
    memcpy(fill, row_ptr, sizeof(int64_t) * (nrows + 1));
    kv* e = (kv*)malloc(sizeof(kv) * (size_t)(nnz ? nnz : 1));
    for (int t = 0; t < n_threads; ++t) {
      u64map* K = &jobs[t].K;
      for (size_t i = 0; i < K->cap; ++i)
        if (K->keys[i]) {
          uint64_t key = K->keys[i] - 1;
          int64_t at = fill[key / nrows]++;
          e[at].key = key;
          memcpy(&e[at].val, &K->vals[i], 8);
        }
    }
    for (uint64_t r = 0; r < nrows; ++r) {
      int64_t b = row_ptr[r], n = row_ptr[r + 1] - b;
      if (n > 1) qsort(e + b, (size_t)n, sizeof(kv), kv_cmp);
      for (int64_t k = b; k < b + n; ++k) {
        col_idx[k] = (int32_t)(e[k].key % nrows);
        values[k] = e[k].val;
      }
    }
    free(e);
    free(fill);
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  for (int t = 0; t < n_threads; ++t) u64map_free(&jobs[t].K);
  free(th);
  free(jobs);
  return st;
}

/* ------------------------------------------------------------------------ */
/* element results (methods_for_element_analysis.rs:27-58)                   */
/* ------------------------------------------------------------------------ */

/* row i of R times a 3-vector as a left-to-right fma chain */
static inline double rrow(const double R[9], int i, const double* u) {
  return fma(R[3 * i + 2], u[2], fma(R[3 * i + 1], u[1], R[3 * i] * u[0]));
}

/* truss.rs:281-333.  One integration point r = 0, B = [dh1, 0, 0, dh2, 0, 0] / (L/2)
 * with dh1 = -1/2, dh2 = 1/2 on the local displacements (R u per node), so the
 * strain is (u2 - u1) / L with u_i the local axial displacement of node i;
 * area = area_at_r(0) = A (+ (A2 - A)/2 when tapered, truss.rs:120-130);
 * ForceR = strain (E area). */
int orc_truss_results(const double x1[3], const double x2[3], double young, double area, int has_area2,
                      double area2, double rel_tol, double abs_tol, const double* u6, double* out1) {
  double R[9];
  int st = orc_truss_rotation(x1, x2, rel_tol, abs_tol, R);
  if (st) return st;
  double d[3];
  sub3(x2, x1, d);
  const double L = norm3(d);
  double a_r = area;
  if (has_area2) a_r = area + (area2 - area) * 0.5;
  const double u1 = rrow(R, 0, u6), u2 = rrow(R, 0, u6 + 3);
  out1[0] = ((u2 - u1) * (1.0 / L)) * (young * a_r);
  return ORC_OK;
}

/* beam.rs:803-993.  One integration point r = 0 (h1 = h2 = 1/2, dh1 = -1/2,
 * dh2 = 1/2, 1/J = 2/L) on the local displacements ul = (R u) per 3-block
 * (u1, th1, u2, th2); with s = 1/L the six strains of beam.rs:260-493 are
 *   e_u   = (ul6 - ul0) s
 *   e_v   = (ul7 - ul1) s - (ul5 + ul11)/2      (dv/dx - th_w)
 *   e_w   = (ul8 - ul2) s - (ul4 + ul10)/2      (dw/dx - th_v)
 *   e_thu = (ul9 - ul3) s, e_thv = (ul10 - ul4) s, e_thw = (ul11 - ul5) s
 * and the results, G = E / (2 (1 + nu)):
 *   ForceR = e_u (E A), ForceS = e_v ((G A) k), ForceT = e_w ((G A) k),
 *   MomentR = e_thu (G It), MomentS = e_thv (E I22p) at mid-length and
 *   +- (L ForceT)/2 at the nodes, MomentT = e_thw (E I11p), +- (L ForceS)/2.
 * out10: ForceR, ForceS, ForceT, MomentR, MomentS (node 1, average, node 2),
 * MomentT (node 1, average, node 2) -- the reference's component order. */
int orc_beam_results(const double x1[3], const double x2[3], double young, double poisson, double area, double i11,
                     double i22, double i12, double it, double shear_factor, const double axis[3], double rel_tol,
                     double abs_tol, const double* u12, double* out10) {
  double R[9], i11p, i22p;
  int st = orc_beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol, R, &i11p, &i22p);
  if (st) return st;
  double d[3];
  sub3(x2, x1, d);
  const double L = norm3(d);
  const double s = 1.0 / L;
  double ul[12];
  for (int b = 0; b < 4; ++b)
    for (int i = 0; i < 3; ++i) ul[3 * b + i] = rrow(R, i, u12 + 3 * b);
  const double G = young / (2.0 * (1.0 + poisson));
  const double gak = (G * area) * shear_factor;
  const double eu = (ul[6] - ul[0]) * s;
  const double ev = fma(ul[7] - ul[1], s, (ul[5] + ul[11]) * -0.5);
  const double ew = fma(ul[8] - ul[2], s, (ul[4] + ul[10]) * -0.5);
  const double fr = eu * (young * area);
  const double fs = ev * gak;
  const double ft = ew * gak;
  const double mr = ((ul[9] - ul[3]) * s) * (G * it);
  const double ms = ((ul[10] - ul[4]) * s) * (young * i22p);
  const double mt = ((ul[11] - ul[5]) * s) * (young * i11p);
  const double hs = (L * ft) * 0.5, ht = (L * fs) * 0.5;
  out10[0] = fr;
  out10[1] = fs;
  out10[2] = ft;
  out10[3] = mr;
  out10[4] = ms + hs;
  out10[5] = ms;
  out10[6] = ms - hs;
  out10[7] = mt + ht;
  out10[8] = mt;
  out10[9] = mt - ht;
  return ORC_OK;
}

/* plate.rs:1196-1409.  The reference sums the strain-displacement matrices
 * (membrane plate.rs:160-274, bending :276-390, assumed-strain shear
 * :392-511) over the four corner points (r, s) = (1,1), (-1,1), (-1,-1),
 * (1,-1) and multiplies the sum by the local displacements (R u per node).
 *
 * At a corner only the corner node and its two edge neighbours have nonzero
 * shape-function derivatives and the Jacobian rows are half the two edge
 * vectors, so dh/dx, dh/dy there is the gradient of the nodal field from its
 * differences along those edges.  With the four edges (local coordinates,
 * node 3 at the origin; head minus tail)
 *   E0 = X1 - X2, E1 = X4 - X3 (the r direction), E2 = X1 - X4, E3 = X2 - X3 (s),
 * corner k has (a, b) = (E0, E2), (E0, E3), (E1, E3), (E1, E2),
 * d_k = a x b = 4 det J, q_k = 1 / d_k, and for a nodal field f with edge
 * differences F:  df/dx|k = q_k (b_y F_a - a_y F_b),  df/dy|k = q_k (a_x F_b - b_x F_a).
 * Each edge belongs to two corners, so the corner sums are edge sums with
 * geometric weights (corner order inside each weight):
 *   Wx0 = y2 q0 + y3 q1    Wy0 = -(x2 q0 + x3 q1)     (xi, yi: components of Ei)
 *   Wx1 = y3 q2 + y2 q3    Wy1 = -(x3 q2 + x2 q3)
 *   Wx2 = -(y0 q0 + y1 q3) Wy2 = x0 q0 + x1 q3
 *   Wx3 = -(y0 q1 + y1 q2) Wy3 = x0 q1 + x1 q2
 * sum_k df/dx = sum_e Wx_e F_e, sum_k df/dy = sum_e Wy_e F_e.  The shear
 * multipliers of plate.rs:443-447 are |b| q_k (gamma_rz) and |a| q_k
 * (gamma_sz), and the tying value of an edge row (plate.rs:452-508) is
 *   Gam_e = (w_h - w_t) + (x_e (thy_h + thy_t) - y_e (thx_h + thx_t)) / 2,
 * so sum_k gamma_rz = Gam0 (l2 q0 + l3 q1) + Gam1 (l3 q2 + l2 q3) and
 * sum_k gamma_sz = Gam2 (l0 q0 + l1 q3) + Gam3 (l0 q1 + l1 q2), l_e = |E_e|.
 * The four q_k share one reciprocal.  Forces: membrane C_m e (t/4) with
 * C_m = E/(1-nu^2) [[1,nu,0],[nu,1,0],[0,0,(1-nu)/2]]; bending C_b k (t^2/24),
 * C_b = E t/(2(1-nu^2)) [same]; shear E/(2(1+nu)) g (t k_s / 4), where
 * e = (du/dx, dv/dy, du/dy + dv/dx), k = (-dthy/dx, dthx/dy, dthx/dx - dthy/dy)
 * and g = (gamma_rz, gamma_sz) are the corner sums.
 * out8: MembraneForceR, MembraneForceS, MembraneForceRS, BendingMomentR (the
 * second bending row), BendingMomentS (the first), BendingMomentRS,
 * ShearForceRT, ShearForceST. */
int orc_plate_results(const double x1[3], const double x2[3], const double x3[3], const double x4[3], double young,
                      double poisson, double thickness, double shear_factor, double rel_tol, double abs_tol,
                      const double* u24, double* out8) {
  double R[9];
  int st = orc_plate_rotation(x2, x3, x4, rel_tol, abs_tol, R);
  if (st) return st;
  const double* X[4] = {x1, x2, x3, x4};
  double xl[4] = {0, 0, 0, 0}, yl[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    if (i == 2) continue;
    double dd[3];
    sub3(X[i], x3, dd);
    xl[i] = (R[0] * dd[0] + R[1] * dd[1]) + R[2] * dd[2];
    yl[i] = (R[3] * dd[0] + R[4] * dd[1]) + R[5] * dd[2];
  }
  /* local nodal fields u, v, w, thx, thy */
  double fu[4], fv[4], fw[4], ftx[4], fty[4];
  for (int i = 0; i < 4; ++i) {
    const double* ui = u24 + 6 * i;
    fu[i] = rrow(R, 0, ui);
    fv[i] = rrow(R, 1, ui);
    fw[i] = rrow(R, 2, ui);
    ftx[i] = rrow(R, 0, ui + 3);
    fty[i] = rrow(R, 1, ui + 3);
  }
  static const int eh[4] = {0, 3, 0, 1}, et[4] = {1, 2, 3, 2};
  double ex[4], ey[4], el[4], Fu[4], Fv[4], Ftx[4], Fty[4], Gm[4];
  for (int e = 0; e < 4; ++e) {
    const int p = eh[e], q = et[e];
    ex[e] = xl[p] - xl[q];
    ey[e] = yl[p] - yl[q];
    el[e] = sqrt(fma(ex[e], ex[e], ey[e] * ey[e]));
    Fu[e] = fu[p] - fu[q];
    Fv[e] = fv[p] - fv[q];
    Ftx[e] = ftx[p] - ftx[q];
    Fty[e] = fty[p] - fty[q];
    Gm[e] = fma(fma(ex[e], fty[p] + fty[q], -(ey[e] * (ftx[p] + ftx[q]))), 0.5, fw[p] - fw[q]);
  }
  double dk[4];
  dk[0] = fma(ex[0], ey[2], -(ey[0] * ex[2]));
  dk[1] = fma(ex[0], ey[3], -(ey[0] * ex[3]));
  dk[2] = fma(ex[1], ey[3], -(ey[1] * ex[3]));
  dk[3] = fma(ex[1], ey[2], -(ey[1] * ex[2]));
  double q[4];
  {
    const double d01 = dk[0] * dk[1], d23 = dk[2] * dk[3];
    const double inv = 1.0 / (d01 * d23);
    q[0] = (dk[1] * d23) * inv;
    q[1] = (dk[0] * d23) * inv;
    q[2] = (dk[3] * d01) * inv;
    q[3] = (dk[2] * d01) * inv;
  }
  const double Wx[4] = {fma(ey[2], q[0], ey[3] * q[1]), fma(ey[3], q[2], ey[2] * q[3]),
                        -fma(ey[0], q[0], ey[1] * q[3]), -fma(ey[0], q[1], ey[1] * q[2])};
  const double Wy[4] = {-fma(ex[2], q[0], ex[3] * q[1]), -fma(ex[3], q[2], ex[2] * q[3]),
                        fma(ex[0], q[0], ex[1] * q[3]), fma(ex[0], q[1], ex[1] * q[2])};
  double e0 = Wx[0] * Fu[0], e1 = Wy[0] * Fv[0], k0 = Wx[0] * Fty[0], k1 = Wy[0] * Ftx[0];
  double e2 = fma(Wx[0], Fv[0], Wy[0] * Fu[0]), k2 = fma(Wx[0], Ftx[0], -(Wy[0] * Fty[0]));
  for (int e = 1; e < 4; ++e) {
    e0 = fma(Wx[e], Fu[e], e0);
    e1 = fma(Wy[e], Fv[e], e1);
    e2 = fma(Wx[e], Fv[e], fma(Wy[e], Fu[e], e2));
    k0 = fma(Wx[e], Fty[e], k0);
    k1 = fma(Wy[e], Ftx[e], k1);
    k2 = fma(-Wy[e], Fty[e], fma(Wx[e], Ftx[e], k2));
  }
  k0 = -k0;
  const double g0 = fma(Gm[1], fma(el[3], q[2], el[2] * q[3]), Gm[0] * fma(el[2], q[0], el[3] * q[1]));
  const double g1 = fma(Gm[3], fma(el[0], q[1], el[1] * q[2]), Gm[2] * fma(el[0], q[0], el[1] * q[3]));
  const double nu = poisson, t = thickness;
  // one division: E / (2 (1 + nu)) = E ((1 - nu) / 2) / (1 - nu^2), and t^2 / 24 by the constant 1/24
  const double dinv = 1.0 / (1.0 - nu * nu);
  const double hn = (1.0 - nu) * 0.5;
  const double cm = (young * dinv) * (t * 0.25);
  const double cbm = ((young * t) * (0.5 * dinv)) * ((t * t) * (1.0 / 24.0));
  const double cs = ((young * hn) * dinv) * ((t * shear_factor) * 0.25);
  out8[0] = cm * fma(nu, e1, e0);
  out8[1] = cm * fma(nu, e0, e1);
  out8[2] = cm * (hn * e2);
  out8[3] = cbm * fma(nu, k0, k1);
  out8[4] = cbm * fma(nu, k1, k0);
  out8[5] = cbm * (hn * k2);
  out8[6] = cs * g0;
  out8[7] = cs * g1;
  return ORC_OK;
}

/* A mesh's element results from a displacements vector (6 per node, node
 * index order), n_threads threads over contiguous element ranges; outputs in
 * element call order (NULL skips a kind); *seconds: wall time. */
typedef struct {
  const orc_mesh_t* m;
  const double* disp;
  double rel_tol, abs_tol;
  double *t_out, *b_out, *p_out;
  size_t t0, t1, b0, b1, p0, p1;
  int status;
} res_job;

static void gather_u(const double* disp, const int32_t* nd, int nn, int per, double* u) {
  for (int i = 0; i < nn; ++i)
    for (int c = 0; c < per; ++c) u[per * i + c] = disp[6 * (size_t)nd[i] + (size_t)c];
}

static void* res_worker(void* arg) {
  res_job* j = (res_job*)arg;
  const orc_mesh_t* m = j->m;
  const double* X = m->xyz;
  double u[24];
  if (j->t_out)
    for (size_t e = j->t0; e < j->t1; ++e) {
      const int32_t* nd = m->t_nodes + 2 * e;
      double a2 = m->t_area2 ? m->t_area2[e] : NAN;
      gather_u(j->disp, nd, 2, 3, u);
      int st = orc_truss_results(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], m->t_young[e], m->t_area[e],
                                 a2 == a2, a2, j->rel_tol, j->abs_tol, u, j->t_out + e);
      if (st) j->status = st;
    }
  if (j->b_out)
    for (size_t e = j->b0; e < j->b1; ++e) {
      const int32_t* nd = m->b_nodes + 2 * e;
      gather_u(j->disp, nd, 2, 6, u);
      int st = orc_beam_results(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], m->b_young[e], m->b_poisson[e],
                                m->b_area[e], m->b_i11[e], m->b_i22[e], m->b_i12[e], m->b_it[e], m->b_shear[e],
                                m->b_axis + 3 * e, j->rel_tol, j->abs_tol, u, j->b_out + 10 * e);
      if (st) j->status = st;
    }
  if (j->p_out)
    for (size_t e = j->p0; e < j->p1; ++e) {
      const int32_t* nd = m->p_nodes + 4 * e;
      gather_u(j->disp, nd, 4, 6, u);
      int st = orc_plate_results(X + 3 * (size_t)nd[0], X + 3 * (size_t)nd[1], X + 3 * (size_t)nd[2],
                                 X + 3 * (size_t)nd[3], m->p_young[e], m->p_poisson[e], m->p_thickness[e],
                                 m->p_shear[e], j->rel_tol, j->abs_tol, u, j->p_out + 8 * e);
      if (st) j->status = st;
    }
  return NULL;
}

int orc_element_results(const orc_mesh_t* mesh, const double* displacements, double rel_tol, double abs_tol,
                        int n_threads, double* truss_out, double* beam_out, double* plate_out, double* seconds) {
  if (n_threads < 1) n_threads = 1;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
  res_job* jobs = (res_job*)calloc((size_t)n_threads, sizeof(res_job));
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < n_threads; ++t) {
    res_job* j = &jobs[t];
    j->m = mesh;
    j->disp = displacements;
    j->rel_tol = rel_tol;
    j->abs_tol = abs_tol;
    j->t_out = truss_out;
    j->b_out = beam_out;
    j->p_out = plate_out;
    j->t0 = mesh->n_truss * (size_t)t / (size_t)n_threads;
    j->t1 = mesh->n_truss * (size_t)(t + 1) / (size_t)n_threads;
    j->b0 = mesh->n_beam * (size_t)t / (size_t)n_threads;
    j->b1 = mesh->n_beam * (size_t)(t + 1) / (size_t)n_threads;
    j->p0 = mesh->n_plate * (size_t)t / (size_t)n_threads;
    j->p1 = mesh->n_plate * (size_t)(t + 1) / (size_t)n_threads;
    pthread_create(&th[t], NULL, res_worker, j);
  }
  int st = ORC_OK;
  for (int t = 0; t < n_threads; ++t) {
    pthread_join(th[t], NULL);
    if (jobs[t].status) st = jobs[t].status;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (seconds) *seconds = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
  free(th);
  free(jobs);
  return st;
}
