// element_math.cuh -- FP64 element arithmetic of the truss, beam and plate
// elements of the Rust crate finite_element_method (src/fem/structs/*.rs,
// src/fem/bar_2n_element_functions.rs,
// src/fem/quadrilateral_4n_element_functions.rs), on the device.
//
// Arithmetic contract: IEEE binary64, round to nearest, compiled with
// --fmad=false so that the only fused multiply-adds are the explicit fma()
// calls below.  Every quantity is evaluated in one fixed order, the same order
// the project's CPU oracle uses, so device results are bit-identical to it.
// Transcendentals are implemented here (Cody-Waite reduction and Taylor series,
// table-based arctangent) rather than taken from the CUDA math library so that
// host and device agree to the last bit.
#pragma once
#include <cstdint>

namespace femgpu {

// pi/2 in three parts (from a 300-bit value of pi), 2/pi, 1/n!, atan(k/8), 1/(2k+1)
__device__ __constant__ static const double kPio2_1 = 0x1.921fb54442d18p+0;
__device__ __constant__ static const double kPio2_2 = 0x1.1a62633145c07p-54;
__device__ __constant__ static const double kPio2_3 = -0x1.f1976b7ed8fbcp-110;
#define FEM_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define FEM_PI_F32 3.1415927410125732
#define FEM_RAD2DEG 0x1.ca5dc1a63c1f8p+5

__device__ __forceinline__ double inv_fact(int n) {
  switch (n) {
    case 2: return 0x1.0000000000000p-1;
    case 3: return 0x1.5555555555555p-3;
    case 4: return 0x1.5555555555555p-5;
    case 5: return 0x1.1111111111111p-7;
    case 6: return 0x1.6c16c16c16c17p-10;
    case 7: return 0x1.a01a01a01a01ap-13;
    case 8: return 0x1.a01a01a01a01ap-16;
    case 9: return 0x1.71de3a556c734p-19;
    case 10: return 0x1.27e4fb7789f5cp-22;
    case 11: return 0x1.ae64567f544e4p-26;
    case 12: return 0x1.1eed8eff8d898p-29;
    case 13: return 0x1.6124613a86d09p-33;
    case 14: return 0x1.93974a8c07c9dp-37;
    case 15: return 0x1.ae7f3e733b81fp-41;
    case 16: return 0x1.ae7f3e733b81fp-45;
    case 17: return 0x1.952c77030ad4ap-49;
    case 18: return 0x1.6827863b97d97p-53;
    case 19: return 0x1.2f49b46814157p-57;
    case 20: return 0x1.e542ba4020225p-62;
    case 21: return 0x1.71b8ef6dcf572p-66;
    default: return 0x1.0ce396db7f853p-70;  // 22
  }
}

__device__ __forceinline__ double atan_k8(int k) {
  switch (k) {
    case 0: return 0.0;
    case 1: return 0x1.fd5ba9aac2f6ep-4;
    case 2: return 0x1.f5b75f92c80ddp-3;
    case 3: return 0x1.6f61941e4def1p-2;
    case 4: return 0x1.dac670561bb4fp-2;
    case 5: return 0x1.1e00babdefeb4p-1;
    case 6: return 0x1.4978fa3269ee1p-1;
    case 7: return 0x1.700a7c5784634p-1;
    default: return 0x1.921fb54442d18p-1;  // 8
  }
}

__device__ __forceinline__ void sincos_reduced(double r, double& s, double& c) {
  double r2 = r * r;
  double ps = inv_fact(21);
  ps = fma(ps, r2, -inv_fact(19));
  ps = fma(ps, r2, inv_fact(17));
  ps = fma(ps, r2, -inv_fact(15));
  ps = fma(ps, r2, inv_fact(13));
  ps = fma(ps, r2, -inv_fact(11));
  ps = fma(ps, r2, inv_fact(9));
  ps = fma(ps, r2, -inv_fact(7));
  ps = fma(ps, r2, inv_fact(5));
  ps = fma(ps, r2, -inv_fact(3));
  s = fma(r * r2, ps, r);
  double pc = -inv_fact(22);
  pc = fma(pc, r2, inv_fact(20));
  pc = fma(pc, r2, -inv_fact(18));
  pc = fma(pc, r2, inv_fact(16));
  pc = fma(pc, r2, -inv_fact(14));
  pc = fma(pc, r2, inv_fact(12));
  pc = fma(pc, r2, -inv_fact(10));
  pc = fma(pc, r2, inv_fact(8));
  pc = fma(pc, r2, -inv_fact(6));
  pc = fma(pc, r2, inv_fact(4));
  pc = fma(pc, r2, -inv_fact(2));
  c = fma(r2, pc, 1.0);
}

__device__ __forceinline__ int reduce_pio2(double x, double& r) {
  double k = rint(x * FEM_TWO_OVER_PI);
  double t = fma(-k, 0x1.921fb54442d18p+0, x);
  t = fma(-k, 0x1.1a62633145c07p-54, t);
  t = fma(-k, -0x1.f1976b7ed8fbcp-110, t);
  r = t;
  return ((int)k) & 3;
}

__device__ __forceinline__ double dsin(double x) {
  double r, s, c;
  int q = reduce_pio2(x, r);
  sincos_reduced(r, s, c);
  return q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
}

__device__ __forceinline__ double dcos(double x) {
  double r, s, c;
  int q = reduce_pio2(x, r);
  sincos_reduced(r, s, c);
  return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}

__device__ __forceinline__ double datan(double t) {
  if (t != t) return t;
  bool neg = t < 0.0;
  double a = neg ? -t : t;
  bool inv = a > 1.0;
  if (inv) a = 1.0 / a;
  double kf = rint(a * 8.0);
  int k = (int)kf;
  double c = kf * 0.125;
  double u = (a - c) / fma(a, c, 1.0);
  double u2 = u * u;
  double p = 0x1.e1e1e1e1e1e1ep-5;     // 1/17
  p = fma(p, u2, -0x1.1111111111111p-4);  // 1/15
  p = fma(p, u2, 0x1.3b13b13b13b14p-4);   // 1/13
  p = fma(p, u2, -0x1.745d1745d1746p-4);  // 1/11
  p = fma(p, u2, 0x1.c71c71c71c71cp-4);   // 1/9
  p = fma(p, u2, -0x1.2492492492492p-3);  // 1/7
  p = fma(p, u2, 0x1.999999999999ap-3);   // 1/5
  p = fma(p, u2, -0x1.5555555555555p-2);  // 1/3
  double res = atan_k8(k) + fma(u * u2, p, u);
  if (inv) res = (0x1.921fb54442d18p+0 - res) + 0x1.1a62633145c07p-54;
  return neg ? -res : res;
}

__device__ __forceinline__ double dacos(double x) { return 2.0 * datan(sqrt((1.0 - x) / (1.0 + x))); }

}  // namespace femgpu
#include "dual.cuh"
namespace femgpu {

// ---------------------------------------------------------------------------
// vectors (plain left-to-right, no fusion)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T dot3(const T a[3], const T b[3]) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
template <class T>
__device__ __forceinline__ T norm3(const T a[3]) { return sqrt(dot3(a, a)); }
template <class T>
__device__ __forceinline__ void sub3(const T a[3], const T b[3], T o[3]) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}
template <class T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
// compare_with_tolerance, math_functions.rs:3-12
template <class T>
__device__ __forceinline__ T cwt(T v, double abs_tol) { return fabs(v) < abs_tol ? 0.0 : v; }
// differentiated: the clamp zeroes the value only -- its plateau (|v| < abs_tol) is far narrower than
// any finite-difference step, so the derivative that central differences see passes through
template <>
__device__ __forceinline__ Dual cwt<Dual>(Dual v, double abs_tol) { return fabs(v.v) < abs_tol ? Dual(0.0, v.d) : v; }

template <class T>
__device__ __forceinline__ void set_identity(T R[9]) {
  R[0] = 1.0; R[1] = 0.0; R[2] = 0.0;
  R[3] = 0.0; R[4] = 1.0; R[5] = 0.0;
  R[6] = 0.0; R[7] = 0.0; R[8] = 1.0;
}

// Rotation taking direction a onto direction b (the reference's
// rotation_matrix_to_align_with_vector of extended_matrix, called at
// structs/truss.rs:80, structs/beam.rs:179 and
// quadrilateral_4n_element_functions.rs:158): Rodrigues rotation about a x b,
// R = c I + [v]x + v v^T / (1 + c); exact parallel -> I; exact anti-parallel ->
// half turn about a x e_z (or a x e_x); entries below abs_tol -> 0.
template <class T>
__device__ __forceinline__ void align_rotation(const T a[3], const T b[3], double abs_tol, T R[9]) {
  T ia = 1.0 / norm3(a), ib = 1.0 / norm3(b);
  T ua[3] = {a[0] * ia, a[1] * ia, a[2] * ia};
  T ub[3] = {b[0] * ib, b[1] * ib, b[2] * ib};
  T v[3];
  cross3(ua, ub, v);
  T c = dot3(ua, ub);
  if (v[0] == 0.0 && v[1] == 0.0 && v[2] == 0.0) {
    // Exactly parallel: the identity.  Differentiated code takes the general
    // formula below instead, which gives the same identity value and the
    // rotation's derivative ([dv]x).
    if (c > 0.0 && !IsDual<T>::value) {
      set_identity(R);
      return;
    }
  }
  if (v[0] == 0.0 && v[1] == 0.0 && v[2] == 0.0 && !(c > 0.0)) {
    T ez[3] = {0.0, 0.0, 1.0}, ex[3] = {1.0, 0.0, 0.0}, n[3];
    cross3(ua, ez, n);
    if (n[0] == 0.0 && n[1] == 0.0 && n[2] == 0.0) cross3(ua, ex, n);
    T in = 1.0 / norm3(n);
    n[0] *= in;
    n[1] *= in;
    n[2] *= in;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T tn = 2.0 * n[i];
        R[3 * i + j] = cwt(i == j ? fma(tn, n[j], -1.0) : tn * n[j], abs_tol);
      }
    return;
  }
  T h = 1.0 / (1.0 + c);
  T hv0 = h * v[0], hv1 = h * v[1], hv2 = h * v[2];
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

template <class T>
__device__ __forceinline__ bool is_identity(const T R[9]) {
  return R[0] == 1.0 && R[1] == 0.0 && R[2] == 0.0 && R[3] == 0.0 && R[4] == 1.0 && R[5] == 0.0 && R[6] == 0.0 &&
         R[7] == 0.0 && R[8] == 1.0;
}
// The same test on the integer pipe (on GB300 an FP64 compare takes a slot of
// the narrow FP64 pipe): 1.0 exactly, +-0.0 exactly.
__device__ __forceinline__ bool bits_one(double v) { return __double_as_longlong(v) == 0x3ff0000000000000ll; }
__device__ __forceinline__ bool bits_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
// v > 0.0 (false for +-0.0 and NaN)
__device__ __forceinline__ bool bits_positive(double v) {
  const long long b = __double_as_longlong(v);
  return b > 0 && b <= 0x7ff0000000000000ll;
}
__device__ __forceinline__ bool is_identity(const double R[9]) {
  return bits_one(R[0]) & bits_zero(R[1]) & bits_zero(R[2]) & bits_zero(R[3]) & bits_one(R[4]) & bits_zero(R[5]) &
         bits_zero(R[6]) & bits_zero(R[7]) & bits_one(R[8]);
}

// symmetric R^T diag(d) R (upper computed, lower mirrored)
template <class T>
__device__ __forceinline__ void rt_diag_r(const T R[9], const T d[3], T out[9]) {
  T t[9];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int i = 0; i < 3; ++i) t[3 * k + i] = R[3 * k + i] * d[k];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      T s = fma(t[6 + i], R[6 + j], fma(t[3 + i], R[3 + j], t[i] * R[j]));
      out[3 * i + j] = s;
      out[3 * j + i] = s;
    }
}

// R^T M R for one 3x3 block (dense fma chains); sym: i <= j computed, mirrored
template <class T>
__device__ __forceinline__ void rt_m_r(const T R[9], const T M[9], T out[9], bool sym) {
  T Y[9];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int b = 0; b < 3; ++b) Y[3 * k + b] = fma(M[3 * k + 2], R[6 + b], fma(M[3 * k + 1], R[3 + b], M[3 * k] * R[b]));
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (sym && b < a) continue;
      T s = fma(R[6 + a], Y[6 + b], fma(R[3 + a], Y[3 + b], R[a] * Y[b]));
      out[3 * a + b] = s;
      if (sym) out[3 * b + a] = s;
    }
}

// ---------------------------------------------------------------------------
// truss (structs/truss.rs:66-214)
// ---------------------------------------------------------------------------
// returns false for coincident nodes
template <class T>
__device__ __forceinline__ bool truss_rotation(const T x1[3], const T x2[3], double abs_tol, T R[9]) {
  T d[3];
  sub3(x2, x1, d);
  T L = norm3(d);
  if (!(L > 0.0)) return false;
  T target[3] = {L, 0.0, 0.0};
  align_rotation(d, target, abs_tol, R);
  return true;
}

// g (3x3, node-pair (1,1) block of the 6x6 truss matrix in global axes);
// blocks: (1,1) = g, (1,2) = (2,1) = -g, (2,2) = g
template <class T>
__device__ __forceinline__ bool truss_block(const T x1[3], const T x2[3], T young, T area,
                                            T area2 /* NaN: none */, double abs_tol, T g[9]) {
  T R[9];
  if (!truss_rotation(x1, x2, abs_tol, R)) return false;
  T d[3];
  sub3(x2, x1, d);
  T L = norm3(d);
  T jac = L * 0.5;
  T inv = 1.0 / jac;
  T b = 0.5 * inv;
  T a_r = area;
  if (area2 == area2) {
    T hh = (area2 - area) * 0.5;
    a_r = area + hh;
  }
  T scalar = ((a_r * young) * jac) * 2.0;
  T q = (b * b) * scalar;
  T m[3] = {R[0] * q, R[1] * q, R[2] * q};
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      T s = m[i] * R[j];
      g[3 * i + j] = s;
      g[3 * j + i] = s;
    }
  return true;
}

// ---------------------------------------------------------------------------
// beam (structs/beam.rs)
// ---------------------------------------------------------------------------
// i12 == 0 (a section symmetric about a local axis): atan(+-0) = +0 (the arctangent's reduction takes a
// signed zero to +0), and cos, sin of +0 are exactly 1 and +0 -- the same bits as the general evaluation,
// without its arctangent and series
template <class T>
__device__ __forceinline__ bool principal_axes_aligned(T i12) {
  if constexpr (IsDual<T>::value) return false;
  else return i12 == 0.0;
}

template <class T>
__device__ __forceinline__ void principal_moments(T i11, T i22, T i12, double rel_tol, T& i11p,
                                                  T& i22p, T& angle_out) {
  T angle, c, s, s2;
  if (principal_axes_aligned(i12)) {
    angle = 0.0;
    c = 1.0;
    s = 0.0;
    s2 = 0.0;
  } else {
    if (i11 != i22) {
      angle = datan((2.0 * i12) / (i22 - i11)) / 2.0;
    } else {
      T i11m, i22m;
      if (i22 < i11) {
        i11m = i11;
        i22m = ((fabs(i22) - fabs(i22) * rel_tol) * i22) / fabs(i22);
      } else {
        i11m = ((fabs(i11) - fabs(i11) * rel_tol) * i11) / fabs(i11);
        i22m = i22;
      }
      angle = datan((2.0 * i12) / (i22m - i11m)) / 2.0;
    }
    c = dcos(angle);
    s = dsin(angle);
    s2 = dsin(2.0 * angle);
  }
  T a = (i11 * (c * c) + i22 * (s * s)) - i12 * s2;
  T bb = (i11 * (s * s) + i22 * (c * c)) + i12 * s2;
  int it = 1;
  while (a < bb && it <= 8) {
    angle = (datan((2.0 * i12) / (i22 - i11)) + FEM_PI_F32 * (T)it) / 2.0;
    c = dcos(angle);
    s = dsin(angle);
    s2 = dsin(2.0 * angle);
    a = (i11 * (c * c) + i22 * (s * s)) - i12 * s2;
    bb = (i11 * (s * s) + i22 * (c * c)) + i12 * s2;
    ++it;
  }
  i11p = a;
  i22p = bb;
  angle_out = angle;
}

// projection_perpendicular_to_vector: a - ((a.b)/(b.b)) b
template <class T>
__device__ __forceinline__ void project_perp(const T a[3], const T b[3], T p[3]) {
  T s = dot3(a, b) / dot3(b, b);
  p[0] = a[0] - s * b[0];
  p[1] = a[1] - s * b[1];
  p[2] = a[2] - s * b[2];
}

// The section twist of find_rotation_matrix_elements (beam.rs:162-258): acos of
// the cosine between the rotated projected axis tp and local z, the cosine
// clamped to [-1, 1].
template <class T>
__device__ __forceinline__ T twist_angle(const T tp[3]) {
  T cosang = tp[2] / norm3(tp);
  if (cosang > 1.0) cosang = 1.0;
  if (cosang < -1.0) cosang = -1.0;
  return dacos(cosang);
}
// Differentiated: the value exactly as above; the derivative written without
// the cancellation in 1 - cos^2, which costs eps / theta^2 of relative
// accuracy at a small twist theta.  With q = tp0^2 + tp1^2 (so sin theta =
// sqrt(q) / |tp|):  theta' = -(tp2' q - tp2 (tp0 tp0' + tp1 tp1')) / (|tp|^2 sqrt(q)),
// and 0 where q = 0 (the kink of acos at +-1, whose symmetric derivative is 0).
template <>
__device__ __forceinline__ Dual twist_angle<Dual>(const Dual tp[3]) {
  const double v[3] = {tp[0].v, tp[1].v, tp[2].v};
  const double theta = twist_angle(v);
  const double q = tp[0].v * tp[0].v + tp[1].v * tp[1].v;
  if (!(q > 0.0)) return Dual(theta, 0.0);
  const double num = tp[2].d * q - tp[2].v * (tp[0].v * tp[0].d + tp[1].v * tp[1].d);
  return Dual(theta, -num / ((q + tp[2].v * tp[2].v) * sqrt(q)));
}

// find_rotation_matrix_elements, beam.rs:162-258 (false: coincident nodes)
template <class T>
__device__ __forceinline__ bool beam_rotation(const T x1[3], const T x2[3], T i11, T i22,
                                              T i12, const T axis[3], double rel_tol, double abs_tol,
                                              T R[9], T& i11p, T& i22p) {
  T angle;
  principal_moments(i11, i22, i12, rel_tol, i11p, i22p, angle);
  T d[3];
  sub3(x2, x1, d);
  T L = norm3(d);
  if (!(L > 0.0)) return false;
  T target[3] = {L, 0.0, 0.0};
  T Ri[9];
  align_rotation(d, target, abs_tol, Ri);
  T p[3];
  project_perp(axis, d, p);
  T tp[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) tp[i] = (Ri[3 * i] * p[0] + Ri[3 * i + 1] * p[1]) + Ri[3 * i + 2] * p[2];
  T total = angle + twist_angle(tp);
  T cx = cwt(d[0] / L, abs_tol), cy = cwt(d[1] / L, abs_tol), cz = cwt(d[2] / L, abs_tol);
  T cxz = cwt(sqrt(cx * cx + cz * cz), abs_tol);
  T c = cwt(dcos(total), abs_tol), s = cwt(dsin(total), abs_tol);
  if (cxz != 0.0) {
    R[0] = cx;
    R[1] = cy;
    R[2] = cz;
    R[3] = ((((-1.0 * cx) * cy) * c) - cz * s) / cxz;
    R[4] = cxz * c;
    R[5] = ((((-1.0 * cy) * cz) * c) + cx * s) / cxz;
    R[6] = (((cx * cy) * s) - cz * c) / cxz;
    R[7] = (-1.0 * cxz) * s;
    R[8] = (((cy * cz) * s) + cx * c) / cxz;
  } else {
    R[0] = 0.0;
    R[1] = cy;
    R[2] = 0.0;
    R[3] = (-1.0 * cy) * c;
    R[4] = 0.0;
    R[5] = s;
    R[6] = cy * s;
    R[7] = 0.0;
    R[8] = c;
  }
  return true;
}

// 3x3 blocks of the beam matrix in global axes (block order u1, th1, u2, th2):
// uu, ut (u1-th1 = u1-th2), th (th1-th1 = th2-th2), tu (th1-u2), thth2 (th1-th2);
// u1-u2 = -uu, u2-u2 = uu, u2-th2 = -ut.
template <class T>
struct BeamBlocksT {
  T uu[9], ut[9], th[9], tu[9], thth2[9];
};
using BeamBlocks = BeamBlocksT<double>;


template <class T>
__device__ __forceinline__ bool beam_blocks(const T x1[3], const T x2[3], T young, T poisson,
                                            T area, T i11, T i22, T i12, T it,
                                            T shear_factor, const T axis[3], double rel_tol, double abs_tol,
                                            BeamBlocksT<T>& B) {
  T R[9], i11p, i22p;
  if (!beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol, R, i11p, i22p)) return false;
  T d[3];
  sub3(x2, x1, d);
  T L = norm3(d);
  T jac = L * 0.5, inv = 1.0 / jac;
  T b = 0.5 * inv;
  T hb = 0.5 * b;
  T b2 = b * b;
  T G = young / (2.0 * (1.0 + poisson));
  T su = ((area * young) * jac) * 2.0;
  T sv = ((((G * area) * shear_factor)) * jac) * 2.0;
  T sw = ((((G * area) * shear_factor)) * jac) * 2.0;
  T stu = ((G * it) * jac) * 2.0;
  T stv = ((young * i22p) * jac) * 2.0;
  T stw = ((young * i11p) * jac) * 2.0;
  T A1 = b2 * su, V1 = b2 * sv, W1 = b2 * sw, T1 = b2 * stu, Y1 = b2 * stv, Z1 = b2 * stw;
  T HV = hb * sv, HW = hb * sw, QV = 0.25 * sv, QW = 0.25 * sw;
  T du[3] = {A1, V1, W1};
  T dth[3] = {T1, QW + Y1, QV + Z1};
  T dth2[3] = {-T1, QW + (-Y1), QV + (-Z1)};
  rt_diag_r(R, du, B.uu);
  rt_diag_r(R, dth, B.th);
  rt_diag_r(R, dth2, B.thth2);
  T P[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) P[3 * i + j] = R[3 + i] * R[6 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      B.ut[3 * i + j] = fma(HW, P[3 * j + i], HV * P[3 * i + j]);
      B.tu[3 * i + j] = fma(-HV, P[3 * j + i], (-HW) * P[3 * i + j]);
    }
  return true;
}

// ---------------------------------------------------------------------------
// plate (structs/plate.rs, quadrilateral_4n_element_functions.rs)
// ---------------------------------------------------------------------------
// find_rotation_matrix_elements_of_quadrilateral, quad.rs:131-171 (false: nodes on a line)
template <class T>
__device__ __forceinline__ bool plate_rotation(const T x2[3], const T x3[3], const T x4[3],
                                               double abs_tol, T R[9]) {
  T e34[3], e32[3], n[3];
  sub3(x4, x3, e34);
  sub3(x2, x3, e32);
  cross3(e34, e32, n);
  if constexpr (!IsDual<T>::value) {
    if (bits_zero(n[0]) & bits_zero(n[1]) & bits_positive(n[2])) {
      set_identity(R);
      return true;
    }
  }
  T ln = norm3(n);
  if (!(ln > 0.0)) return false;
  T target[3] = {0.0, 0.0, ln};
  align_rotation(n, target, abs_tol, R);
  return true;
}

// Local in-plane coordinates of the nodes relative to node 3 (quad.rs:340-378):
// (x, y) of R (X_i - X_3).  When R is exactly the identity they are the
// differences themselves (the same values); otherwise each is one product and
// two fused multiply-adds.
template <class T>
__device__ __forceinline__ void plate_local_xy(const T X[4][3], const T R[9], bool ident, T xl[4], T yl[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    xl[i] = 0.0;
    yl[i] = 0.0;
    if (i == 2) continue;
    if (ident) {
      xl[i] = X[i][0] - X[2][0];
      yl[i] = X[i][1] - X[2][1];
    } else {
      T dd[3];
      sub3(X[i], X[2], dd);
      xl[i] = fma(R[2], dd[2], fma(R[1], dd[1], R[0] * dd[0]));
      yl[i] = fma(R[5], dd[2], fma(R[4], dd[1], R[3] * dd[0]));
    }
  }
}

// Everything the plate's 6x6 node-pair blocks are made of (see
// plate_local_matrix in the oracle for the derivation; scaled Jacobian Jh = 4J,
// D = det Jh, one reciprocal for the four determinants).
template <class T>
struct PlateCoreT {
  T Sxx[10], Syy[10], Sxy[16];  // upper-triangle index for Sxx/Syy
  T tb, gam, nu;  // tb = t^2 / 12: bending over membrane stiffness (the S sums carry the membrane factor)
  T F12[3], G12[3], F43[3];
  T E12[3], E43[3];
  T P14[6], P23[6], P1423[9];  // upper-triangle index for P14/P23
};

using PlateCore = PlateCoreT<double>;

__host__ __device__ constexpr int ut4(int i, int j) {  // 4x4 upper index, i <= j
  return i == 0 ? j : i == 1 ? 3 + j : i == 2 ? 5 + j : 9;
}
__host__ __device__ constexpr int ut3(int a, int b) {  // 3x3 upper index, a <= b
  return a == 0 ? b : a == 1 ? 2 + b : 5;
}

template <class T>
__device__ __forceinline__ void plate_core(const T xl[4], const T yl[4], T young, T poisson,
                                           T thickness, T shear_factor, PlateCoreT<T>& C) {
  const double g = sqrt((double)(1.0f / 3.0f));
  const double al = 1.0 + g, be = 1.0 - g;
  T x1 = xl[0], x2 = xl[1], x4 = xl[3];
  T y1 = yl[0], y2 = yl[1], y4 = yl[3];
  T d12x = x1 - x2, d12y = y1 - y2;
  T ax = d12x + x4, bx = d12x - x4, cx = (x1 + x2) - x4;
  T ay = d12y + y4, by = d12y - y4, cy = (y1 + y2) - y4;
  const double ipr[4] = {g * 1.0, g * -1.0, g * -1.0, g * 1.0};
  const double ips[4] = {g * 1.0, g * 1.0, g * -1.0, g * -1.0};
  T J00[4], J01[4], J10[4], J11[4], D[4], q[4];
#pragma unroll
  for (int ip = 0; ip < 4; ++ip) {
    J00[ip] = fma(ips[ip], bx, ax);
    J01[ip] = fma(ips[ip], by, ay);
    J10[ip] = fma(ipr[ip], bx, cx);
    J11[ip] = fma(ipr[ip], by, cy);
    D[ip] = fma(J00[ip], J11[ip], -(J01[ip] * J10[ip]));
  }
  {
    T D01 = D[0] * D[1], D23 = D[2] * D[3];
    T inv = 1.0 / (D01 * D23);
    q[0] = (D[1] * D23) * inv;
    q[1] = (D[0] * D23) * inv;
    q[2] = (D[3] * D01) * inv;
    q[3] = (D[2] * D01) * inv;
  }
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    C.Sxx[k] = 0.0;
    C.Syy[k] = 0.0;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) C.Sxy[k] = 0.0;
  // material (plate.rs:532-548, :580-597, :629-636), one reciprocal: cm/16 = E t / (16 (1 - nu^2)) scales the
  // membrane sums through the integration-point weights; bending is (t^2 / 12) times membrane; shear c_s/64
  T dinv = 1.0 / (1.0 - poisson * poisson);
  T Et = young * thickness;
  const T cmq = (Et * dinv) * 0.0625;
  C.tb = (thickness * thickness) * 0x1.5555555555555p-4;
  T omn = 1.0 - poisson;
  T cq = ((Et * shear_factor) * omn) * (dinv * 0x1p-7);
  C.gam = omn * 0.5;
  C.nu = poisson;
  T Wr[4], Ws[4];
#pragma unroll
  for (int ip = 0; ip < 4; ++ip) {
    const double sp = 1.0 + ips[ip], sm = 1.0 - ips[ip], rp = 1.0 + ipr[ip], rm = 1.0 - ipr[ip];
    // gx = [J11 sp - J01 rp, -J11 sp - J01 rm, J01 rm - J11 sm, J11 sm + J01 rp],
    // gy = [J00 rp - J10 sp, J00 rm + J10 sp, J10 sm - J00 rm, -J00 rp - J10 sm]: one product and one fma each
    const T P3 = J01[ip] * rp, P4 = J01[ip] * rm, Q1 = J00[ip] * rp, Q2 = J00[ip] * rm;
    T gx[4] = {fma(J11[ip], sp, -P3), fma(-J11[ip], sp, -P4), fma(-J11[ip], sm, P4), fma(J11[ip], sm, P3)};
    T gy[4] = {fma(-J10[ip], sp, Q1), fma(J10[ip], sp, Q2), fma(J10[ip], sm, -Q2), fma(-J10[ip], sm, -Q1)};
    const T qm = cmq * q[ip];
    T a[4], bq[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      a[i] = qm * gx[i];
      bq[i] = qm * gy[i];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i; j < 4; ++j) {
        C.Sxx[ut4(i, j)] = fma(a[i], gx[j], C.Sxx[ut4(i, j)]);
        C.Syy[ut4(i, j)] = fma(bq[i], gy[j], C.Syy[ut4(i, j)]);
      }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) C.Sxy[4 * i + j] = fma(a[i], gy[j], C.Sxy[4 * i + j]);
    Wr[ip] = fma(J11[ip], J11[ip], J10[ip] * J10[ip]) * q[ip];
    Ws[ip] = fma(J01[ip], J01[ip], J00[ip] * J00[ip]) * q[ip];
  }
  const double al2 = al * al, be2 = be * be, ab = al * be;
  T W0p = Wr[0] + Wr[1], W0m = Wr[2] + Wr[3];
  T W1p = Ws[0] + Ws[3], W1m = Ws[1] + Ws[2];
  T A12 = cq * fma(W0p, al2, W0m * be2);
  T A1243 = cq * ((W0p + W0m) * ab);
  T A43 = cq * fma(W0p, be2, W0m * al2);
  T B14 = cq * fma(W1p, al2, W1m * be2);
  T B1423 = cq * ((W1p + W1m) * ab);
  T B23 = cq * fma(W1p, be2, W1m * al2);
  C.E12[0] = 2.0; C.E12[1] = -d12y; C.E12[2] = d12x;
  C.E43[0] = 2.0; C.E43[1] = -y4; C.E43[2] = x4;
  T E14[3] = {2.0, -(y1 - y4), x1 - x4};
  T E23[3] = {2.0, -y2, x2};
  T F14[3], H14[3], F23[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    C.F12[k] = A12 * C.E12[k];
    C.G12[k] = A1243 * C.E12[k];
    C.F43[k] = A43 * C.E43[k];
    F14[k] = B14 * E14[k];
    H14[k] = B1423 * E14[k];
    F23[k] = B23 * E23[k];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (b >= a) {
        C.P14[ut3(a, b)] = F14[a] * E14[b];
        C.P23[ut3(a, b)] = F23[a] * E23[b];
      }
      C.P1423[3 * a + b] = H14[a] * E23[b];
    }
}

// Local 6x6 block (i, j), i <= j, of the plate's 24x24 matrix, row-major.
template <class T>
__device__ __forceinline__ void plate_local_block(const PlateCoreT<T>& C, int i, int j, T blk[36]) {
#pragma unroll
  for (int k = 0; k < 36; ++k) blk[k] = 0.0;
  int lo = i < j ? i : j, hi = i < j ? j : i;
  T Sxx = C.Sxx[ut4(lo, hi)], Syy = C.Syy[ut4(lo, hi)];
  T tuu = fma(C.gam, Syy, Sxx);
  T tvv = fma(C.gam, Sxx, Syy);
  T tuv_ij = fma(C.gam, C.Sxy[4 * j + i], C.nu * C.Sxy[4 * i + j]);
  T tuv_ji = fma(C.gam, C.Sxy[4 * i + j], C.nu * C.Sxy[4 * j + i]);
  blk[0] = tuu;
  blk[7] = tvv;
  blk[1] = tuv_ij;
  blk[6] = (i == j) ? tuv_ij : tuv_ji;
  const int g0i = i < 2 ? 0 : 1, g0j = j < 2 ? 0 : 1;
  const T s0i = (i == 1 || i == 2) ? -1.0 : 1.0, s0j = (j == 1 || j == 2) ? -1.0 : 1.0;
  const int g1i = (i == 0 || i == 3) ? 0 : 1, g1j = (j == 0 || j == 3) ? 0 : 1;
  const T s1i = i >= 2 ? -1.0 : 1.0, s1j = j >= 2 ? -1.0 : 1.0;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (i == j && b < a) continue;
      int l3 = a < b ? a : b, h3 = a < b ? b : a;
      T t1;
      if (g1i == 0 && g1j == 0) t1 = C.P14[ut3(l3, h3)];
      else if (g1i == 1 && g1j == 1) t1 = C.P23[ut3(l3, h3)];
      else if (g1i == 0) t1 = C.P1423[3 * a + b];
      else t1 = C.P1423[3 * b + a];
      T sg1 = (a == 0 ? s1i : 1.0) * (b == 0 ? s1j : 1.0);
      if (sg1 < 0) t1 = -t1;
      T f, e;
      if (g0i == 0 && g0j == 0) { f = C.F12[l3]; e = C.E12[h3]; }
      else if (g0i == 1 && g0j == 1) { f = C.F43[l3]; e = C.E43[h3]; }
      else if (g0i == 0) { f = C.G12[a]; e = C.E43[b]; }
      else { f = C.G12[b]; e = C.E43[a]; }
      T sg0 = (a == 0 ? s0i : 1.0) * (b == 0 ? s0j : 1.0);
      if (sg0 < 0) f = -f;
      T sh = fma(f, e, t1);
      T v = sh;
      if (a >= 1 && b >= 1) {
        if (a == 2 && b == 2) v = fma(C.tb, tuu, sh);
        else if (a == 1 && b == 1) v = fma(C.tb, tvv, sh);
        else if (a == 2 && b == 1) v = fma(-C.tb, tuv_ij, sh);
        else v = fma(-C.tb, tuv_ji, sh);
      }
      blk[6 * (2 + a) + 2 + b] = v;
      if (i == j) blk[6 * (2 + b) + 2 + a] = v;
    }
  if (i == j) blk[35] = 0.0 + 1.0;  // KROT6 (plate.rs:25, :716-721)
}

// The same block with the node pair fixed at compile time: every index, group
// and sign of the assumed-strain shear terms folds to a constant, so the only
// FP64 instructions left are the products and sums themselves (same operations,
// same order, bit-identical to plate_local_block).
template <int I, int J, class T>
__device__ __forceinline__ void plate_block_ct(const PlateCoreT<T>& C, T blk[36]) {
  static_assert(I <= J, "pairs are enumerated with I <= J");
  constexpr int g0i = I < 2 ? 0 : 1, g0j = J < 2 ? 0 : 1;
  constexpr bool n0i = I == 1 || I == 2, n0j = J == 1 || J == 2;
  constexpr int g1i = (I == 0 || I == 3) ? 0 : 1, g1j = (J == 0 || J == 3) ? 0 : 1;
  constexpr bool n1i = I >= 2, n1j = J >= 2;
#pragma unroll
  for (int k = 0; k < 36; ++k) blk[k] = 0.0;
  const T Sxx = C.Sxx[ut4(I, J)], Syy = C.Syy[ut4(I, J)];
  const T tuu = fma(C.gam, Syy, Sxx);
  const T tvv = fma(C.gam, Sxx, Syy);
  const T tuv_ij = fma(C.gam, C.Sxy[4 * J + I], C.nu * C.Sxy[4 * I + J]);
  const T tuv_ji = fma(C.gam, C.Sxy[4 * I + J], C.nu * C.Sxy[4 * J + I]);
  blk[0] = tuu;
  blk[7] = tvv;
  blk[1] = tuv_ij;
  blk[6] = (I == J) ? tuv_ij : tuv_ji;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (I == J && b < a) continue;
      const int l3 = a < b ? a : b, h3 = a < b ? b : a;
      T t1;
      if (g1i == 0 && g1j == 0) t1 = C.P14[ut3(l3, h3)];
      else if (g1i == 1 && g1j == 1) t1 = C.P23[ut3(l3, h3)];
      else if (g1i == 0) t1 = C.P1423[3 * a + b];
      else t1 = C.P1423[3 * b + a];
      const bool neg1 = ((a == 0) && n1i) != ((b == 0) && n1j);
      if (neg1) t1 = -t1;
      T f, e;
      if (g0i == 0 && g0j == 0) { f = C.F12[l3]; e = C.E12[h3]; }
      else if (g0i == 1 && g0j == 1) { f = C.F43[l3]; e = C.E43[h3]; }
      else if (g0i == 0) { f = C.G12[a]; e = C.E43[b]; }
      else { f = C.G12[b]; e = C.E43[a]; }
      const bool neg0 = ((a == 0) && n0i) != ((b == 0) && n0j);
      if (neg0) f = -f;
      const T sh = fma(f, e, t1);
      T v = sh;
      if (a >= 1 && b >= 1) {
        if (a == 2 && b == 2) v = fma(C.tb, tuu, sh);
        else if (a == 1 && b == 1) v = fma(C.tb, tvv, sh);
        else if (a == 2 && b == 1) v = fma(-C.tb, tuv_ij, sh);
        else v = fma(-C.tb, tuv_ji, sh);
      }
      blk[6 * (2 + a) + 2 + b] = v;
      if (I == J) blk[6 * (2 + b) + 2 + a] = v;
    }
  if (I == J) blk[35] = 0.0 + 1.0;  // KROT6 (plate.rs:25, :716-721)
}

// rotate a local node-pair block to global axes: T^T K T restricted to (i, j)
template <class T>
__device__ __forceinline__ void plate_rotate_block(const T R[9], bool diag, const T blk[36], T out[36]) {
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (diag && p == 1 && q == 0) continue;
      T M[9], o[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) M[3 * a + b] = blk[6 * (3 * p + a) + 3 * q + b];
      rt_m_r(R, M, o, diag && p == q);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          out[6 * (3 * p + a) + 3 * q + b] = o[3 * a + b];
          if (diag) out[6 * (3 * q + b) + 3 * p + a] = o[3 * a + b];
        }
    }
}

// R^T M R of one 3x3 sub-block whose zero entries are known at compile time
// (NZ: 9-bit row-major mask of the entries that can be non-zero): the same
// fma chains as rt_m_r with the terms of structural zeros left out.  Leaving out
// a term 0 * x of a chain changes no non-zero result (x + (+-0) = x), only the
// sign of a result that is zero, and zeros are never stored.
template <unsigned NZ, bool SYM, class T>
__device__ __forceinline__ void rt_m_r_sparse(const T R[9], const T M[9], T out[9]) {
  T Y[9];
  bool yrow[3] = {false, false, false};  // row k of Y = M R can be non-zero
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      bool started = false;
      T acc = 0.0;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (!((NZ >> (3 * k + j)) & 1u)) continue;
        acc = started ? fma(M[3 * k + j], R[3 * j + b], acc) : M[3 * k + j] * R[3 * j + b];
        started = true;
      }
      Y[3 * k + b] = acc;
      yrow[k] = yrow[k] || started;
    }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (SYM && b < a) continue;
      bool started = false;
      T acc = 0.0;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (!yrow[k]) continue;
        acc = started ? fma(R[3 * k + a], Y[3 * k + b], acc) : R[3 * k + a] * Y[3 * k + b];
        started = true;
      }
      out[3 * a + b] = acc;
      if (SYM) out[3 * b + a] = acc;
    }
}

// plate_rotate_block for the blocks plate_block_ct builds: in the local block
// only the membrane u-v entries, w-w, the w-thx-thy coupling, thx-thy and (on
// diagonal blocks) thz-thz can be non-zero, so each 3x3 sub-block of R^T K R
// takes only those terms.  Non-zero results are bit-identical to
// plate_rotate_block's.
template <bool DIAG, class T>
__device__ __forceinline__ void plate_rotate_block_ct(const T R[9], const T blk[36], T out[36]) {
  constexpr unsigned kNz00 = 0x11Bu;                  // (u,u) (u,v) (v,u) (v,v) (w,w)
  constexpr unsigned kNz01 = 0x0C0u;                  // (w,thx) (w,thy)
  constexpr unsigned kNz10 = 0x024u;                  // (thx,w) (thy,w)
  constexpr unsigned kNz11 = DIAG ? 0x11Bu : 0x01Bu;  // thx-thy 2x2, thz-thz on diagonal blocks
  T M[9], o[9];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (DIAG && p == 1 && q == 0) continue;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) M[3 * a + b] = blk[6 * (3 * p + a) + 3 * q + b];
      if (p == 0 && q == 0) rt_m_r_sparse<kNz00, DIAG>(R, M, o);
      else if (p == 0) rt_m_r_sparse<kNz01, false>(R, M, o);
      else if (q == 0) rt_m_r_sparse<kNz10, false>(R, M, o);
      else rt_m_r_sparse<kNz11, DIAG>(R, M, o);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          out[6 * (3 * p + a) + 3 * q + b] = o[3 * a + b];
          if (DIAG) out[6 * (3 * q + b) + 3 * p + a] = o[3 * a + b];
        }
    }
}

// ---------------------------------------------------------------------------
// validation (structs/truss.rs:44-64, beam.rs:63-117, plate.rs:58-158)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool quad_on_line(const double* P0, const double* P1, const double* P2, const double* P3) {
  const double* P[4] = {P0, P1, P2, P3};
  const int pairs[4][3] = {{0, 1, 3}, {1, 0, 2}, {2, 1, 3}, {3, 2, 0}};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double u[3], v[3], c[3];
    sub3(P[pairs[k][1]], P[pairs[k][0]], u);
    sub3(P[pairs[k][2]], P[pairs[k][0]], v);
    cross3(u, v, c);
    if (dot3(c, c) == 0.0) return true;  // |c| == 0 exactly when |c|^2 == 0 (no square root needed)
  }
  return false;
}

__device__ __forceinline__ bool quad_on_plane(const double* p1, const double* p2, const double* p3, const double* p4,
                                              double abs_tol) {
  double v32[3], v34[3], n[3];
  sub3(p2, p3, v32);
  sub3(p4, p3, v34);
  cross3(v32, v34, n);
  double d = -1.0 * ((n[0] * p3[0] + n[1] * p3[1]) + n[2] * p3[2]);
  double val = ((n[0] * p1[0] + n[1] * p1[1]) + n[2] * p1[2]) + d;
  return cwt(val, abs_tol) == 0.0;
}

struct HullPt {
  double x, y, key;
};

__device__ __forceinline__ double hull_key(double x, double y) {
  double len = sqrt((0.0 - x) * (0.0 - x) + (0.0 - y) * (0.0 - y));
  double sp = (0.0 - 1.0) * (0.0 - x) + (0.0 - 0.0) * (0.0 - y);
  double c = sp / (1.0 * len);
  return dacos(c) * FEM_RAD2DEG;
}

__device__ __forceinline__ void hull_swap(HullPt* a, int i, int j) {
  HullPt t = a[i];
  a[i] = a[j];
  a[j] = t;
}

// partition / quick_sort of convex_hull_on_plane.rs:14-58 on a 3-point slice
__device__ __forceinline__ int hull_partition(HullPt* a, int low, int high) {
  int pivot = high, store = low - 1, last = high;
  for (int guard = 0; guard < 16; ++guard) {
    store += 1;
    while (store < high && a[store].key < a[pivot].key) store += 1;
    last -= 1;
    while (last >= 0 && a[last].key > a[pivot].key) last -= 1;
    if (store >= last) break;
    hull_swap(a, store, last);
  }
  hull_swap(a, store, pivot);
  return store;
}

__device__ __forceinline__ void hull_sort3(HullPt* a) {
  // _quick_sort(0, 2) unrolled with an explicit stack (depth <= 2)
  int lo[4], hi[4], sp = 0;
  lo[0] = 0;
  hi[0] = 2;
  sp = 1;
  for (int guard = 0; guard < 8 && sp > 0; ++guard) {
    --sp;
    int l = lo[sp], h = hi[sp];
    if (l < h) {
      int p = hull_partition(a, l, h);
      // reference recursion order: left then right; push right first
      if (sp < 3) { lo[sp] = p + 1; hi[sp] = h; ++sp; }
      if (sp < 3) { lo[sp] = l; hi[sp] = p - 1; ++sp; }
    }
  }
}

__device__ __forceinline__ int quad_hull_size(const double* p1, const double* p2, const double* p3, const double* p4,
                                              double abs_tol, bool& ok) {
  double R[9];
  ok = plate_rotation(p2, p3, p4, abs_tol, R);
  if (!ok) return 0;
  const double* P[4] = {p1, p2, p3, p4};
  HullPt pts[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pts[i].key = 0.0;
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
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (pts[i].y < min_y) {
      shift_x = pts[i].x;
      min_y = pts[i].y;
      pos = i;
    }
  hull_swap(pts, 0, pos);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    pts[i].x -= shift_x;
    pts[i].y -= min_y;
  }
#pragma unroll
  for (int i = 1; i < 4; ++i) pts[i].key = hull_key(pts[i].x, pts[i].y);
  hull_sort3(pts + 1);
  int len = 4, i = 0;
  for (int guard = 0; guard < 8 && i + 2 < len; ++guard) {
    const HullPt a = pts[i], b = pts[i + 1], c = pts[i + 2];
    double area2 = (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
    if (area2 <= 0.0) {
      for (int k = i + 1; k + 1 < len; ++k) pts[k] = pts[k + 1];
      len -= 1;
    } else {
      i += 1;
    }
  }
  return len;
}

}  // namespace femgpu
