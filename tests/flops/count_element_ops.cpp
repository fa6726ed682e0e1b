// Floating-point operations of the plate, beam and truss element arithmetic, counted by compiling the device header
// element_math.cuh on the host with an operation-counting number type: the algorithmic work the bench's
// roofline divides by (adds and subtractions, multiplications, divisions and square roots one flop each,
// a fused multiply-add two).  Prints, for a plate in a global plane (R = I: the identity fast path) and a
// plate off the planes (general rotation), the operation counts of the rotation and local coordinates, of
// the element core and of the ten node-pair blocks; and for a beam the counts of its blocks for sections
// with I12 != 0 and with I12 = 0, each with I11 > I22 and with I11 < I22 (one more turn of the
// principal-axes loop); and for a truss the counts of its block for an oblique bar (without and with a
// second area) and a bar along x.  The header's transcendentals are double-only; their Cnt versions below add the operations of
// the double code (the same argument reduction and series).  Test infrastructure:
// tests/test_flop_model.py builds and runs it.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
static inline long long __double_as_longlong(double v) {
  long long b;
  std::memcpy(&b, &v, sizeof b);
  return b;
}

struct Ops {
  long add = 0, mul = 0, fma = 0, div = 0, sqrt = 0;
  long flops() const { return add + mul + 2 * fma + div + sqrt; }
};
static Ops g_ops;

struct Cnt {
  double v;
  Cnt() : v(0.0) {}
  Cnt(double x) : v(x) {}
};
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator+(Cnt a, Cnt b) { ++g_ops.add; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { ++g_ops.add; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { ++g_ops.mul; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { ++g_ops.div; return Cnt(a.v / b.v); }
inline Cnt operator+(Cnt a, double b) { return a + Cnt(b); }
inline Cnt operator+(double a, Cnt b) { return Cnt(a) + b; }
inline Cnt operator-(Cnt a, double b) { return a - Cnt(b); }
inline Cnt operator-(double a, Cnt b) { return Cnt(a) - b; }
inline Cnt operator*(Cnt a, double b) { return a * Cnt(b); }
inline Cnt operator*(double a, Cnt b) { return Cnt(a) * b; }
inline Cnt operator/(Cnt a, double b) { return a / Cnt(b); }
inline Cnt operator/(double a, Cnt b) { return Cnt(a) / b; }
inline Cnt& operator+=(Cnt& a, Cnt b) { return a = a + b; }
inline Cnt& operator-=(Cnt& a, Cnt b) { return a = a - b; }
inline Cnt& operator*=(Cnt& a, Cnt b) { return a = a * b; }
inline Cnt& operator*=(Cnt& a, double b) { return a = a * b; }
inline bool operator<(Cnt a, Cnt b) { return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { return a.v >= b.v; }
inline bool operator==(Cnt a, Cnt b) { return a.v == b.v; }
inline bool operator!=(Cnt a, Cnt b) { return a.v != b.v; }
inline bool operator<(Cnt a, double b) { return a.v < b; }
inline bool operator>(Cnt a, double b) { return a.v > b; }
inline bool operator<=(Cnt a, double b) { return a.v <= b; }
inline bool operator>=(Cnt a, double b) { return a.v >= b; }
inline bool operator==(Cnt a, double b) { return a.v == b; }
inline bool operator!=(Cnt a, double b) { return a.v != b; }
inline Cnt fma(Cnt a, Cnt b, Cnt c) { ++g_ops.fma; return Cnt(std::fma(a.v, b.v, c.v)); }
inline Cnt fma(double a, Cnt b, Cnt c) { return fma(Cnt(a), b, c); }
inline Cnt fma(Cnt a, double b, Cnt c) { return fma(a, Cnt(b), c); }
inline Cnt fma(Cnt a, Cnt b, double c) { return fma(a, b, Cnt(c)); }
inline Cnt fma(Cnt a, double b, double c) { return fma(a, Cnt(b), Cnt(c)); }
inline Cnt fma(double a, Cnt b, double c) { return fma(Cnt(a), b, Cnt(c)); }
inline Cnt fma(double a, double b, Cnt c) { return fma(Cnt(a), Cnt(b), c); }
inline Cnt sqrt(Cnt a) { ++g_ops.sqrt; return Cnt(std::sqrt(a.v)); }
inline Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
// the header's integer tests of exact values (no arithmetic)
inline bool bits_zero(Cnt v) { return (__double_as_longlong(v.v) << 1) == 0; }
inline bool bits_one(Cnt v) { return __double_as_longlong(v.v) == 0x3ff0000000000000ll; }
inline bool bits_positive(Cnt v) { return v.v > 0.0; }

#include "../../finite_element_method_gb300/csrc/element_math.cuh"

using namespace femgpu;

// the header's transcendentals for Cnt: the value of the double code, with its operations counted
// (reduce_pio2: one multiplication and three fmas; sincos_reduced, both series: r^2 and r r^2, nine fmas
// for the sine's polynomial and one to finish it, ten for the cosine's and one to finish it; the
// arctangent: see datan)
inline Cnt dsin(Cnt x) {
  g_ops.mul += 1 + 2;
  g_ops.fma += 3 + 9 + 1 + 10 + 1;
  return Cnt(femgpu::dsin(x.v));
}
inline Cnt dcos(Cnt x) {
  g_ops.mul += 1 + 2;
  g_ops.fma += 3 + 9 + 1 + 10 + 1;
  return Cnt(femgpu::dcos(x.v));
}
inline Cnt datan(Cnt t) {
  const double a = std::fabs(t.v);
  const bool inv = a > 1.0;
  g_ops.div += inv ? 2 : 1;  // 1 / a; (a - c) / (1 + a c)
  g_ops.mul += 4;            // a 8, k / 8, u u, u u^2
  g_ops.add += inv ? 4 : 2;  // a - c, the table value + the series; pi/2 - res + its low part
  g_ops.fma += 9;            // 1 + a c, seven series terms, u + u^3 p
  return Cnt(femgpu::datan(t.v));
}
inline Cnt dacos(Cnt x) { return 2.0 * datan(sqrt((1.0 - x) / (1.0 + x))); }

template <int I, int J, bool ROT>
static void pair(const PlateCoreT<Cnt>& C, const Cnt R[9]) {
  Cnt blk[36];
  plate_block_ct<I, J>(C, blk);
  if (ROT) {
    Cnt o[36];
    plate_rotate_block_ct<I == J>(R, blk, o);
  }
}

template <bool ROT>
static void blocks(const PlateCoreT<Cnt>& C, const Cnt R[9]) {
  pair<0, 0, ROT>(C, R);
  pair<0, 1, ROT>(C, R);
  pair<0, 2, ROT>(C, R);
  pair<0, 3, ROT>(C, R);
  pair<1, 1, ROT>(C, R);
  pair<1, 2, ROT>(C, R);
  pair<1, 3, ROT>(C, R);
  pair<2, 2, ROT>(C, R);
  pair<2, 3, ROT>(C, R);
  pair<3, 3, ROT>(C, R);
}

static void report(const char* what, const Ops& o) {
  std::printf("%s add=%ld mul=%ld fma=%ld div=%ld sqrt=%ld flops=%ld\n", what, o.add, o.mul, o.fma, o.div, o.sqrt,
              o.flops());
}

static void count(const char* name, const double P[4][3]) {
  Cnt X[4][3];
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 3; ++k) X[i][k] = Cnt(P[i][k]);
  g_ops = Ops();
  Cnt R[9];
  if (!plate_rotation(X[1], X[2], X[3], 1e-12, R)) set_identity(R);
  bool ident = true;
  for (int k = 0; k < 9; ++k) ident = ident && R[k].v == ((k % 4 == 0) ? 1.0 : 0.0);
  Cnt xl[4], yl[4];
  plate_local_xy(X, R, ident, xl, yl);
  const Ops geo = g_ops;
  g_ops = Ops();
  PlateCoreT<Cnt> C;
  plate_core(xl, yl, Cnt(70e9), Cnt(0.3), Cnt(0.02), Cnt(5.0 / 6.0), C);
  const Ops core = g_ops;
  g_ops = Ops();
  if (ident)
    blocks<false>(C, R);
  else
    blocks<true>(C, R);
  const Ops blk = g_ops;
  std::printf("%s identity=%d\n", name, ident ? 1 : 0);
  report("  geometry", geo);
  report("  core", core);
  report("  blocks", blk);
  std::printf("  total=%ld\n", geo.flops() + core.flops() + blk.flops());
}

static void count_beam(const char* name, double i11, double i22, double i12) {
  const Cnt x1[3] = {Cnt(0.03), Cnt(-0.02), Cnt(0.01)}, x2[3] = {Cnt(2.98), Cnt(0.05), Cnt(-0.04)};
  const Cnt axis[3] = {Cnt(0.0), Cnt(0.0), Cnt(1.0)};
  g_ops = Ops();
  BeamBlocksT<Cnt> B;
  const bool ok = beam_blocks(x1, x2, Cnt(210e9), Cnt(0.3), Cnt(1e-2), Cnt(i11), Cnt(i22), Cnt(i12), Cnt(2e-5),
                              Cnt(5.0 / 6.0), axis, 1e-6, 1e-12, B);
  std::printf("beam_%s ok=%d\n", name, ok ? 1 : 0);
  report("  blocks", g_ops);
}

static void count_truss(const char* name, const double d[3], double area2) {
  const Cnt x1[3] = {Cnt(0.02), Cnt(-0.01), Cnt(0.03)};
  const Cnt x2[3] = {Cnt(0.02 + d[0]), Cnt(-0.01 + d[1]), Cnt(0.03 + d[2])};
  g_ops = Ops();
  Cnt g[9];
  const bool ok = truss_block(x1, x2, Cnt(200e9), Cnt(3e-4), Cnt(area2), 1e-12, g);
  std::printf("truss_%s ok=%d\n", name, ok ? 1 : 0);
  report("  blocks", g_ops);
}

int main() {
  // a distorted quadrilateral in z = 0, counter-clockwise
  const double flat[4][3] = {{1.1, 1.05, 0.0}, {0.02, 0.97, 0.0}, {-0.03, 0.01, 0.0}, {1.04, -0.02, 0.0}};
  // the same plate turned off the global planes
  const double c = std::cos(0.7), s = std::sin(0.7), c2 = std::cos(0.4), s2 = std::sin(0.4);
  double tilted[4][3];
  for (int i = 0; i < 4; ++i) {
    const double x = flat[i][0], y = flat[i][1];
    const double xr = c * x - s * y, yr = s * x + c * y;
    tilted[i][0] = xr;
    tilted[i][1] = c2 * yr;
    tilted[i][2] = s2 * yr;
  }
  count("flat", flat);
  count("tilted", tilted);
  count_beam("general", 8e-5, 3e-5, 2e-5);
  count_beam("general_turn", 3e-5, 8e-5, 2e-5);
  count_beam("aligned", 8e-5, 3e-5, 0.0);
  count_beam("aligned_turn", 3e-5, 8e-5, 0.0);
  const double oblique[3] = {0.97, 1.04, -0.03}, along_x[3] = {1.0, 0.0, 0.0};
  count_truss("general", oblique, std::nan(""));
  count_truss("general_area2", oblique, 5e-4);
  count_truss("along_x", along_x, std::nan(""));
  return 0;
}
