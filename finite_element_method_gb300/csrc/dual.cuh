// dual.cuh -- forward-mode dual numbers (value + one directional derivative)
// for differentiating the element arithmetic of element_math.cuh.
//
// A Dual carries v (the FP64 value, computed exactly as the plain double code
// computes it) and d (its derivative along one seeded parameter).  Branches
// and clamps follow the value, so the derivative is that of the branch taken;
// where the reference's parametrisation has a kink (acos at +-1, the
// compare_with_tolerance clamps) the derivative is the symmetric one, which is
// what central finite differences measure.
#pragma once
#include <type_traits>

namespace femgpu {

// the double versions stay visible next to the Dual overloads below
using ::fabs;
using ::fma;
using ::sqrt;

struct Dual {
  double v, d;
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(x), d(0.0) {}
  __device__ __forceinline__ Dual(double x, double dx) : v(x), d(dx) {}
};

template <class T>
struct IsDual : std::false_type {};
template <>
struct IsDual<Dual> : std::true_type {};

__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return Dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return Dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return Dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return Dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, fma(a.d, b.v, a.v * b.d)); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual operator/(Dual a, double b) { return Dual(a.v / b, a.d / b); }
__device__ __forceinline__ Dual operator/(double a, Dual b) {
  const double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { return a = a * b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, double b) { return a = a * b; }

__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator<(Dual a, double b) { return a.v < b; }
__device__ __forceinline__ bool operator<(double a, Dual b) { return a < b.v; }
__device__ __forceinline__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
__device__ __forceinline__ bool operator>(Dual a, double b) { return a.v > b; }
__device__ __forceinline__ bool operator>(double a, Dual b) { return a > b.v; }
__device__ __forceinline__ bool operator<=(Dual a, double b) { return a.v <= b; }
__device__ __forceinline__ bool operator>=(Dual a, double b) { return a.v >= b; }
__device__ __forceinline__ bool operator==(Dual a, Dual b) { return a.v == b.v; }
__device__ __forceinline__ bool operator==(Dual a, double b) { return a.v == b; }
__device__ __forceinline__ bool operator!=(Dual a, Dual b) { return a.v != b.v; }
__device__ __forceinline__ bool operator!=(Dual a, double b) { return a.v != b; }

__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) { return Dual(fma(a.v, b.v, c.v), fma(a.d, b.v, fma(a.v, b.d, c.d))); }
__device__ __forceinline__ Dual fma(double a, Dual b, Dual c) { return Dual(fma(a, b.v, c.v), fma(a, b.d, c.d)); }
__device__ __forceinline__ Dual fma(Dual a, double b, Dual c) { return Dual(fma(a.v, b, c.v), fma(a.d, b, c.d)); }
__device__ __forceinline__ Dual fma(Dual a, Dual b, double c) { return Dual(fma(a.v, b.v, c), fma(a.d, b.v, a.v * b.d)); }
__device__ __forceinline__ Dual fma(Dual a, double b, double c) { return Dual(fma(a.v, b, c), a.d * b); }
__device__ __forceinline__ Dual fma(double a, Dual b, double c) { return Dual(fma(a, b.v, c), a * b.d); }
__device__ __forceinline__ Dual fma(double a, double b, Dual c) { return Dual(fma(a, b, c.v), c.d); }

__device__ __forceinline__ Dual sqrt(Dual a) {
  const double s = sqrt(a.v);
  return Dual(s, s > 0.0 ? a.d * (0.5 / s) : 0.0);
}
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? Dual(-a.v, -a.d) : a; }
__device__ __forceinline__ Dual dsin(Dual a) { return Dual(dsin(a.v), dcos(a.v) * a.d); }
__device__ __forceinline__ Dual dcos(Dual a) { return Dual(dcos(a.v), -dsin(a.v) * a.d); }
__device__ __forceinline__ Dual datan(Dual a) { return Dual(datan(a.v), a.d / fma(a.v, a.v, 1.0)); }
// acos: at +-1 the section-angle parametrisation has a kink; its symmetric derivative there is 0
__device__ __forceinline__ Dual dacos(Dual a) {
  const double r = fma(-a.v, a.v, 1.0);
  return Dual(dacos(a.v), r > 0.0 ? -a.d / sqrt(r) : 0.0);
}

}  // namespace femgpu
