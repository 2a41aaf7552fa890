// dual.cuh - forward-mode dual numbers for the tangent step.
//
// A DualT<N> carries a double value and N directional derivatives. Its
// arithmetic runs the value part with exactly the double operation the same
// expression on plain doubles would run (so that, built with --fmad=false,
// every discrete decision - a SAT axis, a clip side, a clamp, the stick test
// - follows the f64 engine), and the derivative parts by the chain rule.
// Comparisons compare values. At 0 the derivative of sqrt is taken as 0 (the
// subgradient of the norm of a vector that is and stays zero, e.g. a friction
// force inside the cone's tip), and fabs takes the sign of the value.
//
// Dual = DualT<kTangentDims> holds every seeded direction; Dual1 = DualT<1>
// holds one, for code where each thread carries one direction (the value,
// computed by every such thread, is the same in all of them).
#pragma once

#include <cmath>

namespace avbd {

constexpr int kTangentDims = 5;

template <int N>
struct DualT {
  double v;
  double d[N];
  __host__ __device__ DualT() : v(0.0) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
  __host__ __device__ DualT(double x) : v(x) {  // NOLINT: constants enter as values
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
};
using Dual = DualT<kTangentDims>;
using Dual1 = DualT<1>;

template <int N>
__host__ __device__ __forceinline__ DualT<N> operator-(const DualT<N> &a) {
  DualT<N> r(-a.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -a.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator+(const DualT<N> &a, const DualT<N> &b) {
  DualT<N> r(a.v + b.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator-(const DualT<N> &a, const DualT<N> &b) {
  DualT<N> r(a.v - b.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator*(const DualT<N> &a, const DualT<N> &b) {
  DualT<N> r(a.v * b.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator/(const DualT<N> &a, const DualT<N> &b) {
  const double q = a.v / b.v;
  DualT<N> r(q);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = (a.d[k] - q * b.d[k]) / b.v;
  return r;
}
// with a plain double: the same value operation, the constant's derivative 0
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator+(const DualT<N> &a, double b) {
  DualT<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator+(double a, const DualT<N> &b) {
  DualT<N> r = b;
  r.v = a + b.v;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator-(const DualT<N> &a, double b) {
  DualT<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator-(double a, const DualT<N> &b) {
  DualT<N> r(a - b.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -b.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator*(const DualT<N> &a, double b) {
  DualT<N> r(a.v * b);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator*(double a, const DualT<N> &b) {
  DualT<N> r(a * b.v);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a * b.d[k];
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator/(const DualT<N> &a, double b) {
  DualT<N> r(a.v / b);
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] / b;
  return r;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> operator/(double a, const DualT<N> &b) {
  return DualT<N>(a) / b;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> &operator+=(DualT<N> &a, const DualT<N> &b) {
  return a = a + b;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> &operator-=(DualT<N> &a, const DualT<N> &b) {
  return a = a - b;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> &operator*=(DualT<N> &a, const DualT<N> &b) {
  return a = a * b;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> &operator/=(DualT<N> &a, const DualT<N> &b) {
  return a = a / b;
}

#define AVBD_DUAL_CMP(op)                                                                         \
  template <int N>                                                                                \
  __host__ __device__ __forceinline__ bool operator op(const DualT<N> &a, const DualT<N> &b) {   \
    return a.v op b.v;                                                                            \
  }                                                                                               \
  template <int N>                                                                                \
  __host__ __device__ __forceinline__ bool operator op(const DualT<N> &a, double b) {            \
    return a.v op b;                                                                              \
  }                                                                                               \
  template <int N>                                                                                \
  __host__ __device__ __forceinline__ bool operator op(double a, const DualT<N> &b) {            \
    return a op b.v;                                                                              \
  }
AVBD_DUAL_CMP(<)
AVBD_DUAL_CMP(>)
AVBD_DUAL_CMP(<=)
AVBD_DUAL_CMP(>=)
AVBD_DUAL_CMP(==)
AVBD_DUAL_CMP(!=)
#undef AVBD_DUAL_CMP

template <int N>
__host__ __device__ __forceinline__ DualT<N> sqrt(const DualT<N> &a) {
  const double r = ::sqrt(a.v);
  DualT<N> o(r);
#pragma unroll
  for (int k = 0; k < N; k++) o.d[k] = r > 0 ? a.d[k] / (2.0 * r) : 0.0;
  return o;
}
template <int N>
__host__ __device__ __forceinline__ DualT<N> fabs(const DualT<N> &a) {
  DualT<N> o = a.v < 0 ? -a : a;
  o.v = ::fabs(a.v);
  return o;
}
template <int N>
__host__ __device__ __forceinline__ bool isfinite(const DualT<N> &a) {
  return ::isfinite(a.v);
}
__host__ __device__ __forceinline__ bool isfinite(double a) { return ::isfinite(a); }
template <int N>
__host__ __device__ __forceinline__ double val(const DualT<N> &a) {
  return a.v;
}
__host__ __device__ __forceinline__ double val(double a) { return a; }

// One direction of a full dual number, and back: every thread of a direction
// group writes the (same) value and its own derivative.
__host__ __device__ __forceinline__ Dual1 dir_of(const Dual &x, int k) {
  Dual1 r(x.v);
  r.d[0] = x.d[k];
  return r;
}
__host__ __device__ __forceinline__ void set_dir(Dual &dst, const Dual1 &x, int k) {
  dst.v = x.v;
  dst.d[k] = x.d[0];
}

}  // namespace avbd
