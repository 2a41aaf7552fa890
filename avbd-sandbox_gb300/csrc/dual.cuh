// dual.cuh - forward-mode dual numbers for the tangent step.
//
// A Dual carries a double value and kTangentDims directional derivatives.
// Its arithmetic runs the value part with exactly the double operation the
// same expression on plain doubles would run (so that, built with
// --fmad=false, every discrete decision - a SAT axis, a clip side, a clamp,
// the stick test - follows the f64 engine), and the derivative parts by the
// chain rule. Comparisons compare values. At 0 the derivative of sqrt is
// taken as 0 (the subgradient of the norm of a vector that is and stays zero,
// e.g. a friction force inside the cone's tip), and fabs takes the sign of
// the value.
#pragma once

#include <cmath>

namespace avbd {

constexpr int kTangentDims = 5;

struct Dual {
  double v;
  double d[kTangentDims];
  __host__ __device__ Dual() : v(0.0) {
#pragma unroll
    for (int k = 0; k < kTangentDims; k++) d[k] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {  // NOLINT: constants enter as values
#pragma unroll
    for (int k = 0; k < kTangentDims; k++) d[k] = 0.0;
  }
};

__host__ __device__ __forceinline__ Dual operator-(const Dual &a) {
  Dual r(-a.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = -a.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator+(const Dual &a, const Dual &b) {
  Dual r(a.v + b.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator-(const Dual &a, const Dual &b) {
  Dual r(a.v - b.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator*(const Dual &a, const Dual &b) {
  Dual r(a.v * b.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator/(const Dual &a, const Dual &b) {
  const double q = a.v / b.v;
  Dual r(q);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = (a.d[k] - q * b.d[k]) / b.v;
  return r;
}
// with a plain double: the same value operation, the constant's derivative 0
__host__ __device__ __forceinline__ Dual operator+(const Dual &a, double b) {
  Dual r = a;
  r.v = a.v + b;
  return r;
}
__host__ __device__ __forceinline__ Dual operator+(double a, const Dual &b) {
  Dual r = b;
  r.v = a + b.v;
  return r;
}
__host__ __device__ __forceinline__ Dual operator-(const Dual &a, double b) {
  Dual r = a;
  r.v = a.v - b;
  return r;
}
__host__ __device__ __forceinline__ Dual operator-(double a, const Dual &b) {
  Dual r(a - b.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = -b.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator*(const Dual &a, double b) {
  Dual r(a.v * b);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a.d[k] * b;
  return r;
}
__host__ __device__ __forceinline__ Dual operator*(double a, const Dual &b) {
  Dual r(a * b.v);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a * b.d[k];
  return r;
}
__host__ __device__ __forceinline__ Dual operator/(const Dual &a, double b) {
  Dual r(a.v / b);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) r.d[k] = a.d[k] / b;
  return r;
}
__host__ __device__ __forceinline__ Dual operator/(double a, const Dual &b) { return Dual(a) / b; }
__host__ __device__ __forceinline__ Dual &operator+=(Dual &a, const Dual &b) { return a = a + b; }
__host__ __device__ __forceinline__ Dual &operator-=(Dual &a, const Dual &b) { return a = a - b; }
__host__ __device__ __forceinline__ Dual &operator*=(Dual &a, const Dual &b) { return a = a * b; }
__host__ __device__ __forceinline__ Dual &operator/=(Dual &a, const Dual &b) { return a = a / b; }

#define AVBD_DUAL_CMP(op)                                                                                          \
  __host__ __device__ __forceinline__ bool operator op(const Dual &a, const Dual &b) { return a.v op b.v; }       \
  __host__ __device__ __forceinline__ bool operator op(const Dual &a, double b) { return a.v op b; }              \
  __host__ __device__ __forceinline__ bool operator op(double a, const Dual &b) { return a op b.v; }
AVBD_DUAL_CMP(<)
AVBD_DUAL_CMP(>)
AVBD_DUAL_CMP(<=)
AVBD_DUAL_CMP(>=)
AVBD_DUAL_CMP(==)
AVBD_DUAL_CMP(!=)
#undef AVBD_DUAL_CMP

__host__ __device__ __forceinline__ Dual sqrt(const Dual &a) {
  const double r = ::sqrt(a.v);
  Dual o(r);
#pragma unroll
  for (int k = 0; k < kTangentDims; k++) o.d[k] = r > 0 ? a.d[k] / (2.0 * r) : 0.0;
  return o;
}
__host__ __device__ __forceinline__ Dual fabs(const Dual &a) {
  Dual o = a.v < 0 ? -a : a;
  o.v = ::fabs(a.v);
  return o;
}
__host__ __device__ __forceinline__ bool isfinite(const Dual &a) { return ::isfinite(a.v); }
__host__ __device__ __forceinline__ double val(const Dual &a) { return a.v; }
__host__ __device__ __forceinline__ double val(double a) { return a; }

}  // namespace avbd
