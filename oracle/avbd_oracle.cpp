/*
 * ORACLE - test infrastructure only. Not part of the product.
 *
 * A C++17 f64 restatement of the AVBD sandbox's CPU engine, the reference
 * `Solver.step()` path:
 *   src/math/maths.js            vec3 / mat3 / quat / solve6
 *   src/physics/rigid.js         mass properties, world moment, constrainedTo
 *   src/physics/collide.js       box-box SAT + clipping, sphere-sphere, sphere-OBB
 *   src/physics/manifold.js      persistent manifolds, warm start, contact rows
 *   src/physics/joint.js         ball socket + angular rows + fracture
 *   src/physics/spring.js        distance spring + Eq. 17 geometric stiffness + tear
 *   src/physics/broadphase.js    spatial hash (brute-force order) / brute force
 *   src/physics/coloring.js      greedy index-order colouring
 *   src/physics/gpu/layout.js:50-57  lowbias32 colour priority
 *   src/physics/solver.js        Algorithm 1 (`step`, :307-493)
 *
 * It is the checker for the CUDA backend: tests, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it; nothing in the product links it.
 *
 * Floating-point operation order follows the reference line by line (it must
 * be compiled with -ffp-contract=off and without -ffast-math) so that it is a
 * faithful f64 restatement. Parity against the JavaScript engine itself cannot
 * be run in this build environment (there is no JavaScript runtime); the
 * oracle is pinned instead by the reference's closed-form tests
 * (test/analytic.mjs, test/fixtures.mjs, test/spheres.mjs), ported in tests/.
 *
 * Compiled with -DORC_TANGENT the same source is the tangent oracle: its
 * scalar is a forward-mode dual number whose value runs the same double
 * operations (values identical to the f64 build's) and which carries ND
 * directional derivatives through the whole step - contact geometry, clamps
 * and all - the exact derivative of the discrete step that an adjoint's
 * gradient is checked against (orc_t_seed / orc_t_read_pos below).
 */

#include "../include/avbd_cuda.h"

// The tangent build's own namespace: no C++ symbol is shared with the f64
// build, so both libraries can live in one process.
#ifdef ORC_TANGENT
#define orc orc_tangent
#endif

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace orc {

// The scalar of the restatement: double, or (built with -DORC_TANGENT, the
// tangent oracle) a forward-mode dual number whose value part runs the very
// same double operations and which carries ND directional derivatives.
#ifdef ORC_TANGENT
constexpr int ND = 5;
struct Real {
  double v;
  double d[ND];
  Real() : v(0), d{} {}
  Real(double x) : v(x), d{} {}  // NOLINT: constants and inputs enter as values
};
inline Real make_real(double v, const double *d) {
  Real r(v);
  for (int k = 0; k < ND; k++) r.d[k] = d[k];
  return r;
}
inline Real operator-(const Real &a) {
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = -a.d[k];
  return make_real(-a.v, d);
}
inline Real operator+(const Real &a, const Real &b) {
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = a.d[k] + b.d[k];
  return make_real(a.v + b.v, d);
}
inline Real operator-(const Real &a, const Real &b) {
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = a.d[k] - b.d[k];
  return make_real(a.v - b.v, d);
}
inline Real operator*(const Real &a, const Real &b) {
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = a.d[k] * b.v + a.v * b.d[k];
  return make_real(a.v * b.v, d);
}
inline Real operator/(const Real &a, const Real &b) {
  const double q = a.v / b.v;
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = (a.d[k] - q * b.d[k]) / b.v;
  return make_real(q, d);
}
inline Real operator+(const Real &a, double b) { return a + Real(b); }
inline Real operator+(double a, const Real &b) { return Real(a) + b; }
inline Real operator-(const Real &a, double b) { return a - Real(b); }
inline Real operator-(double a, const Real &b) { return Real(a) - b; }
inline Real operator*(const Real &a, double b) { return a * Real(b); }
inline Real operator*(double a, const Real &b) { return Real(a) * b; }
inline Real operator/(const Real &a, double b) { return a / Real(b); }
inline Real operator/(double a, const Real &b) { return Real(a) / b; }
inline Real &operator+=(Real &a, const Real &b) { return a = a + b; }
inline Real &operator-=(Real &a, const Real &b) { return a = a - b; }
inline Real &operator*=(Real &a, const Real &b) { return a = a * b; }
inline Real &operator/=(Real &a, const Real &b) { return a = a / b; }
#define ORC_CMP(op)                                                             \
  inline bool operator op(const Real &a, const Real &b) { return a.v op b.v; } \
  inline bool operator op(const Real &a, double b) { return a.v op b; }        \
  inline bool operator op(double a, const Real &b) { return a op b.v; }
ORC_CMP(<) ORC_CMP(>) ORC_CMP(<=) ORC_CMP(>=) ORC_CMP(==) ORC_CMP(!=)
#undef ORC_CMP
// At 0 the derivative of sqrt is taken as 0: the subgradient of the norm of a
// vector that is and stays zero (a friction force inside the cone's tip).
inline Real sqrt(const Real &a) {
  const double r = std::sqrt(a.v);
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = r > 0 ? a.d[k] / (2.0 * r) : 0.0;
  return make_real(r, d);
}
inline Real fabs(const Real &a) {
  double d[ND];
  for (int k = 0; k < ND; k++) d[k] = a.v < 0 ? -a.d[k] : a.d[k];
  return make_real(std::fabs(a.v), d);
}
inline Real floor(const Real &a) { return Real(std::floor(a.v)); }
// Tangents the narrow phase's geometry is denied (orc_t_freeze): bit 0 the
// contact bases, bit 1 the body-local anchors - what an adjoint that holds
// the contact frames constant within a step would compute.
static int g_freeze_geometry = 0;
inline bool isfinite(const Real &a) { return std::isfinite(a.v); }
inline bool isnan(const Real &a) { return std::isnan(a.v); }
inline bool signbit(const Real &a) { return std::signbit(a.v); }
inline double val(const Real &a) { return a.v; }
#else
using Real = double;
using std::fabs;
using std::floor;
using std::isfinite;
using std::isnan;
using std::signbit;
using std::sqrt;
inline double val(double a) { return a; }
#endif
inline int64_t floor_i64(const Real &a) { return (int64_t)std::floor(val(a)); }

static const Real INF = std::numeric_limits<double>::infinity();
static const Real NaN = std::numeric_limits<double>::quiet_NaN();

// ---------------------------------------------------------------------------
// Scalar helpers with JavaScript semantics (src/math/maths.js:34-44)
// ---------------------------------------------------------------------------

// Math.min / Math.max: NaN propagates, -0 < +0.
static inline Real js_min(Real a, Real b) {
  if (a != a || b != b) return NaN;
  if (a < b) return a;
  if (b < a) return b;
  if (a == 0 && b == 0) return (signbit(a) || signbit(b)) ? -0.0 : 0.0;
  return a;
}
static inline Real js_max(Real a, Real b) {
  if (a != a || b != b) return NaN;
  if (a > b) return a;
  if (b > a) return b;
  if (a == 0 && b == 0) return (!signbit(a) || !signbit(b)) ? 0.0 : -0.0;
  return a;
}
static inline Real sign(Real x) { return x < 0 ? -1 : x > 0 ? 1 : 0; }
// clamp(x, a, b) = Math.max(a, Math.min(b, x))  (maths.js:38-40)
static inline Real clamp(Real x, Real a, Real b) { return js_max(a, js_min(b, x)); }
static inline bool is_finite(Real x) { return isfinite(x); }

// ---------------------------------------------------------------------------
// vec3 (maths.js:50-193)
// ---------------------------------------------------------------------------
static inline void v3_set(Real *o, Real x, Real y, Real z) { o[0] = x; o[1] = y; o[2] = z; }
static inline void v3_copy(Real *o, const Real *a) { o[0] = a[0]; o[1] = a[1]; o[2] = a[2]; }
static inline void v3_zero(Real *o) { o[0] = 0; o[1] = 0; o[2] = 0; }
static inline void v3_add(Real *o, const Real *a, const Real *b) {
  o[0] = a[0] + b[0]; o[1] = a[1] + b[1]; o[2] = a[2] + b[2];
}
static inline void v3_sub(Real *o, const Real *a, const Real *b) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static inline void v3_scale(Real *o, const Real *a, Real s) {
  o[0] = a[0] * s; o[1] = a[1] * s; o[2] = a[2] * s;
}
static inline void v3_div(Real *o, const Real *a, Real s) {
  o[0] = a[0] / s; o[1] = a[1] / s; o[2] = a[2] / s;
}
static inline void v3_add_scaled(Real *o, const Real *a, Real s) {
  o[0] += a[0] * s; o[1] += a[1] * s; o[2] += a[2] * s;
}
static inline void v3_negate(Real *o, const Real *a) { o[0] = -a[0]; o[1] = -a[1]; o[2] = -a[2]; }
static inline Real v3_dot(const Real *a, const Real *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline Real v3_len_sq(const Real *a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }
static inline Real v3_len(const Real *a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
static inline void v3_cross(Real *o, const Real *a, const Real *b) {
  const Real ax = a[0], ay = a[1], az = a[2], bx = b[0], by = b[1], bz = b[2];
  o[0] = ay * bz - az * by;
  o[1] = az * bx - ax * bz;
  o[2] = ax * by - ay * bx;
}
static inline void v3_abs(Real *o, const Real *a) {
  o[0] = fabs(a[0]); o[1] = fabs(a[1]); o[2] = fabs(a[2]);
}
static inline void v3_min_scalar(Real *o, const Real *a, Real s) {
  o[0] = js_min(a[0], s); o[1] = js_min(a[1], s); o[2] = js_min(a[2], s);
}
static inline void v3_clamp_scalar(Real *o, const Real *a, Real lo, Real hi) {
  o[0] = clamp(a[0], lo, hi); o[1] = clamp(a[1], lo, hi); o[2] = clamp(a[2], lo, hi);
}

// ---------------------------------------------------------------------------
// mat3, row-major (maths.js:199-435)
// ---------------------------------------------------------------------------
static inline void m3_zero(Real *o) { for (int i = 0; i < 9; i++) o[i] = 0; }
static inline void m3_copy(Real *o, const Real *a) { for (int i = 0; i < 9; i++) o[i] = a[i]; }
static inline void m3_diagonal(Real *o, Real a, Real b, Real c) {
  o[0] = a; o[1] = 0; o[2] = 0; o[3] = 0; o[4] = b; o[5] = 0; o[6] = 0; o[7] = 0; o[8] = c;
}
static inline void m3_add_into(Real *o, const Real *a) { for (int i = 0; i < 9; i++) o[i] += a[i]; }
static inline void m3_scale(Real *o, const Real *a, Real s) { for (int i = 0; i < 9; i++) o[i] = a[i] * s; }
static inline void m3_div(Real *o, const Real *a, Real s) { for (int i = 0; i < 9; i++) o[i] = a[i] / s; }
static inline void m3_negate(Real *o, const Real *a) { for (int i = 0; i < 9; i++) o[i] = -a[i]; }
static inline void m3_get_row(Real *o, const Real *a, int r) { o[0] = a[r * 3]; o[1] = a[r * 3 + 1]; o[2] = a[r * 3 + 2]; }
static inline void m3_mul_vec(Real *o, const Real *a, const Real *v) {
  const Real x = v[0], y = v[1], z = v[2];
  o[0] = a[0] * x + a[1] * y + a[2] * z;
  o[1] = a[3] * x + a[4] * y + a[5] * z;
  o[2] = a[6] * x + a[7] * y + a[8] * z;
}
static inline void m3_mul(Real *o, const Real *a, const Real *b) {
  const Real a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3], a4 = a[4], a5 = a[5], a6 = a[6], a7 = a[7], a8 = a[8];
  const Real b0 = b[0], b1 = b[1], b2 = b[2], b3 = b[3], b4 = b[4], b5 = b[5], b6 = b[6], b7 = b[7], b8 = b[8];
  o[0] = a0 * b0 + a1 * b3 + a2 * b6;
  o[1] = a0 * b1 + a1 * b4 + a2 * b7;
  o[2] = a0 * b2 + a1 * b5 + a2 * b8;
  o[3] = a3 * b0 + a4 * b3 + a5 * b6;
  o[4] = a3 * b1 + a4 * b4 + a5 * b7;
  o[5] = a3 * b2 + a4 * b5 + a5 * b8;
  o[6] = a6 * b0 + a7 * b3 + a8 * b6;
  o[7] = a6 * b1 + a7 * b4 + a8 * b7;
  o[8] = a6 * b2 + a7 * b5 + a8 * b8;
}
static inline void m3_mul_diag_right(Real *o, const Real *a, Real d0, Real d1, Real d2) {
  o[0] = a[0] * d0; o[1] = a[1] * d1; o[2] = a[2] * d2;
  o[3] = a[3] * d0; o[4] = a[4] * d1; o[5] = a[5] * d2;
  o[6] = a[6] * d0; o[7] = a[7] * d1; o[8] = a[8] * d2;
}
static inline void m3_transpose(Real *o, const Real *a) {
  const Real a1 = a[1], a2 = a[2], a5 = a[5];
  o[0] = a[0]; o[4] = a[4]; o[8] = a[8];
  o[1] = a[3]; o[3] = a1;
  o[2] = a[6]; o[6] = a2;
  o[5] = a[7]; o[7] = a5;
}
static inline void m3_outer(Real *o, const Real *a, const Real *b) {
  o[0] = a[0] * b[0]; o[1] = a[0] * b[1]; o[2] = a[0] * b[2];
  o[3] = a[1] * b[0]; o[4] = a[1] * b[1]; o[5] = a[1] * b[2];
  o[6] = a[2] * b[0]; o[7] = a[2] * b[1]; o[8] = a[2] * b[2];
}
static inline void m3_skew(Real *o, const Real *r) {
  const Real rx = r[0], ry = r[1], rz = r[2];
  o[0] = 0; o[1] = -rz; o[2] = ry;
  o[3] = rz; o[4] = 0; o[5] = -rx;
  o[6] = -ry; o[7] = rx; o[8] = 0;
}
static inline void m3_diagonalize(Real *o, const Real *m) {
  const Real c0 = sqrt(m[0] * m[0] + m[3] * m[3] + m[6] * m[6]);
  const Real c1 = sqrt(m[1] * m[1] + m[4] * m[4] + m[7] * m[7]);
  const Real c2 = sqrt(m[2] * m[2] + m[5] * m[5] + m[8] * m[8]);
  o[0] = c0; o[1] = 0; o[2] = 0; o[3] = 0; o[4] = c1; o[5] = 0; o[6] = 0; o[7] = 0; o[8] = c2;
}
// maths.js:389-414
static inline void m3_orthonormal(Real *o, const Real *normal) {
  const Real nx = normal[0], ny = normal[1], nz = normal[2];
  Real t1x, t1y, t1z;
  if (fabs(nx) > fabs(nz)) { t1x = -ny; t1y = nx; t1z = 0; }
  else { t1x = 0; t1y = -nz; t1z = ny; }
  const Real t1len = sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
  t1x /= t1len; t1y /= t1len; t1z /= t1len;
  const Real t2x = ny * t1z - nz * t1y;
  const Real t2y = nz * t1x - nx * t1z;
  const Real t2z = nx * t1y - ny * t1x;
  o[0] = nx; o[1] = ny; o[2] = nz;
  o[3] = t1x; o[4] = t1y; o[5] = t1z;
  o[6] = t2x; o[7] = t2y; o[8] = t2z;
}
// maths.js:417-434
static inline void m3_from_quat(Real *o, const Real *q) {
  const Real x = q[0], y = q[1], z = q[2], w = q[3];
  const Real xx = x * x, yy = y * y, zz = z * z;
  const Real xy = x * y, xz = x * z, yz = y * z;
  const Real wx = w * x, wy = w * y, wz = w * z;
  o[0] = 1 - 2 * (yy + zz);
  o[1] = 2 * (xy + wz);
  o[2] = 2 * (xz - wy);
  o[3] = 2 * (xy - wz);
  o[4] = 1 - 2 * (xx + zz);
  o[5] = 2 * (yz + wx);
  o[6] = 2 * (xz + wy);
  o[7] = 2 * (yz - wx);
  o[8] = 1 - 2 * (xx + yy);
}

// ---------------------------------------------------------------------------
// quat (maths.js:441-627)
// ---------------------------------------------------------------------------
static inline void q_copy(Real *o, const Real *a) { o[0] = a[0]; o[1] = a[1]; o[2] = a[2]; o[3] = a[3]; }
static inline void q_identity(Real *o) { o[0] = 0; o[1] = 0; o[2] = 0; o[3] = 1; }
static inline void q_conjugate(Real *o, const Real *q) { o[0] = -q[0]; o[1] = -q[1]; o[2] = -q[2]; o[3] = q[3]; }
// Eq. 20, maths.js:541-555
static inline void q_subtract(Real *o, const Real *a, const Real *b) {
  const Real lsq = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[3] * b[3];
  const Real ix = -b[0] / lsq, iy = -b[1] / lsq, iz = -b[2] / lsq, iw = b[3] / lsq;
  const Real ax = a[0], ay = a[1], az = a[2], aw = a[3];
  o[0] = (aw * ix + ax * iw + ay * iz - az * iy) * 2;
  o[1] = (aw * iy - ax * iz + ay * iw + az * ix) * 2;
  o[2] = (aw * iz + ax * iy - ay * ix + az * iw) * 2;
}
// Eq. 21, maths.js:568-592 (the "0 * q" terms are kept: they fix -0 handling)
static inline void q_integrate(Real *o, const Real *q, const Real *dw) {
  const Real qx = q[0], qy = q[1], qz = q[2], qw = q[3];
  const Real wx = dw[0], wy = dw[1], wz = dw[2];
  const Real px = 0 * qx + wx * qw + wy * qz - wz * qy;
  const Real py = 0 * qy - wx * qz + wy * qw + wz * qx;
  const Real pz = 0 * qz + wx * qy - wy * qx + wz * qw;
  const Real pw = 0 * qw - wx * qx - wy * qy - wz * qz;
  const Real rx = qx + px * 0.5, ry = qy + py * 0.5, rz = qz + pz * 0.5, rw = qw + pw * 0.5;
  const Real len = sqrt(rx * rx + ry * ry + rz * rz + rw * rw);
  o[0] = rx / len; o[1] = ry / len; o[2] = rz / len; o[3] = rw / len;
}
// maths.js:599-613
static inline void q_rotate(Real *o, const Real *q, const Real *v) {
  const Real ux = q[0], uy = q[1], uz = q[2], w = q[3];
  const Real vx = v[0], vy = v[1], vz = v[2];
  const Real tx = (uy * vz - uz * vy) * 2;
  const Real ty = (uz * vx - ux * vz) * 2;
  const Real tz = (ux * vy - uy * vx) * 2;
  o[0] = vx + tx * w + (uy * tz - uz * ty);
  o[1] = vy + ty * w + (uz * tx - ux * tz);
  o[2] = vz + tz * w + (ux * ty - uy * tx);
}
// maths.js:621-627
static inline void transform_point(Real *o, const Real *lin, const Real *ang, const Real *v) {
  q_rotate(o, ang, v);
  o[0] += lin[0]; o[1] += lin[1]; o[2] += lin[2];
}

// maths.js:660-725, unrolled LDL^T of the 6x6 block system
static void solve6(const Real *aLin, const Real *aAng, const Real *aCross, const Real *bLin,
                   const Real *bAng, Real *xLin, Real *xAng) {
  const Real A11 = aLin[0];
  const Real A21 = aLin[3], A22 = aLin[4];
  const Real A31 = aLin[6], A32 = aLin[7], A33 = aLin[8];
  const Real A41 = aCross[0], A42 = aCross[1], A43 = aCross[2], A44 = aAng[0];
  const Real A51 = aCross[3], A52 = aCross[4], A53 = aCross[5], A54 = aAng[3], A55 = aAng[4];
  const Real A61 = aCross[6], A62 = aCross[7], A63 = aCross[8], A64 = aAng[6], A65 = aAng[7], A66 = aAng[8];

  const Real L21 = A21 / A11, L31 = A31 / A11, L41 = A41 / A11, L51 = A51 / A11, L61 = A61 / A11;
  const Real D1 = A11;
  const Real D2 = A22 - L21 * L21 * D1;
  const Real L32 = (A32 - L21 * L31 * D1) / D2;
  const Real L42 = (A42 - L21 * L41 * D1) / D2;
  const Real L52 = (A52 - L21 * L51 * D1) / D2;
  const Real L62 = (A62 - L21 * L61 * D1) / D2;
  const Real D3 = A33 - (L31 * L31 * D1 + L32 * L32 * D2);
  const Real L43 = (A43 - L31 * L41 * D1 - L32 * L42 * D2) / D3;
  const Real L53 = (A53 - L31 * L51 * D1 - L32 * L52 * D2) / D3;
  const Real L63 = (A63 - L31 * L61 * D1 - L32 * L62 * D2) / D3;
  const Real D4 = A44 - (L41 * L41 * D1 + L42 * L42 * D2 + L43 * L43 * D3);
  const Real L54 = (A54 - L41 * L51 * D1 - L42 * L52 * D2 - L43 * L53 * D3) / D4;
  const Real L64 = (A64 - L41 * L61 * D1 - L42 * L62 * D2 - L43 * L63 * D3) / D4;
  const Real D5 = A55 - (L51 * L51 * D1 + L52 * L52 * D2 + L53 * L53 * D3 + L54 * L54 * D4);
  const Real L65 = (A65 - L51 * L61 * D1 - L52 * L62 * D2 - L53 * L63 * D3 - L54 * L64 * D4) / D5;
  const Real D6 = A66 - (L61 * L61 * D1 + L62 * L62 * D2 + L63 * L63 * D3 + L64 * L64 * D4 + L65 * L65 * D5);

  const Real y1 = bLin[0];
  const Real y2 = bLin[1] - L21 * y1;
  const Real y3 = bLin[2] - L31 * y1 - L32 * y2;
  const Real y4 = bAng[0] - L41 * y1 - L42 * y2 - L43 * y3;
  const Real y5 = bAng[1] - L51 * y1 - L52 * y2 - L53 * y3 - L54 * y4;
  const Real y6 = bAng[2] - L61 * y1 - L62 * y2 - L63 * y3 - L64 * y4 - L65 * y5;

  const Real z1 = y1 / D1, z2 = y2 / D2, z3 = y3 / D3, z4 = y4 / D4, z5 = y5 / D5, z6 = y6 / D6;

  xAng[2] = z6;
  xAng[1] = z5 - L65 * xAng[2];
  xAng[0] = z4 - L54 * xAng[1] - L64 * xAng[2];
  xLin[2] = z3 - L43 * xAng[0] - L53 * xAng[1] - L63 * xAng[2];
  xLin[1] = z2 - L32 * xLin[2] - L42 * xAng[0] - L52 * xAng[1] - L62 * xAng[2];
  xLin[0] = z1 - L21 * xLin[1] - L31 * xLin[2] - L41 * xAng[0] - L51 * xAng[1] - L61 * xAng[2];
}

// lowbias32 integer hash (src/physics/gpu/layout.js:50-57)
static inline uint32_t color_priority(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// ---------------------------------------------------------------------------
// Scene graph
// ---------------------------------------------------------------------------
struct Solver;
struct Force;

struct Body {
  int index = 0;
  int shape = AVBD_SHAPE_BOX;
  Real positionLin[3] = {0, 0, 0};
  Real positionAng[4] = {0, 0, 0, 1};
  Real initialLin[3] = {0, 0, 0};
  Real initialAng[4] = {0, 0, 0, 1};
  Real inertialLin[3] = {0, 0, 0};
  Real inertialAng[4] = {0, 0, 0, 1};
  Real velocityLin[3] = {0, 0, 0};
  Real velocityAng[3] = {0, 0, 0};
  Real prevVelocityLin[3] = {0, 0, 0};
  Real size[3] = {1, 1, 1};
  Real friction = 0.5;
  // contact materials (rigid.js:54-68, 144-214)
  Real staticFriction = 0.5, dynamicFriction = 0.5, restitution = 0, contactOffset = 0.005, restOffset = -0.005;
  // the broad phase's reach: the bounding radius, plus the contact offset
  // under AVBD_CONTACT_MATERIALS (shaders.js:440-442)
  Real reach = 0;
  Real mass = 0;
  Real moment[3] = {0, 0, 0};
  Real radius = 0;
  std::vector<Force *> forces; // creation order; iterate in reverse

  // rigid.js:228-247
  void computeWorldMoment(Real *out, bool rotated) const {
    if (!rotated || shape == AVBD_SHAPE_SPHERE) {
      m3_diagonal(out, moment[0], moment[1], moment[2]);
      return;
    }
    Real R[9], T[9];
    m3_from_quat(R, positionAng);
    m3_transpose(R, R);
    m3_diagonal(T, moment[0], moment[1], moment[2]);
    m3_mul(out, R, T);
    m3_transpose(R, R);
    m3_mul(out, out, R);
  }
  bool constrainedTo(const Body *other) const;
};

enum ForceKind { KIND_MANIFOLD = 0, KIND_JOINT = 1, KIND_SPRING = 2 };

struct Force {
  Solver *solver = nullptr;
  Body *bodyA = nullptr;
  Body *bodyB = nullptr;
  ForceKind kind = KIND_MANIFOLD;
  int id = 0; // index within its kind's array (joints / springs)
  virtual ~Force() {}
  virtual bool isBroken() const { return false; }
  virtual bool initialize() { return true; }
  virtual void updatePrimal(Body *body, Real alpha, Real *lhsLin, Real *lhsAng, Real *lhsCross,
                            Real *rhsLin, Real *rhsAng) = 0;
  virtual void updateDual(Real alpha) = 0;
  virtual Real maxLambda() const { return 0; }
  virtual Real maxPenalty() const { return 0; }
  virtual Real maxConstraintError() const { return 0; }
};

// rigid.js:250-259 (a manifold has no `broken` field, which reads falsy)
bool Body::constrainedTo(const Body *other) const {
  for (int i = (int)forces.size() - 1; i >= 0; i--) {
    const Force *f = forces[i];
    if (f->isBroken()) continue;
    if ((f->bodyA == this && f->bodyB == other) || (f->bodyA == other && f->bodyB == this)) return true;
  }
  return false;
}

struct Params {
  Real dt = 1.0 / 60.0, gravity = -10.0;
  int iterations = 10;
  Real betaLin = 1e4, betaAng = 100, alpha = 0.95, gamma = 0.999;
  bool postStabilize = false;
  Real penaltyMin = 1, penaltyMax = 1e10, collisionMargin = 0.01, stickThreshold = 1e-5;
  bool rotatedInertia = true, springRamp = false, springGeometric = true, cachedJacobians = true;
  int broadphase = 0, hashThreshold = 150, bodyOrderMode = AVBD_ORDER_REFERENCE;
  // the WebGPU engine's contact extensions (AVBD_CONTACT_MATERIALS) and their
  // defaults (solver.js:151-162)
  int contactModel = AVBD_CONTACT_CPU;
  Real contactOffset = 0.005, restOffset = -0.005, restitutionThreshold = 1.0, contactPersistence = 0.002;
};

// ---------------------------------------------------------------------------
// Narrow phase (src/physics/collide.js)
// ---------------------------------------------------------------------------
static const int MAX_CONTACTS = 8;
static const int MAX_POLY_VERTS = 16;
static const Real SAT_AXIS_EPSILON = 1.0e-6;
static const Real SPHERE_DISTANCE_EPSILON_SQ = 1.0e-20;
static const Real PLANE_EPSILON = 1.0e-5;
static const Real CONTACT_MERGE_DIST_SQ = 1.0e-6;
static const int AXIS_FACE_A = 0, AXIS_FACE_B = 1, AXIS_EDGE = 2;

struct Contact {
  uint32_t feature = 0;
  Real rA[3] = {0, 0, 0}, rB[3] = {0, 0, 0};
  Real C0[3] = {0, 0, 0}, penalty[3] = {0, 0, 0}, lambda[3] = {0, 0, 0};
  bool stick = false;
  Real C[3] = {0, 0, 0};
  Real restitutionBias = 0;  // AVBD_CONTACT_MATERIALS: this step's one-frame normal target
  void copyFrom(const Contact &o) { *this = o; }
  void reset() {
    feature = 0;
    v3_zero(penalty); v3_zero(lambda); v3_zero(C0); v3_zero(C);
    stick = false;
    restitutionBias = 0;
  }
};

struct OBB {
  Real center[3], half[3], axis[3][3];
};

struct SatAxis {
  int type = 0, indexA = -1, indexB = -1;
  Real separation = 0;
  Real normalAB[3] = {0, 0, 0};
  bool valid = false;
};

// The module-level scratch of collide.js, gathered in one object.
struct Collider {
  // the pair's contact skin: contacts are generated up to this separation
  // (AVBD_CONTACT_MATERIALS: the WGSL collider's contactDistance,
  // src/physics/gpu/shaders.js:716-886, 1039); 0 for the CPU engine's
  Real skin = 0;
  OBB boxA, boxB;
  Real frameNormal[3], frameCenter[3], frameU[3], frameV[3], frameExtentU, frameExtentV;
  Real faceExtU, faceExtV;
  Real clip0[MAX_POLY_VERTS * 3], clip1[MAX_POLY_VERTS * 3], midpoints[MAX_CONTACTS * 3];
  int stateCount = 0;

  static void makeOBB(OBB &box, const Body &b) {
    static const Real ux[3] = {1, 0, 0}, uy[3] = {0, 1, 0}, uz[3] = {0, 0, 1};
    v3_copy(box.center, b.positionLin);
    v3_scale(box.half, b.size, 0.5);
    q_rotate(box.axis[0], b.positionAng, ux);
    q_rotate(box.axis[1], b.positionAng, uy);
    q_rotate(box.axis[2], b.positionAng, uz);
  }
  static Real absDot(const Real *a, const Real *b) { return fabs(v3_dot(a, b)); }
  static void supportPoint(Real *out, const OBB &box, const Real *dir) {
    const Real sx = v3_dot(dir, box.axis[0]) >= 0 ? 1 : -1;
    const Real sy = v3_dot(dir, box.axis[1]) >= 0 ? 1 : -1;
    const Real sz = v3_dot(dir, box.axis[2]) >= 0 ? 1 : -1;
    v3_copy(out, box.center);
    v3_add_scaled(out, box.axis[0], box.half[0] * sx);
    v3_add_scaled(out, box.axis[1], box.half[1] * sy);
    v3_add_scaled(out, box.axis[2], box.half[2] * sz);
  }
  void getFaceAxes(const OBB &box, int axisIndex, Real *u, Real *v) {
    if (axisIndex == 0) {
      v3_copy(u, box.axis[1]); v3_copy(v, box.axis[2]); faceExtU = box.half[1]; faceExtV = box.half[2];
    } else if (axisIndex == 1) {
      v3_copy(u, box.axis[0]); v3_copy(v, box.axis[2]); faceExtU = box.half[0]; faceExtV = box.half[2];
    } else {
      v3_copy(u, box.axis[0]); v3_copy(v, box.axis[1]); faceExtU = box.half[0]; faceExtV = box.half[1];
    }
  }
  void buildFaceFrame(const OBB &box, int axisIndex, const Real *outwardNormal) {
    const Real s = v3_dot(outwardNormal, box.axis[axisIndex]) >= 0 ? 1 : -1;
    v3_scale(frameNormal, box.axis[axisIndex], s);
    v3_copy(frameCenter, box.center);
    v3_add_scaled(frameCenter, frameNormal, box.half[axisIndex]);
    getFaceAxes(box, axisIndex, frameU, frameV);
    frameExtentU = faceExtU;
    frameExtentV = faceExtV;
  }
  static int chooseIncidentFaceAxis(const OBB &box, const Real *referenceNormal) {
    int axis = 0;
    Real best = -INF;
    for (int i = 0; i < 3; i++) {
      const Real d = absDot(box.axis[i], referenceNormal);
      if (d > best) { best = d; axis = i; }
    }
    return axis;
  }
  void buildIncidentFace(Real *outVerts, const OBB &box, int axisIndex, const Real *referenceNormal) {
    Real t0[3], t1[3], t2[3], t3[3];
    const Real s = v3_dot(box.axis[axisIndex], referenceNormal) > 0 ? -1 : 1;
    v3_scale(t0, box.axis[axisIndex], s);
    v3_copy(t1, box.center);
    v3_add_scaled(t1, t0, box.half[axisIndex]);
    getFaceAxes(box, axisIndex, t2, t3);
    const Real eU = faceExtU, eV = faceExtV;
    for (int i = 0; i < 4; i++) {
      const Real su = (i == 0 || i == 3) ? 1 : -1;
      const Real sv = (i == 0 || i == 1) ? 1 : -1;
      outVerts[i * 3 + 0] = t1[0] + t2[0] * (eU * su) + t3[0] * (eV * sv);
      outVerts[i * 3 + 1] = t1[1] + t2[1] * (eU * su) + t3[1] * (eV * sv);
      outVerts[i * 3 + 2] = t1[2] + t2[2] * (eU * su) + t3[2] * (eV * sv);
    }
  }
  static int clipPolygonAgainstPlane(const Real *inV, int inCount, const Real *pn, Real po, Real *outV) {
    if (inCount <= 0) return 0;
    int outCount = 0;
    Real ax = inV[(inCount - 1) * 3 + 0], ay = inV[(inCount - 1) * 3 + 1], az = inV[(inCount - 1) * 3 + 2];
    Real da = pn[0] * ax + pn[1] * ay + pn[2] * az - po;
    for (int i = 0; i < inCount; i++) {
      const Real bx = inV[i * 3 + 0], by = inV[i * 3 + 1], bz = inV[i * 3 + 2];
      const Real db = pn[0] * bx + pn[1] * by + pn[2] * bz - po;
      const bool aInside = da <= PLANE_EPSILON;
      const bool bInside = db <= PLANE_EPSILON;
      if (aInside != bInside) {
        Real t = 0;
        const Real denom = da - db;
        if (fabs(denom) > SAT_AXIS_EPSILON) t = clamp(da / denom, 0, 1);
        if (outCount < MAX_POLY_VERTS) {
          outV[outCount * 3 + 0] = ax + (bx - ax) * t;
          outV[outCount * 3 + 1] = ay + (by - ay) * t;
          outV[outCount * 3 + 2] = az + (bz - az) * t;
          outCount++;
        }
      }
      if (bInside && outCount < MAX_POLY_VERTS) {
        outV[outCount * 3 + 0] = bx; outV[outCount * 3 + 1] = by; outV[outCount * 3 + 2] = bz;
        outCount++;
      }
      ax = bx; ay = by; az = bz; da = db;
    }
    return outCount;
  }
  // collide.js:254-285
  bool addContact(const Body &A, const Body &B, Contact *contacts, const Real *xA, const Real *xB, uint32_t key) {
    const Real mx = (xA[0] + xB[0]) * 0.5, my = (xA[1] + xB[1]) * 0.5, mz = (xA[2] + xB[2]) * 0.5;
    for (int i = 0; i < stateCount; i++) {
      const Real dx = mx - midpoints[i * 3 + 0], dy = my - midpoints[i * 3 + 1], dz = mz - midpoints[i * 3 + 2];
      if (dx * dx + dy * dy + dz * dz < CONTACT_MERGE_DIST_SQ) return false;
    }
    if (stateCount >= MAX_CONTACTS) return false;
    Contact &c = contacts[stateCount];
    c.feature = key;
    Real inv[4], t[3];
    q_conjugate(inv, A.positionAng);
    v3_sub(t, xA, A.positionLin);
    q_rotate(c.rA, inv, t);
    q_conjugate(inv, B.positionAng);
    v3_sub(t, xB, B.positionLin);
    q_rotate(c.rB, inv, t);
    midpoints[stateCount * 3 + 0] = mx; midpoints[stateCount * 3 + 1] = my; midpoints[stateCount * 3 + 2] = mz;
    stateCount++;
    return true;
  }
  // collide.js:291-324
  bool testAxis(const Real *delta, const Real *axis, int type, int indexA, int indexB, SatAxis &target) {
    const Real lenSq = v3_len_sq(axis);
    if (lenSq < SAT_AXIS_EPSILON) return true;
    const Real invLen = 1.0 / sqrt(lenSq);
    Real n[3];
    v3_scale(n, axis, invLen);
    if (v3_dot(n, delta) < 0) v3_negate(n, n);
    const Real distance = fabs(v3_dot(delta, n));
    const Real rA = boxA.half[0] * absDot(n, boxA.axis[0]) + boxA.half[1] * absDot(n, boxA.axis[1]) +
                      boxA.half[2] * absDot(n, boxA.axis[2]);
    const Real rB = boxB.half[0] * absDot(n, boxB.axis[0]) + boxB.half[1] * absDot(n, boxB.axis[1]) +
                      boxB.half[2] * absDot(n, boxB.axis[2]);
    const Real separation = distance - (rA + rB);
    if (separation > skin) return false;
    if (!target.valid || separation > target.separation) {
      target.valid = true;
      target.type = type; target.indexA = indexA; target.indexB = indexB;
      target.separation = separation;
      v3_copy(target.normalAB, n);
    }
    return true;
  }
  static void supportEdge(const OBB &box, int axisIndex, const Real *dir, Real *edgeA, Real *edgeB) {
    const int axis1 = (axisIndex + 1) % 3, axis2 = (axisIndex + 2) % 3;
    const Real sign1 = v3_dot(dir, box.axis[axis1]) >= 0 ? 1 : -1;
    const Real sign2 = v3_dot(dir, box.axis[axis2]) >= 0 ? 1 : -1;
    Real t[3];
    v3_copy(t, box.center);
    v3_add_scaled(t, box.axis[axis1], box.half[axis1] * sign1);
    v3_add_scaled(t, box.axis[axis2], box.half[axis2] * sign2);
    v3_copy(edgeA, t);
    v3_add_scaled(edgeA, box.axis[axisIndex], -box.half[axisIndex]);
    v3_copy(edgeB, t);
    v3_add_scaled(edgeB, box.axis[axisIndex], box.half[axisIndex]);
  }
  // collide.js:345-393
  static void closestPointsOnSegments(const Real *p0, const Real *p1, const Real *q0, const Real *q1,
                                      Real *c0, Real *c1) {
    const Real d1x = p1[0] - p0[0], d1y = p1[1] - p0[1], d1z = p1[2] - p0[2];
    const Real d2x = q1[0] - q0[0], d2y = q1[1] - q0[1], d2z = q1[2] - q0[2];
    const Real rx = p0[0] - q0[0], ry = p0[1] - q0[1], rz = p0[2] - q0[2];
    const Real a = d1x * d1x + d1y * d1y + d1z * d1z;
    const Real e = d2x * d2x + d2y * d2y + d2z * d2z;
    const Real f = d2x * rx + d2y * ry + d2z * rz;
    Real s = 0, t = 0;
    if (a <= SAT_AXIS_EPSILON && e <= SAT_AXIS_EPSILON) {
      v3_copy(c0, p0); v3_copy(c1, q0);
      return;
    }
    if (a <= SAT_AXIS_EPSILON) {
      t = clamp(f / e, 0, 1);
    } else {
      const Real c = d1x * rx + d1y * ry + d1z * rz;
      if (e <= SAT_AXIS_EPSILON) {
        s = clamp(-c / a, 0, 1);
      } else {
        const Real b = d1x * d2x + d1y * d2y + d1z * d2z;
        const Real denom = a * e - b * b;
        if (fabs(denom) > SAT_AXIS_EPSILON) s = clamp((b * f - c * e) / denom, 0, 1);
        t = (b * s + f) / e;
        if (t < 0) { t = 0; s = clamp(-c / a, 0, 1); }
        else if (t > 1) { t = 1; s = clamp((b - c) / a, 0, 1); }
      }
    }
    c0[0] = p0[0] + d1x * s; c0[1] = p0[1] + d1y * s; c0[2] = p0[2] + d1z * s;
    c1[0] = q0[0] + d2x * t; c1[1] = q0[1] + d2y * t; c1[2] = q0[2] + d2z * t;
  }
  // collide.js:403-472
  int buildFaceManifold(const Body &A, const Body &B, bool referenceIsA, int referenceAxis, const Real *normalAB,
                        Contact *contacts) {
    const OBB &referenceBox = referenceIsA ? boxA : boxB;
    const OBB &incidentBox = referenceIsA ? boxB : boxA;
    Real t0[3];
    if (referenceIsA) v3_copy(t0, normalAB);
    else v3_negate(t0, normalAB);
    buildFaceFrame(referenceBox, referenceAxis, t0);
    const int incidentAxis = chooseIncidentFaceAxis(incidentBox, frameNormal);
    buildIncidentFace(clip0, incidentBox, incidentAxis, frameNormal);
    int count = 4;
    Real pn[3];
    v3_copy(pn, frameU);
    count = clipPolygonAgainstPlane(clip0, count, pn, v3_dot(pn, frameCenter) + frameExtentU, clip1);
    if (!count) return 0;
    v3_negate(pn, frameU);
    count = clipPolygonAgainstPlane(clip1, count, pn, v3_dot(pn, frameCenter) + frameExtentU, clip0);
    if (!count) return 0;
    v3_copy(pn, frameV);
    count = clipPolygonAgainstPlane(clip0, count, pn, v3_dot(pn, frameCenter) + frameExtentV, clip1);
    if (!count) return 0;
    v3_negate(pn, frameV);
    count = clipPolygonAgainstPlane(clip1, count, pn, v3_dot(pn, frameCenter) + frameExtentV, clip0);
    if (!count) return 0;

    stateCount = 0;
    uint32_t featurePrefix = (uint32_t)(referenceIsA ? AXIS_FACE_A : AXIS_FACE_B) << 24;
    featurePrefix |= (uint32_t)(referenceAxis & 0xff) << 16;
    featurePrefix |= (uint32_t)(incidentAxis & 0xff) << 8;
    Real p[3], q[3], xA[3], xB[3];
    for (int i = 0; i < count && stateCount < MAX_CONTACTS; i++) {
      p[0] = clip0[i * 3 + 0]; p[1] = clip0[i * 3 + 1]; p[2] = clip0[i * 3 + 2];
      v3_sub(q, p, frameCenter);
      const Real distance = v3_dot(q, frameNormal);
      if (distance > skin + PLANE_EPSILON) continue;
      v3_copy(q, p);
      v3_add_scaled(q, frameNormal, -distance);
      if (referenceIsA) { v3_copy(xA, q); v3_copy(xB, p); }
      else { v3_copy(xA, p); v3_copy(xB, q); }
      addContact(A, B, contacts, xA, xB, featurePrefix | (uint32_t)(i & 0xff));
    }
    if (!stateCount) {
      Real neg[3];
      supportPoint(xA, boxA, normalAB);
      v3_negate(neg, normalAB);
      supportPoint(xB, boxB, neg);
      addContact(A, B, contacts, xA, xB, featurePrefix);
    }
    return stateCount;
  }
  // collide.js:475-493
  int buildEdgeContact(const Body &A, const Body &B, int axisA, int axisB, const Real *normalAB, Contact *contacts) {
    Real neg[3], eA0[3], eA1[3], eB0[3], eB1[3], xA[3], xB[3];
    v3_negate(neg, normalAB);
    supportEdge(boxA, axisA, normalAB, eA0, eA1);
    supportEdge(boxB, axisB, neg, eB0, eB1);
    closestPointsOnSegments(eA0, eA1, eB0, eB1, xA, xB);
    stateCount = 0;
    const uint32_t key = ((uint32_t)AXIS_EDGE << 24) | ((uint32_t)(axisA & 0xff) << 8) | (uint32_t)(axisB & 0xff);
    addContact(A, B, contacts, xA, xB, key);
    if (!stateCount) {
      supportPoint(xA, boxA, normalAB);
      supportPoint(xB, boxB, neg);
      addContact(A, B, contacts, xA, xB, key);
    }
    return stateCount;
  }
  // collide.js:496-520
  int sphereSphere(const Body &A, const Body &B, Contact *contacts, Real *basisOut) {
    Real delta[3], n[3], t[3], xA[3], xB[3];
    v3_sub(delta, B.positionLin, A.positionLin);
    const Real distanceSq = v3_len_sq(delta);
    const Real radiusSum = A.radius + B.radius + skin;
    if (distanceSq > radiusSum * radiusSum) return 0;
    if (distanceSq > SPHERE_DISTANCE_EPSILON_SQ) v3_scale(n, delta, 1 / sqrt(distanceSq));
    else v3_set(n, 1, 0, 0);
    v3_negate(t, n);
    m3_orthonormal(basisOut, t);
    v3_copy(xA, A.positionLin);
    v3_add_scaled(xA, n, A.radius);
    v3_copy(xB, B.positionLin);
    v3_add_scaled(xB, n, -B.radius);
    stateCount = 0;
    addContact(A, B, contacts, xA, xB, 0x31000001u);
    return stateCount;
  }
  // collide.js:526-600
  int sphereBox(const Body &A, const Body &B, Contact *contacts, Real *basisOut, bool sphereIsA) {
    const Body &sphere = sphereIsA ? A : B;
    const Body &boxBody = sphereIsA ? B : A;
    makeOBB(boxA, boxBody);
    Real delta[3], closest[3], t3[3], n[3], t0[3], xA[3], xB[3];
    v3_sub(delta, sphere.positionLin, boxA.center);
    const Real lx = v3_dot(delta, boxA.axis[0]);
    const Real ly = v3_dot(delta, boxA.axis[1]);
    const Real lz = v3_dot(delta, boxA.axis[2]);
    const Real cx = clamp(lx, -boxA.half[0], boxA.half[0]);
    const Real cy = clamp(ly, -boxA.half[1], boxA.half[1]);
    const Real cz = clamp(lz, -boxA.half[2], boxA.half[2]);
    v3_copy(closest, boxA.center);
    v3_add_scaled(closest, boxA.axis[0], cx);
    v3_add_scaled(closest, boxA.axis[1], cy);
    v3_add_scaled(closest, boxA.axis[2], cz);
    v3_sub(t3, sphere.positionLin, closest);
    const Real distanceSq = v3_len_sq(t3);
    int featureAxis = 0;
    if (distanceSq > SPHERE_DISTANCE_EPSILON_SQ) {
      const Real distance = sqrt(distanceSq);
      if (distance - sphere.radius > skin) return 0;
      v3_scale(n, t3, 1 / distance);
    } else {
      const Real gx = boxA.half[0] - fabs(lx);
      const Real gy = boxA.half[1] - fabs(ly);
      const Real gz = boxA.half[2] - fabs(lz);
      featureAxis = gx < gy ? (gx < gz ? 0 : 2) : (gy < gz ? 1 : 2);
      const Real local = featureAxis == 0 ? lx : featureAxis == 1 ? ly : lz;
      const Real sgn = local >= 0 ? 1 : -1;
      v3_scale(n, boxA.axis[featureAxis], sgn);
      const Real gap = featureAxis == 0 ? gx : featureAxis == 1 ? gy : gz;
      v3_copy(closest, sphere.positionLin);
      v3_add_scaled(closest, n, gap);
    }
    v3_copy(t3, sphere.positionLin);
    v3_add_scaled(t3, n, -sphere.radius);
    if (sphereIsA) {
      v3_copy(xA, t3); v3_copy(xB, closest);
      m3_orthonormal(basisOut, n);
    } else {
      v3_copy(xA, closest); v3_copy(xB, t3);
      v3_negate(t0, n);
      m3_orthonormal(basisOut, t0);
    }
    stateCount = 0;
    int sideX = lx < -boxA.half[0] ? 1 : lx > boxA.half[0] ? 2 : 0;
    int sideY = ly < -boxA.half[1] ? 1 : ly > boxA.half[1] ? 2 : 0;
    int sideZ = lz < -boxA.half[2] ? 1 : lz > boxA.half[2] ? 2 : 0;
    if ((sideX | sideY | sideZ) == 0) {
      const Real local = featureAxis == 0 ? lx : featureAxis == 1 ? ly : lz;
      const int side = local >= 0 ? 2 : 1;
      if (featureAxis == 0) sideX = side;
      else if (featureAxis == 1) sideY = side;
      else sideZ = side;
    }
    const uint32_t region = (uint32_t)(sideX | (sideY << 2) | (sideZ << 4));
    const uint32_t feature = 0x32000000u | (region << 2) | (sphereIsA ? 1u : 2u);
    addContact(A, B, contacts, xA, xB, feature);
    return stateCount;
  }
  // collide.js:612-685
  int collide(const Body &A, const Body &B, Contact *contacts, Real *basisOut) {
    const bool sA = A.shape == AVBD_SHAPE_SPHERE, sB = B.shape == AVBD_SHAPE_SPHERE;
    if (sA && sB) return sphereSphere(A, B, contacts, basisOut);
    if (sA || sB) return sphereBox(A, B, contacts, basisOut, sA);
    makeOBB(boxA, A);
    makeOBB(boxB, B);
    Real delta[3], axis[3], t0[3];
    v3_sub(delta, boxB.center, boxA.center);
    SatAxis bestFace, bestEdge, best;
    bestFace.separation = -INF; bestFace.valid = false;
    bestEdge.separation = -INF; bestEdge.valid = false;
    for (int i = 0; i < 3; i++)
      if (!testAxis(delta, boxA.axis[i], AXIS_FACE_A, i, -1, bestFace)) return 0;
    for (int i = 0; i < 3; i++)
      if (!testAxis(delta, boxB.axis[i], AXIS_FACE_B, -1, i, bestFace)) return 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        v3_cross(axis, boxA.axis[i], boxB.axis[j]);
        if (!testAxis(delta, axis, AXIS_EDGE, i, j, bestEdge)) return 0;
      }
    if (!bestFace.valid) return 0;
    best = bestFace;
    if (bestEdge.valid) {
      const Real edgeRelTol = 0.95, edgeAbsTol = 0.01;
      if (edgeRelTol * bestEdge.separation > bestFace.separation + edgeAbsTol) best = bestEdge;
    }
    v3_negate(t0, best.normalAB);
    m3_orthonormal(basisOut, t0);
    if (best.type == AXIS_EDGE) return buildEdgeContact(A, B, best.indexA, best.indexB, best.normalAB, contacts);
    if (best.type == AXIS_FACE_A) return buildFaceManifold(A, B, true, best.indexA, best.normalAB, contacts);
    return buildFaceManifold(A, B, false, best.indexB, best.normalAB, contacts);
  }
};

// ---------------------------------------------------------------------------
// Solver state
// ---------------------------------------------------------------------------
struct Solver {
  Params p;
  std::vector<Body *> bodies;
  std::vector<Force *> forces;
  std::vector<int32_t> bodyOrder;   // explicit order (AVBD_ORDER_EXPLICIT)
  std::vector<int32_t> lastColorOf; // priority colouring of the last step
  int lastNumColors = 0;
  std::vector<int64_t> lastPairs;   // manifolds initialised in the last step, (A<<32)|B
  Collider collider;
  std::vector<Force *> graveyard;   // removed joints/springs, freed with the solver
  std::vector<Force *> manifoldPool;  // recycled manifolds (solver.js:68-73)
  // The WebGPU backend's mouse grab (src/physics/gpu/shaders.js:2119-2161,
  // src/physics/gpu/backend.js:302-307): a finite ball socket from a world
  // target to a point on one body, with its penalty fixed at the stiffness,
  // no multiplier and no dual update, applied in that body's primal only (no
  // force list, no colouring edge). Null when nothing is grabbed.
  Force *grab = nullptr;
  ~Solver();
};

// ---------------------------------------------------------------------------
// Manifold (src/physics/manifold.js)
// ---------------------------------------------------------------------------
static void transportComponents(Real *out, const Real *value, const Real *oldB, const Real *newB) {
  const Real x = value[0], y = value[1], z = value[2];
  Real r3[3];
  for (int r = 0; r < 3; r++) {
    const int n = r * 3;
    r3[r] = x * (newB[n] * oldB[0] + newB[n + 1] * oldB[1] + newB[n + 2] * oldB[2]) +
            y * (newB[n] * oldB[3] + newB[n + 1] * oldB[4] + newB[n + 2] * oldB[5]) +
            z * (newB[n] * oldB[6] + newB[n + 1] * oldB[7] + newB[n + 2] * oldB[8]);
    out[r] = r3[r];
  }
}
static void transportPenalty(Real *out, const Real *value, const Real *oldB, const Real *newB) {
  const Real x = value[0], y = value[1], z = value[2];
  for (int r = 0; r < 3; r++) {
    const int n = r * 3;
    const Real dx = newB[n] * oldB[0] + newB[n + 1] * oldB[1] + newB[n + 2] * oldB[2];
    const Real dy = newB[n] * oldB[3] + newB[n + 1] * oldB[4] + newB[n + 2] * oldB[5];
    const Real dz = newB[n] * oldB[6] + newB[n + 1] * oldB[7] + newB[n + 2] * oldB[8];
    out[r] = x * dx * dx + y * dy * dy + z * dz * dz;
  }
}

struct Manifold : Force {
  Contact contacts[MAX_CONTACTS];
  Contact newContacts[MAX_CONTACTS];
  Real basis[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int numContacts = 0;
  Real friction = 0;
  // AVBD_CONTACT_MATERIALS: the pair's dynamic friction and whether its
  // contact skin (the sum of the contact offsets) is positive
  Real dynamicFriction = 0;
  bool skin = false;
  Real jacobians[MAX_CONTACTS * 18];
  bool jacobiansValid = false;
  // _beginPass scratch
  Real dqALin[3], dqAAng[3], dqBLin[3], dqBAng[3], jALin[9], jBLin[9], jAAng[9], jBAng[9];
  Real K[9], Cv[3], F[3];

  Manifold() { kind = KIND_MANIFOLD; }

  // manifold.js:214-318
  bool initialize() override {
    Body &A = *bodyA, &B = *bodyB;
    jacobiansValid = false;
    const bool hasSphere = A.shape == AVBD_SHAPE_SPHERE || B.shape == AVBD_SHAPE_SPHERE;
    const bool hadContacts = numContacts > 0;
    Real oldBasis[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if ((hasSphere || solver->p.contactModel == AVBD_CONTACT_MATERIALS) && hadContacts) m3_copy(oldBasis, basis);
    friction = sqrt(A.friction * B.friction);
    for (int i = 0; i < MAX_CONTACTS; i++) newContacts[i].reset();
    const bool materials = solver->p.contactModel == AVBD_CONTACT_MATERIALS;
    solver->collider.skin = materials ? A.contactOffset + B.contactOffset : 0;
    const int newNum = solver->collider.collide(A, B, newContacts, basis);
    if (materials) return initializeMaterials(oldBasis, hadContacts, newNum);
    const bool basisCompatible =
        !hasSphere || !hadContacts || (oldBasis[0] * basis[0] + oldBasis[1] * basis[1] + oldBasis[2] * basis[2]) > 0.85;
    for (int i = 0; i < newNum; i++) {
      for (int j = 0; j < numContacts; j++) {
        if (basisCompatible && newContacts[i].feature == contacts[j].feature) {
          Real nrA[3], nrB[3];
          v3_copy(nrA, newContacts[i].rA);
          v3_copy(nrB, newContacts[i].rB);
          newContacts[i].copyFrom(contacts[j]);
          if (hasSphere) {
            transportComponents(newContacts[i].lambda, newContacts[i].lambda, oldBasis, basis);
            transportPenalty(newContacts[i].penalty, newContacts[i].penalty, oldBasis, basis);
          }
          if (!contacts[j].stick || hasSphere) {
            v3_copy(newContacts[i].rA, nrA);
            v3_copy(newContacts[i].rB, nrB);
          }
          break;
        }
      }
    }
    numContacts = newNum;
    for (int i = 0; i < newNum; i++) contacts[i].copyFrom(newContacts[i]);
#ifdef ORC_TANGENT
    if (g_freeze_geometry & 1)
      for (int k = 0; k < 9; k++) basis[k] = Real(val(basis[k]));
    if (g_freeze_geometry & 2)
      for (int i = 0; i < numContacts; i++)
        for (int k = 0; k < 3; k++) {
          contacts[i].rA[k] = Real(val(contacts[i].rA[k]));
          contacts[i].rB[k] = Real(val(contacts[i].rB[k]));
        }
#endif
    const Params &P = solver->p;
    for (int i = 0; i < numContacts; i++) {
      Contact &c = contacts[i];
      Real xA[3], xB[3], d[3];
      transform_point(xA, A.positionLin, A.positionAng, c.rA);
      transform_point(xB, B.positionLin, B.positionAng, c.rB);
      v3_sub(d, xA, xB);
      m3_mul_vec(c.C0, basis, d);
      c.C0[0] += P.collisionMargin;
      if (!P.postStabilize) {
        v3_scale(c.lambda, c.lambda, P.alpha);
        v3_scale(c.lambda, c.lambda, P.gamma);
      }
      v3_scale(c.penalty, c.penalty, P.gamma);
      v3_clamp_scalar(c.penalty, c.penalty, P.penaltyMin, P.penaltyMax);
    }
    return numContacts > 0;
  }

  // The WebGPU engine's manifold warm start with its contact extensions
  // (src/physics/gpu/shaders.js:1105-1366): pair materials (friction as the
  // geometric mean of static and of dynamic coefficients, restitution as the
  // max, contact and rest offsets summed); each new contact matches the old
  // one with its feature ID, else the nearest old contact within the
  // persistence distance (separation, tangential offset and midpoint
  // distance all within it), each old contact claimed once and only when the
  // normals agree (dot > 0.85); multipliers and penalties are transported
  // into the new basis; a matched static box contact keeps its anchors; a
  // new contact starts static. C0 on the normal is measured to the rest
  // distance, and a new or re-armed impact gets a one-frame restitution bias.
  bool initializeMaterials(const Real *oldBasis, bool hadContacts, int newNum) {
    Body &A = *bodyA, &B = *bodyB;
    const Params &P = solver->p;
    friction = sqrt(A.staticFriction * B.staticFriction);
    dynamicFriction = sqrt(A.dynamicFriction * B.dynamicFriction);
    const Real restitution = js_max(A.restitution, B.restitution);
    const Real contactDistance = A.contactOffset + B.contactOffset;
    const Real restDistance = A.restOffset + B.restOffset;
    skin = contactDistance > 0;
    const Real *newN = &basis[0];
    const Real *oldN = hadContacts ? &oldBasis[0] : newN;
    const bool compatible = hadContacts && v3_dot(oldN, newN) > 0.85;
    const Real minExtent =
        2.0 * js_min(js_min(A.size[0] * 0.5, js_min(A.size[1] * 0.5, A.size[2] * 0.5)),
                     js_min(B.size[0] * 0.5, js_min(B.size[1] * 0.5, B.size[2] * 0.5)));
    const Real persistence = js_max(P.contactPersistence, js_max(contactDistance, minExtent * 0.02));
    const Real persistenceSq = persistence * persistence;
    const bool curved = A.shape == AVBD_SHAPE_SPHERE || B.shape == AVBD_SHAPE_SPHERE;
    unsigned oldUsed = 0;
    for (int c = 0; c < newNum; c++) {
      Contact &nc = newContacts[c];
      Real rA[3], rB[3], pen[3] = {0, 0, 0}, lam[3] = {0, 0, 0};
      v3_copy(rA, nc.rA);
      v3_copy(rB, nc.rB);
      bool priorOutsideRest = false, priorHadBias = false, stick = true;
      bool found = false, exact = false;
      int match = -1;
      Real best = persistenceSq;
      Real nxA[3], nxB[3], mid[3];
      transform_point(nxA, A.positionLin, A.positionAng, rA);
      transform_point(nxB, B.positionLin, B.positionAng, rB);
      for (int k = 0; k < 3; k++) mid[k] = (nxA[k] + nxB[k]) * 0.5;
      if (compatible) {
        for (int o = 0; o < numContacts; o++) {
          if (oldUsed & (1u << o)) continue;
          const Contact &oc = contacts[o];
          const bool same = oc.feature == nc.feature;
          if (curved && same) {
            match = o;
            exact = true;
            break;
          }
          Real oxA[3], oxB[3], od[3], td[3], md[3];
          transform_point(oxA, A.positionLin, A.positionAng, oc.rA);
          transform_point(oxB, B.positionLin, B.positionAng, oc.rB);
          v3_sub(od, oxA, oxB);
          const Real sep = v3_dot(newN, od);
          for (int k = 0; k < 3; k++) td[k] = od[k] - newN[k] * sep;
          if (sep > contactDistance + persistence) continue;
          if (v3_dot(td, td) > persistenceSq) continue;
          for (int k = 0; k < 3; k++) md[k] = mid[k] - (oxA[k] + oxB[k]) * 0.5;
          const Real mdSq = v3_dot(md, md);
          if (mdSq > persistenceSq) continue;
          if (same) {
            match = o;
            exact = true;
            break;
          }
          if (!found || mdSq < best) {
            found = true;
            match = o;
            best = mdSq;
          }
        }
      }
      found = found || exact;
      if (found) {
        const Contact &oc = contacts[match];
        oldUsed |= 1u << match;
        transportMaterials(pen, lam, oc.penalty, oc.lambda, oldBasis, basis);
        stick = oc.stick;
        priorOutsideRest = oc.C0[0] > 0;
        priorHadBias = oc.restitutionBias > 0;
        if (stick && A.shape != AVBD_SHAPE_SPHERE && B.shape != AVBD_SHAPE_SPHERE) {
          v3_copy(rA, oc.rA);
          v3_copy(rB, oc.rB);
        }
      }
      Contact &out = nc;  // newContacts[c] becomes the contact
      v3_copy(out.rA, rA);
      v3_copy(out.rB, rB);
      Real xA[3], xB[3], d[3];
      transform_point(xA, A.positionLin, A.positionAng, rA);
      transform_point(xB, B.positionLin, B.positionAng, rB);
      v3_sub(d, xA, xB);
      out.C0[0] = v3_dot(&basis[0], d) - restDistance;
      out.C0[1] = v3_dot(&basis[3], d);
      out.C0[2] = v3_dot(&basis[6], d);
      Real bias = 0;
      const bool armed = !found || (priorOutsideRest && !priorHadBias);
      if (armed && restitution > 0) {
        Real wA[3], wB[3], vA[3], vB[3], rel[3];
        q_rotate(wA, A.positionAng, rA);
        q_rotate(wB, B.positionAng, rB);
        v3_cross(vA, A.velocityAng, wA);
        v3_cross(vB, B.velocityAng, wB);
        for (int k = 0; k < 3; k++) rel[k] = (A.velocityLin[k] + vA[k]) - (B.velocityLin[k] + vB[k]);
        const Real vn = v3_dot(newN, rel);
        const Real closing = js_max(0.0, -vn * P.dt);
        const Real toRest = js_max(0.0, out.C0[0]);
        if (vn < -P.restitutionThreshold && closing > toRest) bias = restitution * (closing - toRest);
      }
      out.restitutionBias = bias;
      if (!P.postStabilize)
        for (int k = 0; k < 3; k++) lam[k] = lam[k] * P.alpha * P.gamma;
      for (int k = 0; k < 3; k++) out.penalty[k] = js_max(P.penaltyMin, js_min(P.penaltyMax, pen[k] * P.gamma));
      v3_copy(out.lambda, lam);
      out.stick = stick;
    }
    numContacts = newNum;
    for (int i = 0; i < newNum; i++) contacts[i].copyFrom(newContacts[i]);
    return numContacts > 0;
  }
  // transportPenalty / transportComponents of the WebGPU engine
  // (src/physics/gpu/shaders.js:1050-1085): rows of the new basis against the
  // old basis's rows
  static void transportMaterials(Real *pen, Real *lam, const Real *oldPen, const Real *oldLam, const Real *oldB,
                                 const Real *newB) {
    for (int r = 0; r < 3; r++) {
      const Real *n = &newB[r * 3];
      const Real a = v3_dot(n, &oldB[0]), b = v3_dot(n, &oldB[3]), c = v3_dot(n, &oldB[6]);
      pen[r] = oldPen[0] * (a * a) + oldPen[1] * (b * b) + oldPen[2] * (c * c);
      lam[r] = oldLam[0] * a + oldLam[1] * b + oldLam[2] * c;
    }
  }

  // manifold.js:325-350
  static void angularBlocks(const Real *rAW, const Real *rBW, const Real *jALin, const Real *jBLin,
                            Real *jAAng, Real *jBAng) {
    Real row[3], acc[3];
    for (int r = 0; r < 3; r++) {
      m3_get_row(row, jALin, r);
      v3_cross(acc, rAW, row);
      jAAng[r * 3 + 0] = acc[0]; jAAng[r * 3 + 1] = acc[1]; jAAng[r * 3 + 2] = acc[2];
      m3_get_row(row, jBLin, r);
      v3_cross(acc, rBW, row);
      jBAng[r * 3 + 0] = acc[0]; jBAng[r * 3 + 1] = acc[1]; jBAng[r * 3 + 2] = acc[2];
    }
  }
  void beginPass() {
    Body &A = *bodyA, &B = *bodyB;
    v3_sub(dqALin, A.positionLin, A.initialLin);
    q_subtract(dqAAng, A.positionAng, A.initialAng);
    v3_sub(dqBLin, B.positionLin, B.initialLin);
    q_subtract(dqBAng, B.positionAng, B.initialAng);
    m3_copy(jALin, basis);
    m3_negate(jBLin, basis);
    if (solver->p.cachedJacobians && !jacobiansValid) {
      for (int i = 0; i < numContacts; i++) {
        Real rAW[3], rBW[3];
        q_rotate(rAW, A.initialAng, contacts[i].rA);
        q_rotate(rBW, B.initialAng, contacts[i].rB);
        angularBlocks(rAW, rBW, jALin, jBLin, jAAng, jBAng);
        std::memcpy(&jacobians[i * 18], jAAng, sizeof(Real) * 9);
        std::memcpy(&jacobians[i * 18 + 9], jBAng, sizeof(Real) * 9);
      }
      jacobiansValid = true;
    }
  }
  // manifold.js:358-409
  bool evaluate(int i, Real alpha) {
    Contact &c = contacts[i];
    if (solver->p.cachedJacobians) {
      for (int k = 0; k < 9; k++) { jAAng[k] = jacobians[i * 18 + k]; jBAng[k] = jacobians[i * 18 + 9 + k]; }
    } else {
      Real rAW[3], rBW[3];
      q_rotate(rAW, bodyA->positionAng, c.rA);
      q_rotate(rBW, bodyB->positionAng, c.rB);
      angularBlocks(rAW, rBW, jALin, jBLin, jAAng, jBAng);
    }
    m3_diagonal(K, c.penalty[0], c.penalty[1], c.penalty[2]);
    Real acc[3];
    v3_scale(Cv, c.C0, 1 - alpha);
    const bool materials = solver->p.contactModel == AVBD_CONTACT_MATERIALS;
    if (materials) {
      // a positive speculative gap is kept unscaled while the skin is on, and
      // the restitution target applies outside the projection pass
      // (shaders.js:1806-1818)
      if (skin && c.C0[0] > 0) Cv[0] = c.C0[0];
      if (!(solver->p.postStabilize && alpha < 0.5)) Cv[0] = Cv[0] - c.restitutionBias;
    }
    m3_mul_vec(acc, jALin, dqALin); v3_add(Cv, Cv, acc);
    m3_mul_vec(acc, jBLin, dqBLin); v3_add(Cv, Cv, acc);
    m3_mul_vec(acc, jAAng, dqAAng); v3_add(Cv, Cv, acc);
    m3_mul_vec(acc, jBAng, dqBAng); v3_add(Cv, Cv, acc);
    m3_mul_vec(F, K, Cv);
    v3_add(F, F, c.lambda);
    F[0] = js_min(F[0], 0);
    if (materials) {
      // the static cone while the contact was static, else the dynamic one;
      // outside it the force is clamped to the dynamic cone (shaders.js:1826-1845)
      const Real fs = sqrt(F[1] * F[1] + F[2] * F[2]);
      const Real active = fabs(F[0]) * (c.stick ? friction : dynamicFriction);
      const bool within = fs <= active;
      if (!within && fs > 0) {
        const Real dyn = fabs(F[0]) * dynamicFriction;
        F[1] = F[1] * dyn / fs;
        F[2] = F[2] * dyn / fs;
      }
      return within;
    }
    const Real bounds = fabs(F[0]) * friction;
    const Real frictionScale = sqrt(F[1] * F[1] + F[2] * F[2]);
    if (frictionScale > bounds && frictionScale > 0) {
      F[1] *= bounds / frictionScale;
      F[2] *= bounds / frictionScale;
    }
    return frictionScale <= bounds;
  }
  // manifold.js:411-445
  void updatePrimal(Body *body, Real alpha, Real *lhsLin, Real *lhsAng, Real *lhsCross, Real *rhsLin,
                    Real *rhsAng) override {
    const bool isA = body == bodyA;
    beginPass();
    Real jLinT[9], jAngT[9], jAngTk[9], m0[9], acc[3];
    for (int i = 0; i < numContacts; i++) {
      Contact &c = contacts[i];
      evaluate(i, alpha);
      const Real *jLin = isA ? jALin : jBLin;
      const Real *jAng = isA ? jAAng : jBAng;
      m3_transpose(jLinT, jLin);
      m3_transpose(jAngT, jAng);
      m3_mul_diag_right(jAngTk, jAngT, c.penalty[0], c.penalty[1], c.penalty[2]);
      m3_mul_diag_right(m0, jLinT, c.penalty[0], c.penalty[1], c.penalty[2]);
      m3_mul(m0, m0, jLin);
      m3_add_into(lhsLin, m0);
      m3_mul(m0, jAngTk, jAng);
      m3_add_into(lhsAng, m0);
      m3_mul(m0, jAngTk, jLin);
      m3_add_into(lhsCross, m0);
      m3_mul_vec(acc, jLinT, F);
      v3_add(rhsLin, rhsLin, acc);
      m3_mul_vec(acc, jAngT, F);
      v3_add(rhsAng, rhsAng, acc);
    }
  }
  // manifold.js:447-491
  void updateDual(Real alpha) override {
    const Params &P = solver->p;
    beginPass();
    for (int i = 0; i < numContacts; i++) {
      Contact &c = contacts[i];
      const bool within = evaluate(i, alpha);
      v3_copy(c.lambda, F);
      v3_copy(c.C, Cv);
      if (F[0] < 0) c.penalty[0] = js_min(c.penalty[0] + P.betaLin * fabs(Cv[0]), P.penaltyMax);
      if (within) {
        c.penalty[1] = js_min(c.penalty[1] + P.betaLin * fabs(Cv[1]), P.penaltyMax);
        c.penalty[2] = js_min(c.penalty[2] + P.betaLin * fabs(Cv[2]), P.penaltyMax);
        c.stick = sqrt(Cv[1] * Cv[1] + Cv[2] * Cv[2]) < P.stickThreshold;
      } else if (bodyA->shape == AVBD_SHAPE_SPHERE || bodyB->shape == AVBD_SHAPE_SPHERE) {
        c.stick = false;
      }
      if (P.contactModel == AVBD_CONTACT_MATERIALS) c.stick = within;  // static = inside the cone (shaders.js:2253-2260)
    }
  }
  Real maxLambda() const override {
    Real m = 0;
    for (int i = 0; i < numContacts; i++) {
      const Real *l = contacts[i].lambda;
      m = js_max(m, js_max(fabs(l[0]), js_max(fabs(l[1]), fabs(l[2]))));
    }
    return m;
  }
  Real maxPenalty() const override {
    Real m = 0;
    for (int i = 0; i < numContacts; i++) {
      const Real *p = contacts[i].penalty;
      m = js_max(m, js_max(p[0], js_max(p[1], p[2])));
    }
    return m;
  }
  Real maxConstraintError() const override {
    Real m = 0;
    for (int i = 0; i < numContacts; i++) m = js_max(m, js_max(0, -contacts[i].C[0]));
    return m;
  }
};

// ---------------------------------------------------------------------------
// Joint (src/physics/joint.js)
// ---------------------------------------------------------------------------
static void geometricStiffnessBallSocket(Real *out, int k, const Real *v) {
  m3_diagonal(out, -v[k], -v[k], -v[k]);
  out[0 * 3 + k] += v[0];
  out[1 * 3 + k] += v[1];
  out[2 * 3 + k] += v[2];
}

struct Joint : Force {
  Real rA[3], rB[3];
  Real stiffnessLin = INF, stiffnessAng = 0, fracture = INF;
  bool broken = false;
  Real C0Lin[3] = {0, 0, 0}, C0Ang[3] = {0, 0, 0};
  Real penaltyLin[3] = {0, 0, 0}, penaltyAng[3] = {0, 0, 0};
  Real lambdaLin[3] = {0, 0, 0}, lambdaAng[3] = {0, 0, 0};
  Real CLin[3] = {0, 0, 0}, CAng[3] = {0, 0, 0};
  Real torqueArm = 0;

  Joint() { kind = KIND_JOINT; }
  bool isBroken() const override { return broken; }
  void setup() { // joint.js:108-112
    const Real *sA = bodyA ? bodyA->size : nullptr;
    const Real sx = (sA ? sA[0] : 0) + bodyB->size[0];
    const Real sy = (sA ? sA[1] : 0) + bodyB->size[1];
    const Real sz = (sA ? sA[2] : 0) + bodyB->size[2];
    torqueArm = sx * sx + sy * sy + sz * sz;
  }
  void evalLinear(Real *out) const {
    Real pA[3], pB[3];
    if (bodyA) transform_point(pA, bodyA->positionLin, bodyA->positionAng, rA);
    else v3_copy(pA, rA);
    transform_point(pB, bodyB->positionLin, bodyB->positionAng, rB);
    v3_sub(out, pA, pB);
  }
  void evalAngular(Real *out) const {
    static const Real identity[4] = {0, 0, 0, 1};
    q_subtract(out, bodyA ? bodyA->positionAng : identity, bodyB->positionAng);
    v3_scale(out, out, torqueArm);
  }
  // joint.js:131-160
  bool initialize() override {
    const Params &P = solver->p;
    evalLinear(C0Lin);
    evalAngular(C0Ang);
    if (!P.postStabilize) {
      v3_scale(lambdaLin, lambdaLin, P.alpha); v3_scale(lambdaLin, lambdaLin, P.gamma);
      v3_scale(lambdaAng, lambdaAng, P.alpha); v3_scale(lambdaAng, lambdaAng, P.gamma);
    }
    v3_scale(penaltyLin, penaltyLin, P.gamma);
    v3_clamp_scalar(penaltyLin, penaltyLin, P.penaltyMin, P.penaltyMax);
    v3_scale(penaltyAng, penaltyAng, P.gamma);
    v3_clamp_scalar(penaltyAng, penaltyAng, P.penaltyMin, P.penaltyMax);
    v3_min_scalar(penaltyLin, penaltyLin, stiffnessLin);
    v3_min_scalar(penaltyAng, penaltyAng, stiffnessAng);
    return !broken;
  }
  // joint.js:162-253
  void updatePrimal(Body *body, Real alpha, Real *lhsLin, Real *lhsAng, Real *lhsCross, Real *rhsLin,
                    Real *rhsAng) override {
    const bool isA = body == bodyA;
    Real K[9], C[3], F[3], rW[3], r[3], jLin[9], jAng[9], jLinT[9], jAngT[9], jAngTk[9], m0[9], H[9], G[9], acc[3];
    if (v3_len_sq(penaltyLin) > 0) {
      m3_diagonal(K, penaltyLin[0], penaltyLin[1], penaltyLin[2]);
      evalLinear(C);
      if (stiffnessLin == INF) v3_add_scaled(C, C0Lin, -alpha);
      m3_mul_vec(F, K, C);
      v3_add(F, F, lambdaLin);
      if (isA) {
        m3_diagonal(jLin, 1, 1, 1);
        q_rotate(rW, bodyA->positionAng, rA);
        v3_negate(r, rW);
        m3_skew(jAng, r);
        v3_copy(r, rW);
      } else {
        m3_diagonal(jLin, -1, -1, -1);
        q_rotate(rW, bodyB->positionAng, rB);
        m3_skew(jAng, rW);
        v3_negate(r, rW);
      }
      const Real k0 = penaltyLin[0], k1 = penaltyLin[1], k2 = penaltyLin[2];
      m3_transpose(jLinT, jLin);
      m3_transpose(jAngT, jAng);
      m3_mul_diag_right(jAngTk, jAngT, k0, k1, k2);
      m3_mul_diag_right(m0, jLinT, k0, k1, k2);
      m3_mul(m0, m0, jLin);
      m3_add_into(lhsLin, m0);
      m3_mul(m0, jAngTk, jAng);
      m3_add_into(lhsAng, m0);
      m3_mul(m0, jAngTk, jLin);
      m3_add_into(lhsCross, m0);
      m3_zero(H);
      for (int k = 0; k < 3; k++) {
        geometricStiffnessBallSocket(G, k, r);
        m3_scale(G, G, F[k]);
        m3_add_into(H, G);
      }
      m3_diagonalize(G, H);
      m3_add_into(lhsAng, G);
      m3_mul_vec(acc, jLinT, F);
      v3_add(rhsLin, rhsLin, acc);
      m3_mul_vec(acc, jAngT, F);
      v3_add(rhsAng, rhsAng, acc);
    }
    if (v3_len_sq(penaltyAng) > 0) {
      m3_diagonal(K, penaltyAng[0], penaltyAng[1], penaltyAng[2]);
      evalAngular(C);
      if (stiffnessAng == INF) v3_add_scaled(C, C0Ang, -alpha);
      m3_mul_vec(F, K, C);
      v3_add(F, F, lambdaAng);
      const Real s = isA ? torqueArm : -torqueArm;
      m3_diagonal(jAng, s, s, s);
      m3_transpose(jAngT, jAng);
      m3_mul(m0, jAngT, K);
      m3_mul(m0, m0, jAng);
      m3_add_into(lhsAng, m0);
      m3_mul_vec(acc, jAngT, F);
      v3_add(rhsAng, rhsAng, acc);
    }
  }
  // joint.js:255-317
  void updateDual(Real alpha) override {
    const Params &P = solver->p;
    Real K[9], C[3], F[3], acc[3];
    if (v3_len_sq(penaltyLin) > 0) {
      m3_diagonal(K, penaltyLin[0], penaltyLin[1], penaltyLin[2]);
      evalLinear(C);
      if (stiffnessLin == INF) {
        v3_add_scaled(C, C0Lin, -alpha);
        m3_mul_vec(F, K, C);
        v3_add(lambdaLin, F, lambdaLin);
      }
      v3_copy(CLin, C);
      v3_abs(acc, C);
      v3_scale(acc, acc, P.betaLin);
      v3_add(penaltyLin, penaltyLin, acc);
      v3_min_scalar(penaltyLin, penaltyLin, js_min(stiffnessLin, P.penaltyMax));
    }
    if (v3_len_sq(penaltyAng) > 0) {
      m3_diagonal(K, penaltyAng[0], penaltyAng[1], penaltyAng[2]);
      evalAngular(C);
      if (stiffnessAng == INF) {
        v3_add_scaled(C, C0Ang, -alpha);
        m3_mul_vec(F, K, C);
        v3_add(lambdaAng, F, lambdaAng);
      }
      v3_copy(CAng, C);
      v3_abs(acc, C);
      v3_scale(acc, acc, P.betaAng);
      v3_add(penaltyAng, penaltyAng, acc);
      v3_min_scalar(penaltyAng, penaltyAng, js_min(stiffnessAng, P.penaltyMax));
    }
    if (v3_len_sq(lambdaAng) > fracture * fracture) {
      v3_zero(penaltyLin); v3_zero(penaltyAng); v3_zero(lambdaLin); v3_zero(lambdaAng);
      broken = true;
    }
  }
  Real maxLambda() const override { return sqrt(js_max(v3_len_sq(lambdaLin), v3_len_sq(lambdaAng))); }
  Real maxPenalty() const override {
    Real m = penaltyLin[0];
    m = js_max(m, penaltyLin[1]); m = js_max(m, penaltyLin[2]);
    m = js_max(m, penaltyAng[0]); m = js_max(m, penaltyAng[1]); m = js_max(m, penaltyAng[2]);
    return m;
  }
  Real maxConstraintError() const override { return sqrt(v3_len_sq(CLin)); }
};

// ---------------------------------------------------------------------------
// Spring (src/physics/spring.js)
// ---------------------------------------------------------------------------
struct Spring : Force {
  Real rA[3], rB[3];
  Real stiffness = 0, rest = 0, penalty = 0, C = 0;
  Real tearStrain = INF;
  bool broken = false;
  Real peakStrain = 0;
  // _evaluate scratch (module-level in spring.js)
  Real d[3], n[3], rW[3];

  Spring() { kind = KIND_SPRING; }
  bool isBroken() const override { return broken; }
  bool rampEnabled() const { return solver->p.springRamp; }
  bool geometricEnabled() const { return solver->p.springGeometric; }

  Real evaluate() { // spring.js:447-458
    Real pA[3], pB[3];
    transform_point(pA, bodyA->positionLin, bodyA->positionAng, rA);
    transform_point(pB, bodyB->positionLin, bodyB->positionAng, rB);
    v3_sub(d, pA, pB);
    const Real dLen = v3_len(d);
    if (dLen <= 1.0e-6) return NaN;
    v3_div(n, d, dLen);
    return dLen - rest;
  }
  bool updateTearing(Real Cv) { // spring.js:461-470
    if (rest <= 1.0e-6) return false;
    const Real strain = js_max(0, Cv / rest);
    peakStrain = js_max(peakStrain, strain);
    if (strain <= tearStrain) return false;
    broken = true;
    penalty = 0;
    C = 0;
    return true;
  }
  bool initialize() override { // spring.js:472-507
    if (broken) { penalty = 0; C = 0; return true; }
    if (is_finite(tearStrain)) {
      const Real Cv = evaluate();
      if (!(Cv != Cv)) {
        C = Cv;
        if (updateTearing(Cv)) return true;
      }
    }
    const Params &P = solver->p;
    if (!rampEnabled()) {
      penalty = stiffness;
      return stiffness > 0;
    }
    penalty = clamp(penalty * P.gamma, P.penaltyMin, P.penaltyMax);
    penalty = js_min(penalty, stiffness);
    return stiffness > 0;
  }
  void updatePrimal(Body *body, Real alpha, Real *lhsLin, Real *lhsAng, Real *lhsCross, Real *rhsLin,
                    Real *rhsAng) override { // spring.js:509-553
    (void)alpha;
    (void)lhsCross;
    if (broken) return;
    const Real Cv = evaluate();
    if (Cv != Cv) return;
    const bool isA = body == bodyA;
    const Real k = penalty;
    const Real f = k * Cv;
    Real jLin[3], jAng[3], m0[9];
    if (isA) {
      q_rotate(rW, bodyA->positionAng, rA);
      v3_copy(jLin, n);
      v3_cross(jAng, rW, n);
    } else {
      q_rotate(rW, bodyB->positionAng, rB);
      v3_negate(jLin, n);
      v3_cross(jAng, rW, n);
      v3_negate(jAng, jAng);
    }
    m3_outer(m0, jLin, jLin); m3_scale(m0, m0, k); m3_add_into(lhsLin, m0);
    m3_outer(m0, jAng, jAng); m3_scale(m0, m0, k); m3_add_into(lhsAng, m0);
    m3_outer(m0, jAng, jLin); m3_scale(m0, m0, k); m3_add_into(lhsCross, m0);
    v3_add_scaled(rhsLin, jLin, f);
    v3_add_scaled(rhsAng, jAng, f);
    if (geometricEnabled()) stampGeometricStiffness(isA, f, lhsLin, lhsAng);
    C = Cv;
  }
  void stampGeometricStiffness(bool isA, Real f, Real *lhsLin, Real *lhsAng) { // spring.js:564-616
    const Real dLen = v3_len(d);
    const Real s = isA ? 1 : -1;
    Real P[9], S[9], Gll[9], Gla[9], Gal[9], Gaa[9], m0[9];
    m3_outer(P, n, n);
    m3_negate(P, P);
    P[0] += 1; P[4] += 1; P[8] += 1;
    m3_div(P, P, dLen);
    m3_skew(S, rW);
    m3_copy(Gll, P);
    m3_mul(Gla, P, S);
    m3_negate(Gla, Gla);
    m3_mul(Gal, S, P);
    m3_mul(Gaa, S, P);
    m3_mul(Gaa, Gaa, S);
    m3_negate(Gaa, Gaa);
    const Real ndotr = v3_dot(n, rW);
    m3_outer(m0, rW, n);
    m0[0] -= ndotr; m0[4] -= ndotr; m0[8] -= ndotr;
    m3_scale(m0, m0, s);
    m3_add_into(Gaa, m0);
    const Real af = fabs(f);
    for (int c = 0; c < 3; c++) {
      const Real a0 = Gll[c], a1 = Gll[3 + c], a2 = Gll[6 + c];
      const Real a3 = Gal[c], a4 = Gal[3 + c], a5 = Gal[6 + c];
      const Real g = sqrt(a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5) * af;
      lhsLin[c * 3 + c] += g;
    }
    for (int c = 0; c < 3; c++) {
      const Real a0 = Gla[c], a1 = Gla[3 + c], a2 = Gla[6 + c];
      const Real a3 = Gaa[c], a4 = Gaa[3 + c], a5 = Gaa[6 + c];
      const Real g = sqrt(a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5) * af;
      lhsAng[c * 3 + c] += g;
    }
  }
  void updateDual(Real alpha) override { // spring.js:618-634
    (void)alpha;
    if (broken) return;
    const Real Cv = evaluate();
    if (Cv != Cv) return;
    C = Cv;
    if (is_finite(tearStrain) && updateTearing(Cv)) return;
    if (!rampEnabled()) return;
    const Params &P = solver->p;
    penalty = js_min(penalty + P.betaLin * fabs(Cv), js_min(stiffness, P.penaltyMax));
  }
  Real maxLambda() const override { return broken ? 0 : fabs(penalty * C); }
  Real maxPenalty() const override { return broken ? 0 : penalty; }
  Real maxConstraintError() const override { return broken ? 0 : fabs(C); }
};

Solver::~Solver() {
  delete grab;
  for (Body *b : bodies) delete b;
  for (Force *f : forces) delete f;
  for (Force *f : graveyard) delete f;
  for (Force *f : manifoldPool) delete f;
}

// ---------------------------------------------------------------------------
// Broad phase (src/physics/broadphase.js)
// ---------------------------------------------------------------------------
static inline uint32_t hash_cell(int64_t x, int64_t y, int64_t z) { // broadphase.js:231-233
  const uint32_t hx = (uint32_t)(x * 73856093LL), hy = (uint32_t)(y * 19349663LL), hz = (uint32_t)(z * 83492791LL);
  return hx ^ hy ^ hz;
}

template <class Visit>
static void for_each_pair_hash(const std::vector<Body *> &bodies, Visit &&visit) { // broadphase.js:47-215
  const int n = (int)bodies.size();
  if (n < 2) return;
  Real radiusSum = 0;
  for (int i = 0; i < n; i++) radiusSum += bodies[i]->reach;
  const Real meanRadius = radiusSum / n;
  const Real largeThreshold = js_max(meanRadius * 8, 1e-6);
  const Real inv = 1 / js_max(meanRadius * 2, 1e-4);
  std::vector<int32_t> large;
  int64_t insertions = 0;
  for (int i = 0; i < n; i++) {
    const Body &b = *bodies[i];
    if (b.reach > largeThreshold) { large.push_back(i); continue; }
    const Real r = b.reach;
    const Real *p = b.positionLin;
    const int64_t nx = floor_i64((p[0] + r) * inv) - floor_i64((p[0] - r) * inv) + 1;
    const int64_t ny = floor_i64((p[1] + r) * inv) - floor_i64((p[1] - r) * inv) + 1;
    const int64_t nz = floor_i64((p[2] + r) * inv) - floor_i64((p[2] - r) * inv) + 1;
    insertions += nx * ny * nz;
  }
  int64_t tableSize = 64;
  while (tableSize < insertions * 2) tableSize *= 2;
  const uint32_t mask = (uint32_t)(tableSize - 1);
  std::vector<int32_t> counts(tableSize, 0), starts(tableSize, 0), scatter(tableSize, 0);
  std::vector<int32_t> entries(std::max<int64_t>(insertions, 1));
  std::vector<int32_t> lastSeen(n, -1);
  auto cell_range = [&](const Body &b, int64_t *lo, int64_t *hi) {
    const Real r = b.reach;
    const Real *p = b.positionLin;
    for (int a = 0; a < 3; a++) {
      lo[a] = floor_i64((p[a] - r) * inv);
      hi[a] = floor_i64((p[a] + r) * inv);
    }
  };
  for (int i = 0; i < n; i++) {
    const Body &b = *bodies[i];
    if (b.reach > largeThreshold) continue;
    int64_t lo[3], hi[3];
    cell_range(b, lo, hi);
    for (int64_t x = lo[0]; x <= hi[0]; x++)
      for (int64_t y = lo[1]; y <= hi[1]; y++)
        for (int64_t z = lo[2]; z <= hi[2]; z++) counts[hash_cell(x, y, z) & mask]++;
  }
  int32_t running = 0;
  for (int64_t c = 0; c < tableSize; c++) {
    starts[c] = running;
    scatter[c] = running;
    running += counts[c];
  }
  for (int i = 0; i < n; i++) {
    const Body &b = *bodies[i];
    if (b.reach > largeThreshold) continue;
    int64_t lo[3], hi[3];
    cell_range(b, lo, hi);
    for (int64_t x = lo[0]; x <= hi[0]; x++)
      for (int64_t y = lo[1]; y <= hi[1]; y++)
        for (int64_t z = lo[2]; z <= hi[2]; z++) entries[scatter[hash_cell(x, y, z) & mask]++] = i;
  }
  std::vector<int32_t> candidates;
  candidates.reserve(256);
  for (int i = n - 1; i >= 1; i--) {
    Body *bodyA = bodies[i];
    if (bodyA->reach > largeThreshold) {
      for (int j = i - 1; j >= 0; j--) visit(bodyA, bodies[j]);
      continue;
    }
    candidates.clear();
    for (int32_t j : large) {
      if (j < i && lastSeen[j] != i) { lastSeen[j] = i; candidates.push_back(j); }
    }
    int64_t lo[3], hi[3];
    cell_range(*bodyA, lo, hi);
    for (int64_t x = lo[0]; x <= hi[0]; x++)
      for (int64_t y = lo[1]; y <= hi[1]; y++)
        for (int64_t z = lo[2]; z <= hi[2]; z++) {
          const uint32_t b = hash_cell(x, y, z) & mask;
          const int32_t start = starts[b], end = start + counts[b];
          for (int32_t k = start; k < end; k++) {
            const int32_t j = entries[k];
            if (j < i && lastSeen[j] != i) { lastSeen[j] = i; candidates.push_back(j); }
          }
        }
    // descending index order (the reference uses an insertion sort)
    std::sort(candidates.begin(), candidates.end(), [](int32_t a, int32_t b) { return a > b; });
    for (int32_t j : candidates) visit(bodyA, bodies[j]);
  }
}

template <class Visit>
static void for_each_pair_brute(const std::vector<Body *> &bodies, Visit &&visit) { // broadphase.js:236-243
  for (int i = (int)bodies.size() - 1; i >= 1; i--)
    for (int j = i - 1; j >= 0; j--) visit(bodies[i], bodies[j]);
}

// ---------------------------------------------------------------------------
// Colouring
// ---------------------------------------------------------------------------
// Dynamic-dynamic edges of the current force list (after force init).
static void constraint_edges(const Solver &s, std::vector<std::vector<int32_t>> &adj) {
  const int n = (int)s.bodies.size();
  adj.assign(n, {});
  for (const Force *f : s.forces) {
    if (!f->bodyA || !f->bodyB) continue;
    if (f->isBroken()) continue;
    if (f->bodyA->mass <= 0 || f->bodyB->mass <= 0) continue;
    adj[f->bodyA->index].push_back(f->bodyB->index);
    adj[f->bodyB->index].push_back(f->bodyA->index);
  }
}

// Greedy colouring in integer-priority order: a body takes the smallest colour
// not used by its neighbours that precede it in (lowbias32(local index), index)
// order. Statics get -1. This is the fixed point of the reference GPU's Jacobi
// colouring (src/physics/gpu/shaders.js:1558-1656).
static int priority_coloring(const Solver &s, std::vector<int32_t> &colorOf) {
  const int n = (int)s.bodies.size();
  std::vector<std::vector<int32_t>> adj;
  constraint_edges(s, adj);
  std::vector<int32_t> order;
  order.reserve(n);
  for (int i = 0; i < n; i++)
    if (s.bodies[i]->mass > 0) order.push_back(i);
  std::sort(order.begin(), order.end(), [](int32_t a, int32_t b) {
    const uint32_t pa = color_priority((uint32_t)a), pb = color_priority((uint32_t)b);
    return pa < pb || (pa == pb && a < b);
  });
  colorOf.assign(n, -1);
  int numColors = 0;
  std::vector<int32_t> usedStamp(n + 1, -1);
  int stamp = 0;
  for (int32_t i : order) {
    stamp++;
    for (int32_t j : adj[i]) {
      const int32_t c = colorOf[j];
      if (c >= 0) usedStamp[c] = stamp;
    }
    int c = 0;
    while (c < numColors && usedStamp[c] == stamp) c++;
    if (c == numColors) numColors++;
    colorOf[i] = c;
  }
  return numColors;
}

// Coloring.build (src/physics/coloring.js:43-118): greedy in index order.
static int index_coloring(const Solver &s, std::vector<int32_t> &colorOf) {
  const int n = (int)s.bodies.size();
  std::vector<std::vector<int32_t>> adj(n);
  for (const Force *f : s.forces) {
    if (!f->bodyA || !f->bodyB) continue;
    adj[f->bodyA->index].push_back(f->bodyB->index);
    adj[f->bodyB->index].push_back(f->bodyA->index);
  }
  colorOf.assign(n, -1);
  std::vector<int32_t> used(n + 1, -1);
  int stamp = 0, numColors = 0;
  for (int i = 0; i < n; i++) {
    if (s.bodies[i]->mass <= 0) continue;
    stamp++;
    for (int32_t j : adj[i]) {
      const int32_t c = colorOf[j];
      if (c >= 0) used[c] = stamp;
    }
    int c = 0;
    while (c < numColors && used[c] == stamp) c++;
    if (c == numColors) numColors++;
    colorOf[i] = c;
  }
  return numColors;
}

// ---------------------------------------------------------------------------
// Algorithm 1 (src/physics/solver.js:307-493)
// ---------------------------------------------------------------------------
static void step(Solver &s) {
  const Real dt = s.p.dt;
  std::vector<Body *> &bodies = s.bodies;
  const Params &P = s.p;

  // 1. broad phase
  std::vector<Force *> created;
  auto visit = [&](Body *A, Body *B) {
    const Real dx = A->positionLin[0] - B->positionLin[0];
    const Real dy = A->positionLin[1] - B->positionLin[1];
    const Real dz = A->positionLin[2] - B->positionLin[2];
    const Real r = A->reach + B->reach;
    if (dx * dx + dy * dy + dz * dz <= r * r && !A->constrainedTo(B)) {
      if (A->mass > 0 || B->mass > 0) {
        // Manifold.reinit (manifold.js:201-212) on a pooled manifold, or a new one
        Manifold *m;
        if (!s.manifoldPool.empty()) {
          m = static_cast<Manifold *>(s.manifoldPool.back());
          s.manifoldPool.pop_back();
          m->numContacts = 0;
          m->friction = 0;
          for (int i = 0; i < MAX_CONTACTS; i++) m->contacts[i].reset();
        } else {
          m = new Manifold();
        }
        m->solver = &s;
        m->bodyA = A;
        m->bodyB = B;
        s.forces.push_back(m);
        A->forces.push_back(m);
        B->forces.push_back(m);
      }
    }
  };
  const bool useHash = P.broadphase == 1 || (P.broadphase == 0 && (int)bodies.size() > P.hashThreshold);
  if (useHash) for_each_pair_hash(bodies, visit);
  else for_each_pair_brute(bodies, visit);

  s.lastPairs.clear();
  for (Force *f : s.forces)
    if (f->kind == KIND_MANIFOLD)
      s.lastPairs.push_back(((int64_t)f->bodyA->index << 32) | (int64_t)f->bodyB->index);
  std::sort(s.lastPairs.begin(), s.lastPairs.end());

  // 2. force initialisation and warm start
  {
    std::vector<Force *> &forces = s.forces;
    size_t write = 0;
    for (size_t i = 0; i < forces.size(); i++) {
      Force *f = forces[i];
      if (f->initialize()) {
        forces[write++] = f;
      } else {
        for (Body *b : {f->bodyA, f->bodyB}) {
          if (!b) continue;
          auto it = std::find(b->forces.begin(), b->forces.end(), f);
          if (it != b->forces.end()) b->forces.erase(it);
        }
        if (f->kind == KIND_MANIFOLD) s.manifoldPool.push_back(f);
        else s.graveyard.push_back(f);
      }
    }
    forces.resize(write);
  }

  // 3. body initialisation (Eq. 2 + adaptive guess)
  Real gravityVec[3] = {0, 0, P.gravity};
  for (Body *b : bodies) {
    Real tmp[3];
    v3_copy(b->inertialLin, b->positionLin);
    v3_add_scaled(b->inertialLin, b->velocityLin, dt);
    if (b->mass > 0) v3_add_scaled(b->inertialLin, gravityVec, dt * dt);
    v3_scale(tmp, b->velocityAng, dt);
    q_integrate(b->inertialAng, b->positionAng, tmp);
    const Real accelZ = (b->velocityLin[2] - b->prevVelocityLin[2]) / dt;
    const Real accelExt = accelZ * sign(P.gravity);
    Real accelWeight = clamp(accelExt / fabs(P.gravity), 0.0, 1.0);
    if (!is_finite(accelWeight)) accelWeight = 0.0;
    v3_copy(b->initialLin, b->positionLin);
    q_copy(b->initialAng, b->positionAng);
    if (b->mass > 0) {
      v3_add_scaled(b->positionLin, b->velocityLin, dt);
      v3_add_scaled(b->positionLin, gravityVec, accelWeight * dt * dt);
      v3_scale(tmp, b->velocityAng, dt);
      q_integrate(b->positionAng, b->positionAng, tmp);
    }
  }

  // visit order of the primal sweep
  std::vector<int32_t> order;
  const std::vector<int32_t> *orderPtr = nullptr;
  if (P.bodyOrderMode == AVBD_ORDER_EXPLICIT && !s.bodyOrder.empty()) {
    orderPtr = &s.bodyOrder;
  } else if (P.bodyOrderMode == AVBD_ORDER_PRIORITY) {
    s.lastNumColors = priority_coloring(s, s.lastColorOf);
    for (int c = 0; c < s.lastNumColors; c++)
      for (int i = 0; i < (int)bodies.size(); i++)
        if (s.lastColorOf[i] == c) order.push_back(i);
    orderPtr = &order;
  }

  // 4. main loop
  const Real dt2 = dt * dt;
  const int totalIterations = P.iterations + (P.postStabilize ? 1 : 0);
  std::vector<Force *> &forces = s.forces;
  for (int it = 0; it < totalIterations; it++) {
    const Real alpha = P.postStabilize ? (it < P.iterations ? 1.0 : 0.0) : P.alpha;
    const int sweep = orderPtr ? (int)orderPtr->size() : (int)bodies.size();
    for (int si = 0; si < sweep; si++) {
      Body *b = orderPtr ? bodies[(*orderPtr)[si]] : bodies[bodies.size() - 1 - si];
      if (b->mass <= 0) continue;
      Real MLin[9], MAng[9], lhsLin[9], lhsAng[9], lhsCross[9], rhsLin[3], rhsAng[3], tmp[3], dq[3], dxLin[3],
          dxAng[3];
      m3_diagonal(MLin, b->mass, b->mass, b->mass);
      b->computeWorldMoment(MAng, P.rotatedInertia);
      m3_div(lhsLin, MLin, dt2);
      m3_div(lhsAng, MAng, dt2);
      m3_zero(lhsCross);
      v3_sub(tmp, b->positionLin, b->inertialLin);
      m3_mul_vec(rhsLin, lhsLin, tmp);
      q_subtract(dq, b->positionAng, b->inertialAng);
      m3_mul_vec(rhsAng, lhsAng, dq);
      for (int k = (int)b->forces.size() - 1; k >= 0; k--)
        b->forces[k]->updatePrimal(b, alpha, lhsLin, lhsAng, lhsCross, rhsLin, rhsAng);
      if (s.grab && s.grab->bodyB == b) s.grab->updatePrimal(b, alpha, lhsLin, lhsAng, lhsCross, rhsLin, rhsAng);
      v3_negate(rhsLin, rhsLin);
      v3_negate(rhsAng, rhsAng);
      solve6(lhsLin, lhsAng, lhsCross, rhsLin, rhsAng, dxLin, dxAng);
      v3_add(b->positionLin, b->positionLin, dxLin);
      q_integrate(b->positionAng, b->positionAng, dxAng);
    }
    if (it < P.iterations)
      for (int i = (int)forces.size() - 1; i >= 0; i--) forces[i]->updateDual(alpha);
    if (it == P.iterations - 1) {
      for (Body *b : bodies) {
        v3_copy(b->prevVelocityLin, b->velocityLin);
        if (b->mass > 0) {
          v3_sub(b->velocityLin, b->positionLin, b->initialLin);
          v3_div(b->velocityLin, b->velocityLin, dt);
          q_subtract(b->velocityAng, b->positionAng, b->initialAng);
          v3_div(b->velocityAng, b->velocityAng, dt);
        }
      }
    }
  }
}

} // namespace orc

// ===========================================================================
// C ABI for the tests (ctypes). Shares avbd_world with the CUDA backend.
// ===========================================================================
using namespace orc;

struct orc_solver {
  Solver s;
  std::string err;
};

static void params_from(Params &p, const avbd_params *a) {
  p.dt = a->dt; p.gravity = a->gravity; p.iterations = a->iterations; p.postStabilize = a->post_stabilize != 0;
  p.betaLin = a->beta_lin; p.betaAng = a->beta_ang; p.alpha = a->alpha; p.gamma = a->gamma;
  p.penaltyMin = a->penalty_min; p.penaltyMax = a->penalty_max; p.collisionMargin = a->collision_margin;
  p.stickThreshold = a->stick_threshold; p.rotatedInertia = a->rotated_inertia != 0;
  p.springRamp = a->spring_stiffness_ramp != 0; p.springGeometric = a->spring_geometric_stiffness != 0;
  p.cachedJacobians = a->cached_contact_jacobians != 0; p.broadphase = a->broadphase;
  p.hashThreshold = a->hash_threshold; p.bodyOrderMode = a->body_order;
  p.contactModel = a->contact_model; p.contactOffset = a->contact_offset; p.restOffset = a->rest_offset;
  p.restitutionThreshold = a->restitution_threshold; p.contactPersistence = a->contact_persistence;
}

extern "C" {

void orc_default_params(avbd_params *o) {
  std::memset(o, 0, sizeof(*o));
  o->dt = 1.0 / 60.0; o->gravity = -10.0; o->iterations = 10; o->post_stabilize = 0;
  o->beta_lin = 1e4; o->beta_ang = 100; o->alpha = 0.95; o->gamma = 0.999;
  o->penalty_min = 1; o->penalty_max = 1e10; o->collision_margin = 0.01; o->stick_threshold = 1e-5;
  o->rotated_inertia = 1; o->spring_stiffness_ramp = 0; o->spring_geometric_stiffness = 1;
  o->cached_contact_jacobians = 1; o->broadphase = 0; o->hash_threshold = 150;
  o->body_order = AVBD_ORDER_REFERENCE; o->fp64_ratio_threshold = 0; o->schedule = 1;
  o->contact_model = AVBD_CONTACT_CPU; o->contact_offset = 0.005; o->rest_offset = -0.005;
  o->restitution_threshold = 1.0; o->contact_persistence = 0.002;
}

orc_solver *orc_create(const avbd_params *params) {
  orc_solver *o = new orc_solver();
  params_from(o->s.p, params);
  return o;
}

void orc_destroy(orc_solver *o) { delete o; }

int orc_set_params(orc_solver *o, const avbd_params *params) {
  params_from(o->s.p, params);
  return AVBD_OK;
}

const char *orc_last_error(const orc_solver *o) { return o ? o->err.c_str() : ""; }

static void load_manifolds(orc_solver *o, const avbd_manifold_soa &M, std::vector<std::pair<int, Force *>> &ordered,
                           int base) {
  Solver &s = o->s;
  for (int m = 0; m < M.count; m++) {
    Manifold *f = new Manifold();
    f->solver = &s;
    f->bodyA = s.bodies[M.body_a[m]];
    f->bodyB = s.bodies[M.body_b[m]];
    f->numContacts = M.num_contacts[m];
    if (M.basis) for (int k = 0; k < 9; k++) f->basis[k] = M.basis[m * 9 + k];
    f->friction = M.friction ? M.friction[m] : 0;
    for (int i = 0; i < MAX_CONTACTS; i++) {
      Contact &c = f->contacts[i];
      const int slot = m * MAX_CONTACTS + i;
      c.feature = M.feature ? M.feature[slot] : 0;
      for (int k = 0; k < 3; k++) {
        c.rA[k] = M.r_a ? M.r_a[slot * 3 + k] : 0;
        c.rB[k] = M.r_b ? M.r_b[slot * 3 + k] : 0;
        c.penalty[k] = M.penalty ? M.penalty[slot * 3 + k] : 0;
        c.lambda[k] = M.lambda ? M.lambda[slot * 3 + k] : 0;
        c.C0[k] = M.c0 ? M.c0[slot * 3 + k] : 0;
      }
      c.stick = M.stick ? M.stick[slot] != 0 : false;
      c.restitutionBias = M.restitution_bias ? M.restitution_bias[slot] : 0;
    }
    if (s.p.contactModel == AVBD_CONTACT_MATERIALS) {  // the pair's materials, as initializeMaterials sets them
      const Body &A = *f->bodyA, &B = *f->bodyB;
      f->friction = sqrt(A.staticFriction * B.staticFriction);
      f->dynamicFriction = sqrt(A.dynamicFriction * B.dynamicFriction);
      f->skin = A.contactOffset + B.contactOffset > 0;
    }
    ordered.push_back({M.order ? M.order[m] : base + m, f});
  }
}

// Build the scene graph. Forces are ordered by their `order` fields when given,
// else joints, then springs, then manifolds, each in array order.
int orc_load(orc_solver *o, const avbd_world *w) {
  Solver &s = o->s;
  delete s.grab;
  s.grab = nullptr;
  for (Body *b : s.bodies) delete b;
  for (Force *f : s.forces) delete f;
  s.bodies.clear();
  s.forces.clear();
  const avbd_body_soa &B = w->bodies;
  for (int i = 0; i < B.count; i++) {
    Body *b = new Body();
    b->index = i;
    b->shape = B.shape ? B.shape[i] : AVBD_SHAPE_BOX;
    for (int k = 0; k < 3; k++) {
      b->size[k] = B.size[i * 3 + k];
      b->moment[k] = B.moment[i * 3 + k];
      b->positionLin[k] = B.pos[i * 3 + k];
      b->initialLin[k] = B.pos[i * 3 + k];
      b->velocityLin[k] = B.vel ? B.vel[i * 3 + k] : 0;
      b->velocityAng[k] = B.omega ? B.omega[i * 3 + k] : 0;
      b->prevVelocityLin[k] = B.prev_vel ? B.prev_vel[i * 3 + k] : b->velocityLin[k];
    }
    for (int k = 0; k < 4; k++) b->positionAng[k] = B.quat ? B.quat[i * 4 + k] : (k == 3 ? 1 : 0);
    q_copy(b->initialAng, b->positionAng);
    b->mass = B.mass[i];
    b->radius = B.radius[i];
    b->friction = B.friction[i];
    b->staticFriction = B.static_friction ? B.static_friction[i] : b->friction;
    b->dynamicFriction = B.dynamic_friction ? B.dynamic_friction[i] : b->friction;
    b->restitution = B.restitution ? B.restitution[i] : 0;
    b->contactOffset = B.contact_offset ? B.contact_offset[i] : s.p.contactOffset;
    b->restOffset = B.rest_offset ? B.rest_offset[i] : s.p.restOffset;
    b->reach = s.p.contactModel == AVBD_CONTACT_MATERIALS ? b->radius + b->contactOffset : b->radius;
    s.bodies.push_back(b);
  }
  std::vector<std::pair<int, Force *>> ordered;
  const avbd_joint_soa &J = w->joints;
  for (int j = 0; j < J.count; j++) {
    Joint *f = new Joint();
    f->solver = &s;
    f->id = j;
    f->bodyA = J.body_a[j] < 0 ? nullptr : s.bodies[J.body_a[j]];
    f->bodyB = s.bodies[J.body_b[j]];
    for (int k = 0; k < 3; k++) {
      f->rA[k] = J.r_a[j * 3 + k];
      f->rB[k] = J.r_b[j * 3 + k];
      f->penaltyLin[k] = J.penalty_lin ? J.penalty_lin[j * 3 + k] : 0;
      f->penaltyAng[k] = J.penalty_ang ? J.penalty_ang[j * 3 + k] : 0;
      f->lambdaLin[k] = J.lambda_lin ? J.lambda_lin[j * 3 + k] : 0;
      f->lambdaAng[k] = J.lambda_ang ? J.lambda_ang[j * 3 + k] : 0;
    }
    f->stiffnessLin = J.stiffness_lin[j];
    f->stiffnessAng = J.stiffness_ang[j];
    f->fracture = J.fracture[j];
    f->broken = J.broken ? J.broken[j] != 0 : false;
    f->setup();
    ordered.push_back({J.order ? J.order[j] : j, f});
  }
  const avbd_spring_soa &S = w->springs;
  for (int j = 0; j < S.count; j++) {
    Spring *f = new Spring();
    f->solver = &s;
    f->id = j;
    f->bodyA = s.bodies[S.body_a[j]];
    f->bodyB = s.bodies[S.body_b[j]];
    for (int k = 0; k < 3; k++) {
      f->rA[k] = S.r_a[j * 3 + k];
      f->rB[k] = S.r_b[j * 3 + k];
    }
    f->stiffness = S.stiffness[j];
    f->rest = S.rest[j];
    f->tearStrain = S.tear_strain ? S.tear_strain[j] : INF;
    f->penalty = S.penalty ? S.penalty[j] : 0;
    f->peakStrain = S.peak_strain ? S.peak_strain[j] : 0;
    f->broken = S.broken ? S.broken[j] != 0 : false;
    ordered.push_back({S.order ? S.order[j] : J.count + j, f});
  }
  load_manifolds(o, w->manifolds, ordered, J.count + S.count);
  std::stable_sort(ordered.begin(), ordered.end(),
                   [](const std::pair<int, Force *> &a, const std::pair<int, Force *> &b) { return a.first < b.first; });
  for (auto &e : ordered) {
    Force *f = e.second;
    s.forces.push_back(f);
    if (f->bodyA) f->bodyA->forces.push_back(f);
    if (f->bodyB) f->bodyB->forces.push_back(f);
  }
  return AVBD_OK;
}

int orc_set_body_order(orc_solver *o, const int32_t *order, int32_t n) {
  o->s.bodyOrder.assign(order, order + n);
  return AVBD_OK;
}

int orc_step(orc_solver *o, int32_t n) {
  for (int i = 0; i < n; i++) step(o->s);
  return AVBD_OK;
}

// Writes body state, joint/spring state (by id) and, when pointers are given,
// the manifolds in force-list order (count = number of manifolds).
int orc_read_state(orc_solver *o, avbd_world *w) {
  Solver &s = o->s;
  avbd_body_soa &B = w->bodies;
  const int n = std::min<int>(B.count, (int)s.bodies.size());
  for (int i = 0; i < n; i++) {
    const Body *b = s.bodies[i];
    for (int k = 0; k < 3; k++) {
      if (B.pos) B.pos[i * 3 + k] = val(b->positionLin[k]);
      if (B.vel) B.vel[i * 3 + k] = val(b->velocityLin[k]);
      if (B.omega) B.omega[i * 3 + k] = val(b->velocityAng[k]);
      if (B.prev_vel) B.prev_vel[i * 3 + k] = val(b->prevVelocityLin[k]);
    }
    if (B.quat) for (int k = 0; k < 4; k++) B.quat[i * 4 + k] = val(b->positionAng[k]);
  }
  avbd_manifold_soa &M = w->manifolds;
  int m = 0, pos = 0;
  for (const Force *f : s.forces) {
    if (f->kind == KIND_JOINT) {
      const Joint *j = static_cast<const Joint *>(f);
      avbd_joint_soa &J = w->joints;
      if (j->id < J.count) {
        for (int k = 0; k < 3; k++) {
          if (J.penalty_lin) J.penalty_lin[j->id * 3 + k] = val(j->penaltyLin[k]);
          if (J.penalty_ang) J.penalty_ang[j->id * 3 + k] = val(j->penaltyAng[k]);
          if (J.lambda_lin) J.lambda_lin[j->id * 3 + k] = val(j->lambdaLin[k]);
          if (J.lambda_ang) J.lambda_ang[j->id * 3 + k] = val(j->lambdaAng[k]);
        }
        if (J.broken) J.broken[j->id] = j->broken ? 1 : 0;
        if (J.order) J.order[j->id] = pos;
      }
    } else if (f->kind == KIND_SPRING) {
      const Spring *sp = static_cast<const Spring *>(f);
      avbd_spring_soa &S = w->springs;
      if (sp->id < S.count) {
        if (S.penalty) S.penalty[sp->id] = val(sp->penalty);
        if (S.peak_strain) S.peak_strain[sp->id] = val(sp->peakStrain);
        if (S.broken) S.broken[sp->id] = sp->broken ? 1 : 0;
        if (S.order) S.order[sp->id] = pos;
      }
    } else {
      const Manifold *mf = static_cast<const Manifold *>(f);
      if (m < M.capacity) {
        if (M.body_a) M.body_a[m] = val(mf->bodyA->index);
        if (M.body_b) M.body_b[m] = val(mf->bodyB->index);
        if (M.num_contacts) M.num_contacts[m] = val(mf->numContacts);
        if (M.basis) for (int k = 0; k < 9; k++) M.basis[m * 9 + k] = val(mf->basis[k]);
        if (M.friction) M.friction[m] = val(mf->friction);
        for (int i = 0; i < MAX_CONTACTS; i++) {
          const Contact &c = mf->contacts[i];
          const int slot = m * MAX_CONTACTS + i;
          if (M.feature) M.feature[slot] = i < mf->numContacts ? c.feature : 0;
          for (int k = 0; k < 3; k++) {
            const bool live = i < mf->numContacts;
            if (M.r_a) M.r_a[slot * 3 + k] = live ? val(c.rA[k]) : 0;
            if (M.r_b) M.r_b[slot * 3 + k] = live ? val(c.rB[k]) : 0;
            if (M.c0) M.c0[slot * 3 + k] = live ? val(c.C0[k]) : 0;
            if (M.penalty) M.penalty[slot * 3 + k] = live ? val(c.penalty[k]) : 0;
            if (M.lambda) M.lambda[slot * 3 + k] = live ? val(c.lambda[k]) : 0;
          }
          if (M.stick) M.stick[slot] = (i < mf->numContacts && c.stick) ? 1 : 0;
          if (M.restitution_bias) M.restitution_bias[slot] = i < mf->numContacts ? val(c.restitutionBias) : 0;
        }
        if (M.order) M.order[m] = pos;
      }
      m++;
    }
    pos++;
  }
  M.count = m;
  // Broken joints left the force list (joint.js:159 returns !broken); report
  // their final state too.
  for (const Force *f : s.graveyard) {
    if (f->kind != KIND_JOINT) continue;
    const Joint *j = static_cast<const Joint *>(f);
    avbd_joint_soa &J = w->joints;
    if (j->id >= J.count) continue;
    for (int k = 0; k < 3; k++) {
      if (J.penalty_lin) J.penalty_lin[j->id * 3 + k] = val(j->penaltyLin[k]);
      if (J.penalty_ang) J.penalty_ang[j->id * 3 + k] = val(j->penaltyAng[k]);
      if (J.lambda_lin) J.lambda_lin[j->id * 3 + k] = val(j->lambdaLin[k]);
      if (J.lambda_ang) J.lambda_ang[j->id * 3 + k] = val(j->lambdaAng[k]);
    }
    if (J.broken) J.broken[j->id] = j->broken ? 1 : 0;
    if (J.order) J.order[j->id] = -1;
  }
  return AVBD_OK;
}

// Joints/springs that were removed from the force list (broken joints) keep
// the state they had when removed; report them via this accessor.
// The uniform mouse grab (src/physics/gpu/shaders.js:2119-2161): body < 0
// releases it. Applies from the next step on.
int orc_set_grab(orc_solver *o, int32_t body, const double *local, const double *target, double stiffness) {
  Solver &s = o->s;
  delete s.grab;
  s.grab = nullptr;
  if (body < 0) return AVBD_OK;
  if (body >= (int32_t)s.bodies.size() || !(stiffness > 0)) return AVBD_ERR_ARG;
  Joint *j = new Joint();
  j->solver = &s;
  j->bodyA = nullptr;
  j->bodyB = s.bodies[body];
  for (int k = 0; k < 3; k++) {
    j->rA[k] = target[k];
    j->rB[k] = local[k];
    j->penaltyLin[k] = stiffness;
  }
  j->stiffnessLin = stiffness;
  j->stiffnessAng = 0;
  j->setup();
  s.grab = j;
  return AVBD_OK;
}

int orc_num_forces(orc_solver *o, int32_t *joints, int32_t *springs, int32_t *manifolds) {
  int j = 0, sp = 0, m = 0;
  for (const Force *f : o->s.forces) {
    if (f->kind == KIND_JOINT) j++;
    else if (f->kind == KIND_SPRING) sp++;
    else m++;
  }
  *joints = j; *springs = sp; *manifolds = m;
  return AVBD_OK;
}

int orc_read_coloring(orc_solver *o, int32_t *color_of, int32_t *num_colors) {
  const Solver &s = o->s;
  for (size_t i = 0; i < s.bodies.size(); i++) color_of[i] = i < s.lastColorOf.size() ? s.lastColorOf[i] : -1;
  *num_colors = s.lastNumColors;
  return AVBD_OK;
}

// Colourings of the CURRENT force list, without stepping.
int orc_priority_coloring(orc_solver *o, int32_t *color_of, int32_t *num_colors) {
  std::vector<int32_t> c;
  *num_colors = priority_coloring(o->s, c);
  std::memcpy(color_of, c.data(), c.size() * sizeof(int32_t));
  return AVBD_OK;
}
int orc_index_coloring(orc_solver *o, int32_t *color_of, int32_t *num_colors) {
  std::vector<int32_t> c;
  *num_colors = index_coloring(o->s, c);
  std::memcpy(color_of, c.data(), c.size() * sizeof(int32_t));
  return AVBD_OK;
}

// Pairs whose manifolds were initialised in the last step (new and persisting),
// sorted by (A, B); A is the higher index.
int orc_read_pairs(orc_solver *o, int32_t *a, int32_t *b, int64_t capacity, int64_t *count) {
  const std::vector<int64_t> &p = o->s.lastPairs;
  *count = (int64_t)p.size();
  for (int64_t i = 0; i < (int64_t)p.size() && i < capacity; i++) {
    a[i] = (int32_t)(p[i] >> 32);
    b[i] = (int32_t)(p[i] & 0xffffffff);
  }
  return AVBD_OK;
}

int orc_stats(orc_solver *o, avbd_stats *st) {
  const Solver &s = o->s;
  std::memset(st, 0, sizeof(*st));
  st->bodies = (int64_t)s.bodies.size();
  Real maxErr = 0, maxL = 0, maxP = 0;
  for (const Force *f : s.forces) {
    if (f->kind == KIND_MANIFOLD) {
      st->manifolds++;
      st->contacts += static_cast<const Manifold *>(f)->numContacts;
    }
    maxErr = js_max(maxErr, f->maxConstraintError());
    maxL = js_max(maxL, f->maxLambda());
    maxP = js_max(maxP, f->maxPenalty());
    if (f->kind == KIND_SPRING && static_cast<const Spring *>(f)->broken) st->springs_broken++;
  }
  for (const Force *f : s.graveyard)
    if (f->kind == KIND_JOINT && static_cast<const Joint *>(f)->broken) st->joints_broken++;
  st->candidate_pairs = (int64_t)s.lastPairs.size();
  st->colors = s.lastNumColors;
  st->max_constraint_error = val(maxErr);
  st->max_lambda = val(maxL);
  st->max_penalty = val(maxP);
  return AVBD_OK;
}

// Broken joints leave the force list; read their final state here.
int orc_read_joint(orc_solver *o, int32_t id, double *penalty_lin, double *lambda_ang, int32_t *broken) {
  auto scan = [&](const std::vector<Force *> &list) -> bool {
    for (const Force *f : list)
      if (f->kind == KIND_JOINT && f->id == id) {
        const Joint *j = static_cast<const Joint *>(f);
        for (int k = 0; k < 3; k++) { penalty_lin[k] = val(j->penaltyLin[k]); lambda_ang[k] = val(j->lambdaAng[k]); }
        *broken = j->broken ? 1 : 0;
        return true;
      }
    return false;
  };
  if (scan(o->s.forces) || scan(o->s.graveyard)) return AVBD_OK;
  return AVBD_ERR_ARG;
}

#ifndef ORC_TANGENT  // the f64 build's golden-vector helpers
// World-space inertia of body i (rigid.js:228-247).
int orc_world_moment(orc_solver *o, int32_t i, int32_t rotated, double *out9) {
  o->s.bodies[i]->computeWorldMoment(out9, rotated != 0);
  return AVBD_OK;
}

// Direct narrow-phase call on bodies a and b of the loaded scene
// (collide.js:612): contact count, basis, features and body-local anchors.
int orc_collide(orc_solver *o, int32_t a, int32_t b, double *basis9, uint32_t *features8, double *rA24,
                double *rB24) {
  Contact c[MAX_CONTACTS];
  for (auto &x : c) x.reset();
  double basis[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const Body &A = *o->s.bodies[a], &B = *o->s.bodies[b];
  o->s.collider.skin = o->s.p.contactModel == AVBD_CONTACT_MATERIALS ? val(A.contactOffset + B.contactOffset) : 0.0;
  const int n = o->s.collider.collide(A, B, c, basis);
  for (int k = 0; k < 9; k++) basis9[k] = basis[k];
  for (int i = 0; i < MAX_CONTACTS; i++) {
    features8[i] = c[i].feature;
    for (int k = 0; k < 3; k++) { rA24[i * 3 + k] = c[i].rA[k]; rB24[i * 3 + k] = c[i].rB[k]; }
  }
  return n;
}

// Math primitives, exposed for golden-vector tests of the restatement.
void orc_solve6(const double *aLin, const double *aAng, const double *aCross, const double *bLin,
                const double *bAng, double *xLin, double *xAng) {
  solve6(aLin, aAng, aCross, bLin, bAng, xLin, xAng);
}
void orc_quat_subtract(double *out3, const double *a, const double *b) { q_subtract(out3, a, b); }
void orc_quat_integrate(double *out4, const double *q, const double *dw) { q_integrate(out4, q, dw); }
void orc_quat_rotate(double *out3, const double *q, const double *v) { q_rotate(out3, q, v); }
void orc_orthonormal(double *out9, const double *n) { m3_orthonormal(out9, n); }
#endif
uint32_t orc_color_priority(uint32_t i) { return color_priority(i); }

// The normal row of every live contact's last evaluated constraint C (the
// `contact.C` of manifold.js:479, what test/convergence.mjs:57-71 reads as
// penetration), in force order; `count` returns the total.
int orc_contact_normal_c(orc_solver *o, double *out, int64_t capacity, int64_t *count) {
  int64_t k = 0;
  for (const Force *f : o->s.forces) {
    if (f->kind != KIND_MANIFOLD) continue;
    const Manifold *m = static_cast<const Manifold *>(f);
    for (int i = 0; i < m->numContacts; i++, k++)
      if (out && k < capacity) out[k] = val(m->contacts[i].C[0]);
  }
  *count = k;
  return AVBD_OK;
}

#ifdef ORC_TANGENT
// The tangent oracle's inputs and outputs. A seed sets direction `dir`
// (0..ND-1) of one input to 1, after orc_load:
//   what 0: linear velocity component `comp` of body `index` (its previous
//           velocity too: a scene starts with the two equal, rigid.js:51)
//   what 1: the friction of body `index`
//   what 2: the penalty cap penalty_max
int orc_t_dims() { return ND; }
void orc_t_freeze(int32_t mode) { g_freeze_geometry = mode; }
int orc_t_seed(orc_solver *o, int32_t what, int32_t index, int32_t comp, int32_t dir) {
  if (dir < 0 || dir >= ND) return AVBD_ERR_ARG;
  Solver &s = o->s;
  const bool body = what == 0 || what == 1;
  if (body && (index < 0 || index >= (int32_t)s.bodies.size())) return AVBD_ERR_ARG;
  if (what == 0) {
    if (comp < 0 || comp > 2) return AVBD_ERR_ARG;
    s.bodies[index]->velocityLin[comp].d[dir] = 1.0;
    s.bodies[index]->prevVelocityLin[comp].d[dir] = 1.0;
  } else if (what == 1) {
    s.bodies[index]->friction.d[dir] = 1.0;
  } else if (what == 2) {
    s.p.penaltyMax.d[dir] = 1.0;
  } else if (what == 3) {
    // joint `index`'s finite stiffnesses (joint.js:95-96; the caps of the
    // penalty ramp, joint.js:283-301)
    Joint *hit = nullptr;
    for (Force *f : s.forces)
      if (f->kind == KIND_JOINT && static_cast<Joint *>(f)->id == index) hit = static_cast<Joint *>(f);
    if (!hit) return AVBD_ERR_ARG;
    if (std::isfinite(hit->stiffnessLin.v)) hit->stiffnessLin.d[dir] = 1.0;
    if (std::isfinite(hit->stiffnessAng.v)) hit->stiffnessAng.d[dir] = 1.0;
  } else {
    return AVBD_ERR_ARG;
  }
  return AVBD_OK;
}
// Body positions (n x 3) and their tangents (n x 3 x ND).
int orc_t_read_pos(orc_solver *o, double *pos, double *tangents) {
  const Solver &s = o->s;
  for (size_t i = 0; i < s.bodies.size(); i++)
    for (int k = 0; k < 3; k++) {
      const Real &x = s.bodies[i]->positionLin[k];
      pos[i * 3 + k] = x.v;
      for (int d = 0; d < ND; d++) tangents[(i * 3 + k) * ND + d] = x.d[d];
    }
  return AVBD_OK;
}
#endif

} // extern "C"
