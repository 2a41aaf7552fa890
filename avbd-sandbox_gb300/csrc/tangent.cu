// tangent.cu - the differentiable AVBD step: forward-mode tangents through
// the whole world step, on the device.
//
// Every scalar of the step is a Dual (dual.cuh): a double value and
// kTangentDims directional derivatives along inputs the caller seeds (a
// body's initial velocity, a body's friction, the penalty cap, a joint's
// stiffness). The value part runs in f64 with the reference engine's
// operations (this unit is built with --fmad=false), so the discrete
// decisions of a step - the candidate pairs, the SAT axis and clip topology,
// the feature-ID warm start, the colouring, the cone and normal clamps, the
// stick test, the penalty caps - are the f64 engine's, and the derivatives
// follow the continuous path those decisions select: contact geometry as a
// function of the poses at the step's start (collider.cuh on Dual),
// warm start, every primal 6x6 solve and every dual update of every
// iteration, and the BDF1 velocity. Forward mode carries all seeded
// directions in one pass, so no checkpoints are needed; the backward of the
// C ABI contracts these columns with an upstream gradient.
//
// Reference path (src/physics/solver.js:307-493):
//   broad phase      solver.js:316-336, rigid.js:250-259 (constrainedTo)
//   narrow phase     collide.js:612-685 (collider.cuh), manifold.js:214-318
//   force init       joint.js:131-160, spring.js:472-507
//   body init        solver.js:366-401
//   primal           solver.js:418-458, manifold.js:325-445, joint.js:162-253,
//                    spring.js:509-616, maths.js:660-725 (solve6), :568-592
//   dual             manifold.js:447-491, joint.js:255-317, spring.js:618-634
//   velocity         solver.js:476-488
// Bodies are visited in the colour order of the integer-priority greedy
// colouring (src/physics/gpu/layout.js:50-66), as the CUDA backend's step.
//
// Layout: small scenes (the differentiable workloads: hundreds of bodies),
// structure of records. GB300's FP64 issue costs an SM sub-partition the same
// per warp instruction however few of its lanes are active, so the kernels
// compute in Dual1 - the value and one tangent direction - on five lanes per
// item, one direction a lane (every lane also computes the value and takes
// the same branches), and give each kind of work its own warps: the narrow
// phase, the force and body initialisations and the dual updates an item per
// five-lane group; the iterations one cooperative block per SM, a body
// update per block (its constraint rows on five-lane groups by kind, their
// addends summed in the f64 engine's order, the 6x6 LDL^T on six lanes a
// direction), bounded grid barriers between colour phases.
#include <cub/cub.cuh>

#include <cstdio>
#include <vector>

#include "../../include/avbd_cuda.h"
#include "avbd_device.cuh"
#include "collider.cuh"
#include "dual.cuh"

namespace avbd {
namespace tg {

using R = Dual;
constexpr int K8 = kMaxContacts;
constexpr int kBlock = 256;  // threads of the single-block kernels

struct TBody {
  R p[3], q[4];    // the iterate x (positionLin / positionAng)
  R dqL[3], dqA[3];  // p - p0 and qsub(q, q0) of the current iterate (what contact rows read), kept with p, q
  R v[3], w[3];    // velocity, angular velocity
  R pv[3];         // previous velocity
  R p0[3], q0[4];  // x_t (initialLin / initialAng)
  R q0i[4];        // q0's inverse q0* / |q0|^2, the right factor of every q_subtract(., q0) of the step
  R yqi[4];        // yq's inverse, likewise for the inertial terms
  R qi[4];         // q's inverse, kept with q during the iterations (the joints' angular rows)
  R yl[3], yq[4];  // inertial target y
};
struct TBodyStatic {
  double mass, moment[3], half[3], radius;
  R friction;
  int shape;
  int cStart, cEnd;  // joint/spring references (make_ref layout)
};
struct TJoint {
  int a, b;  // a = -1: rA is a world point
  R rA[3], rB[3];
  R stiffLin, stiffAng;
  double fracture, torqueArm;
  R penLin[3], penAng[3], lamLin[3], lamAng[3], C0Lin[3], C0Ang[3];
  int broken, removed;
};
struct TSpring {
  int a, b;
  R rA[3], rB[3];
  R stiffness;
  double rest, tear;
  R penalty, peak;
  int broken;
};
struct TContact {
  R rA[3], rB[3], C0[3], pen[3], lam[3];
  uint32_t feature;
  int stick;
};
struct TManifold {
  int a, b, count;
  R basis[9];
  R friction;
  TContact c[K8];
};

struct TParams {
  double dt, gravity, alpha, gamma, betaLin, betaAng, penaltyMin, margin, stickThreshold;
  R penaltyMax;
  int iterations, postStabilize, rotatedInertia, springRamp, springGeometric, cachedJacobians;
};

// Everything the tangent kernels touch (device pointers).
struct TWorld {
  TParams P;
  int n, nj, ns;
  TBody *b;
  // per contact slot of the current manifolds (manifold * 8 + contact): the
  // angular Jacobian rows of A and B at the x_t orientations (the cached
  // Jacobians of manifold.js:325-350), computed once per step
  R *jac;
  // per body: the 33 inertial entries of its next update's system (they
  // depend only on the body's own iterate, so they are formed in the phase
  // before its colour's)
  R *inert;
  TBodyStatic *bs;
  const uint32_t *cRef;
  TJoint *j;
  TSpring *s;
  // candidate pairs of the step and the manifolds (double-buffered by pair key)
  int mcap;
  int *pairCount, *pairStart;  // n + 1
  uint64_t *key;               // current candidates (mcap)
  TManifold *cur, *prev;
  uint64_t *prevKey;
  int *commitAt;  // per candidate: its slot among the step's live manifolds, or -1
  int *ctl;  // [0] candidates, [1] previous candidates, [2] overflow, [3] colours
  // adjacency of the solve (per dynamic body: its forces) and the colouring
  int *fStart, *fCount;  // n + 1
  uint32_t *fRef;        // (type << 30) | (index << 1) | side; type 0 = manifold
  int fcap;
  int *color, *order, *colorStart;  // colour per body; bodies by (colour, index); kMaxColors + 1
  uint32_t *prio;
};

// ---------------------------------------------------------------------------
// vec3 / mat3 / quaternion on R (maths.js: the operation order of the reference)
// ---------------------------------------------------------------------------
template <class S>
__device__ __forceinline__ S js_min(S a, S b) {
  if (a != a || b != b) return S(NAN);
  if (a < b) return a;
  if (b < a) return b;
  return a;
}
template <class S>
__device__ __forceinline__ S js_max(S a, S b) {
  if (a != a || b != b) return S(NAN);
  if (a > b) return a;
  if (b > a) return b;
  return a;
}
template <class S>
__device__ __forceinline__ S clampR(S x, S a, S b) { return js_max(a, js_min(b, x)); }
template <class S>
__device__ __forceinline__ void v3_sub(S *o, const S *a, const S *b) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
template <class S>
__device__ __forceinline__ void v3_add(S *o, const S *a, const S *b) {
  o[0] = a[0] + b[0]; o[1] = a[1] + b[1]; o[2] = a[2] + b[2];
}
// o += a * s; `o` an R array or a recording row (RecRow) of a body's system
template <class O, class S>
__device__ __forceinline__ void v3_add_scaled(O &&o, const S *a, S s) {
  o[0] += a[0] * s; o[1] += a[1] * s; o[2] += a[2] * s;
}
template <class O, class S>
__device__ __forceinline__ void v3_add_into(O &&o, const S *a) {
  o[0] += a[0]; o[1] += a[1]; o[2] += a[2];
}
template <class S>
__device__ __forceinline__ S v3_dot(const S *a, const S *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
template <class S>
__device__ __forceinline__ S v3_len_sq(const S *a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2]; }
template <class S>
__device__ __forceinline__ void v3_cross(S *o, const S *a, const S *b) {
  const S ax = a[0], ay = a[1], az = a[2], bx = b[0], by = b[1], bz = b[2];
  o[0] = ay * bz - az * by;
  o[1] = az * bx - ax * bz;
  o[2] = ax * by - ay * bx;
}
template <class S>
__device__ __forceinline__ void m3_zero(S *o) {
  for (int i = 0; i < 9; i++) o[i] = 0.0;
}
template <class S>
__device__ __forceinline__ void m3_diag(S *o, S a, S b, S c) {
  m3_zero(o);
  o[0] = a; o[4] = b; o[8] = c;
}
template <class S>
__device__ __forceinline__ void m3_mul_vec(S *o, const S *a, const S *v) {
  const S x = v[0], y = v[1], z = v[2];
  o[0] = a[0] * x + a[1] * y + a[2] * z;
  o[1] = a[3] * x + a[4] * y + a[5] * z;
  o[2] = a[6] * x + a[7] * y + a[8] * z;
}
template <class S>
__device__ void m3_mul(S *o, const S *a, const S *b) {
  S t[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) t[r * 3 + c] = a[r * 3] * b[c] + a[r * 3 + 1] * b[3 + c] + a[r * 3 + 2] * b[6 + c];
  for (int i = 0; i < 9; i++) o[i] = t[i];
}
template <class S>
__device__ __forceinline__ void m3_transpose(S *o, const S *a) {
  S t[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) t[c * 3 + r] = a[r * 3 + c];
  for (int i = 0; i < 9; i++) o[i] = t[i];
}
template <class S>
__device__ __forceinline__ void m3_skew(S *o, const S *r) {
  o[0] = 0.0; o[1] = -r[2]; o[2] = r[1];
  o[3] = r[2]; o[4] = 0.0; o[5] = -r[0];
  o[6] = -r[1]; o[7] = r[0]; o[8] = 0.0;
}
template <class O, class S>
__device__ __forceinline__ void m3_add_into(O &&o, const S *a) {
  for (int i = 0; i < 9; i++) o[i] += a[i];
}
// Eq. 20 (maths.js:541-555)
// q_subtract's second half: 2 (a * b^-1).xyz with b^-1 = (ix, iy, iz, iw)
template <class S>
__device__ __forceinline__ void q_mul_inv(S *o, const S *a, const S *inv) {
  const S ix = inv[0], iy = inv[1], iz = inv[2], iw = inv[3];
  const S ax = a[0], ay = a[1], az = a[2], aw = a[3];
  o[0] = (aw * ix + ax * iw + ay * iz - az * iy) * 2.0;
  o[1] = (aw * iy - ax * iz + ay * iw + az * ix) * 2.0;
  o[2] = (aw * iz + ax * iy - ay * ix + az * iw) * 2.0;
}
// b^-1 = b* / |b|^2
template <class S>
__device__ __forceinline__ void q_inverse(S *o, const S *b) {
  const S lsq = b[0] * b[0] + b[1] * b[1] + b[2] * b[2] + b[3] * b[3];
  o[0] = -b[0] / lsq;
  o[1] = -b[1] / lsq;
  o[2] = -b[2] / lsq;
  o[3] = b[3] / lsq;
}
template <class S>
__device__ void q_subtract(S *o, const S *a, const S *b) {
  S inv[4];
  q_inverse(inv, b);
  q_mul_inv(o, a, inv);
}
// Eq. 21 (maths.js:568-592), its "0 * q" terms kept
template <class S>
__device__ void q_integrate(S *o, const S *q, const S *dw) {
  const S qx = q[0], qy = q[1], qz = q[2], qw = q[3];
  const S wx = dw[0], wy = dw[1], wz = dw[2];
  const S px = 0.0 * qx + wx * qw + wy * qz - wz * qy;
  const S py = 0.0 * qy - wx * qz + wy * qw + wz * qx;
  const S pz = 0.0 * qz + wx * qy - wy * qx + wz * qw;
  const S pw = 0.0 * qw - wx * qx - wy * qy - wz * qz;
  const S rx = qx + px * 0.5, ry = qy + py * 0.5, rz = qz + pz * 0.5, rw = qw + pw * 0.5;
  const S len = sqrt(rx * rx + ry * ry + rz * rz + rw * rw);
  o[0] = rx / len; o[1] = ry / len; o[2] = rz / len; o[3] = rw / len;
}
// maths.js:599-613
template <class S>
__device__ void q_rotate(S *o, const S *q, const S *v) {
  const S ux = q[0], uy = q[1], uz = q[2], w = q[3];
  const S vx = v[0], vy = v[1], vz = v[2];
  const S tx = (uy * vz - uz * vy) * 2.0;
  const S ty = (uz * vx - ux * vz) * 2.0;
  const S tz = (ux * vy - uy * vx) * 2.0;
  o[0] = vx + tx * w + (uy * tz - uz * ty);
  o[1] = vy + ty * w + (uz * tx - ux * tz);
  o[2] = vz + tz * w + (ux * ty - uy * tx);
}
// maths.js:621-627
template <class S>
__device__ __forceinline__ void transform_point(S *o, const S *lin, const S *ang, const S *v) {
  q_rotate(o, ang, v);
  o[0] += lin[0]; o[1] += lin[1]; o[2] += lin[2];
}
// R I R^T of a body (rigid.js:228-247), maths.js:417-434 for R
template <class S>
__device__ void world_moment(S *out, const TBodyStatic &st, const S *q, bool rotated) {
  if (!rotated || st.shape == AVBD_SHAPE_SPHERE) {
    m3_diag(out, S(st.moment[0]), S(st.moment[1]), S(st.moment[2]));
    return;
  }
  const S x = q[0], y = q[1], z = q[2], w = q[3];
  const S xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y, wz = w * z;
  S Rm[9];
  Rm[0] = 1.0 - 2.0 * (yy + zz); Rm[1] = 2.0 * (xy + wz); Rm[2] = 2.0 * (xz - wy);
  Rm[3] = 2.0 * (xy - wz); Rm[4] = 1.0 - 2.0 * (xx + zz); Rm[5] = 2.0 * (yz + wx);
  Rm[6] = 2.0 * (xz + wy); Rm[7] = 2.0 * (yz - wx); Rm[8] = 1.0 - 2.0 * (xx + yy);
  S T[9], Rt[9];
  m3_transpose(Rt, Rm);
  m3_diag(T, S(st.moment[0]), S(st.moment[1]), S(st.moment[2]));
  m3_mul(out, Rt, T);
  m3_mul(out, out, Rm);
}
// maths.js:660-725, unrolled LDL^T of the 6x6 block system
template <class S>
__device__ void solve6(const S *aLin, const S *aAng, const S *aCross, const S *bLin, const S *bAng, S *xLin, S *xAng) {
  const S A11 = aLin[0];
  const S A21 = aLin[3], A22 = aLin[4];
  const S A31 = aLin[6], A32 = aLin[7], A33 = aLin[8];
  const S A41 = aCross[0], A42 = aCross[1], A43 = aCross[2], A44 = aAng[0];
  const S A51 = aCross[3], A52 = aCross[4], A53 = aCross[5], A54 = aAng[3], A55 = aAng[4];
  const S A61 = aCross[6], A62 = aCross[7], A63 = aCross[8], A64 = aAng[6], A65 = aAng[7], A66 = aAng[8];
  const S L21 = A21 / A11, L31 = A31 / A11, L41 = A41 / A11, L51 = A51 / A11, L61 = A61 / A11;
  const S D1 = A11;
  const S D2 = A22 - L21 * L21 * D1;
  const S L32 = (A32 - L21 * L31 * D1) / D2;
  const S L42 = (A42 - L21 * L41 * D1) / D2;
  const S L52 = (A52 - L21 * L51 * D1) / D2;
  const S L62 = (A62 - L21 * L61 * D1) / D2;
  const S D3 = A33 - (L31 * L31 * D1 + L32 * L32 * D2);
  const S L43 = (A43 - L31 * L41 * D1 - L32 * L42 * D2) / D3;
  const S L53 = (A53 - L31 * L51 * D1 - L32 * L52 * D2) / D3;
  const S L63 = (A63 - L31 * L61 * D1 - L32 * L62 * D2) / D3;
  const S D4 = A44 - (L41 * L41 * D1 + L42 * L42 * D2 + L43 * L43 * D3);
  const S L54 = (A54 - L41 * L51 * D1 - L42 * L52 * D2 - L43 * L53 * D3) / D4;
  const S L64 = (A64 - L41 * L61 * D1 - L42 * L62 * D2 - L43 * L63 * D3) / D4;
  const S D5 = A55 - (L51 * L51 * D1 + L52 * L52 * D2 + L53 * L53 * D3 + L54 * L54 * D4);
  const S L65 = (A65 - L51 * L61 * D1 - L52 * L62 * D2 - L53 * L63 * D3 - L54 * L64 * D4) / D5;
  const S D6 = A66 - (L61 * L61 * D1 + L62 * L62 * D2 + L63 * L63 * D3 + L64 * L64 * D4 + L65 * L65 * D5);
  const S y1 = bLin[0];
  const S y2 = bLin[1] - L21 * y1;
  const S y3 = bLin[2] - L31 * y1 - L32 * y2;
  const S y4 = bAng[0] - L41 * y1 - L42 * y2 - L43 * y3;
  const S y5 = bAng[1] - L51 * y1 - L52 * y2 - L53 * y3 - L54 * y4;
  const S y6 = bAng[2] - L61 * y1 - L62 * y2 - L63 * y3 - L64 * y4 - L65 * y5;
  const S z1 = y1 / D1, z2 = y2 / D2, z3 = y3 / D3, z4 = y4 / D4, z5 = y5 / D5, z6 = y6 / D6;
  xAng[2] = z6;
  xAng[1] = z5 - L65 * xAng[2];
  xAng[0] = z4 - L54 * xAng[1] - L64 * xAng[2];
  xLin[2] = z3 - L43 * xAng[0] - L53 * xAng[1] - L63 * xAng[2];
  xLin[1] = z2 - L32 * xLin[2] - L42 * xAng[0] - L52 * xAng[1] - L62 * xAng[2];
  xLin[0] = z1 - L21 * xLin[1] - L31 * xLin[2] - L41 * xAng[0] - L51 * xAng[1] - L61 * xAng[2];
}

// A body's 6x6 system, accumulated by its forces: 33 entries in this order.
template <class S>
struct Sys6T {
  S lin[9], ang[9], cross[9], bl[3], ba[3];
};
using Sys6 = Sys6T<R>;
constexpr int kSysEntries = 33;
static_assert(sizeof(Sys6) == kSysEntries * sizeof(R), "Sys6 is 33 contiguous entries");
static_assert(sizeof(Sys6T<Dual1>) == kSysEntries * sizeof(Dual1), "33 contiguous entries");

// A stored value as a thread computing in S sees it: the whole dual number,
// or its value and the derivative of tangent direction k.
template <class S>
__device__ __forceinline__ S ld(const R &x, int k);
template <>
__device__ __forceinline__ R ld<R>(const R &x, int) { return x; }
template <>
__device__ __forceinline__ Dual1 ld<Dual1>(const R &x, int k) { return dir_of(x, k); }
template <class S>
__device__ __forceinline__ void ldn(S *o, const R *x, int n, int k) {
  for (int c = 0; c < n; c++) o[c] = ld<S>(x[c], k);
}
// A body's iterate (p, q) as seen in S by direction k.
template <class S>
__device__ __forceinline__ void body_pose(const TWorld &w, int i, S *p, S *q, int k) {
  ldn(p, w.b[i].p, 3, k);
  ldn(q, w.b[i].q, 4, k);
}
// Per-item work of the kernels below runs on five-lane groups, a tangent
// direction a lane, six groups a warp (30 of its 32 lanes).
constexpr int kGroupsPerWarp = 6;

// The recording form of a body's system: one constraint's contribution as
// the sequence of addends it adds to each entry, so that the addends of many
// constraints, computed by different threads, are summed afterwards in the
// f64 engine's order. An entry has room for the most addends one row makes
// to it: a joint's angular diagonal gets its rows, its geometric stiffness
// and its angular rows (3), the angular off-diagonal and the angular
// right-hand side two, a spring's linear diagonal two (its geometric
// stiffness), every other entry one - 51 slots per row.
constexpr int kMaxAdd = 3;
// room per entry: lin (diagonal 2), ang (diagonal 3, off-diagonal 2), cross, bl, ba
__device__ __forceinline__ int rec_cap(int e) {
  return e < 9 ? ((e == 0 || e == 4 || e == 8) ? 2 : 1)
       : e < 18 ? ((e == 9 || e == 13 || e == 17) ? 3 : 2)
       : e < 30 ? 1
       : 2;
}
// first slot of entry e: the caps above summed
__device__ __forceinline__ int rec_off(int e) {
  if (e < 9) return e + (e > 0) + (e > 4);             // lin: 12 slots
  if (e < 18) {                                         // ang: 21 slots from 12
    const int k = e - 9;
    return 12 + 2 * k + (k > 0) + (k > 4);
  }
  if (e < 30) return 33 + (e - 18);                     // cross, bl: 12 slots from 33
  return 45 + 2 * (e - 30);                             // ba: 6 slots from 45
}
constexpr int kRecSlots = 51;
// One addend of tangent direction dir, recorded into its slot of the full
// dual number: direction 0 also writes the value (the same in every
// direction), so each thread owns the doubles it writes.
struct RecElem {
  R *slot;
  unsigned char *cnt;
  int cap, dir;
  __device__ void operator+=(const Dual1 &x) const {
    const int k = *cnt;
    if (k < cap) {
      if (dir == 0) slot[k].v = x.v;
      slot[k].d[dir] = x.d[0];
    }
    *cnt = (unsigned char)(k + 1);  // above the entry's room: reported by the replay
  }
};
struct RecRow {
  R *slot;
  unsigned char *cnt;
  int base, dir;  // first entry of the row
  __device__ RecElem operator[](int e) const {
    return RecElem{slot + rec_off(base + e), cnt + base + e, rec_cap(base + e), dir};
  }
};
struct RecSys6 {
  RecRow lin, ang, cross, bl, ba;
  __device__ RecSys6(R *slots, unsigned char *cnt, int dir)
      : lin{slots, cnt, 0, dir}, ang{slots, cnt, 9, dir}, cross{slots, cnt, 18, dir}, bl{slots, cnt, 27, dir},
        ba{slots, cnt, 30, dir} {}
};

__device__ __forceinline__ bool is_dynamic(const TWorld &w, int i) { return i >= 0 && w.bs[i].mass > 0; }
__device__ __forceinline__ uint64_t pair_key(int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; }

// Index of `key` in the sorted array, or -1.
__device__ int find_key(const uint64_t *keys, int n, uint64_t key) {
  int l = 0, h = n;
  while (l < h) {
    const int m = (l + h) >> 1;
    if (keys[m] < key) l = m + 1;
    else h = m;
  }
  return l < n && keys[l] == key ? l : -1;
}

// A live joint or spring joins a and b (rigid.js:250-259).
__device__ bool constrained(const TWorld &w, int a, int b) {
  const TBodyStatic &s = w.bs[a];
  for (int k = s.cStart; k < s.cEnd; k++) {
    const uint32_t ref = w.cRef[k];
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu;
    int x, y;
    if (type == kRefJoint) {
      const TJoint &j = w.j[idx];
      if (j.broken) continue;
      x = j.a; y = j.b;
    } else {
      const TSpring &sp = w.s[idx];
      if (sp.broken) continue;
      x = sp.a; y = sp.b;
    }
    if ((x == a && y == b) || (x == b && y == a)) return true;
  }
  return false;
}

// solver.js:316-336: pairs (a, b), b < a, whose bounding spheres overlap (f64
// values), not both static and not joined, and every pair that held contacts
// in the previous step (its manifold stays in the force list).
__device__ bool is_candidate(const TWorld &w, int a, int b, int prevCount) {
  if (!(w.bs[a].mass > 0 || w.bs[b].mass > 0)) return false;
  if (find_key(w.prevKey, prevCount, pair_key(a, b)) >= 0) return true;
  // the values of the dual positions' difference (the test reads values only)
  const double dx = w.b[a].p[0].v - w.b[b].p[0].v, dy = w.b[a].p[1].v - w.b[b].p[1].v,
               dz = w.b[a].p[2].v - w.b[b].p[2].v;
  const double r = w.bs[a].radius + w.bs[b].radius;
  if (!(dx * dx + dy * dy + dz * dz <= r * r)) return false;
  return !constrained(w, a, b);
}

// The candidate pairs (a, b), b < a, a warp per body a, its lanes over b in
// rounds of 32: a ballot counts them, and its prefix places them in
// increasing b.
__global__ void pairs_count_kernel(TWorld w) {
  const int prevCount = w.ctl[1], lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int a = blockIdx.x + gridDim.x * (threadIdx.x >> 5); a < w.n; a += warps) {
    int c = 0;
    for (int b0 = 0; b0 < a; b0 += 32) {
      const int b = b0 + lane;
      c += __popc(__ballot_sync(0xffffffffu, b < a && is_candidate(w, a, b, prevCount)));
    }
    if (lane == 0) w.pairCount[a] = c;
  }
}

__global__ void pairs_write_kernel(TWorld w) {
  const int prevCount = w.ctl[1], lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int a = blockIdx.x + gridDim.x * (threadIdx.x >> 5); a < w.n; a += warps) {
    int at = w.pairStart[a];
    for (int b0 = 0; b0 < a; b0 += 32) {
      const int b = b0 + lane;
      const bool cand = b < a && is_candidate(w, a, b, prevCount);
      const unsigned ballot = __ballot_sync(0xffffffffu, cand);
      if (cand) {
        const int k = at + __popc(ballot & ((1u << lane) - 1u));
        if (k < w.mcap) w.key[k] = pair_key(a, b);
      }
      at += __popc(ballot);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int total = w.pairStart[w.n];
    w.ctl[0] = total < w.mcap ? total : w.mcap;
    if (total > w.mcap) w.ctl[2] = 1;
  }
}

// manifold.js:222-270, the sphere pairs' transport of lambda and k into the new basis
template <class S>
__device__ void transport(S *lam, S *pen, const S *oldB, const S *newB) {
  const S x = lam[0], y = lam[1], z = lam[2];
  S o[3];
  for (int r = 0; r < 3; r++) {
    const int n = r * 3;
    o[r] = x * (newB[n] * oldB[0] + newB[n + 1] * oldB[1] + newB[n + 2] * oldB[2]) +
           y * (newB[n] * oldB[3] + newB[n + 1] * oldB[4] + newB[n + 2] * oldB[5]) +
           z * (newB[n] * oldB[6] + newB[n + 1] * oldB[7] + newB[n + 2] * oldB[8]);
  }
  lam[0] = o[0]; lam[1] = o[1]; lam[2] = o[2];
  const S px = pen[0], py = pen[1], pz = pen[2];
  for (int r = 0; r < 3; r++) {
    const int n = r * 3;
    const S dx = newB[n] * oldB[0] + newB[n + 1] * oldB[1] + newB[n + 2] * oldB[2];
    const S dy = newB[n] * oldB[3] + newB[n + 1] * oldB[4] + newB[n + 2] * oldB[5];
    const S dz = newB[n] * oldB[6] + newB[n + 1] * oldB[7] + newB[n + 2] * oldB[8];
    o[r] = px * dx * dx + py * dy * dy + pz * dz * dz;
  }
  pen[0] = o[0]; pen[1] = o[1]; pen[2] = o[2];
}

// body i's collision geometry as tangent direction dir sees it
__device__ geo::BodyT<Dual1> body_geo(const TWorld &w, int i, int dir) {
  geo::BodyT<Dual1> g;
  const TBody &b = w.b[i];
  const TBodyStatic &s = w.bs[i];
  g.p = geo::D3T<Dual1>{dir_of(b.p[0], dir), dir_of(b.p[1], dir), dir_of(b.p[2], dir)};
  g.q = geo::QDT<Dual1>{dir_of(b.q[0], dir), dir_of(b.q[1], dir), dir_of(b.q[2], dir), dir_of(b.q[3], dir)};
  g.half = geo::D3T<Dual1>{Dual1(s.half[0]), Dual1(s.half[1]), Dual1(s.half[2])};
  g.radius = s.radius;
  g.sphere = s.shape == AVBD_SHAPE_SPHERE;
  return g;
}

// Manifold.initialize (manifold.js:214-318) of candidate c, at x_t.
// manifold.js:325-350: the angular Jacobian rows of a contact, rows of
// rA_world x n_r (A) and rB_world x (-n_r) (B), into out[0..8] and out[9..17]
template <class S>
__device__ void contact_jacobians(S *out, const S *basis, const S *qA, const S *qB, const S *rA, const S *rB) {
  S rAW[3], rBW[3], row[3], acc[3];
  q_rotate(rAW, qA, rA);
  q_rotate(rBW, qB, rB);
  for (int r = 0; r < 3; r++) {
    row[0] = basis[r * 3]; row[1] = basis[r * 3 + 1]; row[2] = basis[r * 3 + 2];
    v3_cross(acc, rAW, row);
    out[r * 3] = acc[0]; out[r * 3 + 1] = acc[1]; out[r * 3 + 2] = acc[2];
    row[0] = -basis[r * 3]; row[1] = -basis[r * 3 + 1]; row[2] = -basis[r * 3 + 2];
    v3_cross(acc, rBW, row);
    out[9 + r * 3] = acc[0]; out[9 + r * 3 + 1] = acc[1]; out[9 + r * 3 + 2] = acc[2];
  }
}

// One candidate pair per five-lane group, a tangent direction per lane
// (each lane also computes the values, so every lane takes the same
// branches); lane 0 writes the value parts and the integers. Nothing the
// kernel writes is read back: the manifold's data stay in registers.
__global__ void narrow_kernel(TWorld w) {
  using S = Dual1;
  const int total = w.ctl[0], prevCount = w.ctl[1];
  const TParams &P = w.P;
  const int lane = threadIdx.x & 31, slot = lane / kTangentDims, dir = lane % kTangentDims;
  if (slot >= kGroupsPerWarp) return;
  const int nWarps = gridDim.x * (blockDim.x >> 5), wg = blockIdx.x + gridDim.x * (threadIdx.x >> 5);
  // pairs spread over the warps (and SMs) first, then over a warp's groups
  for (int c = slot * nWarps + wg; c < total; c += nWarps * kGroupsPerWarp) {
    const uint64_t key = w.key[c];
    const int ia = (int)(key >> 32), ib = (int)(key & 0xffffffffu);
    TManifold &m = w.cur[c];
    const int pi = find_key(w.prevKey, prevCount, key);
    const TManifold *old = pi >= 0 ? &w.prev[pi] : nullptr;
    const int oldNum = old ? old->count : 0;
    const bool hasSphere = w.bs[ia].shape == AVBD_SHAPE_SPHERE || w.bs[ib].shape == AVBD_SHAPE_SPHERE;
    set_dir(m.friction, sqrt(dir_of(w.bs[ia].friction, dir) * dir_of(w.bs[ib].friction, dir)), dir);
    const geo::BodyT<S> A = body_geo(w, ia, dir), B = body_geo(w, ib, dir);
    geo::NewContactT<S> nc[K8];
    S basis[9];
    for (int k = 0; k < 9; k++) basis[k] = 0.0;
    geo::ColliderT<S> col(A, B, nc);
    const int num = col.collide(basis);
    bool compatible = true;
    if (hasSphere && oldNum > 0)
      compatible = (old->basis[0].v * basis[0].v + old->basis[1].v * basis[1].v + old->basis[2].v * basis[2].v) > 0.85;
    for (int k = 0; k < 9; k++) set_dir(m.basis[k], basis[k], dir);
    if (dir == 0) {
      m.a = ia;
      m.b = ib;
      m.count = num;
    }
    S pA[3], qA[4], pB[3], qB[4];
    body_pose(w, ia, pA, qA, dir);
    body_pose(w, ib, pB, qB, dir);
    for (int i = 0; i < num; i++) {
      TContact &t = m.c[i];
      S rA[3] = {nc[i].rA.x, nc[i].rA.y, nc[i].rA.z}, rB[3] = {nc[i].rB.x, nc[i].rB.y, nc[i].rB.z};
      S pen[3] = {S(0.0), S(0.0), S(0.0)}, lam[3] = {S(0.0), S(0.0), S(0.0)};
      int stick = 0;
      for (int j = 0; j < oldNum; j++) {
        const TContact &o = old->c[j];
        if (compatible && nc[i].feature == o.feature) {
          ldn(pen, o.pen, 3, dir);
          ldn(lam, o.lam, 3, dir);
          stick = o.stick;
          if (hasSphere) {
            S ob[9];
            ldn(ob, old->basis, 9, dir);
            transport(lam, pen, ob, basis);
          }
          if (o.stick && !hasSphere) {  // a stuck box contact keeps its anchors (manifold.js:279-282)
            ldn(rA, o.rA, 3, dir);
            ldn(rB, o.rB, 3, dir);
          }
          break;
        }
      }
      // C*(x_t) + margin, warm start (manifold.js:292-315)
      S xA[3], xB[3], d[3], C0[3];
      transform_point(xA, pA, qA, rA);
      transform_point(xB, pB, qB, rB);
      v3_sub(d, xA, xB);
      m3_mul_vec(C0, basis, d);
      C0[0] = C0[0] + P.margin;
      const S pMax = dir_of(P.penaltyMax, dir);
      for (int k = 0; k < 3; k++) {
        if (!P.postStabilize) lam[k] = (lam[k] * P.alpha) * P.gamma;
        pen[k] = clampR(pen[k] * P.gamma, S(P.penaltyMin), pMax);
        set_dir(t.rA[k], rA[k], dir);
        set_dir(t.rB[k], rB[k], dir);
        set_dir(t.C0[k], C0[k], dir);
        set_dir(t.pen[k], pen[k], dir);
        set_dir(t.lam[k], lam[k], dir);
      }
      if (dir == 0) {
        t.feature = nc[i].feature;
        t.stick = stick;
      }
      if (P.cachedJacobians) {  // the orientations here are the step's x_t ones
        S jc[18];
        contact_jacobians(jc, basis, qA, qB, rA, rB);
        R *out = &w.jac[((size_t)c * K8 + i) * 18];
        for (int q = 0; q < 18; q++) set_dir(out[q], jc[q], dir);
      }
    }
  }
}

// Joint.initialize (joint.js:131-160) and Spring.initialize (spring.js:472-507).
template <class S>
__device__ void joint_eval_lin(const TWorld &w, const TJoint &j, S *out, int dir = 0) {
  S pA[3], pB[3], p[3], q[4], r[3];
  ldn(r, j.rA, 3, dir);
  if (j.a >= 0) {
    body_pose(w, j.a, p, q, dir);
    transform_point(pA, p, q, r);
  } else {
    pA[0] = r[0]; pA[1] = r[1]; pA[2] = r[2];
  }
  ldn(r, j.rB, 3, dir);
  body_pose(w, j.b, p, q, dir);
  transform_point(pB, p, q, r);
  v3_sub(out, pA, pB);
}
template <class S>
__device__ void joint_eval_ang(const TWorld &w, const TJoint &j, S *out, int dir = 0) {
  S qA[4] = {S(0.0), S(0.0), S(0.0), S(1.0)}, qB[4];
  if (j.a >= 0) ldn(qA, w.b[j.a].q, 4, dir);
  ldn(qB, w.b[j.b].q, 4, dir);
  q_subtract(out, qA, qB);
  for (int k = 0; k < 3; k++) out[k] = out[k] * j.torqueArm;
}
// the same during the iterations, with body b's inverse kept beside its q
template <class S>
__device__ void joint_eval_ang_iter(const TWorld &w, const TJoint &j, S *out, int dir) {
  S qA[4] = {S(0.0), S(0.0), S(0.0), S(1.0)}, qBi[4];
  if (j.a >= 0) ldn(qA, w.b[j.a].q, 4, dir);
  ldn(qBi, w.b[j.b].qi, 4, dir);
  q_mul_inv(out, qA, qBi);  // q_subtract(out, qA, qB)
  for (int k = 0; k < 3; k++) out[k] = out[k] * j.torqueArm;
}
// spring.js:447-458: C = |d| - rest, n = d / |d| (NaN C when |d| <= 1e-6)
// (rW: if given, the rotated anchor of end `side`)
template <class S>
__device__ S spring_eval(const TWorld &w, const TSpring &s, S *d, S *n, int dir = 0, int side = 0,
                         S *rW = nullptr) {
  S pA[3], pB[3], p[3], q[4], r[3];
  ldn(r, s.rA, 3, dir);
  body_pose(w, s.a, p, q, dir);
  q_rotate(pA, q, r);
  if (rW && side == 0)
    for (int k = 0; k < 3; k++) rW[k] = pA[k];
  for (int k = 0; k < 3; k++) pA[k] += p[k];
  ldn(r, s.rB, 3, dir);
  body_pose(w, s.b, p, q, dir);
  q_rotate(pB, q, r);
  if (rW && side == 1)
    for (int k = 0; k < 3; k++) rW[k] = pB[k];
  for (int k = 0; k < 3; k++) pB[k] += p[k];
  v3_sub(d, pA, pB);
  const S len = sqrt(v3_len_sq(d));
  if (len <= 1.0e-6) return S(NAN);
  for (int k = 0; k < 3; k++) n[k] = d[k] / len;
  return len - s.rest;
}

// The per-item kernels below run an item on a five-lane group, a tangent
// direction a lane: every lane reads the item, the group synchronises, and
// then each lane writes its direction (lane 0 the value parts and flags).
struct GroupLane {
  int dir, first, stride;
  unsigned mask;
  bool on;
  __device__ GroupLane() {
    const int lane = threadIdx.x & 31, slot = lane / kTangentDims;
    const int nWarps = gridDim.x * (blockDim.x >> 5), wg = blockIdx.x + gridDim.x * (threadIdx.x >> 5);
    dir = lane % kTangentDims;
    on = slot < kGroupsPerWarp;
    mask = on ? 0x1fu << (slot * kTangentDims) : 0u;
    first = slot * nWarps + wg;  // items over the warps (and SMs) first
    stride = nWarps * kGroupsPerWarp;
  }
};

// Joint.initialize (joint.js:131-160) and Spring.initialize (spring.js:472-507).
__global__ void forces_init_kernel(TWorld w) {
  using S = Dual1;
  const TParams &P = w.P;
  const GroupLane g;
  if (!g.on) return;
  const int k = g.dir;
  const S pMin(P.penaltyMin), pMax = dir_of(P.penaltyMax, k);
  for (int idx = g.first; idx < w.nj; idx += g.stride) {
    TJoint &j = w.j[idx];
    if (j.removed) continue;
    S C0L[3], C0A[3], lamL[3], lamA[3], penL[3], penA[3];
    joint_eval_lin(w, j, C0L, k);
    joint_eval_ang(w, j, C0A, k);
    ldn(lamL, j.lamLin, 3, k);
    ldn(lamA, j.lamAng, 3, k);
    ldn(penL, j.penLin, 3, k);
    ldn(penA, j.penAng, 3, k);
    const S stiffL = dir_of(j.stiffLin, k), stiffA = dir_of(j.stiffAng, k);
    const bool broken = j.broken != 0;
    __syncwarp(g.mask);
    for (int c = 0; c < 3; c++) {
      if (!P.postStabilize) {
        lamL[c] = (lamL[c] * P.alpha) * P.gamma;
        lamA[c] = (lamA[c] * P.alpha) * P.gamma;
      }
      penL[c] = js_min(clampR(penL[c] * P.gamma, pMin, pMax), stiffL);
      penA[c] = js_min(clampR(penA[c] * P.gamma, pMin, pMax), stiffA);
      set_dir(j.C0Lin[c], C0L[c], k);
      set_dir(j.C0Ang[c], C0A[c], k);
      set_dir(j.lamLin[c], lamL[c], k);
      set_dir(j.lamAng[c], lamA[c], k);
      set_dir(j.penLin[c], penL[c], k);
      set_dir(j.penAng[c], penA[c], k);
    }
    if (broken && k == 0) j.removed = 1;  // returns !broken: leaves the force list
  }
  for (int idx = g.first; idx < w.ns; idx += g.stride) {
    TSpring &sp = w.s[idx];
    const bool broken = sp.broken != 0;
    S penalty = dir_of(sp.penalty, k), peak = dir_of(sp.peak, k);
    const S stiffness = dir_of(sp.stiffness, k);
    bool torn = false;
    if (!broken && isfinite(sp.tear)) {
      S d[3], n[3];
      const S Cv = spring_eval(w, sp, d, n, k);
      if (!(Cv != Cv) && sp.rest > 1.0e-6) {  // the tear test (spring.js:461-470)
        const S strain = js_max(S(0.0), Cv / sp.rest);
        peak = js_max(peak, strain);
        torn = !(strain <= sp.tear);
      }
    }
    __syncwarp(g.mask);
    if (broken || torn) penalty = S(0.0);
    else if (!P.springRamp) penalty = stiffness;
    else penalty = js_min(clampR(penalty * P.gamma, pMin, pMax), stiffness);
    set_dir(sp.penalty, penalty, k);
    set_dir(sp.peak, peak, k);
    if (torn && k == 0) sp.broken = 1;
  }
}

// solver.js:366-401: y = x + v dt + g dt^2 (z), the adaptive initial guess.
__global__ void bodies_init_kernel(TWorld w) {
  using S = Dual1;
  const TParams &P = w.P;
  const double dt = P.dt;
  const GroupLane g;
  if (!g.on) return;
  const int k = g.dir;
  for (int i = g.first; i < w.n; i += g.stride) {
    TBody &b = w.b[i];
    const bool dyn = w.bs[i].mass > 0;
    S p[3], q[4], v[3], om[3];
    ldn(p, b.p, 3, k);
    ldn(q, b.q, 4, k);
    ldn(v, b.v, 3, k);
    ldn(om, b.w, 3, k);
    const S pv2 = dir_of(b.pv[2], k);
    __syncwarp(g.mask);
    const S gv[3] = {S(0.0), S(0.0), S(P.gravity)};
    S yl[3], yq[4], tmp[3];
    for (int c = 0; c < 3; c++) yl[c] = p[c];
    v3_add_scaled(yl, v, S(dt));
    if (dyn) v3_add_scaled(yl, gv, S(dt * dt));
    for (int c = 0; c < 3; c++) tmp[c] = om[c] * dt;
    q_integrate(yq, q, tmp);
    const S accelZ = (v[2] - pv2) / dt;
    const double sgn = P.gravity < 0 ? -1.0 : (P.gravity > 0 ? 1.0 : 0.0);
    const S accelExt = accelZ * sgn;
    S weight = clampR(accelExt / ::fabs(P.gravity), S(0.0), S(1.0));
    if (!isfinite(weight)) weight = 0.0;
    S p0[3], q0[4], q0i[4], yqi[4];
    for (int c = 0; c < 3; c++) p0[c] = p[c];
    for (int c = 0; c < 4; c++) q0[c] = q[c];
    q_inverse(q0i, q0);  // q_subtract's inverses of the step's constant quaternions
    q_inverse(yqi, yq);
    if (dyn) {
      v3_add_scaled(p, v, S(dt));
      v3_add_scaled(p, gv, weight * dt * dt);
      S q1[4];
      q_integrate(q1, q, tmp);
      for (int c = 0; c < 4; c++) q[c] = q1[c];
    }
    S dqL[3], dqA[3], qi[4];
    v3_sub(dqL, p, p0);
    q_subtract(dqA, q, q0);
    q_inverse(qi, q);
    for (int c = 0; c < 3; c++) {
      set_dir(b.yl[c], yl[c], k);
      set_dir(b.p0[c], p0[c], k);
      set_dir(b.p[c], p[c], k);
      set_dir(b.dqL[c], dqL[c], k);
      set_dir(b.dqA[c], dqA[c], k);
    }
    for (int c = 0; c < 4; c++) {
      set_dir(b.yq[c], yq[c], k);
      set_dir(b.q0[c], q0[c], k);
      set_dir(b.q0i[c], q0i[c], k);
      set_dir(b.yqi[c], yqi[c], k);
      set_dir(b.q[c], q[c], k);
      set_dir(b.qi[c], qi[c], k);
    }
  }
}

// ---------------------------------------------------------------------------
// Adjacency, colouring (single block)
// ---------------------------------------------------------------------------
// The forces of the step after initialisation (solver.js:346-360): live
// manifolds, joints that did not leave, every spring (a broken one stays and
// does nothing). Per dynamic body its list of (type, index, side).
// Slot g of the force list - the manifolds with contacts, then the live
// joints, then every spring - or false for a slot that holds no force;
// base: the force's reference without its side bit.
__device__ bool force_at(const TWorld &w, int total, int g, uint32_t &base, int &a, int &b) {
  if (g < total) {
    const TManifold &m = w.cur[g];
    if (m.count <= 0) return false;
    base = (uint32_t)g << 1;
    a = m.a;
    b = m.b;
    return true;
  }
  g -= total;
  if (g < w.nj) {
    const TJoint &j = w.j[g];
    if (j.removed) return false;
    base = (kRefJoint << 30) | ((uint32_t)g << 1);
    a = j.a;
    b = j.b;
    return true;
  }
  g -= w.nj;
  const TSpring &sp = w.s[g];
  base = (kRefSpring << 30) | ((uint32_t)g << 1);
  a = sp.a;
  b = sp.b;
  return true;
}

// Exclusive prefix sum of cnt[0, n) into start[0, n] by one block, in
// chunks of its threads (Hillis-Steele in shared memory).
__device__ void block_exclusive_scan(const int *cnt, int *start, int n, int *scan, int &carry) {
  const int t = threadIdx.x, bd = blockDim.x;
  if (t == 0) carry = 0;
  for (int base = 0; base < n; base += bd) {
    __syncthreads();
    const int i = base + t, v = i < n ? cnt[i] : 0;
    scan[t] = v;
    __syncthreads();
    for (int off = 1; off < bd; off <<= 1) {
      const int x = t >= off ? scan[t - off] : 0;
      __syncthreads();
      scan[t] += x;
      __syncthreads();
    }
    if (i < n) start[i] = carry + scan[t] - v;
    __syncthreads();
    if (t == bd - 1) carry += scan[t];
  }
  __syncthreads();
  if (t == 0) start[n] = carry;
  __syncthreads();
}

// The integer-priority greedy colouring (statics -1), computed as the fixed
// point of Jacobi rounds (the CUDA step's colouring; the oracle's
// priority_coloring); colour edges: forces between two dynamic bodies,
// broken ones excluded (oracle constraint_edges). One block: the per-body
// force lists are filled stably (force-list order) a chunk of forces at a
// time, each force's rank among its chunk's earlier forces on the same body
// counted in shared memory; the (colour, index) order likewise.
__global__ void __launch_bounds__(kBlock) adjacency_coloring_kernel(TWorld w) {
  const int n = w.n, total = w.ctl[0], nForces = total + w.nj + w.ns;
  const int t = threadIdx.x, bd = blockDim.x;
  __shared__ int scan[kBlock], ea[kBlock], eb[kBlock], carry;
  __shared__ int colorCount[kMaxColors], colorRun[kMaxColors], numColors, changed;
  for (int i = t; i <= n; i += bd) w.fCount[i] = 0;
  __syncthreads();
  for (int g = t; g < nForces; g += bd) {  // forces per body
    uint32_t fb;
    int a, b;
    if (!force_at(w, total, g, fb, a, b)) continue;
    if (a >= 0 && w.bs[a].mass > 0) atomicAdd(&w.fCount[a], 1);
    if (w.bs[b].mass > 0) atomicAdd(&w.fCount[b], 1);
  }
  __syncthreads();
  block_exclusive_scan(w.fCount, w.fStart, n, scan, carry);
  for (int i = t; i < n; i += bd) w.fCount[i] = 0;  // now the forces placed so far
  if (t == 0 && w.fStart[n] > w.fcap) w.ctl[2] = 1;
  __syncthreads();
  if (w.ctl[2]) return;
  for (int base = 0; base < nForces; base += bd) {
    const int g = base + t;
    uint32_t fb = 0;
    int a = -1, b = -1;
    const bool has = g < nForces && force_at(w, total, g, fb, a, b);
    const int xa = has && a >= 0 && w.bs[a].mass > 0 ? a : -1;
    const int xb = has && w.bs[b].mass > 0 ? b : -1;
    ea[t] = xa;
    eb[t] = xb;
    __syncthreads();
    int ra = 0, rb = 0;  // earlier forces of the chunk on the same body
    for (int k = 0; k < t; k++) {
      const int pa = ea[k], pb = eb[k];
      ra += xa >= 0 && (pa == xa || pb == xa);
      rb += xb >= 0 && (pa == xb || pb == xb);
    }
    if (xa >= 0) w.fRef[w.fStart[xa] + w.fCount[xa] + ra] = fb | 0u;
    if (xb >= 0) w.fRef[w.fStart[xb] + w.fCount[xb] + rb] = fb | 1u;
    __syncthreads();
    if (xa >= 0) atomicAdd(&w.fCount[xa], 1);
    if (xb >= 0) atomicAdd(&w.fCount[xb], 1);
    __syncthreads();
  }
  for (int i = t; i < n; i += bd) w.color[i] = is_dynamic(w, i) ? 0 : -1;
  for (int round = 0; round < 4096; round++) {
    __syncthreads();
    if (t == 0) changed = 0;
    __syncthreads();
    for (int i = t; i < n; i += bd) {
      if (!is_dynamic(w, i)) continue;
      const uint32_t pi = w.prio[i];
      int c = -1;
      for (int base = 0; c < 0 && base < kMaxColors; base += 64) {
        unsigned long long used = 0ull;
        for (int e = w.fStart[i]; e < w.fStart[i + 1]; e++) {
          const uint32_t ref = w.fRef[e];
          const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
          int a, b;
          bool broken = false;
          if (type == 0) { a = w.cur[idx].a; b = w.cur[idx].b; }
          else if (type == kRefJoint) { a = w.j[idx].a; b = w.j[idx].b; }
          else { a = w.s[idx].a; b = w.s[idx].b; broken = w.s[idx].broken != 0; }
          const int o = side ? a : b;
          if (broken || !is_dynamic(w, o)) continue;
          const uint32_t po = w.prio[o];
          if (!(po < pi || (po == pi && o < i))) continue;
          const int co = w.color[o];
          if (co >= base && co < base + 64) used |= 1ull << (co - base);
        }
        if (~used) c = base + __ffsll((long long)~used) - 1;
      }
      if (c < 0) c = kMaxColors - 1;
      if (c != w.color[i]) {
        w.color[i] = c;
        changed = 1;
      }
    }
    __syncthreads();
    if (!changed) break;
  }
  // bodies in (colour, index) order
  for (int c = t; c < kMaxColors; c += bd) colorCount[c] = colorRun[c] = 0;
  if (t == 0) numColors = 0;
  __syncthreads();
  for (int i = t; i < n; i += bd) {
    const int c = w.color[i];
    if (c < 0) continue;
    atomicAdd(&colorCount[c], 1);
    atomicMax(&numColors, c + 1);
  }
  __syncthreads();
  block_exclusive_scan(colorCount, w.colorStart, numColors, scan, carry);
  for (int base = 0; base < n; base += bd) {
    const int i = base + t, c = i < n ? w.color[i] : -1;
    ea[t] = c;
    __syncthreads();
    if (c >= 0) {
      int r = 0;
      for (int k = 0; k < t; k++) r += ea[k] == c;
      w.order[w.colorStart[c] + colorRun[c] + r] = i;
    }
    __syncthreads();
    if (c >= 0) atomicAdd(&colorRun[c], 1);
    __syncthreads();
  }
  if (t == 0) w.ctl[3] = numColors;
}

// ---------------------------------------------------------------------------
// Primal (solver.js:418-458) and dual (solver.js:466-470) of one iteration
// ---------------------------------------------------------------------------
// Manifold._evaluate (manifold.js:358-409) of contact i with cached
// Jacobians from the x_t orientations: C = (1 - alpha) C0 + J (x - x_t).
// Computed in S by tangent direction dir (S = R: every direction).
template <class S>
struct ContactEvalT {
  S C[3], F[3];
  bool within;
};
template <class S>
__device__ ContactEvalT<S> contact_eval(const TWorld &w, const TManifold &m, int i, R alpha, S *basis, S *jAAng,
                                        S *jBAng, int dir = 0) {
  const TBody &A = w.b[m.a], &B = w.b[m.b];
  const TContact &c = m.c[i];
  // the bodies' displacements from x_t, kept with their iterates
  S dqALin[3], dqAAng[3], dqBLin[3], dqBAng[3];
  ldn(dqALin, A.dqL, 3, dir);
  ldn(dqAAng, A.dqA, 3, dir);
  ldn(dqBLin, B.dqL, 3, dir);
  ldn(dqBAng, B.dqA, 3, dir);
  ldn(basis, m.basis, 9, dir);
  S jBLin[9], acc[3];
  for (int k = 0; k < 9; k++) jBLin[k] = -basis[k];
  if (w.P.cachedJacobians) {  // computed once per step at the x_t orientations (narrow_kernel)
    const R *jc = &w.jac[((size_t)(&m - w.cur) * K8 + i) * 18];
    ldn(jAAng, jc, 9, dir);
    ldn(jBAng, jc + 9, 9, dir);
  } else {
    S jc[18], qA[4], qB[4], rA[3], rB[3];
    ldn(qA, A.q, 4, dir);
    ldn(qB, B.q, 4, dir);
    ldn(rA, c.rA, 3, dir);
    ldn(rB, c.rB, 3, dir);
    contact_jacobians(jc, basis, qA, qB, rA, rB);
    for (int k = 0; k < 9; k++) {
      jAAng[k] = jc[k];
      jBAng[k] = jc[9 + k];
    }
  }
  ContactEvalT<S> e;
  const S keep = 1.0 - ld<S>(alpha, dir);
  for (int k = 0; k < 3; k++) e.C[k] = ld<S>(c.C0[k], dir) * keep;
  m3_mul_vec(acc, basis, dqALin); v3_add(e.C, e.C, acc);
  m3_mul_vec(acc, jBLin, dqBLin); v3_add(e.C, e.C, acc);
  m3_mul_vec(acc, jAAng, dqAAng); v3_add(e.C, e.C, acc);
  m3_mul_vec(acc, jBAng, dqBAng); v3_add(e.C, e.C, acc);
  for (int k = 0; k < 3; k++) e.F[k] = ld<S>(c.pen[k], dir) * e.C[k] + ld<S>(c.lam[k], dir);
  e.F[0] = js_min(e.F[0], S(0.0));
  const S bounds = fabs(e.F[0]) * ld<S>(m.friction, dir);
  const S fs = sqrt(e.F[1] * e.F[1] + e.F[2] * e.F[2]);
  if (fs > bounds && fs > 0.0) {
    e.F[1] *= bounds / fs;
    e.F[2] *= bounds / fs;
  }
  e.within = fs <= bounds;
  return e;
}

// H += J_lin^T K J_lin etc. of one 3-row block with diagonal K: entry (r, c)
// is sum_k (J[k][r] K[k]) J[k][c] over k = 0, 1, 2 in order, the terms of
// transpose, column scale and 3x3 product, and f += J^T F likewise.
template <class S, class Sink>
__device__ void stamp_rows(Sink &s, const S *jLin, const S *jAng, const S *Kd, const S *F) {
  for (int r = 0; r < 3; r++) {
    const S l0 = jLin[r] * Kd[0], l1 = jLin[3 + r] * Kd[1], l2 = jLin[6 + r] * Kd[2];
    const S a0 = jAng[r] * Kd[0], a1 = jAng[3 + r] * Kd[1], a2 = jAng[6 + r] * Kd[2];
    for (int c = 0; c < 3; c++) {
      s.lin[r * 3 + c] += l0 * jLin[c] + l1 * jLin[3 + c] + l2 * jLin[6 + c];
      s.ang[r * 3 + c] += a0 * jAng[c] + a1 * jAng[3 + c] + a2 * jAng[6 + c];
      s.cross[r * 3 + c] += a0 * jLin[c] + a1 * jLin[3 + c] + a2 * jLin[6 + c];
    }
  }
  for (int r = 0; r < 3; r++) {
    s.bl[r] += jLin[r] * F[0] + jLin[3 + r] * F[1] + jLin[6 + r] * F[2];
    s.ba[r] += jAng[r] * F[0] + jAng[3 + r] * F[1] + jAng[6 + r] * F[2];
  }
}

// stamp_rows for a ball socket's rows, J_lin = sgn I and J_ang = the skew J
// (zero diagonal): each entry's nonzero terms in stamp_rows's order and no
// products with the zeros and ones (the sums lose only exact zero terms, so
// the values are stamp_rows's); every entry still gets its one addend.
template <class S, class Sink>
__device__ void stamp_joint_rows(Sink &s, double sgn, const S *J, const S *Kd, const S *F) {
  const S one(sgn), zero(0.0);
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      s.lin[r * 3 + c] += r == c ? (one * Kd[r]) * one : zero;
      if (r == c) {
        const int k1 = r == 0 ? 1 : 0, k2 = r == 2 ? 1 : 2;
        s.ang[r * 3 + c] += (J[k1 * 3 + r] * Kd[k1]) * J[k1 * 3 + c] + (J[k2 * 3 + r] * Kd[k2]) * J[k2 * 3 + c];
      } else {
        const int k = 3 - r - c;
        s.ang[r * 3 + c] += (J[k * 3 + r] * Kd[k]) * J[k * 3 + c];
      }
      s.cross[r * 3 + c] += (J[c * 3 + r] * Kd[c]) * one;
    }
  for (int r = 0; r < 3; r++) {
    const int k1 = r == 0 ? 1 : 0, k2 = r == 2 ? 1 : 2;
    s.bl[r] += one * F[r];
    s.ba[r] += J[k1 * 3 + r] * F[k1] + J[k2 * 3 + r] * F[k2];
  }
}

// manifold.js:411-445, contact i of the manifold
template <class S, class Sink>
__device__ void contact_primal(const TWorld &w, const TManifold &m, int i, int side, R alpha, Sink &s, int dir) {
  S basis[9], jAAng[9], jBAng[9], pen[3];
  const ContactEvalT<S> e = contact_eval(w, m, i, alpha, basis, jAAng, jBAng, dir);
  for (int k = 0; k < 9; k++) {  // body B's rows: -basis and its angular Jacobian
    if (side) basis[k] = -basis[k];
    jAAng[k] = side ? jBAng[k] : jAAng[k];
  }
  ldn(pen, m.c[i].pen, 3, dir);
  stamp_rows(s, basis, jAAng, pen, e.F);
}

// joint.js:214-221: the geometric stiffness of a ball socket, lumped
template <class S>
__device__ void ball_socket_geometric(S *G, const S *r, const S *F) {
  S H[9];
  m3_zero(H);
  for (int k = 0; k < 3; k++) {  // geometricStiffnessBallSocket(v = r, k) * F[k]
    S g[9];
    m3_diag(g, -r[k], -r[k], -r[k]);
    g[0 * 3 + k] += r[0];
    g[1 * 3 + k] += r[1];
    g[2 * 3 + k] += r[2];
    for (int q = 0; q < 9; q++) H[q] += g[q] * F[k];
  }
  const S c0 = sqrt(H[0] * H[0] + H[3] * H[3] + H[6] * H[6]);
  const S c1 = sqrt(H[1] * H[1] + H[4] * H[4] + H[7] * H[7]);
  const S c2 = sqrt(H[2] * H[2] + H[5] * H[5] + H[8] * H[8]);
  m3_diag(G, c0, c1, c2);
}

// the value of |x|^2 > 0 (the branch tests of the joint's rows)
__device__ __forceinline__ bool nonzero3(const R *x) {
  return x[0].v * x[0].v + x[1].v * x[1].v + x[2].v * x[2].v > 0.0;
}

// joint.js:162-253
template <class S, class Sink>
__device__ void joint_primal(const TWorld &w, const TJoint &j, int side, R alpha, Sink &s, int dir) {
  S C[3], F[3], pen[3];
  if (nonzero3(j.penLin)) {
    // joint_eval_lin, keeping the rotated anchors (the rows' lever arms)
    S rAW[3], rBW[3], pA[3], pB[3], p[3], q[4], rl[3];
    ldn(rl, j.rA, 3, dir);
    if (j.a >= 0) {
      body_pose(w, j.a, p, q, dir);
      q_rotate(rAW, q, rl);
      for (int k = 0; k < 3; k++) pA[k] = rAW[k] + p[k];
    } else {
      for (int k = 0; k < 3; k++) pA[k] = rl[k];
    }
    ldn(rl, j.rB, 3, dir);
    body_pose(w, j.b, p, q, dir);
    q_rotate(rBW, q, rl);
    for (int k = 0; k < 3; k++) pB[k] = rBW[k] + p[k];
    v3_sub(C, pA, pB);
    if (j.stiffLin.v == INFINITY) {
      const S na = -ld<S>(alpha, dir);
      for (int k = 0; k < 3; k++) C[k] = C[k] + ld<S>(j.C0Lin[k], dir) * na;
    }
    ldn(pen, j.penLin, 3, dir);
    for (int k = 0; k < 3; k++) F[k] = pen[k] * C[k] + ld<S>(j.lamLin[k], dir);
    S jAng[9], r[3];  // J_lin = I (body a) or -I (body b)
    if (!side) {  // body a (j.a >= 0)
      for (int k = 0; k < 3; k++) r[k] = -rAW[k];
      m3_skew(jAng, r);
      for (int k = 0; k < 3; k++) r[k] = rAW[k];
    } else {
      m3_skew(jAng, rBW);
      for (int k = 0; k < 3; k++) r[k] = -rBW[k];
    }
    stamp_joint_rows(s, side ? -1.0 : 1.0, jAng, pen, F);
    S G[9];
    ball_socket_geometric(G, r, F);
    m3_add_into(s.ang, G);
  }
  if (nonzero3(j.penAng)) {
    joint_eval_ang_iter(w, j, C, dir);
    if (j.stiffAng.v == INFINITY) {
      const S na = -ld<S>(alpha, dir);
      for (int k = 0; k < 3; k++) C[k] = C[k] + ld<S>(j.C0Ang[k], dir) * na;
    }
    ldn(pen, j.penAng, 3, dir);
    for (int k = 0; k < 3; k++) F[k] = pen[k] * C[k] + ld<S>(j.lamAng[k], dir);
    const double sg = side ? -j.torqueArm : j.torqueArm;
    // jAng = sg I: H_ang += sg K sg, f_ang += sg F
    for (int k = 0; k < 3; k++) {
      s.ang[k * 3 + k] += (sg * pen[k]) * sg;
      s.ba[k] += F[k] * sg;
    }
  }
}

// spring.js:509-616
template <class S, class Sink>
__device__ void spring_primal(const TWorld &w, const TSpring &sp, int side, Sink &s, const TParams &P, int dir) {
  if (sp.broken) return;
  S d[3], n[3], rW[3];
  const S Cv = spring_eval(w, sp, d, n, dir, side, rW);
  if (Cv != Cv) return;
  const S k = ld<S>(sp.penalty, dir);
  const S f = k * Cv;
  S jLin[3], jAng[3];
  if (!side) {
    for (int c = 0; c < 3; c++) jLin[c] = n[c];
    v3_cross(jAng, rW, n);
  } else {
    for (int c = 0; c < 3; c++) jLin[c] = -n[c];
    v3_cross(jAng, rW, n);
    for (int c = 0; c < 3; c++) jAng[c] = -jAng[c];
  }
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      s.lin[r * 3 + c] += (jLin[r] * jLin[c]) * k;
      s.ang[r * 3 + c] += (jAng[r] * jAng[c]) * k;
      s.cross[r * 3 + c] += (jAng[r] * jLin[c]) * k;
    }
  v3_add_scaled(s.bl, jLin, f);
  v3_add_scaled(s.ba, jAng, f);
  if (!P.springGeometric) return;
  const S dLen = sqrt(v3_len_sq(d));
  const double sg = side ? -1.0 : 1.0;
  S Pm[9], Sk[9], Gla[9], Gal[9], Gaa[9], m0[9];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) Pm[r * 3 + c] = -(n[r] * n[c]);
  Pm[0] = Pm[0] + 1.0; Pm[4] = Pm[4] + 1.0; Pm[8] = Pm[8] + 1.0;
  for (int q = 0; q < 9; q++) Pm[q] = Pm[q] / dLen;
  m3_skew(Sk, rW);
  m3_mul(Gla, Pm, Sk);
  for (int q = 0; q < 9; q++) Gla[q] = -Gla[q];
  m3_mul(Gal, Sk, Pm);
  m3_mul(Gaa, Sk, Pm);
  m3_mul(Gaa, Gaa, Sk);
  for (int q = 0; q < 9; q++) Gaa[q] = -Gaa[q];
  const S ndotr = v3_dot(n, rW);
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) m0[r * 3 + c] = rW[r] * n[c];
  m0[0] = m0[0] - ndotr; m0[4] = m0[4] - ndotr; m0[8] = m0[8] - ndotr;
  for (int q = 0; q < 9; q++) Gaa[q] += m0[q] * sg;
  const S af = fabs(f);
  for (int c = 0; c < 3; c++) {
    const S a0 = Pm[c], a1 = Pm[3 + c], a2 = Pm[6 + c], a3 = Gal[c], a4 = Gal[3 + c], a5 = Gal[6 + c];
    s.lin[c * 3 + c] += sqrt(a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5) * af;
  }
  for (int c = 0; c < 3; c++) {
    const S a0 = Gla[c], a1 = Gla[3 + c], a2 = Gla[6 + c], a3 = Gaa[c], a4 = Gaa[3 + c], a5 = Gaa[6 + c];
    s.ang[c * 3 + c] += sqrt(a0 * a0 + a1 * a1 + a2 * a2 + a3 * a3 + a4 * a4 + a5 * a5) * af;
  }
}

// One body's update (solver.js:425-457) by one block of kBodyThreads. The
// body's constraint rows - each contact of each manifold, each joint, each
// spring, newest force first - go to the threads up to kRowsPerPass at a
// time, five threads per row (one per tangent direction, each also
// computing the value). A warp holds six such groups, and the rows of one
// kind (contact, joint, spring) start on a warp of their own: a warp's
// threads then follow one instruction stream, and the kinds run side by
// side on the SM's sub-partitions (an FP64 instruction costs the same
// however few of its lanes are active). Every thread records its
// direction of the addends its row makes to each of the 33 system entries
// (RecSys6), and then each double of each entry (its value or one
// derivative) is summed by one thread row after row in force order: every
// entry is summed in the f64 engine's order, so the values stay the serial
// update's. The inertial terms (the entries' first values) were formed in
// the phase before (inertial_terms).
constexpr int kBodyThreads = 256;  // two warps per SM sub-partition: 255 registers a thread
constexpr int kRowsPerPass = kBodyThreads / 32 * kGroupsPerWarp;
constexpr int kDualDoubles = kTangentDims + 1;
static_assert(kGroupsPerWarp * kTangentDims <= 32, "a row's five threads in one warp");
static_assert(sizeof(R) == kDualDoubles * sizeof(double), "a dual number is its value and its derivatives");
struct BodySmem {
  R rec[kRowsPerPass][kRecSlots];                                 // a row's addends per entry
  unsigned char cnt[kRowsPerPass * kTangentDims][kSysEntries + 3];  // a (row, direction)'s addends per entry
  R acc[kSysEntries];                                             // the entries, summed so far
  uint32_t items[kRowsPerPass];                                   // (force entry << 3) | contact, force order
  signed char groupRow[kRowsPerPass];                             // the row of a thread group, or -1
  Dual1 ldl[kTangentDims][6][6];                                  // L of the 6x6 solve, per direction
  int nItems, cursorE, cursorC;
};

__device__ __forceinline__ int round_up_groups(int g) { return (g + kGroupsPerWarp - 1) / kGroupsPerWarp * kGroupsPerWarp; }

// The next rows of body i's force list, from the cursor: as many as fit the
// groups with each kind starting on a warp boundary.
__device__ void next_rows(const TWorld &w, int i, BodySmem &sm) {
  int n = 0, e = sm.cursorE, c = sm.cursorC, per[3] = {0, 0, 0};
  const int e0 = w.fStart[i];
  while (e >= e0) {
    const uint32_t ref = w.fRef[e];
    const int kind = (ref >> 30) == 0 ? 0 : ((ref >> 30) == kRefJoint ? 1 : 2);
    if (kind == 0 && c >= w.cur[(ref >> 1) & 0x1fffffffu].count) {  // the manifold's contacts are done
      e--;
      c = 0;
      continue;
    }
    per[kind]++;
    if (round_up_groups(per[0]) + round_up_groups(per[1]) + per[2] > kRowsPerPass) {
      per[kind]--;
      break;
    }
    if (kind == 0) {
      sm.items[n++] = ((uint32_t)e << 3) | (uint32_t)c;
      c++;
    } else {
      sm.items[n++] = (uint32_t)e << 3;
      e--;
      c = 0;
    }
  }
  // contacts from group 0, joints and springs each from the next warp
  int at[3] = {0, round_up_groups(per[0]), round_up_groups(per[0]) + round_up_groups(per[1])};
  for (int g = 0; g < kRowsPerPass; g++) sm.groupRow[g] = -1;
  for (int r = 0; r < n; r++) {
    const uint32_t ref = w.fRef[sm.items[r] >> 3];
    const int kind = (ref >> 30) == 0 ? 0 : ((ref >> 30) == kRefJoint ? 1 : 2);
    const int g = at[kind]++;
    sm.groupRow[g] = (signed char)r;
  }
  sm.nItems = n;
  sm.cursorE = e;
  sm.cursorC = c;
}

// The lanes of the six-lane row groups: 30 of warp 0's lanes, one row of
// the 6x6 system and one tangent direction each.
constexpr unsigned kSolveLanes = 0x3fffffffu;
static_assert(kTangentDims * 6 <= 32, "the row groups fit one warp");
__device__ __forceinline__ Dual1 shfl_dual(const Dual1 &a, int src) {
  Dual1 o(__shfl_sync(kSolveLanes, a.v, src));
  o.d[0] = __shfl_sync(kSolveLanes, a.d[0], src);
  return o;
}

// a[i] of four values, i in [0, 4), by selects (no local memory)
__device__ __forceinline__ Dual1 pick4(const Dual1 *a, int i) {
  return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

// solve6 above spread over the six rows of the system: lane r of direction
// dir's group holds row r and forms L(r, j) as soon as D(j) is known, the
// rows' divisions of one column at once. Every L, D, y, z and x is formed by
// the same operations in the same order as in solve6 (the terms of a sum
// left to right, a product's factors commuting exactly), so the values are
// the serial solve's. acc: the 33 entries; returns x(r).
__device__ Dual1 solve6_lanes(const R *acc, int dir, int r, Dual1 (&Lsm)[6][6]) {
  using S = Dual1;
  const int base = dir * 6;
  S A[6], L[6], num[6];
  for (int c = 0; c < 6; c++) {  // A(r, c), c <= r: lin, then cross and ang below the diagonal
    const int e = r < 3 ? r * 3 + c : (c < 3 ? 18 + (r - 3) * 3 + c : 9 + (r - 3) * 3 + (c - 3));
    A[c] = c <= r ? dir_of(acc[e], dir) : S(0.0);
    L[c] = S(0.0);
    num[c] = A[c];
  }
  const S b = -(r < 3 ? dir_of(acc[27 + r], dir) : dir_of(acc[30 + (r - 3)], dir));  // -bl, -ba
  S D[6], dacc(0.0), Dr(0.0);
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const S Dj = j == 0 ? A[0] : A[j] - dacc;  // meaningful in lane j: D1 = A11, Dj = Ajj - (sum)
    if (r == j) Dr = Dj;
    D[j] = shfl_dual(Dj, base + j);
    if (r > j) L[j] = num[j] / D[j];
#pragma unroll
    for (int c = j + 1; c < 6; c++) {  // column j of L from the lanes below
      const S Lcj = shfl_dual(L[j], base + c);
      if (r > c) num[c] = num[c] - (Lcj * L[j]) * D[j];
    }
    if (r > j) dacc = j == 0 ? (L[0] * L[0]) * D[0] : dacc + (L[j] * L[j]) * D[j];
  }
  // forward substitution: y(r) = b(r) - L(r,0) y(0) - L(r,1) y(1) - ...
  S y = b;
#pragma unroll
  for (int j = 0; j < 5; j++) {
    const S yj = shfl_dual(y, base + j);
    if (r > j) y = y - L[j] * yj;
  }
  const S z = y / Dr;
  // back substitution: x(r) = z(r) - L(r+1,r) x(r+1) - L(r+2,r) x(r+2) - ...
  for (int c = 0; c < r; c++) Lsm[r][c] = L[c];
  __syncwarp(kSolveLanes);
  S x = z, xs[6];
#pragma unroll
  for (int c = 5; c > 0; c--) {
    xs[c] = shfl_dual(x, base + c);  // final: its lane finished in the round before
    if (r == c - 1)
      for (int m = c; m < 6; m++) x = x - Lsm[m][r] * xs[m];
  }
  return x;
}

// solver.js:425-433: the inertial terms M/dt^2 and M (x - y)/dt^2 of body
// i's system, tangent direction k, into its entries of w.inert (the value
// by direction 0).
__device__ void inertial_terms(const TWorld &w, int i, int k) {
  using S = Dual1;
  const TParams &P = w.P;
  const TBody &b = w.b[i];
  const TBodyStatic &st = w.bs[i];
  const double dt2 = P.dt * P.dt;
  S p[3], yl[3], q[4], yqi[4];
  for (int c = 0; c < 3; c++) {
    p[c] = dir_of(b.p[c], k);
    yl[c] = dir_of(b.yl[c], k);
  }
  for (int c = 0; c < 4; c++) {
    q[c] = dir_of(b.q[c], k);
    yqi[c] = dir_of(b.yqi[c], k);
  }
  Sys6T<S> s;
  S MAng[9], tmp[3], dq[3];
  m3_diag(s.lin, S(st.mass / dt2), S(st.mass / dt2), S(st.mass / dt2));
  world_moment(MAng, st, q, P.rotatedInertia != 0);
  for (int c = 0; c < 9; c++) s.ang[c] = MAng[c] / dt2;
  m3_zero(s.cross);
  v3_sub(tmp, p, yl);
  m3_mul_vec(s.bl, s.lin, tmp);
  q_mul_inv(dq, q, yqi);  // q_subtract(dq, q, yq)
  m3_mul_vec(s.ba, s.ang, dq);
  const S *e = &s.lin[0];
  R *o = &w.inert[(size_t)i * kSysEntries];
  for (int c = 0; c < kSysEntries; c++) {
    if (k == 0) o[c].v = e[c].v;
    o[c].d[k] = e[c].d[0];
  }
}

__device__ void body_update_block(const TWorld &w, int i, R alpha, BodySmem &sm) {
  const TParams &P = w.P;
  const int t = threadIdx.x, nt = blockDim.x;
  for (int q = t; q < kSysEntries * kDualDoubles; q += nt)  // the inertial terms, formed ahead
    reinterpret_cast<double *>(sm.acc)[q] = reinterpret_cast<const double *>(&w.inert[(size_t)i * kSysEntries])[q];
  if (t == 0) {
    sm.cursorE = w.fStart[i + 1] - 1;  // the body's forces, newest first
    sm.cursorC = 0;
    next_rows(w, i, sm);
  }
  __syncthreads();
  for (;;) {
    const int n = sm.nItems;
    if (n == 0) break;
    const int lane = t & 31, group = (t >> 5) * kGroupsPerWarp + lane / kTangentDims, dir = lane % kTangentDims;
    const int row = lane < kGroupsPerWarp * kTangentDims ? sm.groupRow[group] : -1;
    if (row >= 0) {
      unsigned char *cnt = sm.cnt[row * kTangentDims + dir];
      for (int k = 0; k < kSysEntries; k++) cnt[k] = 0;
      RecSys6 rs(sm.rec[row], cnt, dir);
      const uint32_t item = sm.items[row];
      const uint32_t ref = w.fRef[item >> 3];
      const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
      if (type == 0) contact_primal<Dual1>(w, w.cur[idx], (int)(item & 7u), (int)side, alpha, rs, dir);
      else if (type == kRefJoint) joint_primal<Dual1>(w, w.j[idx], (int)side, alpha, rs, dir);
      else spring_primal<Dual1>(w, w.s[idx], (int)side, rs, P, dir);
    }
    __syncwarp();  // each warp whole again (its lanes took different rows) before the block barrier
    __syncthreads();
    for (int q = t; q < kSysEntries * kDualDoubles; q += nt) {  // one double of one entry per thread
      const int entry = q / kDualDoubles, part = q % kDualDoubles;
      double *accp = reinterpret_cast<double *>(&sm.acc[entry]) + part;
      double a = *accp;
      const int cap = rec_cap(entry), off = rec_off(entry);
      for (int it = 0; it < n; it++) {
        const int k = sm.cnt[it * kTangentDims][entry];  // the same count in every direction
        if (k > cap) w.ctl[7] = 1;  // more addends than recorded: the result is not the serial sum
        const double *r = reinterpret_cast<const double *>(&sm.rec[it][off]) + part;
        for (int m = 0; m < k && m < cap; m++) a += r[m * kDualDoubles];
      }
      *accp = a;
    }
    if (t == nt - 1) next_rows(w, i, sm);  // the rows are recorded; the replay reads only rec and cnt
    __syncthreads();
  }
  if (t < kTangentDims * 6) {  // the 6x6 solve over six lanes a direction, then the update
    using S = Dual1;
    const int k = t / 6, r = t % 6;
    S x = solve6_lanes(sm.acc, k, r, sm.ldl[k]);
    // the update (solver.js:450-457), one component a lane: rows 0-2 the
    // position, 0-3 the orientation (q_integrate, then q_subtract against
    // q0 with its inverse formed at the step's start); each component by the
    // operations of the serial functions, a - b written a + (-b), which is
    // exact
    S xa[3];
    for (int c = 0; c < 3; c++) xa[c] = shfl_dual(x, k * 6 + 3 + c);
    TBody &b = w.b[i];
    const int c3 = r < 3 ? r : 0, c4 = r < 4 ? r : 0;
    S q[4], qi[4];
    for (int c = 0; c < 4; c++) {
      q[c] = dir_of(b.q[c], k);
      qi[c] = dir_of(b.q0i[c], k);
    }
    const S p = dir_of(b.p[c3], k), p0 = dir_of(b.p0[c3], k);
    __syncwarp(kSolveLanes);  // every lane has read the body before any writes it
    // q_integrate: p_c = 0 q_c + wx q_. + wy q_. + wz q_. (quaternion product
    // signs), r_c = q_c + p_c / 2, q1_c = r_c / |r|
    constexpr unsigned kIntIdx = (3u << 0) | (2u << 2) | (1u << 4) | (2u << 6) | (3u << 8) | (0u << 10) |
                                 (1u << 12) | (0u << 14) | (3u << 16) | (0u << 18) | (1u << 20) | (2u << 22);
    constexpr unsigned kIntNeg = (1u << 2) | (1u << 3) | (1u << 7) | (1u << 9) | (1u << 10) | (1u << 11);
    S pc = 0.0 * pick4(q, c4);
    for (int m = 0; m < 3; m++) {
      const int bit = 3 * c4 + m;
      const S wm = (kIntNeg >> bit) & 1u ? -xa[m] : xa[m];
      pc = pc + wm * pick4(q, (int)((kIntIdx >> (2 * bit)) & 3u));
    }
    const S rc = pick4(q, c4) + pc * 0.5;
    S rq[4];
    for (int m = 0; m < 4; m++) rq[m] = shfl_dual(rc, k * 6 + m);
    const S len = sqrt(rq[0] * rq[0] + rq[1] * rq[1] + rq[2] * rq[2] + rq[3] * rq[3]);
    const S q1 = rc / len;
    S a[4];  // q1 (x, y, z, w)
    for (int m = 0; m < 4; m++) a[m] = shfl_dual(q1, k * 6 + m);
    // q_subtract(q1, q0) = 2 (q1 * q0^-1).xyz: terms aw, ax, ay, az in order
    constexpr unsigned kSubIdx = (0u << 0) | (3u << 2) | (2u << 4) | (1u << 6) | (1u << 8) | (2u << 10) |
                                 (3u << 12) | (0u << 14) | (2u << 16) | (1u << 18) | (0u << 20) | (3u << 22);
    constexpr unsigned kSubNeg = (1u << 3) | (1u << 5) | (1u << 10);
    S dqa = a[3] * pick4(qi, (int)(kSubIdx >> (8 * c3)) & 3);
    for (int m = 1; m < 4; m++) {
      const int bit = 4 * c3 + m;
      const S am = (kSubNeg >> bit) & 1u ? -a[m - 1] : a[m - 1];
      dqa = dqa + am * pick4(qi, (int)((kSubIdx >> (2 * bit)) & 3u));
    }
    dqa = dqa * 2.0;
    if (r < 3) {
      const S pn = p + x;
      set_dir(b.p[r], pn, k);
      set_dir(b.dqL[r], pn - p0, k);
      set_dir(b.dqA[r], dqa, k);
    }
    if (r < 4) {
      const S lsq = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3];  // q_inverse of q1
      set_dir(b.q[r], q1, k);
      set_dir(b.qi[r], (r < 3 ? -pick4(a, r) : a[3]) / lsq, k);
    }
  }
  __syncthreads();
}

// The dual updates, one tangent direction per thread of a five-lane group
// (mask: the group's lanes). Every thread reads the force, the group
// synchronises, and then each thread writes its direction (direction 0 the
// value and the flags), so that no read sees a half-written dual number.
// manifold.js:447-491, contact i of the manifold (the contacts' dual updates
// are independent of one another)
__device__ void contact_dual_dir(const TWorld &w, TManifold &m, int i, R alpha, int dir, unsigned mask) {
  using S = Dual1;
  const TParams &P = w.P;
  const bool sphere = w.bs[m.a].shape == AVBD_SHAPE_SPHERE || w.bs[m.b].shape == AVBD_SHAPE_SPHERE;
  S basis[9], jAAng[9], jBAng[9], pen[3];
  const ContactEvalT<S> e = contact_eval(w, m, i, alpha, basis, jAAng, jBAng, dir);
  TContact &c = m.c[i];
  ldn(pen, c.pen, 3, dir);
  const S pMax = ld<S>(P.penaltyMax, dir);
  int stick = c.stick;
  if (e.F[0] < 0.0) pen[0] = js_min(pen[0] + P.betaLin * fabs(e.C[0]), pMax);
  if (e.within) {
    pen[1] = js_min(pen[1] + P.betaLin * fabs(e.C[1]), pMax);
    pen[2] = js_min(pen[2] + P.betaLin * fabs(e.C[2]), pMax);
    stick = sqrt(e.C[1] * e.C[1] + e.C[2] * e.C[2]) < P.stickThreshold ? 1 : 0;
  } else if (sphere) {
    stick = 0;
  }
  __syncwarp(mask);
  for (int k = 0; k < 3; k++) {
    set_dir(c.lam[k], e.F[k], dir);
    set_dir(c.pen[k], pen[k], dir);
  }
  if (dir == 0) c.stick = stick;
}

// joint.js:255-317
__device__ void joint_dual_dir(const TWorld &w, TJoint &j, R alpha, int dir, unsigned mask) {
  using S = Dual1;
  const TParams &P = w.P;
  S C[3], penL[3], penA[3], lamL[3], lamA[3];
  ldn(penL, j.penLin, 3, dir);
  ldn(penA, j.penAng, 3, dir);
  ldn(lamL, j.lamLin, 3, dir);
  ldn(lamA, j.lamAng, 3, dir);
  const S pMax = ld<S>(P.penaltyMax, dir);
  if (nonzero3(j.penLin)) {
    joint_eval_lin(w, j, C, dir);
    if (j.stiffLin.v == INFINITY) {
      const S na = -ld<S>(alpha, dir);
      for (int k = 0; k < 3; k++) C[k] = C[k] + ld<S>(j.C0Lin[k], dir) * na;
      for (int k = 0; k < 3; k++) lamL[k] = penL[k] * C[k] + lamL[k];
    }
    const S cap = js_min(ld<S>(j.stiffLin, dir), pMax);
    for (int k = 0; k < 3; k++) penL[k] = js_min(penL[k] + fabs(C[k]) * P.betaLin, cap);
  }
  if (nonzero3(j.penAng)) {
    joint_eval_ang_iter(w, j, C, dir);
    if (j.stiffAng.v == INFINITY) {
      const S na = -ld<S>(alpha, dir);
      for (int k = 0; k < 3; k++) C[k] = C[k] + ld<S>(j.C0Ang[k], dir) * na;
      for (int k = 0; k < 3; k++) lamA[k] = penA[k] * C[k] + lamA[k];
    }
    const S cap = js_min(ld<S>(j.stiffAng, dir), pMax);
    for (int k = 0; k < 3; k++) penA[k] = js_min(penA[k] + fabs(C[k]) * P.betaAng, cap);
  }
  const bool broken = v3_len_sq(lamA) > j.fracture * j.fracture;
  if (broken)
    for (int k = 0; k < 3; k++) penL[k] = penA[k] = lamL[k] = lamA[k] = S(0.0);
  __syncwarp(mask);
  for (int k = 0; k < 3; k++) {
    set_dir(j.penLin[k], penL[k], dir);
    set_dir(j.penAng[k], penA[k], dir);
    set_dir(j.lamLin[k], lamL[k], dir);
    set_dir(j.lamAng[k], lamA[k], dir);
  }
  if (broken && dir == 0) j.broken = 1;
}

// spring.js:618-634 (the tear test of spring.js:461-470 inline)
__device__ void spring_dual_dir(const TWorld &w, TSpring &s, int dir, unsigned mask) {
  using S = Dual1;
  if (s.broken) return;
  S d[3], n[3];
  const S Cv = spring_eval(w, s, d, n, dir);
  if (Cv != Cv) return;
  S peak = ld<S>(s.peak, dir), penalty = ld<S>(s.penalty, dir);
  bool torn = false;
  if (isfinite(s.tear) && s.rest > 1.0e-6) {  // the tear test (spring.js:461-470)
    const S strain = js_max(S(0.0), Cv / s.rest);
    peak = js_max(peak, strain);
    if (!(strain <= s.tear)) {
      torn = true;
      penalty = S(0.0);
    }
  }
  if (!torn && w.P.springRamp)
    penalty = js_min(penalty + fabs(Cv) * w.P.betaLin, js_min(ld<S>(s.stiffness, dir), ld<S>(w.P.penaltyMax, dir)));
  __syncwarp(mask);
  set_dir(s.peak, peak, dir);
  set_dir(s.penalty, penalty, dir);
  if (torn && dir == 0) s.broken = 1;
}

// Bounded grid barrier of the cooperative iterate kernel (ctl[4] arrivals,
// ctl[5] generation, ctl[6] set when a wait gave up: the kernel returns and
// the host reports AVBD_ERR_TIMEOUT).
constexpr long long kGridWaitLimit = 1ll << 25;
__device__ bool tg_grid_sync(const TWorld &w) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile int *gen = (volatile int *)&w.ctl[5];
    const int g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd((unsigned *)&w.ctl[4], 1u) + 1u;
    if (arrived == gridDim.x) {
      w.ctl[4] = 0;
      __threadfence();
      atomicAdd(&w.ctl[5], 1);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > kGridWaitLimit || *((volatile int *)&w.ctl[6])) {
          atomicOr(&w.ctl[6], 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*((volatile int *)&w.ctl[6])) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

// The iterations of one step (cooperative: one block of kBodyThreads per SM,
// latency being the bound): per iteration the colour phases (a block per
// body; bodies of one colour are independent), then every force's
// dual update (a thread per contact, joint, spring), and on the last
// iteration the BDF1 velocity (solver.js:476-488); a grid barrier between
// phases.
__global__ void __launch_bounds__(kBodyThreads, 1) iterate_kernel(TWorld w) {
  if (w.ctl[2]) return;
  extern __shared__ __align__(16) unsigned char smemRaw[];
  BodySmem &sm = *reinterpret_cast<BodySmem *>(smemRaw);
  const TParams &P = w.P;
  const int numColors = w.ctl[3], total = w.ctl[0];
  const int total_it = P.iterations + (P.postStabilize ? 1 : 0);
  // thread index spread so that consecutive items land on different SMs
  const int g = blockIdx.x + gridDim.x * threadIdx.x, gs = gridDim.x * blockDim.x;
  // The per-force phases run on five-lane groups, one tangent direction a
  // lane, six groups a warp, each kind of item (contacts, joints, springs,
  // inertial terms) from its own warps so that their instruction streams run
  // side by side.
  const int lane = threadIdx.x & 31, dir = lane % kTangentDims, slot = lane / kTangentDims;
  const int rows = blockDim.x >> 5, v = threadIdx.x >> 5;  // a block's warps
  const bool grouped = slot < kGroupsPerWarp;
  const unsigned mask = grouped ? 0x1fu << (slot * kTangentDims) : 0u;
  const int nGroups = rows * gridDim.x * kGroupsPerWarp;
  // a kind's n-th warp: warp rho(v) of block n % gridDim.x; contacts fill the
  // blocks' warps from the first, joints, inertial terms and springs from
  // the last three (warp v runs on sub-partition v % 4)
  auto group_of = [&](int rho) { return (rho * (int)gridDim.x + (int)blockIdx.x) * kGroupsPerWarp + slot; };
  const int gContact = group_of(v);
  const int gJoint = group_of(rows - 1 - v);
  const int gInert = group_of((2 * rows - 2 - v) % rows);
  const int gSpring = group_of((2 * rows - 3 - v) % rows);
  if (grouped)
    for (int q = gInert; q < w.n; q += nGroups)
      if (w.bs[q].mass > 0) inertial_terms(w, q, dir);
  if (!tg_grid_sync(w)) return;
  for (int it = 0; it < total_it; it++) {
    const R alpha = P.postStabilize ? (it < P.iterations ? 1.0 : 0.0) : P.alpha;
    for (int c = 0; c < numColors; c++) {
      const int c0 = w.colorStart[c], cn = w.colorStart[c + 1] - c0;
      for (int k = blockIdx.x; k < cn; k += gridDim.x) body_update_block(w, w.order[c0 + k], alpha, sm);
      if (!tg_grid_sync(w)) return;
    }
    if (it < P.iterations) {
      if (grouped) {
        for (int k = gContact; k < total * kMaxContacts; k += nGroups) {
          TManifold &m = w.cur[k / kMaxContacts];
          const int i = k % kMaxContacts;
          if (i < m.count) contact_dual_dir(w, m, i, alpha, dir, mask);
        }
        for (int k = gJoint; k < w.nj; k += nGroups)
          if (!w.j[k].removed) joint_dual_dir(w, w.j[k], alpha, dir, mask);
        for (int k = gSpring; k < w.ns; k += nGroups) spring_dual_dir(w, w.s[k], dir, mask);
        if (it + 1 < total_it)  // the next iteration's inertial terms (the iterates are final for this one)
          for (int q = gInert; q < w.n; q += nGroups)
            if (w.bs[q].mass > 0) inertial_terms(w, q, dir);
      }
      if (!tg_grid_sync(w)) return;
    }
    if (it == P.iterations - 1) {
      for (int i = g; i < w.n; i += gs) {
        TBody &b = w.b[i];
        for (int k = 0; k < 3; k++) b.pv[k] = b.v[k];
        if (w.bs[i].mass > 0) {
          for (int k = 0; k < 3; k++) b.v[k] = (b.p[k] - b.p0[k]) / P.dt;
          R dq[3];
          q_subtract(dq, b.q, b.q0);
          for (int k = 0; k < 3; k++) b.w[k] = dq[k] / P.dt;
        }
      }
      if (!tg_grid_sync(w)) return;
    }
  }
}

// This step's manifolds become the next step's previous ones: keys of the
// live ones, in key order (candidates are in key order already).
__global__ void __launch_bounds__(kBlock) commit_index_kernel(TWorld w) {
  if (w.ctl[2]) return;
  const int total = w.ctl[0];
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  typedef cub::BlockScan<int, kBlock> Scan;
  __shared__ typename Scan::TempStorage tmp;
  for (int c0 = 0; c0 < total; c0 += kBlock) {
    const int c = c0 + threadIdx.x;
    const int live = c < total && w.cur[c].count > 0 ? 1 : 0;
    int at, tot;
    Scan(tmp).ExclusiveSum(live, at, tot);
    if (c < total) w.commitAt[c] = live ? base + at : -1;
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) w.ctl[1] = base;
}
// The live manifolds into the previous-step arrays, a warp per manifold.
__global__ void commit_copy_kernel(TWorld w) {
  if (w.ctl[2]) return;
  const int total = w.ctl[0], lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  static_assert(sizeof(TManifold) % sizeof(unsigned long long) == 0, "a manifold is whole words");
  constexpr int kWords = (int)(sizeof(TManifold) / sizeof(unsigned long long));
  for (int c = blockIdx.x + gridDim.x * (threadIdx.x >> 5); c < total; c += warps) {
    const int at = w.commitAt[c];
    if (at < 0) continue;
    const unsigned long long *src = reinterpret_cast<const unsigned long long *>(&w.cur[c]);
    unsigned long long *dst = reinterpret_cast<unsigned long long *>(&w.prev[at]);
    for (int k = lane; k < kWords; k += 32) dst[k] = src[k];
    if (lane == 0) w.prevKey[at] = w.key[c];
  }
}

// grad[d] = sum over bodies and components of g[i][k] * dx_i,k / d theta_d
__global__ void backward_kernel(TWorld w, const double *g, double *grad) {
  __shared__ double acc[kTangentDims];
  if (threadIdx.x < kTangentDims) acc[threadIdx.x] = 0.0;
  __syncthreads();
  double part[kTangentDims] = {};
  for (int i = threadIdx.x; i < w.n; i += blockDim.x)
    for (int k = 0; k < 3; k++)
      for (int d = 0; d < kTangentDims; d++) part[d] += g[i * 3 + k] * w.b[i].p[k].d[d];
  for (int d = 0; d < kTangentDims; d++) atomicAdd(&acc[d], part[d]);
  __syncthreads();
  if (threadIdx.x < kTangentDims) grad[threadIdx.x] = acc[threadIdx.x];
}

__global__ void read_kernel(TWorld w, double *pos, double *dpos, double *quat) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; k++) {
      pos[i * 3 + k] = w.b[i].p[k].v;
      if (dpos)
        for (int d = 0; d < kTangentDims; d++) dpos[(i * 3 + k) * kTangentDims + d] = w.b[i].p[k].d[d];
    }
    if (quat)
      for (int k = 0; k < 4; k++) quat[i * 4 + k] = w.b[i].q[k].v;
  }
}

}  // namespace tg

// ---------------------------------------------------------------------------
// Host side: the differentiable step's own device state, packed from a host
// world (f64) with the caller's seeds.
// ---------------------------------------------------------------------------
struct TangentCtx {
  tg::TWorld w{};
  std::vector<void *> allocs;
  int smCount = 0;
  int iterGrid = 0;  // blocks of the cooperative iterate kernel (kBodyThreads each)
  ~TangentCtx() {
    for (void *p : allocs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T **p, size_t count) {
    void *q = nullptr;
    const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return e;
    cudaMemset(q, 0, std::max<size_t>(count, 1) * sizeof(T));
    allocs.push_back(q);
    *p = (T *)q;
    return cudaSuccess;
  }
};

void tangent_destroy(TangentCtx *t) { delete t; }

static tg::R dual_of(double v) { return tg::R(v); }

// Pack `world` and seed its inputs. Returns 0 or an AVBD_ERR_* with `msg`.
int tangent_pack(TangentCtx **out, const avbd_world *world, const avbd_params &P, const avbd_tangent_seed *seeds,
                 int nSeeds, char *msg, size_t msgLen, cudaStream_t st) {
  using namespace tg;
  const avbd_body_soa &B = world->bodies;
  const avbd_joint_soa &J = world->joints;
  const avbd_spring_soa &S = world->springs;
  const int n = B.count, nj = J.count, ns = S.count;
  if (n <= 0 || !B.pos || !B.size || !B.mass || !B.moment || !B.radius || !B.friction) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: bodies need count > 0 and size/mass/moment/radius/friction/pos");
    return AVBD_ERR_ARG;
  }
  if (world->num_scenes > 1) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: one scene per call");
    return AVBD_ERR_ARG;
  }
  std::vector<TBody> hb(n);
  std::vector<TBodyStatic> hs(n);
  std::vector<std::vector<uint32_t>> refs(n);
  std::vector<TJoint> hj(nj);
  std::vector<TSpring> hsp(ns);
  for (int i = 0; i < n; i++) {
    TBody &b = hb[i];
    TBodyStatic &s = hs[i];
    for (int k = 0; k < 3; k++) {
      b.p[k] = dual_of(B.pos[i * 3 + k]);
      b.v[k] = dual_of(B.vel ? B.vel[i * 3 + k] : 0.0);
      b.w[k] = dual_of(B.omega ? B.omega[i * 3 + k] : 0.0);
      b.pv[k] = dual_of(B.prev_vel ? B.prev_vel[i * 3 + k] : (B.vel ? B.vel[i * 3 + k] : 0.0));
      s.moment[k] = B.moment[i * 3 + k];
      s.half[k] = B.size[i * 3 + k] * 0.5;
    }
    for (int k = 0; k < 4; k++) b.q[k] = dual_of(B.quat ? B.quat[i * 4 + k] : (k == 3 ? 1.0 : 0.0));
    s.mass = B.mass[i];
    s.radius = B.radius[i];
    s.friction = dual_of(B.friction[i]);
    s.shape = B.shape ? B.shape[i] : AVBD_SHAPE_BOX;
  }
  for (int k = 0; k < nj; k++) {
    TJoint &j = hj[k];
    j.a = J.body_a[k];
    j.b = J.body_b[k];
    if (j.b < 0 || j.b >= n || j.a >= n || j.a == j.b) {
      snprintf(msg, msgLen, "avbd_adjoint_forward: joint %d: bad body indices", k);
      return AVBD_ERR_ARG;
    }
    for (int c = 0; c < 3; c++) {
      j.rA[c] = dual_of(J.r_a[k * 3 + c]);
      j.rB[c] = dual_of(J.r_b[k * 3 + c]);
      j.penLin[c] = dual_of(J.penalty_lin ? J.penalty_lin[k * 3 + c] : 0.0);
      j.penAng[c] = dual_of(J.penalty_ang ? J.penalty_ang[k * 3 + c] : 0.0);
      j.lamLin[c] = dual_of(J.lambda_lin ? J.lambda_lin[k * 3 + c] : 0.0);
      j.lamAng[c] = dual_of(J.lambda_ang ? J.lambda_ang[k * 3 + c] : 0.0);
    }
    j.stiffLin = dual_of(J.stiffness_lin[k]);
    j.stiffAng = dual_of(J.stiffness_ang[k]);
    j.fracture = J.fracture[k];
    const double sx = (j.a >= 0 ? B.size[j.a * 3] : 0) + B.size[j.b * 3];
    const double sy = (j.a >= 0 ? B.size[j.a * 3 + 1] : 0) + B.size[j.b * 3 + 1];
    const double sz = (j.a >= 0 ? B.size[j.a * 3 + 2] : 0) + B.size[j.b * 3 + 2];
    j.torqueArm = sx * sx + sy * sy + sz * sz;  // joint.js:108-112
    j.broken = J.broken && J.broken[k] ? 1 : 0;
    if (j.a >= 0) refs[j.a].push_back(make_ref(kRefJoint, k, 0));
    refs[j.b].push_back(make_ref(kRefJoint, k, 1));
  }
  for (int k = 0; k < ns; k++) {
    TSpring &s = hsp[k];
    s.a = S.body_a[k];
    s.b = S.body_b[k];
    if (s.a < 0 || s.b < 0 || s.a >= n || s.b >= n || s.a == s.b || !(S.rest[k] >= 0)) {
      snprintf(msg, msgLen, "avbd_adjoint_forward: spring %d: bad body indices or unresolved rest length", k);
      return AVBD_ERR_ARG;
    }
    for (int c = 0; c < 3; c++) {
      s.rA[c] = dual_of(S.r_a[k * 3 + c]);
      s.rB[c] = dual_of(S.r_b[k * 3 + c]);
    }
    s.stiffness = dual_of(S.stiffness[k]);
    s.rest = S.rest[k];
    s.tear = S.tear_strain ? S.tear_strain[k] : INFINITY;
    s.penalty = dual_of(S.penalty ? S.penalty[k] : 0.0);
    s.peak = dual_of(S.peak_strain ? S.peak_strain[k] : 0.0);
    s.broken = S.broken && S.broken[k] ? 1 : 0;
    refs[s.a].push_back(make_ref(kRefSpring, k, 0));
    refs[s.b].push_back(make_ref(kRefSpring, k, 1));
  }
  std::vector<uint32_t> cRef;
  for (int i = 0; i < n; i++) {
    hs[i].cStart = (int)cRef.size();
    cRef.insert(cRef.end(), refs[i].begin(), refs[i].end());
    hs[i].cEnd = (int)cRef.size();
  }
  TParams tp{};
  tp.dt = P.dt; tp.gravity = P.gravity; tp.alpha = P.alpha; tp.gamma = P.gamma; tp.betaLin = P.beta_lin;
  tp.betaAng = P.beta_ang; tp.penaltyMin = P.penalty_min; tp.margin = P.collision_margin;
  tp.stickThreshold = P.stick_threshold; tp.penaltyMax = dual_of(P.penalty_max); tp.iterations = P.iterations;
  tp.postStabilize = P.post_stabilize; tp.rotatedInertia = P.rotated_inertia; tp.springRamp = P.spring_stiffness_ramp;
  tp.springGeometric = P.spring_geometric_stiffness;
  tp.cachedJacobians = P.cached_contact_jacobians;
  // seeds
  for (int k = 0; k < nSeeds; k++) {
    const avbd_tangent_seed &sd = seeds[k];
    const int d = sd.dir;
    if (d < 0 || d >= kTangentDims) {
      snprintf(msg, msgLen, "avbd_adjoint_forward: seed %d: direction %d outside 0..%d", k, d, kTangentDims - 1);
      return AVBD_ERR_ARG;
    }
    if (sd.kind == AVBD_SEED_VELOCITY) {
      if (sd.index < 0 || sd.index >= n || sd.comp < 0 || sd.comp > 2) {
        snprintf(msg, msgLen, "avbd_adjoint_forward: seed %d: bad body or component", k);
        return AVBD_ERR_ARG;
      }
      hb[sd.index].v[sd.comp].d[d] = 1.0;
      hb[sd.index].pv[sd.comp].d[d] = 1.0;  // a scene starts with the two equal (rigid.js:51)
    } else if (sd.kind == AVBD_SEED_FRICTION) {
      if (sd.index < 0 || sd.index >= n) {
        snprintf(msg, msgLen, "avbd_adjoint_forward: seed %d: bad body", k);
        return AVBD_ERR_ARG;
      }
      hs[sd.index].friction.d[d] = 1.0;
    } else if (sd.kind == AVBD_SEED_PENALTY_MAX) {
      tp.penaltyMax.d[d] = 1.0;
    } else if (sd.kind == AVBD_SEED_JOINT_STIFFNESS) {
      if (sd.index < 0 || sd.index >= nj) {
        snprintf(msg, msgLen, "avbd_adjoint_forward: seed %d: bad joint", k);
        return AVBD_ERR_ARG;
      }
      if (std::isfinite(hj[sd.index].stiffLin.v)) hj[sd.index].stiffLin.d[d] = 1.0;
      if (std::isfinite(hj[sd.index].stiffAng.v)) hj[sd.index].stiffAng.d[d] = 1.0;
    } else {
      snprintf(msg, msgLen, "avbd_adjoint_forward: seed %d: unknown kind %d", k, sd.kind);
      return AVBD_ERR_ARG;
    }
  }
  TangentCtx *t = new TangentCtx();
  TWorld &w = t->w;
  w.P = tp;
  w.n = n; w.nj = nj; w.ns = ns;
  w.mcap = std::max(16 * n, 256);
  w.fcap = 2 * w.mcap + 2 * (nj + ns) + 64;
  cudaError_t e = cudaSuccess;
  uint32_t *cRefD = nullptr;
  std::vector<uint32_t> prio(n);
  for (int i = 0; i < n; i++) prio[i] = color_priority((uint32_t)i);
  uint32_t *prioD = nullptr;
  if ((e = t->alloc(&w.b, n)) || (e = t->alloc(&w.bs, n)) || (e = t->alloc(&cRefD, cRef.size())) ||
      (e = t->alloc(&w.j, nj)) || (e = t->alloc(&w.s, ns)) || (e = t->alloc(&w.pairCount, n + 1)) ||
      (e = t->alloc(&w.pairStart, n + 1)) || (e = t->alloc(&w.key, w.mcap)) || (e = t->alloc(&w.cur, w.mcap)) ||
      (e = t->alloc(&w.prev, w.mcap)) || (e = t->alloc(&w.prevKey, w.mcap)) || (e = t->alloc(&w.commitAt, w.mcap)) ||
      (e = t->alloc(&w.ctl, 8)) ||
      (e = t->alloc(&w.fStart, n + 1)) || (e = t->alloc(&w.fCount, n + 1)) || (e = t->alloc(&w.fRef, w.fcap)) ||
      (e = t->alloc(&w.color, n)) || (e = t->alloc(&w.order, n)) || (e = t->alloc(&w.colorStart, kMaxColors + 1)) ||
      (e = t->alloc(&prioD, n)) || (e = t->alloc(&w.jac, (size_t)w.mcap * K8 * 18)) ||
      (e = t->alloc(&w.inert, (size_t)n * kSysEntries))) {
    delete t;
    snprintf(msg, msgLen, "avbd_adjoint_forward: cudaMalloc: %s", cudaGetErrorString(e));
    return AVBD_ERR_CUDA;
  }
  w.cRef = cRefD;
  w.prio = prioD;
  cudaMemcpyAsync(w.b, hb.data(), sizeof(TBody) * n, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(w.bs, hs.data(), sizeof(TBodyStatic) * n, cudaMemcpyHostToDevice, st);
  if (!cRef.empty()) cudaMemcpyAsync(cRefD, cRef.data(), sizeof(uint32_t) * cRef.size(), cudaMemcpyHostToDevice, st);
  if (nj) cudaMemcpyAsync(w.j, hj.data(), sizeof(TJoint) * nj, cudaMemcpyHostToDevice, st);
  if (ns) cudaMemcpyAsync(w.s, hsp.data(), sizeof(TSpring) * ns, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(prioD, prio.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice, st);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&t->smCount, cudaDevAttrMultiProcessorCount, dev);
  // the iterate kernel: one warp and one BodySmem per block, all blocks resident
  int perSm = 0;
  e = cudaFuncSetAttribute(iterate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BodySmem));
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, iterate_kernel, kBodyThreads, sizeof(BodySmem));
  if (e != cudaSuccess || perSm < 1) {
    delete t;
    snprintf(msg, msgLen, "avbd_adjoint_forward: the iterate kernel cannot be made resident (%s)",
             e != cudaSuccess ? cudaGetErrorString(e) : "no block fits an SM");
    return AVBD_ERR_CUDA;
  }
  t->iterGrid = std::max(1, std::min(t->smCount, std::max(n, 1)));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    delete t;
    snprintf(msg, msgLen, "avbd_adjoint_forward: %s", cudaGetErrorString(e));
    return AVBD_ERR_CUDA;
  }
  *out = t;
  return AVBD_OK;
}

// `steps` differentiable steps; the scan of the pair counts on the stream.
int tangent_step(TangentCtx *t, int steps, void *temp, size_t tempBytes, char *msg, size_t msgLen, cudaStream_t st) {
  using namespace tg;
  TWorld &w = t->w;
  const int blocks = std::max(1, std::min((w.n + 127) / 128, t->smCount * 4));
  const int pairBlocks = std::max(1, std::min((w.n + 3) / 4, t->smCount * 8));  // a warp per body
  for (int s = 0; s < steps; s++) {
    cudaMemsetAsync(w.pairCount + w.n, 0, sizeof(int), st);
    pairs_count_kernel<<<pairBlocks, 128, 0, st>>>(w);
    size_t tb = tempBytes;
    cub::DeviceScan::ExclusiveSum(temp, tb, w.pairCount, w.pairStart, w.n + 1, st);
    pairs_write_kernel<<<pairBlocks, 128, 0, st>>>(w);
    narrow_kernel<<<t->smCount * 2, 64, 0, st>>>(w);
    forces_init_kernel<<<t->smCount * 2, 64, 0, st>>>(w);
    bodies_init_kernel<<<t->smCount * 2, 64, 0, st>>>(w);
    adjacency_coloring_kernel<<<1, kBlock, 0, st>>>(w);
    {
      void *args[] = {(void *)&w};
      const cudaError_t le = cudaLaunchCooperativeKernel((const void *)iterate_kernel, dim3(t->iterGrid), dim3(kBodyThreads),
                                                         args, sizeof(BodySmem), st);
      if (le != cudaSuccess) {
        snprintf(msg, msgLen, "avbd_adjoint_forward: cooperative launch: %s", cudaGetErrorString(le));
        return AVBD_ERR_CUDA;
      }
    }
    commit_index_kernel<<<1, kBlock, 0, st>>>(w);
    commit_copy_kernel<<<t->smCount, 128, 0, st>>>(w);
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: %s", cudaGetErrorString(e));
    return AVBD_ERR_CUDA;
  }
  int ctl[8];
  cudaMemcpy(ctl, w.ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  if (ctl[6]) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: a grid barrier of the iterations gave up");
    return AVBD_ERR_TIMEOUT;
  }
  if (ctl[7]) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: a constraint row made more than %d addends to one system entry",
             kMaxAdd);
    return AVBD_ERR_STATE;
  }
  if (ctl[2]) {
    snprintf(msg, msgLen, "avbd_adjoint_forward: candidate pairs or force lists exceed the differentiable step's "
                          "arenas (%d pair slots)", w.mcap);
    return AVBD_ERR_CAPACITY;
  }
  return AVBD_OK;
}

size_t tangent_temp_bytes(const TangentCtx *t) {
  size_t a = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int *)nullptr, t->w.n + 1);
  return a;
}

int tangent_read(TangentCtx *t, double *pos, double *dpos, double *quat, cudaStream_t st) {
  const int n = t->w.n;
  double *d = nullptr;
  const size_t bytes = sizeof(double) * ((size_t)n * 3 + (size_t)n * 3 * kTangentDims + (size_t)n * 4);
  if (cudaMalloc(&d, bytes) != cudaSuccess) return AVBD_ERR_CUDA;
  double *dp = d, *dd = d + (size_t)n * 3, *dq = dd + (size_t)n * 3 * kTangentDims;
  tg::read_kernel<<<std::max(1, (n + 255) / 256), 256, 0, st>>>(t->w, dp, dd, dq);
  cudaMemcpyAsync(pos ? pos : nullptr, dp, pos ? sizeof(double) * n * 3 : 0, cudaMemcpyDeviceToHost, st);
  if (dpos) cudaMemcpyAsync(dpos, dd, sizeof(double) * n * 3 * kTangentDims, cudaMemcpyDeviceToHost, st);
  if (quat) cudaMemcpyAsync(quat, dq, sizeof(double) * n * 4, cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(d);
  return e == cudaSuccess ? AVBD_OK : AVBD_ERR_CUDA;
}

int tangent_backward(TangentCtx *t, const double *gradPos, double *gradParams, cudaStream_t st) {
  const int n = t->w.n;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * ((size_t)n * 3 + kTangentDims)) != cudaSuccess) return AVBD_ERR_CUDA;
  cudaMemcpyAsync(d, gradPos, sizeof(double) * n * 3, cudaMemcpyHostToDevice, st);
  tg::backward_kernel<<<1, 256, 0, st>>>(t->w, d, d + (size_t)n * 3);
  cudaMemcpyAsync(gradParams, d + (size_t)n * 3, sizeof(double) * kTangentDims, cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  cudaFree(d);
  return e == cudaSuccess ? AVBD_OK : AVBD_ERR_CUDA;
}

int tangent_dims() { return kTangentDims; }

}  // namespace avbd
