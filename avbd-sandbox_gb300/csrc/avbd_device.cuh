// avbd_device.cuh - device data layout and shared math of the GB300 AVBD step.
//
// Layout in HBM (all structure-of-arrays, 16-byte vectors where the solver
// streams them):
//   bodies      x_t in f64 (D4), iterate displacement delta = x - x_t and
//               orientation q in f32 (float4), f64 shadows for FP64 bodies
//   manifolds   double-buffered (previous / current step), sorted by the
//               64-bit pair key (A << 32) | B, 8 contact slots each; the solver
//               record of one contact is 4 x float4 = 64 B
//   joints /    f32 penalties, f64 multipliers (the fracture test reads them)
//   springs
// Conventions follow src/math/maths.js: quat = (x, y, z, w), row-major mat3.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace avbd {

// 32-byte aligned f64 4-vector (CUDA 13 deprecates the 16-byte-aligned D4).
struct __align__(32) D4 {
  double x, y, z, w;
};
__host__ __device__ inline D4 mkd4(double x, double y, double z, double w) { return D4{x, y, z, w}; }

constexpr int kMaxContacts = 8;
// Colours the device colouring can hold. The greedy colouring needs at most
// (largest number of dynamic neighbours of a body) + 1; per-colour loops run
// over the colours in use only.
constexpr int kMaxColors = 1024;
constexpr int kLaneBuckets = 8;     // log2 of the lanes of a body's group: 0..7
constexpr int kLaneMaxGroup = 128;  // largest group: one solve block

// Overflow / error bits in Control::flags (mirrors AVBD_OVF_* of the ABI).
constexpr unsigned kOvfCells = 0x1u;
constexpr unsigned kOvfPairs = 0x2u;
constexpr unsigned kOvfAdj = 0x4u;
constexpr unsigned kOvfColors = 0x8u;
constexpr unsigned kOvfTimeout = 0x10u;
constexpr unsigned kErrNaN = 0x100u;
constexpr unsigned kErrColoring = 0x200u;  // an uploaded colouring was not proper (AVBD_ERR_COLORING)

// Body flag bits.
constexpr int kBodyDynamic = 0x1;
constexpr int kBodyFp64 = 0x2;
constexpr int kBodyLarge = 0x4;
constexpr int kBodySphere = 0x8;

// Static-adjacency entry: (type << 30) | (index << 1) | side.
constexpr uint32_t kRefJoint = 1u;
constexpr uint32_t kRefSpring = 2u;
__host__ __device__ inline uint32_t make_ref(uint32_t type, uint32_t idx, uint32_t side) {
  return (type << 30) | (idx << 1) | side;
}

// Joint / spring state bits.
constexpr int kBroken = 0x1;
constexpr int kRemoved = 0x2;  // dropped from the solver (Force.initialize() false)

struct SolverParams {
  double dt, gravity;
  int iterations, postStabilize;
  double betaLin, betaAng, alpha, gamma, penaltyMin, penaltyMax, margin, stickThreshold;
  int rotatedInertia, springRamp, springGeometric, cachedJacobians;
  double fp64Ratio;
  int schedule;  // 0: colour phases + grid barrier, 1: dependency wavefront
  int lanes;     // lanes per body of the colour-phase solve; 0: per body, from its constraint count
  int solveBlocksPerSm;  // resident blocks per SM of the solve launch (grid = this x SMs)
  long long barrierLimit, waitLimit;  // polls before a grid barrier / a neighbour wait gives up
  int tailDiv;   // colours of at most (grid / tailDiv) chunks form the tail segment; 0 automatic, < 0 none
  // AVBD_CONTACT_MATERIALS (the WebGPU engine's contact extensions) when 1
  int contactModel;
  double restitutionThreshold, contactPersistence;
};

// Device scalars shared by all kernels of a step.
struct Control {
  unsigned flags;          // overflow / error bits (sticky until pack)
  unsigned barrierCount;   // grid barrier
  unsigned barrierGen;
  int numCandidates;
  int numColors;
  int colorChanged;
  int liveManifolds;
  int liveContacts;
  int fp64Bodies;
  int adjTotal;
  int prevCandidates;  // candidates (= manifold slots) of the previous step
  int npCount[3];      // narrow-phase work lists: face, edge, exact
  int colorBad;        // this step's uploaded colouring has a conflict
  int laneTotal;       // lanes of one iteration's colour phases (sum over bodies)
  int pad[4];
  // Candidate overflow: a step whose candidate pairs exceed the arena is
  // skipped as a whole (every kernel after the broad phase returns at once, so
  // body, joint, spring and warm-start state stay as they were before the
  // step), and so is every step queued after it until the host has regrown
  // the arenas and queued the skipped steps again.
  int skip;            // sticky: set by the broad phase, cleared by the host
  int stepsSkipped;    // steps skipped since the host last cleared `skip`
  int wantCandidates;  // candidate pairs the last broad phase found (may exceed the arena)
};

struct Bodies {
  int n;
  // static
  const D4 *size;   // full widths xyz, w = bounding radius (f64)
  const D4 *massD;  // mass, Ix, Iy, Iz (f64)
  const float4 *massF;   // mass, Ix, Iy, Iz (f32)
  const double *friction;
  const int *flags0;     // static flag bits (dynamic, large, sphere)
  const int *scene;
  const uint32_t *priority;  // lowbias32(local index)
  // persistent dynamic state
  D4 *pos;   // x_t, f64
  float4 *quat;   // iterate q (= q_t at step start)
  float4 *vel, *omega, *prevVel;
  // per-step
  float4 *quatT;  // q_t
  float4 *dp;     // delta = p - p_t
  float4 *dang;   // qsub(q, q_t) of the current iterate (f32), what neighbours read
  float4 *yLin;   // y - p_t
  float4 *yAng;   // q of the inertial prediction
  D4 *dpD, *quatD;  // f64 shadows (FP64 bodies)
  int *flags;     // per-step flags (static bits | kBodyFp64)
  int *color;     // colour, -1 for static bodies
  int *progress;  // iterations completed in the current step (wavefront schedule)
  // contact materials (AVBD_CONTACT_MATERIALS only, else null): static and
  // dynamic friction, restitution, rest offset; contact offset
  const D4 *mat;
  const double *contactOffset;
};

struct Manifolds {
  int cap;
  uint64_t *key;
  int *count;
  float4 *basis0, *basis1, *basis2;  // rows; basis0.w = friction
  double *basisD;                    // 9 per manifold, f64 (next step's sphere transport)
  uint32_t *feat;                    // 8 per manifold
  float4 *rA, *rB;                   // body-local anchors (persistent)
  float4 *cA;  // rA world at x_t, C0.x
  float4 *cB;  // rB world at x_t, C0.y
  float4 *cK;  // penalty xyz, C0.z
  float4 *cL;  // lambda xyz, stick
  float *cX;   // restitution bias (AVBD_CONTACT_MATERIALS); basis1.w bit 1 then marks
               // a positive contact skin and basis2.w holds the dynamic friction
};

struct Joints {
  int n;
  const int2 *bodies;      // a (-1 = world anchor), b
  const D4 *rAD, *rBD;
  const float4 *rAF, *rBF;
  const D4 *stiff;    // stiffnessLin, stiffnessAng, fracture, torqueArm
  float4 *penLin, *penAng;
  D4 *lamLin, *lamAng;
  float4 *c0Lin, *c0Ang;   // per step, C*(x_t)
  float4 *dpt;             // per step, p_A(t) - p_B(t) (or world anchor - p_B(t))
  D4 *dptD;
  int *state;              // kBroken | kRemoved
};

struct Springs {
  int n;
  const int2 *bodies;
  const D4 *rAD, *rBD;
  const float4 *rAF, *rBF;
  const D4 *prm;      // stiffness, rest, tearStrain, -
  float *penalty;
  double *peak;
  int *state;
  float4 *dpt;
  D4 *dptD;
};

// One hash-grid insertion: the body's exact broad-phase inputs travel with
// it, so the sphere test needs no further loads. b2 = (body << 1) | dynamic;
// loc = f32 offset of the centre from its cell's corner, w = radius (f32).
struct __align__(16) Entry {
  double x, y, z, r;
  float4 loc;
  int b2, cx, cy, cz;
};
constexpr int kPairScratch = 128;     // partner row of a step's broad phase
constexpr int kLargeChunk = 1024;     // bodies a block tests against one large body
constexpr int kStaticPairRow = 64;    // partner row of the allocation-free query

struct Grid {
  int numScenes;
  const int *sceneStart;     // numScenes + 1
  const double *invCell;     // per scene
  const int *largeStart;     // per scene CSR of large bodies
  const int *largeList;
  int *largeChunk;           // per large body, maxChunks counts / offsets of its partner chunks
  int maxChunks;             // partner chunks of kLargeChunk bodies per large body
  int4 *cellLo;              // per body: centre cell, w = scene
  float4 *loc;               // per body: f32 offset from the cell corner, w = radius
  const float *cellF;        // per scene: cell edge (f32 of 1 / invCell)
  unsigned tableMask;
  int *tableCount, *tableStart, *tableCursor;
  struct Entry *entries;
  int entryCap;
  uint32_t *scratch;  // per body: sorted lower-index partners (kPairScratch each)
  int hasConstraints; // any joint or spring in the world
  int *pairCount, *pairStart;  // per body, pairStart has n + 1 entries
  uint64_t *candKey;
  int *candPrev;
  int candCap;
  // narrow-phase work lists (candidate index + winning axis), candCap each
  int2 *npFace, *npEdge;
  int *npExact;
  // static joint/spring adjacency (pack time)
  const int *cStart;
  const uint32_t *cRef;
};

struct Adjacency {
  int *start;   // n + 1
  int *count;   // n
  int *cursor;  // n
  uint32_t *entry;  // (manifold << 1) | side
  int cap;
  // per-contact adjacency of dynamic bodies: (slot << 1 | side, other body),
  // slot = manifold * 8 + contact; in manifold order, then contact order
  int *cstart;   // n + 1
  int *ccount;   // n
  int2 *centry;
  int ccap;
  int *hpEntry;      // per body, within its manifold range: dynamic neighbours of higher colouring priority
  int *hpCount;      // n
  const int *colorOverride;  // uploaded colours (avbd_set_coloring), or null
  int *colorStart;   // kMaxColors + 1 (entries past the colours in use hold the total)
  int *colorBodies;  // dynamic bodies sorted by (colour, index)
  int4 *colorRec;    // per colour position: body, contact range begin, end, 0
  int *blockHist;    // colouring counting sort scratch
  // lane layout of the colour-phase solve: per colour, its bodies' lane
  // groups (G lanes, a power of two, aligned to G) in decreasing G, cut into
  // chunks of kLaneMaxGroup lanes (one solve block each); entry per lane:
  // record << 4 | FP64 << 3 | log2 G, or -1 past the colour's last group
  int *laneTab;      // kLaneMaxGroup * (n + kMaxColors): never overflows
  int *colorChunk;   // kMaxColors + 1: first chunk of each colour
  int *laneHist;     // 2 * kMaxColors * kLaneBuckets: group counts, then lane cursors
};

// The uniform mouse grab (src/physics/gpu/shaders.js:2119-2161): a finite
// ball socket from a world target to a body-local point of one body, penalty
// fixed at the stiffness, no multiplier, applied in that body's primal only.
struct __align__(32) Grab {
  D4 target;     // world point, f64
  D4 localD;     // body-local anchor, f64 (FP64 bodies)
  float4 local;  // the same, f32
  double k;      // stiffness
  int body;      // -1: nothing grabbed
};

// Everything a kernel may touch.
struct World {
  SolverParams p;
  Bodies b;
  Joints j;
  Springs s;
  Manifolds cur, prev;
  Grid g;
  Adjacency a;
  Control *ctl;
  Grab *grab;
};

// ---------------------------------------------------------------------------
// Small vector math, templated on the scalar (float / double). Operation order
// follows src/math/maths.js.
// ---------------------------------------------------------------------------
template <class T>
struct V3 {
  T x, y, z;
};
template <class T>
struct Q4 {
  T x, y, z, w;
};

template <class T>
__host__ __device__ inline V3<T> v3(T x, T y, T z) {
  return V3<T>{x, y, z};
}
template <class T>
__host__ __device__ inline V3<T> operator+(V3<T> a, V3<T> b) {
  return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class T>
__host__ __device__ inline V3<T> operator-(V3<T> a, V3<T> b) {
  return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class T>
__host__ __device__ inline V3<T> operator-(V3<T> a) {
  return {-a.x, -a.y, -a.z};
}
template <class T>
__host__ __device__ inline V3<T> operator*(V3<T> a, T s) {
  return {a.x * s, a.y * s, a.z * s};
}
template <class T>
__host__ __device__ inline T dot(V3<T> a, V3<T> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
__host__ __device__ inline V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Eq. 20 (maths.js:541-555): vector part of 2 q_a q_b^-1.
template <class T>
__host__ __device__ inline V3<T> qsub(Q4<T> a, Q4<T> b) {
  const T lsq = b.x * b.x + b.y * b.y + b.z * b.z + b.w * b.w;
  T ix, iy, iz, iw;
  if constexpr (sizeof(T) == 4) {  // FP32 solver path: one reciprocal
    const T r = T(1) / lsq;
    ix = -b.x * r; iy = -b.y * r; iz = -b.z * r; iw = b.w * r;
  } else {
    ix = -b.x / lsq; iy = -b.y / lsq; iz = -b.z / lsq; iw = b.w / lsq;
  }
  V3<T> o;
  o.x = (a.w * ix + a.x * iw + a.y * iz - a.z * iy) * T(2);
  o.y = (a.w * iy - a.x * iz + a.y * iw + a.z * ix) * T(2);
  o.z = (a.w * iz + a.x * iy - a.y * ix + a.z * iw) * T(2);
  return o;
}
// Eq. 21 (maths.js:568-592): normalize(q + 1/2 (0, dw) q).
template <class T>
__host__ __device__ inline Q4<T> qintegrate(Q4<T> q, V3<T> w) {
  const T px = w.x * q.w + w.y * q.z - w.z * q.y;
  const T py = -w.x * q.z + w.y * q.w + w.z * q.x;
  const T pz = w.x * q.y - w.y * q.x + w.z * q.w;
  const T pw = -w.x * q.x - w.y * q.y - w.z * q.z;
  const T rx = q.x + px * T(0.5), ry = q.y + py * T(0.5), rz = q.z + pz * T(0.5), rw = q.w + pw * T(0.5);
  if constexpr (sizeof(T) == 4) {  // FP32 solver path: one reciprocal square root
    const T il = rsqrtf(rx * rx + ry * ry + rz * rz + rw * rw);
    return Q4<T>{rx * il, ry * il, rz * il, rw * il};
  } else {
    const T len = sqrt(rx * rx + ry * ry + rz * rz + rw * rw);
    return Q4<T>{rx / len, ry / len, rz / len, rw / len};
  }
}
// maths.js:599-613
template <class T>
__host__ __device__ inline V3<T> qrotate(Q4<T> q, V3<T> v) {
  const T tx = (q.y * v.z - q.z * v.y) * T(2);
  const T ty = (q.z * v.x - q.x * v.z) * T(2);
  const T tz = (q.x * v.y - q.y * v.x) * T(2);
  return V3<T>{v.x + tx * q.w + (q.y * tz - q.z * ty), v.y + ty * q.w + (q.z * tx - q.x * tz),
               v.z + tz * q.w + (q.x * ty - q.y * tx)};
}

__device__ inline V3<float> f3(float4 v) { return V3<float>{v.x, v.y, v.z}; }
__device__ inline Q4<float> q4(float4 v) { return Q4<float>{v.x, v.y, v.z, v.w}; }
__device__ inline V3<double> d3(D4 v) { return V3<double>{v.x, v.y, v.z}; }
__device__ inline Q4<double> dq4(D4 v) { return Q4<double>{v.x, v.y, v.z, v.w}; }
template <class T>
__device__ inline V3<T> cvt3(V3<float> v) {
  return V3<T>{T(v.x), T(v.y), T(v.z)};
}
template <class T>
__device__ inline Q4<T> cvtq(Q4<float> v) {
  return Q4<T>{T(v.x), T(v.y), T(v.z), T(v.w)};
}

// Read-only-path loads (data not written during the kernel).
template <class T>
__device__ inline T ld(const T *p) {
  return __ldg(p);
}
__device__ inline D4 ld(const D4 *p) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
  const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
  return D4{a.x, a.y, b.x, b.y};
}
// L2-coherent loads/stores for state written earlier in the same persistent
// kernel by other blocks (L1 is not coherent across SMs).
__device__ inline float4 ldcg(const float4 *p) { return __ldcg(p); }
__device__ inline D4 ldcg(const D4 *p) {
  const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
  const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
  return D4{a.x, a.y, b.x, b.y};
}
__device__ inline void stcg(D4 *p, D4 v) {
  __stcg(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y));
  __stcg(reinterpret_cast<double2 *>(p) + 1, make_double2(v.z, v.w));
}

// lowbias32 integer hash: the colouring priority (src/physics/gpu/layout.js:50-57).
__host__ __device__ inline uint32_t color_priority(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// Kernel launchers (defined in the .cu files; all asynchronous on `st`).
size_t broadphase_temp_bytes(int n, int tableSize);
void launch_broadphase_impl(const World &w, int numLarge, void *temp, size_t tempBytes, cudaStream_t st,
                            int smCount);
void launch_narrowphase(const World &w, cudaStream_t st, int smCount);
size_t solver_temp_bytes(int n);
void launch_prepare(const World &w, void *temp, size_t tempBytes, cudaStream_t st, int smCount);
cudaError_t launch_coloring(const World &w, cudaStream_t st, int blocks);
int coloring_grid(int smCount);  // blocks of the cooperative colouring launch
cudaError_t launch_solve(const World &w, int lanesPerBody, int blocksPerSm, cudaStream_t st, int smCount);
int solve_max_blocks_per_sm(int lanesPerBody);
void launch_commit(const World &w, cudaStream_t st, int smCount);
void launch_stats(const World &w, double *out3, cudaStream_t st, int smCount);
cudaError_t launch_joint_anchor(const World &w, int joint, double x, double y, double z, cudaStream_t st);
cudaError_t launch_set_grab(const World &w, int body, const double *local, const double *target, double k,
                            cudaStream_t st);
// Identity-preserving repack (repack.cu): the dynamic state of carried
// bodies, joints and springs gathered from the old arrays (maps new -> old
// index, -1 = keep what the pack uploaded), and the old warm-start arena's
// live manifolds between surviving bodies renumbered into the new one.
// `flag`/`at` hold oldSlots + 1 ints each; the carried count ends up in
// ctl->prevCandidates.
cudaError_t launch_repack_state(const World &oldW, const World &newW, const int *oldBody, const int *oldJoint,
                                const int *oldSpring, cudaStream_t st);
cudaError_t launch_repack_manifolds(const Manifolds &oldM, const Manifolds &newM, int oldSlots, const int *newOf,
                                    int *flag, int *at, Control *ctl, cudaStream_t st);
// Error text of a context-free ABI call (read back by avbd_last_error(NULL)).
int set_context_free_error(int code, const char *msg);
// The differentiable step (tangent.cu).
struct TangentCtx;
void tangent_destroy(TangentCtx *t);
size_t tangent_temp_bytes(const TangentCtx *t);
int tangent_step(TangentCtx *t, int steps, void *temp, size_t tempBytes, char *msg, size_t msgLen, cudaStream_t st);
int tangent_read(TangentCtx *t, double *pos, double *dpos, double *quat, cudaStream_t st);
int tangent_backward(TangentCtx *t, const double *gradPos, double *gradParams, cudaStream_t st);

}  // namespace avbd
