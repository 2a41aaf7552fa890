// host.cu - the C ABI of include/avbd_cuda.h: context, pack, step orchestration,
// state readback. Replaces `GpuBackend` (src/physics/gpu/backend.js:243-2226).
//
// One context = one CUDA stream on the current device. A step is a fixed
// launch sequence with all sizes resident on the device (no host round trip):
//   broadphase (hash grid + candidate keys) -> narrowphase (certified f32,
//   f64 where a decision is not certain) -> prepare (forces, bodies,
//   adjacency) -> colouring and the solve's lane layout (cooperative) ->
//   solve (cooperative persistent: iterations x colours, fused dual,
//   velocity) -> commit (x_{t+1} = x_t + delta in f64)
// Manifold arenas are double-buffered and swapped on the host after each step.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/avbd_cuda.h"
#include "avbd_device.cuh"

using namespace avbd;

namespace avbd {
int tangent_pack(TangentCtx **out, const avbd_world *world, const avbd_params &P, const avbd_tangent_seed *seeds,
                 int nSeeds, char *msg, size_t msgLen, cudaStream_t st);
}

namespace {

const char *g_create_error = "";
std::string g_create_error_buf;

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
};

}  // namespace


struct avbd_ctx {
  avbd_params params{};
  cudaStream_t stream = nullptr;
  int device = 0;
  int smCount = 0;
  std::string err;
  bool packed = false;
  bool profiling = false;
  int64_t launches = 0;
  int steps = 0;
  std::vector<void *> allocs;

  // sizes
  int n = 0, nj = 0, ns = 0, numScenes = 1, numLarge = 0;
  int candCap = 0, entryCap = 0, tableSize = 0, adjCap = 0, colorBlocks = 0;
  int lanes = 8, blocksPerSm = 1;
  size_t bpTempBytes = 0, svTempBytes = 0;
  void *bpTemp = nullptr, *svTemp = nullptr;
  double *statsOut = nullptr;
  World w{};
  Manifolds mA{}, mB{};
  int curIsA = 1;
  avbd_profile prof{};
  cudaEvent_t ev[8]{};
  // the per-step body state as the caller's f64 arrays, on the device: pos
  // (3n), quat (4n), vel, omega, prev_vel (3n each), and the first body with
  // a non-finite position of an upload (hBad: its pinned copy)
  double *d64 = nullptr;
  int *dBad = nullptr, *hBad = nullptr;
  // of the latest completed step (pinned, written by the stream): [0] steps
  // skipped for a candidate overflow since the last regrow, [1] candidates
  int *hCand = nullptr;
  bool autoLanes = false;  // lanes_per_body 0: chosen per body by the colouring
  int nDyn = 0;
  std::vector<void *> growable;  // arenas sized by the candidate capacity
  int64_t regrows = 0;
  int *colorOverride = nullptr;  // device copy of an uploaded colouring (n)
  // The host runs at most kRunAhead steps ahead of the device, so the
  // candidate count the regrow check reads is at most that many steps old.
  static constexpr int kRunAhead = 4;
  cudaEvent_t stepEv[8]{};
  int64_t stepSeq = 0;
  // CUDA graphs of one step, one per manifold-arena parity (the arenas swap
  // every step, and their pointers are part of the launches' arguments);
  // rebuilt after anything that changes a launch (pack, regrow, an uploaded
  // colouring, a new schedule)
  cudaGraphExec_t graphExec[2]{};
  bool graphFailed = false;  // a capture failed: this context launches directly
  int stepKernels = 0;       // own kernels of one step (the launch count)
  int64_t graphSteps = 0;    // steps run as a graph
  int maxBlocksPerSm = 1;    // resident solve blocks per SM at most
  bool capturing = false;    // a graph capture is recording the step
  bool lastViaGraph = false; // the last step ran as a graph
  TangentCtx *tangent = nullptr;  // the differentiable step (avbd_adjoint_forward)
  void *tanTemp = nullptr;
  size_t tanTempBytes = 0;
};

namespace {

int fail(avbd_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(ctx, AVBD_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(avbd_ctx *ctx, T **p, size_t count) {
  void *q = nullptr;
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return fail(ctx, AVBD_ERR_CUDA, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  cudaMemset(q, 0, bytes);
  ctx->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return AVBD_OK;
}

template <class T>
int galloc(avbd_ctx *ctx, T **p, size_t count) {
  int rc = dalloc(ctx, p, count);
  if (rc) return rc;
  ctx->allocs.pop_back();
  ctx->growable.push_back(*p);
  return AVBD_OK;
}

template <class T>
int upload(avbd_ctx *ctx, T **p, const std::vector<T> &h) {
  int rc = dalloc(ctx, p, h.size());
  if (rc) return rc;
  if (!h.empty()) CK(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
  return AVBD_OK;
}

void invalidate_graphs(avbd_ctx *ctx);

void free_all(avbd_ctx *ctx) {
  invalidate_graphs(ctx);
  for (void *p : ctx->allocs) cudaFree(p);
  ctx->allocs.clear();
  for (void *p : ctx->growable) cudaFree(p);
  ctx->growable.clear();
  if (ctx->hCand) cudaFreeHost(ctx->hCand);
  ctx->hCand = nullptr;
  if (ctx->hBad) cudaFreeHost(ctx->hBad);
  ctx->hBad = nullptr;
  ctx->d64 = nullptr;  // (in allocs)
  ctx->dBad = nullptr;
  ctx->packed = false;
}

void set_world_manifolds(avbd_ctx *ctx) {
  ctx->w.cur = ctx->curIsA ? ctx->mA : ctx->mB;
  ctx->w.prev = ctx->curIsA ? ctx->mB : ctx->mA;
}

int alloc_manifolds(avbd_ctx *ctx, Manifolds &m, int cap) {
  int rc = 0;
  m.cap = cap;
  const size_t S = (size_t)cap * kMaxContacts;
  if ((rc = galloc(ctx, &m.key, cap)) || (rc = galloc(ctx, &m.count, cap)) || (rc = galloc(ctx, &m.basis0, cap)) ||
      (rc = galloc(ctx, &m.basis1, cap)) || (rc = galloc(ctx, &m.basis2, cap)) ||
      (rc = galloc(ctx, &m.basisD, (size_t)cap * 9)) || (rc = galloc(ctx, &m.feat, S)) ||
      (rc = galloc(ctx, &m.rA, S)) || (rc = galloc(ctx, &m.rB, S)) || (rc = galloc(ctx, &m.cA, S)) ||
      (rc = galloc(ctx, &m.cB, S)) || (rc = galloc(ctx, &m.cK, S)) || (rc = galloc(ctx, &m.cL, S)) ||
      (rc = galloc(ctx, &m.cX, S)))
    return rc;
  return AVBD_OK;
}

// Arenas whose size follows the candidate capacity: both manifold buffers,
// the candidate keys and the per-body adjacency.
int alloc_candidate_arenas(avbd_ctx *ctx, int cap) {
  int rc;
  World &w = ctx->w;
  ctx->candCap = cap;
  ctx->adjCap = (int)std::min<long long>(2LL * cap, 0x3fffffff);
  w.g.candCap = cap;
  w.a.cap = ctx->adjCap;
  w.a.ccap = (int)std::min<long long>(2LL * kMaxContacts * cap, 0x7fffffff);
  if ((rc = alloc_manifolds(ctx, ctx->mA, cap)) || (rc = alloc_manifolds(ctx, ctx->mB, cap)) ||
      (rc = galloc(ctx, &w.g.candKey, cap)) || (rc = galloc(ctx, &w.g.candPrev, cap)) ||
      (rc = galloc(ctx, &w.g.npFace, cap)) || (rc = galloc(ctx, &w.g.npEdge, cap)) ||
      (rc = galloc(ctx, &w.g.npExact, cap)) ||
      (rc = galloc(ctx, &w.a.entry, ctx->adjCap)) || (rc = galloc(ctx, &w.a.hpEntry, ctx->adjCap)) ||
      (rc = galloc(ctx, &w.a.centry, w.a.ccap)))
    return rc;
  return AVBD_OK;
}

// Arena regrow (src/physics/gpu/backend.js:1683-1739): the candidate arenas
// are reallocated with `cap` slots and the manifolds of the step that has
// been stepped last (`old`, `keep` of them: the warm-start state of the next
// step) move into the new "previous" arena.
int grow_arenas(avbd_ctx *ctx, int cap, const Manifolds old, int keep) {
  invalidate_graphs(ctx);
  std::vector<void *> oldBufs;
  oldBufs.swap(ctx->growable);
  int rc = alloc_candidate_arenas(ctx, cap);
  if (rc) {
    for (void *p : oldBufs) cudaFree(p);
    return rc;
  }
  ctx->curIsA = 1;  // the new "previous" arena is mB
  Manifolds &pm = ctx->mB;
  const size_t K = kMaxContacts;
  if (keep > 0) {
    CK(cudaMemcpy(pm.key, old.key, keep * sizeof(uint64_t), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.count, old.count, keep * sizeof(int), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.basis0, old.basis0, keep * sizeof(float4), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.basis1, old.basis1, keep * sizeof(float4), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.basis2, old.basis2, keep * sizeof(float4), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.basisD, old.basisD, keep * 9 * sizeof(double), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.feat, old.feat, keep * K * sizeof(uint32_t), cudaMemcpyDeviceToDevice));
    float4 *dst[6] = {pm.rA, pm.rB, pm.cA, pm.cB, pm.cK, pm.cL};
    float4 *src[6] = {old.rA, old.rB, old.cA, old.cB, old.cK, old.cL};
    for (int k = 0; k < 6; k++) CK(cudaMemcpy(dst[k], src[k], keep * K * sizeof(float4), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(pm.cX, old.cX, keep * K * sizeof(float), cudaMemcpyDeviceToDevice));
  }
  CK(cudaDeviceSynchronize());
  for (void *p : oldBufs) cudaFree(p);
  set_world_manifolds(ctx);
  ctx->regrows++;
  return AVBD_OK;
}

int one_step(avbd_ctx *ctx);

// Steps skipped for a candidate overflow (Control::skip): the arenas grow to
// twice what the broad phase asked for, the manifolds of the last step that
// did run become the warm-start state again, and the skipped steps are queued
// once more. The state of a skipped step is the state before it, so the
// result equals a run whose arenas were large enough from the start.
int resolve_skips(avbd_ctx *ctx) {
  for (int round = 0; round < 4; round++) {
    CK(cudaStreamSynchronize(ctx->stream));
    // the stream copied each step's skip count to hCand[0] (pinned): nothing
    // skipped, nothing to read back
    if (round == 0 && ctx->hCand[0] <= 0) return AVBD_OK;
    Control c{};
    CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    ctx->hCand[0] = 0;
    if (c.stepsSkipped <= 0) return AVBD_OK;
    const int S = c.stepsSkipped;
    // the host flipped the arenas once per queued step; the first skipped step
    // found the valid warm-start manifolds in its "previous" arena
    const bool firstCurIsA = (ctx->curIsA ^ (S & 1)) != 0;
    const Manifolds valid = firstCurIsA ? ctx->mB : ctx->mA;
    const long long want = std::max<long long>(c.wantCandidates, ctx->candCap);
    const int cap = (int)std::min<long long>(std::max<long long>(2LL * want, 2LL * ctx->candCap), 0x3fffffff);
    if (cap <= ctx->candCap)
      return fail(ctx, AVBD_ERR_CAPACITY, "%lld candidate pairs exceed the largest arena (%d)", want, ctx->candCap);
    int rc = grow_arenas(ctx, cap, valid, c.prevCandidates);
    if (rc) return rc;
    c.skip = 0;
    c.stepsSkipped = 0;
    c.flags &= ~kOvfPairs;
    CK(cudaMemcpy(ctx->w.ctl, &c, sizeof(Control), cudaMemcpyHostToDevice));
    ctx->steps -= S;
    for (int k = 0; k < S; k++) {
      rc = one_step(ctx);
      if (rc) return rc;
    }
  }
  return fail(ctx, AVBD_ERR_CAPACITY, "candidate arena overflow persists after regrowing");
}

// Regrow ahead of overflow: when the last completed step used more than 70%
// of the candidate capacity, the arenas double and the previous step's
// manifolds (the warm-start state) move into the new ones. A step that did
// overflow has been skipped: resolve_skips regrows and steps it again.
int maybe_regrow(avbd_ctx *ctx) {
  if (*((volatile int *)&ctx->hCand[0]) > 0) return resolve_skips(ctx);
  const int last = *((volatile int *)&ctx->hCand[1]);
  if (last * 10LL <= ctx->candCap * 7LL) return AVBD_OK;
  CK(cudaStreamSynchronize(ctx->stream));
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  if (c.stepsSkipped > 0) return resolve_skips(ctx);
  const Manifolds old = ctx->curIsA ? ctx->mB : ctx->mA;  // last step's arena
  const int cap = (int)std::min<long long>(std::max<long long>(2LL * ctx->candCap, 2LL * last), 0x3fffffff);
  return grow_arenas(ctx, cap, old, c.prevCandidates);
}

inline uint32_t priority_of(uint32_t local) { return color_priority(local); }

bool finite3(const double *p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }


int record(avbd_ctx *ctx, int k) {
  if (ctx->profiling && !ctx->capturing) CK(cudaEventRecord(ctx->ev[k], ctx->stream));
  return AVBD_OK;
}

// Upload the dynamic state (bodies, joints, springs, and manifolds when
// given) of `world` into already-sized arenas.
// The body state between the caller's f64 arrays (copied as they are) and
// the device layout: positions D4, the rest float4 (round to nearest, as a
// host (float) cast), absent arrays as the host path defaulted them.
__global__ void state_check_kernel(const double *pos, int n, int *bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!(isfinite(pos[i * 3]) && isfinite(pos[i * 3 + 1]) && isfinite(pos[i * 3 + 2]))) atomicMin(bad, i);
}
__global__ void state_in_kernel(const double *d64, int n, unsigned present, const int *bad, D4 *pos, float4 *quat,
                                float4 *vel, float4 *omega, float4 *prev) {
  if (*bad < n) return;  // a non-finite position: the state stays as it was
  const double *p = d64, *q = d64 + 3 * (size_t)n, *v = q + 4 * (size_t)n, *om = v + 3 * (size_t)n,
               *pv = om + 3 * (size_t)n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    pos[i] = mkd4(p[i * 3], p[i * 3 + 1], p[i * 3 + 2], 0.0);
    quat[i] = present & 1u ? make_float4((float)q[i * 4], (float)q[i * 4 + 1], (float)q[i * 4 + 2], (float)q[i * 4 + 3])
                           : make_float4(0.f, 0.f, 0.f, 1.f);
    const float4 vv = present & 2u ? make_float4((float)v[i * 3], (float)v[i * 3 + 1], (float)v[i * 3 + 2], 0.f)
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
    vel[i] = vv;
    omega[i] = present & 4u ? make_float4((float)om[i * 3], (float)om[i * 3 + 1], (float)om[i * 3 + 2], 0.f)
                            : make_float4(0.f, 0.f, 0.f, 0.f);
    prev[i] = present & 8u ? make_float4((float)pv[i * 3], (float)pv[i * 3 + 1], (float)pv[i * 3 + 2], 0.f) : vv;
  }
}
__global__ void state_out_kernel(const D4 *pos, const float4 *quat, const float4 *vel, const float4 *omega,
                                 const float4 *prev, int n, double *d64) {
  double *p = d64, *q = d64 + 3 * (size_t)n, *v = q + 4 * (size_t)n, *om = v + 3 * (size_t)n, *pv = om + 3 * (size_t)n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const D4 a = pos[i];
    p[i * 3] = a.x; p[i * 3 + 1] = a.y; p[i * 3 + 2] = a.z;
    const float4 b = quat[i];
    q[i * 4] = b.x; q[i * 4 + 1] = b.y; q[i * 4 + 2] = b.z; q[i * 4 + 3] = b.w;
    const float4 c = vel[i], d = omega[i], e = prev[i];
    v[i * 3] = c.x; v[i * 3 + 1] = c.y; v[i * 3 + 2] = c.z;
    om[i * 3] = d.x; om[i * 3 + 1] = d.y; om[i * 3 + 2] = d.z;
    pv[i * 3] = e.x; pv[i * 3 + 1] = e.y; pv[i * 3 + 2] = e.z;
  }
}

int write_state(avbd_ctx *ctx, const avbd_world *world, bool keepManifolds) {
  const avbd_body_soa &B = world->bodies;
  const int n = ctx->n;
  World &w = ctx->w;
  cudaStream_t st = ctx->stream;
  {  // the caller's arrays straight to the device (GB300: host memory over NVLink-C2C), converted there
    const size_t N = (size_t)n;
    double *p = ctx->d64, *q = p + 3 * N, *v = q + 4 * N, *om = v + 3 * N, *pv = om + 3 * N;
    const unsigned present = (B.quat ? 1u : 0u) | (B.vel ? 2u : 0u) | (B.omega ? 4u : 0u) | (B.prev_vel ? 8u : 0u);
    CK(cudaMemcpyAsync(p, B.pos, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    if (B.quat) CK(cudaMemcpyAsync(q, B.quat, 4 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    if (B.vel) CK(cudaMemcpyAsync(v, B.vel, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    if (B.omega) CK(cudaMemcpyAsync(om, B.omega, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    if (B.prev_vel) CK(cudaMemcpyAsync(pv, B.prev_vel, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(ctx->dBad, 0x7f, sizeof(int), st));  // 0x7f7f7f7f: above any body index
    const int grid = std::max(1, std::min((n + 255) / 256, ctx->smCount * 4));
    state_check_kernel<<<grid, 256, 0, st>>>(p, n, ctx->dBad);
    state_in_kernel<<<grid, 256, 0, st>>>(ctx->d64, n, present, ctx->dBad, w.b.pos, w.b.quat, w.b.vel, w.b.omega,
                                          w.b.prevVel);
    CK(cudaMemcpyAsync(ctx->hBad, ctx->dBad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    if (*ctx->hBad < n) return fail(ctx, AVBD_ERR_NAN, "body %d: non-finite position", *ctx->hBad);
  }

  const avbd_joint_soa &J = world->joints;
  if (ctx->nj) {
    std::vector<float4> kl(ctx->nj), ka(ctx->nj);
    std::vector<D4> ll(ctx->nj), la(ctx->nj);
    std::vector<int> st(ctx->nj);
    for (int j = 0; j < ctx->nj; j++) {
      auto f = [&](const double *a) { return a ? make_float4((float)a[j * 3], (float)a[j * 3 + 1], (float)a[j * 3 + 2], 0.f)
                                               : make_float4(0, 0, 0, 0); };
      auto d = [&](const double *a) { return a ? mkd4(a[j * 3], a[j * 3 + 1], a[j * 3 + 2], 0.0)
                                               : mkd4(0, 0, 0, 0); };
      kl[j] = f(J.penalty_lin);
      ka[j] = f(J.penalty_ang);
      ll[j] = d(J.lambda_lin);
      la[j] = d(J.lambda_ang);
      // a broken joint is warm-started once more by the next step, then leaves
      // the force list (Joint.initialize, src/physics/joint.js:131-160)
      st[j] = (J.broken && J.broken[j]) ? kBroken : 0;
    }
    CK(cudaMemcpy(w.j.penLin, kl.data(), ctx->nj * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.j.penAng, ka.data(), ctx->nj * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.j.lamLin, ll.data(), ctx->nj * sizeof(D4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.j.lamAng, la.data(), ctx->nj * sizeof(D4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.j.state, st.data(), ctx->nj * sizeof(int), cudaMemcpyHostToDevice));
  }
  const avbd_spring_soa &S = world->springs;
  if (ctx->ns) {
    std::vector<float> pen(ctx->ns);
    std::vector<double> peak(ctx->ns);
    std::vector<int> st(ctx->ns);
    for (int s = 0; s < ctx->ns; s++) {
      pen[s] = S.penalty ? (float)S.penalty[s] : 0.f;
      peak[s] = S.peak_strain ? S.peak_strain[s] : 0.0;
      st[s] = (S.broken && S.broken[s]) ? kBroken : 0;
    }
    CK(cudaMemcpy(w.s.penalty, pen.data(), ctx->ns * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.s.peak, peak.data(), ctx->ns * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(w.s.state, st.data(), ctx->ns * sizeof(int), cudaMemcpyHostToDevice));
  }

  // warm-start manifolds -> the "previous step" arena, sorted by pair key
  const avbd_manifold_soa &M = world->manifolds;
  int live = 0;
  Manifolds &pm = ctx->curIsA ? ctx->mB : ctx->mA;
  if (M.count > 0) {
    if (M.count > ctx->candCap) return fail(ctx, AVBD_ERR_CAPACITY, "%d manifolds exceed capacity %d", M.count, ctx->candCap);
    std::vector<int> idx;
    for (int m = 0; m < M.count; m++) {
      const int a = M.body_a[m], b = M.body_b[m];
      if (a <= b || a >= n || b < 0) return fail(ctx, AVBD_ERR_ARG, "manifold %d: body_a must exceed body_b", m);
      if (M.num_contacts[m] > 0) idx.push_back(m);
    }
    std::sort(idx.begin(), idx.end(), [&](int x, int y) {
      return ((uint64_t)M.body_a[x] << 32 | (uint32_t)M.body_b[x]) < ((uint64_t)M.body_a[y] << 32 | (uint32_t)M.body_b[y]);
    });
    live = (int)idx.size();
    const size_t K = kMaxContacts;
    std::vector<uint64_t> key(live);
    std::vector<int> cnt(live);
    std::vector<double> basisD((size_t)live * 9);
    std::vector<uint32_t> feat(live * K, 0);
    std::vector<float4> rA(live * K), rB(live * K), cK(live * K), cL(live * K);
    std::vector<float> cX(live * K, 0.f);
    std::vector<float4> cA(live * K, make_float4(0.f, 0.f, 0.f, 0.f));  // .w: C0 on the normal
    for (int t = 0; t < live; t++) {
      const int m = idx[t];
      key[t] = (uint64_t)M.body_a[m] << 32 | (uint32_t)M.body_b[m];
      cnt[t] = std::min(M.num_contacts[m], (int)K);
      for (int k = 0; k < 9; k++) basisD[t * 9 + k] = M.basis ? M.basis[m * 9 + k] : 0.0;
      for (size_t s = 0; s < K; s++) {
        const size_t src = (size_t)m * K + s, dst = (size_t)t * K + s;
        feat[dst] = M.feature ? M.feature[src] : 0u;
        auto f3 = [&](const double *a, float wv) {
          return a ? make_float4((float)a[src * 3], (float)a[src * 3 + 1], (float)a[src * 3 + 2], wv) : make_float4(0, 0, 0, wv);
        };
        rA[dst] = f3(M.r_a, 0.f);
        rB[dst] = f3(M.r_b, 0.f);
        cK[dst] = f3(M.penalty, 0.f);
        cL[dst] = f3(M.lambda, (M.stick && M.stick[src]) ? 1.f : 0.f);
        cX[dst] = M.restitution_bias ? (float)M.restitution_bias[src] : 0.f;
        cA[dst].w = M.c0 ? (float)M.c0[src * 3] : 0.f;  // re-arms restitution (AVBD_CONTACT_MATERIALS)
      }
    }
    CK(cudaMemcpy(pm.key, key.data(), live * sizeof(uint64_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.count, cnt.data(), live * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.basisD, basisD.data(), basisD.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.feat, feat.data(), feat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.rA, rA.data(), rA.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.rB, rB.data(), rB.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.cK, cK.data(), cK.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.cL, cL.data(), cL.size() * sizeof(float4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.cX, cX.data(), cX.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(pm.cA, cA.data(), cA.size() * sizeof(float4), cudaMemcpyHostToDevice));
  }
  if (M.count > 0 || !keepManifolds) {
    Control c{};
    CK(cudaMemcpy(&c, w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    c.prevCandidates = live;
    c.numCandidates = 0;
    CK(cudaMemcpy(w.ctl, &c, sizeof(Control), cudaMemcpyHostToDevice));
  }
  return AVBD_OK;
}

// Lanes per body of the wavefront schedule (launch_solve's argument); the
// colour-phase schedule takes each body's lanes from the colouring's layout.
int wave_lanes(const avbd_ctx *ctx) { return ctx->autoLanes ? 32 : ctx->lanes; }

void invalidate_graphs(avbd_ctx *ctx) {
  for (auto &g : ctx->graphExec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// The launch sequence of one step on the context's stream (what a graph
// captures); the profiling events between the phases only when profiling.
int enqueue_step(avbd_ctx *ctx) {
  World &w = ctx->w;
  cudaStream_t st = ctx->stream;
  // per-step counters: numCandidates .. adjTotal
  CK(cudaMemsetAsync(&w.ctl->numCandidates, 0, sizeof(int) * 7, st));
  int rc;
  if ((rc = record(ctx, 0))) return rc;
  launch_broadphase_impl(w, ctx->numLarge, ctx->bpTemp, ctx->bpTempBytes, st, ctx->smCount);
  if ((rc = record(ctx, 1))) return rc;
  launch_narrowphase(w, st, ctx->smCount);
  if ((rc = record(ctx, 2))) return rc;
  launch_prepare(w, ctx->svTemp, ctx->svTempBytes, st, ctx->smCount);
  if ((rc = record(ctx, 3))) return rc;
  CK(launch_coloring(w, st, ctx->colorBlocks));
  if ((rc = record(ctx, 4))) return rc;
  CK(launch_solve(w, wave_lanes(ctx), ctx->blocksPerSm, st, ctx->smCount));
  if ((rc = record(ctx, 5))) return rc;
  launch_commit(w, st, ctx->smCount);
  // (commit_kernel made this step's candidates the next step's previous
  // manifolds, unless the step was skipped)
  CK(cudaMemcpyAsync(ctx->hCand, &w.ctl->stepsSkipped, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  return record(ctx, 6);
}

// Own kernels of one step: broad phase 6 (+4 with large bodies; its two scans
// are library code), narrow phase 4, prepare 5, colouring 1 (+2 with an
// uploaded colouring), solve 1, commit 1.
int step_kernels(const avbd_ctx *ctx) {
  return 6 + (ctx->numLarge > 0 ? 4 : 0) + 4 + 5 + 1 + (ctx->w.a.colorOverride ? 2 : 0) + 1 + 1;
}

// One step as a CUDA graph (captured on first use for this arena parity).
// Returns false when graphs are off, profiling is on, or capture failed (the
// context then launches directly from now on).
bool launch_step_graph(avbd_ctx *ctx, int *rc) {
  *rc = AVBD_OK;
  if (!ctx->params.graph || ctx->graphFailed) return false;
  const int slot = ctx->curIsA ? 1 : 0;
  cudaStream_t st = ctx->stream;
  if (!ctx->graphExec[slot]) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      ctx->graphFailed = true;
      return false;
    }
    ctx->capturing = true;
    const int erc = enqueue_step(ctx);
    ctx->capturing = false;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    cudaGraphExec_t exec = nullptr;
    if (erc == AVBD_OK && e == cudaSuccess && g && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess) {
      ctx->graphExec[slot] = exec;
    } else {
      cudaGetLastError();  // a launch this stream cannot capture: launch directly
      ctx->graphFailed = true;
    }
    if (g) cudaGraphDestroy(g);
    if (ctx->graphFailed) return false;
  }
  const cudaError_t e = cudaGraphLaunch(ctx->graphExec[slot], st);
  if (e != cudaSuccess) *rc = fail(ctx, AVBD_ERR_CUDA, "cudaGraphLaunch: %s", cudaGetErrorString(e));
  ctx->graphSteps++;
  return true;
}

int one_step(avbd_ctx *ctx) {
  if (ctx->stepSeq >= avbd_ctx::kRunAhead)
    CK(cudaEventSynchronize(ctx->stepEv[(ctx->stepSeq - avbd_ctx::kRunAhead) % 8]));
  int rg = maybe_regrow(ctx);
  if (rg) return rg;
  World &w = ctx->w;
  set_world_manifolds(ctx);
  cudaStream_t st = ctx->stream;
  // a profiled graph step has the whole step's events only (no phase split)
  int rc = AVBD_OK;
  if (ctx->params.graph && !ctx->graphFailed && (rc = record(ctx, 0))) return rc;
  ctx->lastViaGraph = launch_step_graph(ctx, &rc);
  if (rc) return rc;
  if (ctx->lastViaGraph) rc = record(ctx, 6);
  else rc = enqueue_step(ctx);
  if (rc) return rc;
  ctx->launches += step_kernels(ctx);
  CK(cudaEventRecord(ctx->stepEv[ctx->stepSeq % 8], st));
  ctx->stepSeq++;
  CK(cudaGetLastError());
  ctx->curIsA ^= 1;
  ctx->steps++;
  if (ctx->profiling) {
    CK(cudaEventSynchronize(ctx->ev[6]));
    float t[5] = {0, 0, 0, 0, 0};
    if (!ctx->lastViaGraph)
      for (int k = 0; k < 5; k++) cudaEventElapsedTime(&t[k], ctx->ev[k], ctx->ev[k + 1]);
    ctx->prof.via_graph = ctx->lastViaGraph ? 1 : 0;
    ctx->prof.broadphase_ms = t[0];
    ctx->prof.narrowphase_ms = t[1];
    ctx->prof.prepare_ms = t[2];
    ctx->prof.coloring_ms = t[3];
    ctx->prof.solve_ms = t[4];
    float tot = 0;
    cudaEventElapsedTime(&tot, ctx->ev[0], ctx->ev[6]);
    ctx->prof.step_ms = tot;
    Control c{};
    CK(cudaMemcpy(&c, w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    if (c.stepsSkipped > 0) return resolve_skips(ctx);  // the step runs again (and is profiled then)
    ctx->prof.candidate_pairs = c.numCandidates;
    ctx->prof.manifolds = c.liveManifolds;
    ctx->prof.contacts = c.liveContacts;
    ctx->prof.colors = c.numColors;
    ctx->prof.fp64_bodies = c.fp64Bodies;
    ctx->prof.np_face = c.npCount[0];
    ctx->prof.np_edge = c.npCount[1];
    ctx->prof.np_exact = c.npCount[2];
    ctx->prof.lanes_per_body = ctx->params.schedule == 1 || !ctx->autoLanes
                                   ? wave_lanes(ctx)
                                   : (c.laneTotal + std::max(ctx->nDyn, 1) / 2) / std::max(ctx->nDyn, 1);
  }
  return AVBD_OK;
}

int check_flags(avbd_ctx *ctx) {
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  if (c.flags & kOvfTimeout)
    return fail(ctx, AVBD_ERR_TIMEOUT, "a device wait (grid barrier or neighbour progress) gave up; repack to continue");
  if (c.flags & (kOvfCells | kOvfPairs | kOvfAdj | kOvfColors)) {
    // grow the arenas that overflowed for the next pack; this state is invalid
    if (c.flags & kOvfPairs) ctx->params.max_pairs_per_body = std::max(ctx->params.max_pairs_per_body, 16) * 2;
    if (c.flags & kOvfAdj) ctx->params.max_adjacency = std::max(ctx->params.max_adjacency, 2) * 2;
    if (c.flags & kOvfCells) ctx->params.grid_factor = std::max(ctx->params.grid_factor, 1) * 2;
    return fail(ctx, AVBD_ERR_CAPACITY, "device arena overflow (flags 0x%x); capacities grown, repack to retry",
                c.flags);
  }
  if (c.flags & kErrNaN) return fail(ctx, AVBD_ERR_NAN, "non-finite body state produced");
  if (c.flags & kErrColoring) {  // reported once: the steps used their own colouring
    c.flags &= ~kErrColoring;
    CK(cudaMemcpy(&ctx->w.ctl->flags, &c.flags, sizeof(unsigned), cudaMemcpyHostToDevice));
    return fail(ctx, AVBD_ERR_ARG,
                "the uploaded colouring gives two neighbours one colour (or a colour >= %d) in this step's "
                "constraint graph; those steps used the device's own colouring",
                kMaxColors);
  }
  return AVBD_OK;
}

// --- autotuner --------------------------------------------------------------
// The device arrays a step changes, as (address, bytes): body state and
// colours (the colouring's seed), joint and spring state, the warm-start
// manifolds (`keep` of them, in the arena the next step reads) and the
// control block. Saved and put back around the tuner's trial steps.
std::vector<std::pair<void *, size_t>> mutable_regions(avbd_ctx *ctx, int keep) {
  World &w = ctx->w;
  const size_t n = ctx->n, nj = ctx->nj, ns = ctx->ns, K = kMaxContacts, m = keep;
  const Manifolds &pm = ctx->curIsA ? ctx->mB : ctx->mA;
  std::vector<std::pair<void *, size_t>> r = {
      {w.b.pos, n * sizeof(D4)}, {w.b.quat, n * sizeof(float4)}, {w.b.vel, n * sizeof(float4)},
      {w.b.omega, n * sizeof(float4)}, {w.b.prevVel, n * sizeof(float4)}, {w.b.color, n * sizeof(int)},
      {w.j.penLin, nj * sizeof(float4)}, {w.j.penAng, nj * sizeof(float4)}, {w.j.lamLin, nj * sizeof(D4)},
      {w.j.lamAng, nj * sizeof(D4)}, {w.j.state, nj * sizeof(int)}, {w.s.penalty, ns * sizeof(float)},
      {w.s.peak, ns * sizeof(double)}, {w.s.state, ns * sizeof(int)}, {pm.key, m * sizeof(uint64_t)},
      {pm.count, m * sizeof(int)}, {pm.basis0, m * sizeof(float4)}, {pm.basis1, m * sizeof(float4)},
      {pm.basis2, m * sizeof(float4)}, {pm.basisD, m * 9 * sizeof(double)}, {pm.feat, m * K * sizeof(uint32_t)},
      {pm.rA, m * K * sizeof(float4)}, {pm.rB, m * K * sizeof(float4)}, {pm.cA, m * K * sizeof(float4)},
      {pm.cB, m * K * sizeof(float4)}, {pm.cK, m * K * sizeof(float4)}, {pm.cL, m * K * sizeof(float4)},
      {w.ctl, sizeof(Control)}};
  return r;
}

struct Snapshot {
  void *blob = nullptr;
  int keep = 0, steps = 0;
  ~Snapshot() {
    if (blob) cudaFree(blob);
  }
};

int take_snapshot(avbd_ctx *ctx, Snapshot &s) {
  int rc = resolve_skips(ctx);
  if (rc) return rc;
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  s.keep = c.prevCandidates;
  s.steps = ctx->steps;
  size_t total = 0;
  for (auto &r : mutable_regions(ctx, s.keep)) total += (r.second + 255) & ~size_t(255);
  CK(cudaMalloc(&s.blob, std::max<size_t>(total, 256)));
  size_t at = 0;
  for (auto &r : mutable_regions(ctx, s.keep)) {
    if (r.second) CK(cudaMemcpyAsync((char *)s.blob + at, r.first, r.second, cudaMemcpyDeviceToDevice, ctx->stream));
    at += (r.second + 255) & ~size_t(255);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return AVBD_OK;
}

int restore_snapshot(avbd_ctx *ctx, const Snapshot &s) {
  int rc = resolve_skips(ctx);
  if (rc) return rc;
  size_t at = 0;
  for (auto &r : mutable_regions(ctx, s.keep)) {
    if (r.second) CK(cudaMemcpyAsync(r.first, (char *)s.blob + at, r.second, cudaMemcpyDeviceToDevice, ctx->stream));
    at += (r.second + 255) & ~size_t(255);
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->hCand[0] = 0;
  ctx->hCand[1] = 0;
  ctx->steps = s.steps;
  return AVBD_OK;
}

struct TuneConfig {
  int schedule, lanes, tailDiv, blocksPerSm;
};

void apply_config(avbd_ctx *ctx, const TuneConfig &c) {
  avbd_params &P = ctx->params;
  P.schedule = c.schedule;
  P.lanes_per_body = c.lanes;
  P.tail_div = c.tailDiv;
  P.blocks_per_sm = c.blocksPerSm;
  ctx->w.p.schedule = c.schedule == 1 ? 1 : 0;
  ctx->w.p.lanes = c.lanes > 0 ? c.lanes : 0;
  ctx->w.p.tailDiv = c.tailDiv;
  ctx->autoLanes = c.lanes <= 0;
  ctx->lanes = c.lanes > 0 ? c.lanes : 32;
  ctx->blocksPerSm = c.blocksPerSm;
  ctx->w.p.solveBlocksPerSm = c.blocksPerSm;
  invalidate_graphs(ctx);
}

// Mean device time of `steps` steps from the snapshot's state (one untimed
// step first, which also captures the graphs), then the snapshot restored.
int time_config(avbd_ctx *ctx, const Snapshot &snap, int steps, double *ms) {
  int rc;
  if ((rc = restore_snapshot(ctx, snap)) || (rc = one_step(ctx)) || (rc = restore_snapshot(ctx, snap))) return rc;
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, ctx->stream));
  for (int k = 0; k < steps && !rc; k++) rc = one_step(ctx);
  cudaEventRecord(b, ctx->stream);
  cudaEventSynchronize(b);
  float t = 0;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if ((rc = check_flags(ctx))) return rc;
  *ms = t / std::max(steps, 1);
  return restore_snapshot(ctx, snap);
}

}  // namespace

extern "C" {

void avbd_default_params(avbd_params *o) {
  std::memset(o, 0, sizeof(*o));
  o->dt = 1.0 / 60.0;
  o->gravity = -10.0;
  o->iterations = 10;
  o->beta_lin = 1e4;
  o->beta_ang = 100;
  o->alpha = 0.95;
  o->gamma = 0.999;
  o->penalty_min = 1;
  o->penalty_max = 1e10;
  o->collision_margin = 0.01;
  o->stick_threshold = 1e-5;
  o->rotated_inertia = 1;
  o->spring_geometric_stiffness = 1;
  o->cached_contact_jacobians = 1;
  o->hash_threshold = 150;
  o->body_order = AVBD_ORDER_PRIORITY;
  o->fp64_ratio_threshold = 1e5;
  o->schedule = 0;
}

int avbd_create(const avbd_params *params, avbd_ctx **out) {
  if (!params || !out) {
    g_create_error = "avbd_create: NULL argument";
    return AVBD_ERR_ARG;
  }
  if (!(params->dt > 0) || params->iterations < 0) {
    g_create_error = "avbd_create: dt must be > 0 and iterations >= 0";
    return AVBD_ERR_ARG;
  }
  avbd_ctx *ctx = new avbd_ctx();
  ctx->params = *params;
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, ctx->device);
  int coop = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  for (int k = 0; k < 8 && e == cudaSuccess; k++) e = cudaEventCreate(&ctx->ev[k]);
  for (int k = 0; k < 8 && e == cudaSuccess; k++) e = cudaEventCreateWithFlags(&ctx->stepEv[k], cudaEventDisableTiming);
  if (e != cudaSuccess || !coop) {
    g_create_error_buf = std::string("avbd_create: ") + (e != cudaSuccess ? cudaGetErrorString(e)
                                                                          : "device lacks cooperative launch");
    g_create_error = g_create_error_buf.c_str();
    delete ctx;
    return AVBD_ERR_CUDA;
  }
  *out = ctx;
  return AVBD_OK;
}

int avbd_destroy(avbd_ctx *ctx) {
  if (!ctx) return AVBD_OK;
  cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  if (ctx->tangent) tangent_destroy(ctx->tangent);
  if (ctx->tanTemp) cudaFree(ctx->tanTemp);
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : ctx->stepEv)
    if (e) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return AVBD_OK;
}

int avbd_pack(avbd_ctx *ctx, const avbd_world *world) {
  if (!ctx || !world) return fail(ctx, AVBD_ERR_ARG, "avbd_pack: NULL argument");
  const avbd_body_soa &B = world->bodies;
  const int n = B.count;
  if (n <= 0 || !B.size || !B.mass || !B.moment || !B.radius || !B.friction || !B.pos)
    return fail(ctx, AVBD_ERR_ARG, "avbd_pack: bodies need count > 0 and size/mass/moment/radius/friction/pos");
  cudaStreamSynchronize(ctx->stream);
  free_all(ctx);
  ctx->colorOverride = nullptr;
  ctx->w.a.colorOverride = nullptr;
  ctx->n = n;
  ctx->nj = world->joints.count;
  ctx->ns = world->springs.count;
  // scenes
  std::vector<int> sceneStart;
  if (world->num_scenes > 1 && world->scene_start) {
    sceneStart.assign(world->scene_start, world->scene_start + world->num_scenes + 1);
  } else {
    sceneStart = {0, n};
  }
  const int S = (int)sceneStart.size() - 1;
  if (sceneStart.front() != 0 || sceneStart.back() != n)
    return fail(ctx, AVBD_ERR_ARG, "avbd_pack: scene_start must run from 0 to the body count");
  for (int s = 0; s < S; s++)
    if (sceneStart[s + 1] < sceneStart[s]) return fail(ctx, AVBD_ERR_ARG, "avbd_pack: scene_start not monotone");
  ctx->numScenes = S;
  std::vector<int> scene(n);
  for (int s = 0; s < S; s++)
    for (int i = sceneStart[s]; i < sceneStart[s + 1]; i++) scene[i] = s;

  // The broad phase's reach per body: the bounding radius, plus the contact
  // offset under AVBD_CONTACT_MATERIALS (pairs within the skin are candidates,
  // src/physics/gpu/shaders.js:440-442).
  const bool materials = ctx->params.contact_model == AVBD_CONTACT_MATERIALS;
  std::vector<double> reach(n);
  for (int i = 0; i < n; i++) {
    reach[i] = B.radius[i];
    if (materials) {
      const double co = B.contact_offset ? B.contact_offset[i] : ctx->params.contact_offset;
      if (!(co >= 0) || !std::isfinite(co)) return fail(ctx, AVBD_ERR_ARG, "body %d: contact offset must be >= 0", i);
      reach[i] = B.radius[i] + co;
      const int shape = B.shape ? B.shape[i] : AVBD_SHAPE_BOX;
      if (shape == AVBD_SHAPE_SPHERE && B.radius[i] != B.size[i * 3] * 0.5)
        return fail(ctx, AVBD_ERR_ARG, "body %d: a sphere's radius must be half its size (Rigid.sphere)", i);
    }
  }

  // static body tables
  std::vector<D4> size(n), massD(n);
  std::vector<float4> massF(n);
  std::vector<double> friction(n), invCell(S);
  std::vector<int> flags0(n);
  std::vector<uint32_t> prio(n);
  std::vector<std::vector<int>> large(S);
  for (int s = 0; s < S; s++) {
    // Large bodies: bounding radius above twice the scene's 95th-percentile
    // radius (a ground box, a wrecking ball). Grid cell: twice the largest
    // remaining radius, padded so rounding cannot separate overlapping bodies
    // by more than one cell.
    const int cnt = sceneStart[s + 1] - sceneStart[s];
    std::vector<double> radii(reach.begin() + sceneStart[s], reach.begin() + sceneStart[s + 1]);
    double r95 = 1.0;
    if (cnt > 0) {
      const size_t k = std::min<size_t>((size_t)(0.95 * (cnt - 1)), (size_t)cnt - 1);
      std::nth_element(radii.begin(), radii.begin() + k, radii.end());
      r95 = radii[k];
    }
    const double thr = 2.0 * r95;
    double rmax = 0;
    for (int i = sceneStart[s]; i < sceneStart[s + 1]; i++)
      if (reach[i] <= thr) rmax = std::max(rmax, reach[i]);
    const double cell = std::max(2.0 * rmax * (1.0 + 1e-6) + 1e-9, 1e-4);
    invCell[s] = 1.0 / cell;
    for (int i = sceneStart[s]; i < sceneStart[s + 1]; i++) {
      const int shape = B.shape ? B.shape[i] : AVBD_SHAPE_BOX;
      if (!(B.mass[i] >= 0) || !std::isfinite(B.mass[i]))
        return fail(ctx, AVBD_ERR_ARG, "body %d: mass must be finite and >= 0", i);
      if (!(B.radius[i] >= 0) || !std::isfinite(B.radius[i]))
        return fail(ctx, AVBD_ERR_ARG, "body %d: radius must be finite and >= 0", i);
      size[i] = mkd4(B.size[i * 3], B.size[i * 3 + 1], B.size[i * 3 + 2], reach[i]);
      massD[i] = mkd4(B.mass[i], B.moment[i * 3], B.moment[i * 3 + 1], B.moment[i * 3 + 2]);
      massF[i] = make_float4((float)B.mass[i], (float)B.moment[i * 3], (float)B.moment[i * 3 + 1],
                             (float)B.moment[i * 3 + 2]);
      friction[i] = B.friction[i];
      int f = 0;
      if (B.mass[i] > 0) f |= kBodyDynamic;
      if (shape == AVBD_SHAPE_SPHERE) f |= kBodySphere;
      if (reach[i] > thr) {
        f |= kBodyLarge;
        large[s].push_back(i);
      }
      flags0[i] = f;
      prio[i] = priority_of((uint32_t)(i - sceneStart[s]));
    }
  }
  std::vector<int> largeStart(S + 1, 0), largeList;
  for (int s = 0; s < S; s++) {
    largeStart[s] = (int)largeList.size();
    largeList.insert(largeList.end(), large[s].begin(), large[s].end());
  }
  largeStart[S] = (int)largeList.size();
  ctx->numLarge = (int)largeList.size();
  int maxChunks = 1;
  for (int li = 0; li < ctx->numLarge; li++) {
    const int a = largeList[li];
    const int lower = a - sceneStart[scene[a]];
    maxChunks = std::max(maxChunks, (lower + kLargeChunk - 1) / kLargeChunk);
  }

  // joints / springs
  const avbd_joint_soa &J = world->joints;
  const avbd_spring_soa &SP = world->springs;
  std::vector<int2> jb(ctx->nj), sb(ctx->ns);
  std::vector<D4> jrA(ctx->nj), jrB(ctx->nj), jst(ctx->nj), srA(ctx->ns), srB(ctx->ns), sprm(ctx->ns);
  std::vector<float4> jrAf(ctx->nj), jrBf(ctx->nj), srAf(ctx->ns), srBf(ctx->ns);
  std::vector<std::vector<uint32_t>> refs(n);
  for (int j = 0; j < ctx->nj; j++) {
    const int a = J.body_a[j], b = J.body_b[j];
    if (b < 0 || b >= n || a >= n || a == b) return fail(ctx, AVBD_ERR_ARG, "joint %d: bad body indices", j);
    if (a >= 0 && scene[a] != scene[b]) return fail(ctx, AVBD_ERR_ARG, "joint %d crosses scenes", j);
    jb[j] = make_int2(a, b);
    jrA[j] = mkd4(J.r_a[j * 3], J.r_a[j * 3 + 1], J.r_a[j * 3 + 2], 0);
    jrB[j] = mkd4(J.r_b[j * 3], J.r_b[j * 3 + 1], J.r_b[j * 3 + 2], 0);
    jrAf[j] = make_float4((float)jrA[j].x, (float)jrA[j].y, (float)jrA[j].z, 0);
    jrBf[j] = make_float4((float)jrB[j].x, (float)jrB[j].y, (float)jrB[j].z, 0);
    // torqueArm = |size_A + size_B|^2 (joint.js:108-112)
    const double sx = (a >= 0 ? B.size[a * 3] : 0) + B.size[b * 3];
    const double sy = (a >= 0 ? B.size[a * 3 + 1] : 0) + B.size[b * 3 + 1];
    const double sz = (a >= 0 ? B.size[a * 3 + 2] : 0) + B.size[b * 3 + 2];
    jst[j] = mkd4(J.stiffness_lin[j], J.stiffness_ang[j], J.fracture[j], sx * sx + sy * sy + sz * sz);
    if (a >= 0) refs[a].push_back(make_ref(kRefJoint, j, 0));
    refs[b].push_back(make_ref(kRefJoint, j, 1));
  }
  for (int s = 0; s < ctx->ns; s++) {
    const int a = SP.body_a[s], b = SP.body_b[s];
    if (a < 0 || b < 0 || a >= n || b >= n || a == b) return fail(ctx, AVBD_ERR_ARG, "spring %d: bad body indices", s);
    if (scene[a] != scene[b]) return fail(ctx, AVBD_ERR_ARG, "spring %d crosses scenes", s);
    if (!(SP.rest[s] >= 0)) return fail(ctx, AVBD_ERR_ARG, "spring %d: rest length must be resolved (>= 0)", s);
    sb[s] = make_int2(a, b);
    srA[s] = mkd4(SP.r_a[s * 3], SP.r_a[s * 3 + 1], SP.r_a[s * 3 + 2], 0);
    srB[s] = mkd4(SP.r_b[s * 3], SP.r_b[s * 3 + 1], SP.r_b[s * 3 + 2], 0);
    srAf[s] = make_float4((float)srA[s].x, (float)srA[s].y, (float)srA[s].z, 0);
    srBf[s] = make_float4((float)srB[s].x, (float)srB[s].y, (float)srB[s].z, 0);
    sprm[s] = mkd4(SP.stiffness[s], SP.rest[s], SP.tear_strain ? SP.tear_strain[s] : INFINITY, 0);
    refs[a].push_back(make_ref(kRefSpring, s, 0));
    refs[b].push_back(make_ref(kRefSpring, s, 1));
  }
  std::vector<int> cStart(n + 1, 0);
  std::vector<uint32_t> cRef;
  for (int i = 0; i < n; i++) {
    cStart[i] = (int)cRef.size();
    cRef.insert(cRef.end(), refs[i].begin(), refs[i].end());
  }
  cStart[n] = (int)cRef.size();

  // capacities: one grid insertion per regular body
  long long insertions = 0;
  for (int i = 0; i < n; i++)
    if (!(flags0[i] & kBodyLarge)) insertions++;
  const int pairsPerBody = ctx->params.max_pairs_per_body > 0 ? ctx->params.max_pairs_per_body : 16;
  const int cellFactor = std::max(ctx->params.grid_factor, 1);
  ctx->candCap = (int)std::min<long long>((long long)n * pairsPerBody + 256 + world->manifolds.count, 0x3fffffff);
  ctx->entryCap = (int)std::min<long long>(insertions * 2 * cellFactor + 4096, 0x3fffffff);
  ctx->tableSize = 1024;
  while (ctx->tableSize < ctx->entryCap * 2) ctx->tableSize *= 2;

  World &w = ctx->w;
  w = World{};
  const avbd_params &P = ctx->params;
  w.p = SolverParams{P.dt, P.gravity, P.iterations, P.post_stabilize, P.beta_lin, P.beta_ang, P.alpha, P.gamma,
                     P.penalty_min, P.penalty_max, P.collision_margin, P.stick_threshold, P.rotated_inertia,
                     P.spring_stiffness_ramp, P.spring_geometric_stiffness, P.cached_contact_jacobians,
                     P.fp64_ratio_threshold, P.schedule == 1 ? 1 : 0, P.lanes_per_body > 0 ? P.lanes_per_body : 0, 1,
                     P.wait_limit > 0 ? (long long)P.wait_limit : 20000000LL,
                     P.neighbor_wait_limit > 0 ? (long long)P.neighbor_wait_limit
                                               : (P.wait_limit > 0 ? (long long)P.wait_limit : 4000000LL),
                     P.tail_div, P.contact_model == AVBD_CONTACT_MATERIALS ? 1 : 0,
                     P.restitution_threshold, P.contact_persistence};
  int rc = 0;
  D4 *sizeP, *massDP;
  float4 *massFP;
  double *fricP, *invCellP;
  float *cellFP;
  int *flags0P, *sceneP, *sceneStartP, *largeStartP, *largeListP, *cStartP;
  uint32_t *prioP, *cRefP;
  std::vector<float> cellF(S);
  for (int s = 0; s < S; s++) cellF[s] = (float)(1.0 / invCell[s]);
  if ((rc = upload(ctx, &sizeP, size)) || (rc = upload(ctx, &massDP, massD)) || (rc = upload(ctx, &massFP, massF)) ||
      (rc = upload(ctx, &fricP, friction)) || (rc = upload(ctx, &flags0P, flags0)) || (rc = upload(ctx, &sceneP, scene)) ||
      (rc = upload(ctx, &prioP, prio)) || (rc = upload(ctx, &invCellP, invCell)) || (rc = upload(ctx, &cellFP, cellF)) ||
      (rc = upload(ctx, &sceneStartP, sceneStart)) || (rc = upload(ctx, &largeStartP, largeStart)) ||
      (rc = upload(ctx, &largeListP, largeList)) || (rc = upload(ctx, &cStartP, cStart)) || (rc = upload(ctx, &cRefP, cRef)))
    return rc;
  w.b.n = n;
  w.b.mat = nullptr;
  w.b.contactOffset = nullptr;
  if (P.contact_model == AVBD_CONTACT_MATERIALS) {
    // contact materials (Rigid.setMaterial, src/physics/rigid.js:144-214)
    std::vector<D4> mat(n);
    std::vector<double> cofs(n);
    for (int i = 0; i < n; i++) {
      const double sf = B.static_friction ? B.static_friction[i] : B.friction[i];
      const double df = B.dynamic_friction ? B.dynamic_friction[i] : B.friction[i];
      const double e = B.restitution ? B.restitution[i] : 0.0;
      const double ro = B.rest_offset ? B.rest_offset[i] : P.rest_offset;
      const double co = B.contact_offset ? B.contact_offset[i] : P.contact_offset;
      if (!(sf >= 0) || !(df >= 0) || df > sf || !(e >= 0 && e <= 1) || !(co >= 0) || !std::isfinite(ro) ||
          !std::isfinite(sf) || !std::isfinite(co))
        return fail(ctx, AVBD_ERR_ARG, "body %d: contact material out of range (friction >= 0, dynamic <= static, "
                                       "restitution in [0, 1], contact offset >= 0, finite rest offset)", i);
      mat[i] = mkd4(sf, df, e, ro);
      cofs[i] = co;
    }
    D4 *matP;
    double *cofsP;
    if ((rc = upload(ctx, &matP, mat)) || (rc = upload(ctx, &cofsP, cofs))) return rc;
    w.b.mat = matP;
    w.b.contactOffset = cofsP;
  }
  w.b.size = sizeP; w.b.massD = massDP; w.b.massF = massFP; w.b.friction = fricP; w.b.flags0 = flags0P;
  w.b.scene = sceneP; w.b.priority = prioP;
  if ((rc = dalloc(ctx, &w.b.pos, n)) || (rc = dalloc(ctx, &w.b.quat, n)) || (rc = dalloc(ctx, &w.b.vel, n)) ||
      (rc = dalloc(ctx, &w.b.omega, n)) || (rc = dalloc(ctx, &w.b.prevVel, n)) || (rc = dalloc(ctx, &w.b.quatT, n)) ||
      (rc = dalloc(ctx, &w.b.dp, n)) || (rc = dalloc(ctx, &w.b.dang, n)) || (rc = dalloc(ctx, &w.b.yLin, n)) || (rc = dalloc(ctx, &w.b.yAng, n)) ||
      (rc = dalloc(ctx, &w.b.dpD, n)) || (rc = dalloc(ctx, &w.b.quatD, n)) || (rc = dalloc(ctx, &w.b.flags, n)) ||
      (rc = dalloc(ctx, &w.b.color, n)) || (rc = dalloc(ctx, &w.b.progress, n)))
    return rc;
  // joints
  w.j.n = ctx->nj;
  {
    int2 *jbP; D4 *a, *b, *c; float4 *af, *bf;
    if ((rc = upload(ctx, &jbP, jb)) || (rc = upload(ctx, &a, jrA)) || (rc = upload(ctx, &b, jrB)) ||
        (rc = upload(ctx, &c, jst)) || (rc = upload(ctx, &af, jrAf)) || (rc = upload(ctx, &bf, jrBf)))
      return rc;
    w.j.bodies = jbP; w.j.rAD = a; w.j.rBD = b; w.j.stiff = c; w.j.rAF = af; w.j.rBF = bf;
    if ((rc = dalloc(ctx, &w.j.penLin, ctx->nj)) || (rc = dalloc(ctx, &w.j.penAng, ctx->nj)) ||
        (rc = dalloc(ctx, &w.j.lamLin, ctx->nj)) || (rc = dalloc(ctx, &w.j.lamAng, ctx->nj)) ||
        (rc = dalloc(ctx, &w.j.c0Lin, ctx->nj)) || (rc = dalloc(ctx, &w.j.c0Ang, ctx->nj)) ||
        (rc = dalloc(ctx, &w.j.dpt, ctx->nj)) || (rc = dalloc(ctx, &w.j.dptD, ctx->nj)) ||
        (rc = dalloc(ctx, &w.j.state, ctx->nj)))
      return rc;
  }
  w.s.n = ctx->ns;
  {
    int2 *sbP; D4 *a, *b, *c; float4 *af, *bf;
    if ((rc = upload(ctx, &sbP, sb)) || (rc = upload(ctx, &a, srA)) || (rc = upload(ctx, &b, srB)) ||
        (rc = upload(ctx, &c, sprm)) || (rc = upload(ctx, &af, srAf)) || (rc = upload(ctx, &bf, srBf)))
      return rc;
    w.s.bodies = sbP; w.s.rAD = a; w.s.rBD = b; w.s.prm = c; w.s.rAF = af; w.s.rBF = bf;
    if ((rc = dalloc(ctx, &w.s.penalty, ctx->ns)) || (rc = dalloc(ctx, &w.s.peak, ctx->ns)) ||
        (rc = dalloc(ctx, &w.s.state, ctx->ns)) || (rc = dalloc(ctx, &w.s.dpt, ctx->ns)) ||
        (rc = dalloc(ctx, &w.s.dptD, ctx->ns)))
      return rc;
  }
  // grid
  w.g.numScenes = S;
  w.g.sceneStart = sceneStartP; w.g.invCell = invCellP; w.g.cellF = cellFP; w.g.largeStart = largeStartP; w.g.largeList = largeListP;
  w.g.maxChunks = maxChunks;
  if ((rc = dalloc(ctx, &w.g.largeChunk, (size_t)std::max(ctx->numLarge, 1) * maxChunks))) return rc;
  w.g.cStart = cStartP; w.g.cRef = cRefP;
  w.g.tableMask = (unsigned)(ctx->tableSize - 1);
  w.g.entryCap = ctx->entryCap;
  w.g.candCap = ctx->candCap;
  if ((rc = dalloc(ctx, &w.g.cellLo, n)) || (rc = dalloc(ctx, &w.g.loc, n)) ||
      (rc = dalloc(ctx, &w.g.tableCount, ctx->tableSize)) || (rc = dalloc(ctx, &w.g.tableStart, ctx->tableSize)) ||
      (rc = dalloc(ctx, &w.g.tableCursor, ctx->tableSize)) || (rc = dalloc(ctx, &w.g.entries, ctx->entryCap)) ||
      (rc = dalloc(ctx, &w.g.pairCount, n + 1)) || (rc = dalloc(ctx, &w.g.pairStart, n + 1)) ||
      (rc = dalloc(ctx, &w.g.scratch, (size_t)n * kPairScratch)))
    return rc;
  w.g.hasConstraints = (ctx->nj + ctx->ns) > 0 ? 1 : 0;
  // adjacency + colouring
  w.a.cap = ctx->adjCap;
  ctx->colorBlocks = std::max(1, coloring_grid(ctx->smCount));
  if ((rc = dalloc(ctx, &w.a.start, n + 1)) || (rc = dalloc(ctx, &w.a.count, n + 1)) ||
      (rc = dalloc(ctx, &w.a.hpCount, n)) ||
      (rc = dalloc(ctx, &w.a.cursor, n + 1)) || (rc = dalloc(ctx, &w.a.cstart, n + 1)) ||
      (rc = dalloc(ctx, &w.a.ccount, n + 1)) ||
      (rc = dalloc(ctx, &w.a.colorStart, kMaxColors + 1)) || (rc = dalloc(ctx, &w.a.colorBodies, n)) ||
      (rc = dalloc(ctx, &w.a.colorRec, n)) ||
      (rc = dalloc(ctx, &w.a.blockHist, (size_t)ctx->colorBlocks * kMaxColors)) ||
      (rc = dalloc(ctx, &w.a.laneTab, (size_t)kLaneMaxGroup * ((size_t)n + kMaxColors))) ||
      (rc = dalloc(ctx, &w.a.colorChunk, kMaxColors + 1)) ||
      (rc = dalloc(ctx, &w.a.laneHist, 2 * kMaxColors * kLaneBuckets + kMaxColors)))
    return rc;
  // manifolds (double-buffered), candidate keys, adjacency
  if ((rc = alloc_candidate_arenas(ctx, ctx->candCap))) return rc;
  CK(cudaMallocHost((void **)&ctx->hCand, 2 * sizeof(int)));
  ctx->hCand[0] = ctx->hCand[1] = 0;
  ctx->curIsA = 1;
  set_world_manifolds(ctx);
  if ((rc = dalloc(ctx, &w.ctl, 1)) || (rc = dalloc(ctx, &ctx->statsOut, 3)) || (rc = dalloc(ctx, &w.grab, 1)))
    return rc;
  CK(launch_set_grab(w, -1, nullptr, nullptr, 0.0, ctx->stream));  // nothing grabbed
  // scratch of the scans
  ctx->bpTempBytes = broadphase_temp_bytes(n, ctx->tableSize);
  ctx->svTempBytes = solver_temp_bytes(n);
  if ((rc = dalloc(ctx, (char **)&ctx->bpTemp, ctx->bpTempBytes)) || (rc = dalloc(ctx, (char **)&ctx->svTemp, ctx->svTempBytes)))
    return rc;
  // launch shape of the persistent solve
  const int maxPerSm = solve_max_blocks_per_sm(ctx->lanes);
  ctx->autoLanes = P.lanes_per_body <= 0;
  ctx->lanes = P.lanes_per_body > 0 ? P.lanes_per_body : 32;
  ctx->nDyn = 0;
  for (int i = 0; i < n; i++) ctx->nDyn += B.mass[i] > 0 ? 1 : 0;
  if (ctx->lanes != 1 && ctx->lanes != 2 && ctx->lanes != 4 && ctx->lanes != 8 && ctx->lanes != 16 && ctx->lanes != 32)
    return fail(ctx, AVBD_ERR_ARG, "lanes_per_body must be a power of two <= 32");
  ctx->blocksPerSm = P.blocks_per_sm > 0 ? std::min(P.blocks_per_sm, maxPerSm) : maxPerSm;
  ctx->maxBlocksPerSm = maxPerSm;
  if (ctx->blocksPerSm < 1) return fail(ctx, AVBD_ERR_CUDA, "solve kernel cannot be made resident");
  w.p.solveBlocksPerSm = ctx->blocksPerSm;
  // colours start at 0 for dynamic bodies
  CK(cudaMemset(w.b.color, 0, sizeof(int) * n));
  if ((rc = dalloc(ctx, &ctx->d64, (size_t)16 * n)) || (rc = dalloc(ctx, &ctx->dBad, 1))) return rc;
  CK(cudaMallocHost((void **)&ctx->hBad, sizeof(int)));
  // dalloc's zero fills run on the legacy default stream, which the context's
  // non-blocking stream does not wait for: finish them before the upload
  CK(cudaDeviceSynchronize());
  ctx->packed = true;
  ctx->stepSeq = 0;
  ctx->steps = 0;
  ctx->launches = 0;
  ctx->graphSteps = 0;
  ctx->graphFailed = false;
  rc = write_state(ctx, world, false);
  if (rc) return rc;
  CK(cudaDeviceSynchronize());
  return AVBD_OK;
}

int avbd_step(avbd_ctx *ctx, int32_t n_steps) {
  if (!ctx) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_step before avbd_pack");
  for (int s = 0; s < n_steps; s++) {
    int rc = one_step(ctx);
    if (rc) return rc;
  }
  return AVBD_OK;
}

int avbd_synchronize(avbd_ctx *ctx) {
  if (!ctx) return AVBD_ERR_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  if (!ctx->packed) return AVBD_OK;
  int rc = resolve_skips(ctx);
  if (rc) return rc;
  return check_flags(ctx);
}

int avbd_read_state(avbd_ctx *ctx, avbd_world *out) {
  if (!ctx || !out) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_read_state before avbd_pack");
  int rs = resolve_skips(ctx);  // steps skipped for an overflow run again first
  if (rs) return rs;
  const World &w = ctx->w;
  const int n = ctx->n;
  avbd_body_soa &B = out->bodies;
  if (B.count < n) return fail(ctx, AVBD_ERR_ARG, "avbd_read_state: body arrays hold %d < %d", B.count, n);
  cudaStream_t st = ctx->stream;
  {  // converted on the device, then straight into the caller's arrays
    const size_t N = (size_t)n;
    const double *p = ctx->d64, *q = p + 3 * N, *v = q + 4 * N, *om = v + 3 * N, *pv = om + 3 * N;
    const int grid = std::max(1, std::min((n + 255) / 256, ctx->smCount * 4));
    state_out_kernel<<<grid, 256, 0, st>>>(w.b.pos, w.b.quat, w.b.vel, w.b.omega, w.b.prevVel, n, ctx->d64);
    if (B.pos) CK(cudaMemcpyAsync(B.pos, p, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (B.quat) CK(cudaMemcpyAsync(B.quat, q, 4 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (B.vel) CK(cudaMemcpyAsync(B.vel, v, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (B.omega) CK(cudaMemcpyAsync(B.omega, om, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (B.prev_vel) CK(cudaMemcpyAsync(B.prev_vel, pv, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
  }
  avbd_joint_soa &J = out->joints;
  if (ctx->nj && J.count >= ctx->nj) {
    std::vector<float4> kl(ctx->nj), ka(ctx->nj);
    std::vector<D4> ll(ctx->nj), la(ctx->nj);
    std::vector<int> st(ctx->nj);
    CK(cudaMemcpy(kl.data(), w.j.penLin, ctx->nj * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ka.data(), w.j.penAng, ctx->nj * sizeof(float4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ll.data(), w.j.lamLin, ctx->nj * sizeof(D4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(la.data(), w.j.lamAng, ctx->nj * sizeof(D4), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(st.data(), w.j.state, ctx->nj * sizeof(int), cudaMemcpyDeviceToHost));
    for (int j = 0; j < ctx->nj; j++) {
      const float kv[6] = {kl[j].x, kl[j].y, kl[j].z, ka[j].x, ka[j].y, ka[j].z};
      const double lv[6] = {ll[j].x, ll[j].y, ll[j].z, la[j].x, la[j].y, la[j].z};
      for (int k = 0; k < 3; k++) {
        if (J.penalty_lin) J.penalty_lin[j * 3 + k] = kv[k];
        if (J.penalty_ang) J.penalty_ang[j * 3 + k] = kv[3 + k];
        if (J.lambda_lin) J.lambda_lin[j * 3 + k] = lv[k];
        if (J.lambda_ang) J.lambda_ang[j * 3 + k] = lv[3 + k];
      }
      if (J.broken) J.broken[j] = (st[j] & kBroken) ? 1 : 0;
    }
  }
  avbd_spring_soa &SP = out->springs;
  if (ctx->ns && SP.count >= ctx->ns) {
    std::vector<float> pen(ctx->ns);
    std::vector<double> peak(ctx->ns);
    std::vector<int> st(ctx->ns);
    CK(cudaMemcpy(pen.data(), w.s.penalty, ctx->ns * sizeof(float), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(peak.data(), w.s.peak, ctx->ns * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(st.data(), w.s.state, ctx->ns * sizeof(int), cudaMemcpyDeviceToHost));
    for (int s = 0; s < ctx->ns; s++) {
      if (SP.penalty) SP.penalty[s] = pen[s];
      if (SP.peak_strain) SP.peak_strain[s] = peak[s];
      if (SP.broken) SP.broken[s] = (st[s] & kBroken) ? 1 : 0;
    }
  }
  // manifolds of the last step (now the "previous" arena)
  avbd_manifold_soa &M = out->manifolds;
  if (M.body_a || M.num_contacts) {
    Control c{};
    CK(cudaMemcpy(&c, w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
    const int total = c.prevCandidates;
    const Manifolds &pm = ctx->curIsA ? ctx->mB : ctx->mA;
    std::vector<uint64_t> key(total);
    std::vector<int> cnt(total);
    if (total) {
      CK(cudaMemcpy(key.data(), pm.key, total * sizeof(uint64_t), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cnt.data(), pm.count, total * sizeof(int), cudaMemcpyDeviceToHost));
    }
    std::vector<int> live;
    for (int m = 0; m < total; m++)
      if (cnt[m] > 0) live.push_back(m);
    M.count = (int)live.size();
    const int wrote = std::min<int>(M.count, M.capacity);
    const size_t K = kMaxContacts;
    std::vector<double> basisD((size_t)total * 9);
    std::vector<float4> b0(total);
    std::vector<uint32_t> feat((size_t)total * K);
    std::vector<float4> rA(total * K), rB(total * K), cA(total * K), cB(total * K), cK(total * K), cL(total * K);
    std::vector<float> cX(total * K);
    if (total) {
      CK(cudaMemcpy(basisD.data(), pm.basisD, basisD.size() * sizeof(double), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(b0.data(), pm.basis0, total * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(feat.data(), pm.feat, feat.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(rA.data(), pm.rA, rA.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(rB.data(), pm.rB, rB.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cA.data(), pm.cA, cA.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cB.data(), pm.cB, cB.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cK.data(), pm.cK, cK.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cL.data(), pm.cL, cL.size() * sizeof(float4), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cX.data(), pm.cX, cX.size() * sizeof(float), cudaMemcpyDeviceToHost));
    }
    for (int t = 0; t < wrote; t++) {
      const int m = live[t];
      if (M.body_a) M.body_a[t] = (int)(key[m] >> 32);
      if (M.body_b) M.body_b[t] = (int)(key[m] & 0xffffffffu);
      if (M.num_contacts) M.num_contacts[t] = cnt[m];
      if (M.basis) for (int k = 0; k < 9; k++) M.basis[t * 9 + k] = basisD[(size_t)m * 9 + k];
      if (M.friction) M.friction[t] = b0[m].w;
      for (size_t s = 0; s < K; s++) {
        const size_t d = (size_t)t * K + s, src = (size_t)m * K + s;
        const bool on = (int)s < cnt[m];
        if (M.feature) M.feature[d] = on ? feat[src] : 0u;
        const float4 v[5] = {rA[src], rB[src], make_float4(cA[src].w, cB[src].w, cK[src].w, 0), cK[src], cL[src]};
        double *dst[5] = {M.r_a, M.r_b, M.c0, M.penalty, M.lambda};
        for (int f = 0; f < 5; f++)
          if (dst[f]) {
            dst[f][d * 3] = on ? v[f].x : 0;
            dst[f][d * 3 + 1] = on ? v[f].y : 0;
            dst[f][d * 3 + 2] = on ? v[f].z : 0;
          }
        if (M.stick) M.stick[d] = (on && cL[src].w != 0.f) ? 1 : 0;
        if (M.restitution_bias) M.restitution_bias[d] = on ? cX[src] : 0.0;
      }
      if (M.order) M.order[t] = t;
    }
  }
  return AVBD_OK;
}

int avbd_repack(avbd_ctx *ctx, const avbd_world *world, const int32_t *old_body, const int32_t *old_joint,
                const int32_t *old_spring, int64_t *carried) {
  if (!ctx || !world) return fail(ctx, AVBD_ERR_ARG, "avbd_repack: NULL argument");
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_repack before avbd_pack");
  if (world->num_scenes > 1 || ctx->numScenes > 1)
    return fail(ctx, AVBD_ERR_ARG, "avbd_repack: one scene (batches are packed whole)");
  int rc = resolve_skips(ctx);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  const int on = ctx->n, onj = ctx->nj, ons = ctx->ns;
  const int n = world->bodies.count, nj = world->joints.count, ns = world->springs.count;
  // the maps: every old element carried at most once; survivors in their old
  // relative order keep the warm-start manifolds (their A/B roles and the
  // arena's key order stay valid), otherwise the contacts start afresh
  std::vector<int> newOf(std::max(on, 1), -1);
  bool monotone = true;
  int last = -1, survivors = 0;
  for (int i = 0; i < n && old_body; i++) {
    const int o = old_body[i];
    if (o < -1 || o >= on) return fail(ctx, AVBD_ERR_ARG, "avbd_repack: old_body[%d] = %d outside -1..%d", i, o, on - 1);
    if (o < 0) continue;
    if (newOf[o] >= 0) return fail(ctx, AVBD_ERR_ARG, "avbd_repack: old body %d carried twice", o);
    newOf[o] = i;
    monotone = monotone && o > last;
    last = o;
    survivors++;
  }
  auto check_map = [&](const int32_t *m, int count, int oldCount, const char *what) -> int {
    if (!m) return AVBD_OK;
    std::vector<char> seen(std::max(oldCount, 1), 0);
    for (int k = 0; k < count; k++) {
      const int o = m[k];
      if (o < -1 || o >= oldCount)
        return fail(ctx, AVBD_ERR_ARG, "avbd_repack: old_%s[%d] = %d outside -1..%d", what, k, o, oldCount - 1);
      if (o >= 0 && seen[o]++) return fail(ctx, AVBD_ERR_ARG, "avbd_repack: old %s %d carried twice", what, o);
    }
    return AVBD_OK;
  };
  if ((rc = check_map(old_joint, nj, onj, "joint")) || (rc = check_map(old_spring, ns, ons, "spring"))) return rc;
  Control oc{};
  CK(cudaMemcpy(&oc, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  const int oldSlots = (monotone && survivors > 0) ? oc.prevCandidates : 0;

  // keep the old device arrays alive through the pack: the carried state is
  // gathered from them on the device, then they are freed
  const World ow = ctx->w;
  const Manifolds opm = ctx->curIsA ? ctx->mB : ctx->mA;
  std::vector<void *> oldAllocs, oldGrowable;
  oldAllocs.swap(ctx->allocs);
  oldGrowable.swap(ctx->growable);
  auto free_old = [&]() {
    cudaStreamSynchronize(ctx->stream);
    for (void *p : oldAllocs) cudaFree(p);
    for (void *p : oldGrowable) cudaFree(p);
    oldAllocs.clear();
    oldGrowable.clear();
  };
  avbd_world nw = *world;
  nw.manifolds.count = 0;
  rc = avbd_pack(ctx, &nw);
  if (!rc && oldSlots > ctx->candCap)
    rc = grow_arenas(ctx, (int)std::min<long long>(2LL * oldSlots, 0x3fffffff), ctx->mB, 0);
  if (rc) {
    free_old();
    return rc;
  }
  // the maps on the device, then one gather per kind and the arena remap
  World &w = ctx->w;
  cudaStream_t st = ctx->stream;
  int *dMaps = nullptr;
  const size_t mapInts = (size_t)n + nj + ns + on + 2 * (size_t)oldSlots + 2;
  if (cudaMalloc(&dMaps, mapInts * sizeof(int)) != cudaSuccess) {
    free_old();
    return fail(ctx, AVBD_ERR_CUDA, "avbd_repack: cudaMalloc of the maps failed");
  }
  int *dBody = dMaps, *dJoint = dBody + n, *dSpring = dJoint + nj, *dNewOf = dSpring + ns;
  int *dFlag = dNewOf + on, *dAt = dFlag + oldSlots + 1;
  std::vector<int> hb(n, -1), hj(nj, -1), hs(ns, -1);
  if (old_body) std::copy(old_body, old_body + n, hb.begin());
  if (old_joint) std::copy(old_joint, old_joint + nj, hj.begin());
  if (old_spring) std::copy(old_spring, old_spring + ns, hs.begin());
  cudaError_t e = cudaSuccess;
  if (n) e = cudaMemcpyAsync(dBody, hb.data(), n * sizeof(int), cudaMemcpyHostToDevice, st);
  if (!e && nj) e = cudaMemcpyAsync(dJoint, hj.data(), nj * sizeof(int), cudaMemcpyHostToDevice, st);
  if (!e && ns) e = cudaMemcpyAsync(dSpring, hs.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st);
  if (!e && on) e = cudaMemcpyAsync(dNewOf, newOf.data(), on * sizeof(int), cudaMemcpyHostToDevice, st);
  if (!e) e = launch_repack_state(ow, w, dBody, dJoint, dSpring, st);
  int carriedSlots = 0;
  if (!e && oldSlots > 0) {
    Manifolds npm = ctx->curIsA ? ctx->mB : ctx->mA;  // the new context's warm-start arena
    e = launch_repack_manifolds(opm, npm, oldSlots, dNewOf, dFlag, dAt, w.ctl, st);
    int tot[2] = {0, 0};
    if (!e) e = cudaMemcpyAsync(tot, dAt + oldSlots - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(tot + 1, dFlag + oldSlots - 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    carriedSlots = tot[0] + tot[1];
  }
  if (!e) e = cudaStreamSynchronize(st);
  cudaFree(dMaps);
  free_old();
  if (e != cudaSuccess) return fail(ctx, AVBD_ERR_CUDA, "avbd_repack: %s", cudaGetErrorString(e));
  if (carried) *carried = carriedSlots;
  return AVBD_OK;
}

int avbd_write_state(avbd_ctx *ctx, const avbd_world *world) {
  if (!ctx || !world) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_write_state before avbd_pack");
  if (world->bodies.count != ctx->n || world->joints.count != ctx->nj || world->springs.count != ctx->ns)
    return fail(ctx, AVBD_ERR_ARG, "avbd_write_state: topology differs from the packed world");
  int rs = resolve_skips(ctx);
  if (rs) return rs;
  return write_state(ctx, world, true);
}

int avbd_read_coloring(avbd_ctx *ctx, int32_t *color_of, int32_t *num_colors) {
  if (!ctx || !ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_read_coloring before avbd_pack");
  int rs = resolve_skips(ctx);
  if (rs) return rs;
  if (color_of) CK(cudaMemcpy(color_of, ctx->w.b.color, ctx->n * sizeof(int), cudaMemcpyDeviceToHost));
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  if (num_colors) *num_colors = c.numColors;
  return AVBD_OK;
}

int avbd_read_pairs(avbd_ctx *ctx, int32_t *body_a, int32_t *body_b, int64_t capacity, int64_t *count) {
  if (!ctx || !ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_read_pairs before avbd_pack");
  int rs = resolve_skips(ctx);
  if (rs) return rs;
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  const int total = c.prevCandidates;
  if (count) *count = total;
  const int k = (int)std::min<int64_t>(total, capacity);
  if (k > 0) {
    const Manifolds &pm = ctx->curIsA ? ctx->mB : ctx->mA;
    std::vector<uint64_t> key(k);
    CK(cudaMemcpy(key.data(), pm.key, k * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    for (int i = 0; i < k; i++) {
      if (body_a) body_a[i] = (int)(key[i] >> 32);
      if (body_b) body_b[i] = (int)(key[i] & 0xffffffffu);
    }
  }
  return AVBD_OK;
}

int avbd_read_stats(avbd_ctx *ctx, avbd_stats *out) {
  if (!ctx || !out) return AVBD_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  if (!ctx->packed) return AVBD_OK;
  int rs = resolve_skips(ctx);
  if (rs) return rs;
  const World &w = ctx->w;
  World sw = w;
  const Manifolds &pm = ctx->curIsA ? ctx->mB : ctx->mA;
  sw.cur = pm;
  Control c{};
  CK(cudaMemcpy(&c, w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  // the stats kernel reads numCandidates: point it at the last step's count
  Control tmp = c;
  tmp.numCandidates = c.prevCandidates;
  CK(cudaMemcpy(w.ctl, &tmp, sizeof(Control), cudaMemcpyHostToDevice));
  launch_stats(sw, ctx->statsOut, ctx->stream, ctx->smCount);
  double st3[3];
  CK(cudaMemcpyAsync(st3, ctx->statsOut, sizeof(st3), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(w.ctl, &c, sizeof(Control), cudaMemcpyHostToDevice));
  out->bodies = ctx->n;
  out->manifolds = c.liveManifolds;
  out->contacts = c.liveContacts;
  out->candidate_pairs = c.prevCandidates;
  out->colors = c.numColors;
  out->fp64_bodies = c.fp64Bodies;
  out->overflow = c.flags;
  out->steps = ctx->steps;
  out->max_constraint_error = st3[0];
  out->max_lambda = st3[1];
  out->max_penalty = st3[2];
  out->graph_steps = ctx->graphSteps;
  if (ctx->nj) {
    std::vector<int> st(ctx->nj);
    CK(cudaMemcpy(st.data(), w.j.state, ctx->nj * sizeof(int), cudaMemcpyDeviceToHost));
    for (int s : st) out->joints_broken += (s & kBroken) ? 1 : 0;
  }
  if (ctx->ns) {
    std::vector<int> st(ctx->ns);
    CK(cudaMemcpy(st.data(), w.s.state, ctx->ns * sizeof(int), cudaMemcpyDeviceToHost));
    for (int s : st) out->springs_broken += (s & kBroken) ? 1 : 0;
  }
  return AVBD_OK;
}

int avbd_set_profiling(avbd_ctx *ctx, int32_t on) {
  if (!ctx) return AVBD_ERR_ARG;
  ctx->profiling = on != 0;
  return AVBD_OK;
}

int avbd_read_profile(avbd_ctx *ctx, avbd_profile *out) {
  if (!ctx || !out) return AVBD_ERR_ARG;
  *out = ctx->prof;
  return AVBD_OK;
}

int avbd_kernel_launches(avbd_ctx *ctx, int64_t *out) {
  if (!ctx || !out) return AVBD_ERR_ARG;
  *out = ctx->launches;
  return AVBD_OK;
}

int avbd_set_coloring(avbd_ctx *ctx, const int32_t *color_of) {
  if (!ctx) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_set_coloring before avbd_pack");
  int rs = resolve_skips(ctx);
  if (rs) return rs;
  invalidate_graphs(ctx);  // the step's launch sequence changes
  if (!color_of) {
    ctx->w.a.colorOverride = nullptr;
    return AVBD_OK;
  }
  if (!ctx->colorOverride) {
    int rc = dalloc(ctx, &ctx->colorOverride, ctx->n);
    if (rc) return rc;
  }
  CK(cudaMemcpy(ctx->colorOverride, color_of, sizeof(int32_t) * ctx->n, cudaMemcpyHostToDevice));
  ctx->w.a.colorOverride = ctx->colorOverride;
  return AVBD_OK;
}

int avbd_update_joint_anchor(avbd_ctx *ctx, int32_t joint, const double r_a[3]) {
  if (!ctx || !r_a) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_update_joint_anchor before avbd_pack");
  if (joint < 0 || joint >= ctx->nj) return fail(ctx, AVBD_ERR_ARG, "joint %d out of range (%d joints)", joint, ctx->nj);
  if (!std::isfinite(r_a[0]) || !std::isfinite(r_a[1]) || !std::isfinite(r_a[2]))
    return fail(ctx, AVBD_ERR_NAN, "joint %d: non-finite anchor", joint);
  int rs = resolve_skips(ctx);  // the new anchor applies after the steps already queued
  if (rs) return rs;
  CK(launch_joint_anchor(ctx->w, joint, r_a[0], r_a[1], r_a[2], ctx->stream));
  ctx->launches += 1;
  return AVBD_OK;
}

int avbd_set_grab(avbd_ctx *ctx, int32_t body, const double local[3], const double target[3], double stiffness) {
  if (!ctx) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_set_grab before avbd_pack");
  if (body >= ctx->n) return fail(ctx, AVBD_ERR_ARG, "grab body %d out of range (%d bodies)", body, ctx->n);
  if (body >= 0) {
    if (!local || !target) return fail(ctx, AVBD_ERR_ARG, "avbd_set_grab: NULL anchor");
    if (!finite3(local) || !finite3(target) || !(stiffness > 0) || !std::isfinite(stiffness))
      return fail(ctx, AVBD_ERR_ARG, "avbd_set_grab: anchors must be finite and the stiffness finite and > 0");
  }
  int rs = resolve_skips(ctx);  // the grab applies after the steps already queued
  if (rs) return rs;
  CK(launch_set_grab(ctx->w, body < 0 ? -1 : body, local, target, stiffness, ctx->stream));
  ctx->launches += 1;
  return AVBD_OK;
}

int avbd_device_views_get(avbd_ctx *ctx, avbd_device_views *out) {
  if (!ctx || !out) return AVBD_ERR_ARG;
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_device_views_get before avbd_pack");
  out->body_pos = reinterpret_cast<const double *>(ctx->w.b.pos);
  out->body_quat = reinterpret_cast<const float *>(ctx->w.b.quat);
  out->body_count = ctx->n;
  out->joint_state = ctx->w.j.state;
  out->joint_count = ctx->nj;
  out->spring_state = ctx->w.s.state;
  out->spring_count = ctx->ns;
  return AVBD_OK;
}

const char *avbd_last_error(const avbd_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error; }

int avbd_adjoint_forward(avbd_ctx *ctx, const avbd_world *world, int32_t steps, const avbd_tangent_seed *seeds,
                         int32_t n_seeds) {
  if (!ctx || !world || steps < 0 || n_seeds < 0 || (n_seeds > 0 && !seeds))
    return fail(ctx, AVBD_ERR_ARG, "avbd_adjoint_forward: NULL argument or negative count");
  if (ctx->params.contact_model != AVBD_CONTACT_CPU)
    return fail(ctx, AVBD_ERR_ARG, "avbd_adjoint_forward: the differentiable step follows the CPU contact model "
                                   "(contact_model = AVBD_CONTACT_CPU)");
  char msg[256] = "";
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->tangent) {
    tangent_destroy(ctx->tangent);
    ctx->tangent = nullptr;
  }
  TangentCtx *t = nullptr;
  int rc = tangent_pack(&t, world, ctx->params, seeds, n_seeds, msg, sizeof(msg), ctx->stream);
  if (rc) return fail(ctx, rc, "%s", msg);
  ctx->tangent = t;
  const size_t need = tangent_temp_bytes(t);
  if (need > ctx->tanTempBytes) {
    if (ctx->tanTemp) cudaFree(ctx->tanTemp);
    ctx->tanTemp = nullptr;
    ctx->tanTempBytes = 0;
    CK(cudaMalloc(&ctx->tanTemp, need));
    ctx->tanTempBytes = need;
  }
  rc = tangent_step(t, steps, ctx->tanTemp, ctx->tanTempBytes, msg, sizeof(msg), ctx->stream);
  if (rc) return fail(ctx, rc, "%s", msg);
  ctx->launches += (int64_t)steps * 9;
  return AVBD_OK;
}

int avbd_adjoint_read(avbd_ctx *ctx, double *pos, double *dpos, double *quat) {
  if (!ctx) return AVBD_ERR_ARG;
  if (!ctx->tangent) return fail(ctx, AVBD_ERR_STATE, "avbd_adjoint_read before avbd_adjoint_forward");
  if (!pos) return fail(ctx, AVBD_ERR_ARG, "avbd_adjoint_read: NULL positions");
  const int rc = tangent_read(ctx->tangent, pos, dpos, quat, ctx->stream);
  return rc ? fail(ctx, rc, "avbd_adjoint_read: CUDA error") : AVBD_OK;
}

int avbd_adjoint_backward(avbd_ctx *ctx, const double *grad_pos, double *grad_params) {
  if (!ctx || !grad_pos || !grad_params) return fail(ctx, AVBD_ERR_ARG, "avbd_adjoint_backward: NULL argument");
  if (!ctx->tangent) return fail(ctx, AVBD_ERR_STATE, "avbd_adjoint_backward before avbd_adjoint_forward");
  const int rc = tangent_backward(ctx->tangent, grad_pos, grad_params, ctx->stream);
  return rc ? fail(ctx, rc, "avbd_adjoint_backward: CUDA error") : AVBD_OK;
}

int avbd_autotune(avbd_ctx *ctx, int32_t trial_steps, avbd_tuning *out) {
  if (!ctx || !out || trial_steps < 1) return fail(ctx, AVBD_ERR_ARG, "avbd_autotune: NULL argument or trial_steps < 1");
  if (!ctx->packed) return fail(ctx, AVBD_ERR_STATE, "avbd_autotune before avbd_pack");
  const bool profiling = ctx->profiling;
  ctx->profiling = false;
  Snapshot snap;
  int rc = take_snapshot(ctx, snap);
  if (rc) return rc;
  const TuneConfig start{ctx->params.schedule == 1 ? 1 : 0, ctx->autoLanes ? 0 : ctx->lanes, ctx->params.tail_div,
                         ctx->blocksPerSm};
  std::vector<TuneConfig> cands = {start};
  const int maxB = ctx->maxBlocksPerSm;
  for (int b = maxB; b >= std::max(1, maxB - 1); b--) {
    for (int lanes : {0, 32})
      for (int td : {0, -1, 4, 8, 16}) cands.push_back({0, lanes, td, b});  // automatic, no tail, explicit
    for (int lanes : {16, 32}) cands.push_back({1, lanes, 8, b});
  }
  std::memset(out, 0, sizeof(*out));
  double best = 0, first = 0;
  TuneConfig pick = start;
  int tried = 0;
  for (size_t k = 0; k < cands.size(); k++) {
    if (k > 0 && std::memcmp(&cands[k], &start, sizeof(TuneConfig)) == 0) continue;
    apply_config(ctx, cands[k]);
    double ms = 0;
    rc = time_config(ctx, snap, trial_steps, &ms);
    if (rc) break;
    tried++;
    if (k == 0) first = ms;
    if (k == 0 || ms < best) {
      best = ms;
      pick = cands[k];
    }
  }
  apply_config(ctx, rc ? start : pick);
  const int rr = restore_snapshot(ctx, snap);
  ctx->profiling = profiling;
  if (rc) return rc;
  if (rr) return rr;
  Control c{};
  CK(cudaMemcpy(&c, ctx->w.ctl, sizeof(Control), cudaMemcpyDeviceToHost));
  out->schedule = pick.schedule;
  out->lanes_per_body = pick.lanes;
  out->tail_div = pick.tailDiv;
  out->blocks_per_sm = pick.blocksPerSm;
  out->candidates = tried;
  out->trial_steps = trial_steps;
  out->default_ms = first;
  out->best_ms = best;
  out->bodies = ctx->n;
  out->manifolds = c.prevCandidates;
  return AVBD_OK;
}

}  // extern "C"

namespace avbd {
int set_context_free_error(int code, const char *msg) {
  g_create_error_buf = msg;
  g_create_error = g_create_error_buf.c_str();
  return code;
}
}  // namespace avbd
