// solver.cu - per-step preparation, constraint adjacency, integer-priority
// colouring and the persistent primal/dual solve of one AVBD step.
//
// Reference path (src/physics/solver.js:340-489):
//   force init   manifold.js:214-318 (narrowphase.cu), joint.js:131-160,
//                spring.js:472-507                      -> prepare_forces_kernel
//   body init    solver.js:366-401 (Eq. 2 + adaptive guess) -> prepare_bodies_kernel
//   primal       solver.js:418-458, manifold.js:411-445, joint.js:162-253,
//                spring.js:509-616, maths.js:660-725    -> solve_kernel
//   dual         manifold.js:447-491, joint.js:255-317, spring.js:618-634
//   velocity     solver.js:476-488 (BDF1)
//
// GB300 design:
//   * the primal and dual iterations of a step are ONE cooperative persistent
//     kernel; colour phases are separated by a bounded grid barrier, and the
//     last, thin colours run as one dependency-driven segment per iteration
//   * a group of G lanes assembles one body's 6x6 system (each lane takes up
//     to four of the incident constraints per staging round), reduces it with
//     warp shuffles (2-4 warps: through shared memory) and every lane solves
//     the LDL^T in registers; G (4..128) is chosen per body by the colouring,
//     which lays out each colour's groups in 128-lane chunks
//   * the dual update of a constraint is fused into the primal phase of its
//     endpoint with the larger colour: both endpoints are final for the
//     iteration at that moment, so this equals the reference's separate
//     dual sweep (solver.js:466-470) without another barrier per iteration
//   * positions are iterated as delta = x - x_t in f32 (x_t in f64), so the
//     f32 rounding is relative to the step's displacement, not to |x|
//   * bodies whose constraint stiffness dwarfs their inertia (k / (m/dt^2)
//     above a threshold) are assembled and factored in f64 from f64 shadows
#include <cooperative_groups.h>
#include <cub/cub.cuh>

#include "avbd_device.cuh"

namespace avbd {
namespace {

constexpr int kSolveBlock = 128;   // threads of a solve block (3 blocks per SM)
static_assert(kSolveBlock == kLaneMaxGroup, "a lane chunk is one solve block");
constexpr int kStageSlots = 4;     // contacts a lane stages in shared memory at a time
constexpr int kStageVecs = 9;      // float4 per staged contact
constexpr size_t kSolveSmem = (size_t)kSolveBlock * kStageSlots * kStageVecs * sizeof(float4);  // 73,728 B

// ---------------------------------------------------------------------------
// Bounded grid barrier (all blocks are co-resident: cooperative launch).
// Returns false when the wait gave up or another block reported a timeout;
// the caller must then return.
// ---------------------------------------------------------------------------
__device__ bool grid_barrier(Control *ctl, long long limit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned *gen = &ctl->barrierGen;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(&ctl->barrierCount, 1u) + 1u;
    if (arrived == gridDim.x) {
      ctl->barrierCount = 0;
      __threadfence();
      atomicAdd(&ctl->barrierGen, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        // give up after `limit` polls, or at once when another block gave up
        if (++spins > limit || (*((volatile unsigned *)&ctl->flags) & kOvfTimeout)) {
          atomicOr(&ctl->flags, kOvfTimeout);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*((volatile unsigned *)&ctl->flags) & kOvfTimeout) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

// ---------------------------------------------------------------------------
// Preparation
// ---------------------------------------------------------------------------
// A step skipped for a candidate overflow (Control::skip): its kernels after
// the broad phase return at once and leave every state array untouched.
__device__ __forceinline__ bool step_skipped(const World &w) { return *((volatile int *)&w.ctl->skip) != 0; }

__device__ inline double jsmin(double a, double b) { return a < b ? a : (b < a ? b : a); }
__device__ inline double jsmax(double a, double b) { return a > b ? a : (b > a ? b : a); }
__device__ inline double clampd(double x, double a, double b) { return x != x ? x : jsmax(a, jsmin(b, x)); }

__device__ inline Q4<double> body_q_t(const World &w, int i) {
  const float4 q = w.b.quat[i];
  return Q4<double>{q.x, q.y, q.z, q.w};
}

// joint.js:131-160 / spring.js:472-507, plus the f64 offsets p_A(t) - p_B(t).
__global__ void prepare_forces_kernel(World w) {
  if (step_skipped(w)) return;
  const SolverParams &P = w.p;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int j = tid; j < w.j.n; j += stride) {
    const int st = w.j.state[j];
    if (st & kRemoved) continue;  // left the force list in an earlier step
    if (st & kBroken) {
      // Joint.initialize still warm-starts a joint broken in the last step
      // (lambda = alpha gamma 0, k = min(clamp(gamma 0, kmin, kmax), stiffness)),
      // then returns !broken and the joint leaves the force list
      // (solver.js:346-360)
      const D4 sf = w.j.stiff[j];
      auto warm0 = [&](float k, double cap) {
        return (float)jsmin(clampd((double)k * P.gamma, P.penaltyMin, P.penaltyMax), cap);
      };
      const float4 kl = w.j.penLin[j], ka = w.j.penAng[j];
      w.j.penLin[j] = make_float4(warm0(kl.x, sf.x), warm0(kl.y, sf.x), warm0(kl.z, sf.x), 0.f);
      w.j.penAng[j] = make_float4(warm0(ka.x, sf.y), warm0(ka.y, sf.y), warm0(ka.z, sf.y), 0.f);
      if (!P.postStabilize) {
        D4 ll = w.j.lamLin[j], la = w.j.lamAng[j];
        ll.x = ll.x * P.alpha * P.gamma; ll.y = ll.y * P.alpha * P.gamma; ll.z = ll.z * P.alpha * P.gamma;
        la.x = la.x * P.alpha * P.gamma; la.y = la.y * P.alpha * P.gamma; la.z = la.z * P.alpha * P.gamma;
        w.j.lamLin[j] = ll;
        w.j.lamAng[j] = la;
      }
      w.j.state[j] = st | kRemoved;
      continue;
    }
    const int2 ab = w.j.bodies[j];
    const D4 rA = w.j.rAD[j], rB = w.j.rBD[j], sf = w.j.stiff[j];
    const Q4<double> qB = body_q_t(w, ab.y);
    const D4 pB = w.b.pos[ab.y];
    V3<double> pa, dpt;
    Q4<double> qA{0, 0, 0, 1};
    if (ab.x >= 0) {
      qA = body_q_t(w, ab.x);
      const D4 p = w.b.pos[ab.x];
      const V3<double> r = qrotate(qA, V3<double>{rA.x, rA.y, rA.z});
      pa = V3<double>{r.x + p.x, r.y + p.y, r.z + p.z};
      dpt = V3<double>{p.x - pB.x, p.y - pB.y, p.z - pB.z};
    } else {
      pa = V3<double>{rA.x, rA.y, rA.z};
      dpt = V3<double>{rA.x - pB.x, rA.y - pB.y, rA.z - pB.z};
    }
    const V3<double> rb = qrotate(qB, V3<double>{rB.x, rB.y, rB.z});
    const V3<double> pb{rb.x + pB.x, rb.y + pB.y, rb.z + pB.z};
    const V3<double> c0l = pa - pb;
    const V3<double> c0a = qsub(qA, qB) * sf.w;
    w.j.c0Lin[j] = make_float4((float)c0l.x, (float)c0l.y, (float)c0l.z, 0.f);
    w.j.c0Ang[j] = make_float4((float)c0a.x, (float)c0a.y, (float)c0a.z, 0.f);
    w.j.dpt[j] = make_float4((float)dpt.x, (float)dpt.y, (float)dpt.z, 0.f);
    w.j.dptD[j] = mkd4(dpt.x, dpt.y, dpt.z, 0.0);
    D4 ll = w.j.lamLin[j], la = w.j.lamAng[j];
    if (!P.postStabilize) {
      ll.x = ll.x * P.alpha * P.gamma; ll.y = ll.y * P.alpha * P.gamma; ll.z = ll.z * P.alpha * P.gamma;
      la.x = la.x * P.alpha * P.gamma; la.y = la.y * P.alpha * P.gamma; la.z = la.z * P.alpha * P.gamma;
    }
    w.j.lamLin[j] = ll;
    w.j.lamAng[j] = la;
    float4 kl = w.j.penLin[j], ka = w.j.penAng[j];
    auto warm = [&](float k, double cap) {
      return (float)jsmin(clampd((double)k * P.gamma, P.penaltyMin, P.penaltyMax), cap);
    };
    kl = make_float4(warm(kl.x, sf.x), warm(kl.y, sf.x), warm(kl.z, sf.x), 0.f);
    ka = make_float4(warm(ka.x, sf.y), warm(ka.y, sf.y), warm(ka.z, sf.y), 0.f);
    w.j.penLin[j] = kl;
    w.j.penAng[j] = ka;
  }
  for (int s = tid; s < w.s.n; s += stride) {
    int st = w.s.state[s];
    if (st & kRemoved) continue;
    const int2 ab = w.s.bodies[s];
    const D4 prm = w.s.prm[s];
    const D4 pA = w.b.pos[ab.x], pB = w.b.pos[ab.y];
    const V3<double> dpt{pA.x - pB.x, pA.y - pB.y, pA.z - pB.z};
    w.s.dpt[s] = make_float4((float)dpt.x, (float)dpt.y, (float)dpt.z, 0.f);
    w.s.dptD[s] = mkd4(dpt.x, dpt.y, dpt.z, 0.0);
    if (st & kBroken) {
      w.s.penalty[s] = 0.f;
      continue;
    }
    if (isfinite(prm.z)) {  // tear check at x_t (spring.js:484-490)
      const D4 rA = w.s.rAD[s], rB = w.s.rBD[s];
      const V3<double> ra = qrotate(body_q_t(w, ab.x), V3<double>{rA.x, rA.y, rA.z});
      const V3<double> rb = qrotate(body_q_t(w, ab.y), V3<double>{rB.x, rB.y, rB.z});
      const V3<double> d{(ra.x + pA.x) - (rb.x + pB.x), (ra.y + pA.y) - (rb.y + pB.y),
                         (ra.z + pA.z) - (rb.z + pB.z)};
      const double len = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
      if (len > 1.0e-6 && prm.y > 1.0e-6) {
        const double strain = jsmax(0.0, (len - prm.y) / prm.y);
        w.s.peak[s] = jsmax(w.s.peak[s], strain);
        if (strain > prm.z) {
          w.s.state[s] = st | kBroken;
          w.s.penalty[s] = 0.f;
          continue;
        }
      }
    }
    if (!P.springRamp) {
      w.s.penalty[s] = (float)prm.x;
    } else {
      double k = clampd((double)w.s.penalty[s] * P.gamma, P.penaltyMin, P.penaltyMax);
      w.s.penalty[s] = (float)jsmin(k, prm.x);
    }
    if (!(prm.x > 0)) w.s.state[s] = st | kRemoved;
  }
}

// solver.js:369-401, in delta form.
__global__ void prepare_bodies_kernel(World w) {
  if (step_skipped(w)) return;
  const SolverParams &P = w.p;
  const double dt = P.dt, g = P.gravity;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x) {
    const float4 qf = w.b.quat[i], vf = w.b.vel[i], wf = w.b.omega[i], pv = w.b.prevVel[i];
    const double mass = w.b.massD[i].x;
    const Q4<double> q{qf.x, qf.y, qf.z, qf.w};
    const V3<double> wdt{(double)wf.x * dt, (double)wf.y * dt, (double)wf.z * dt};
    V3<double> y{(double)vf.x * dt, (double)vf.y * dt, (double)vf.z * dt};
    if (mass > 0) y.z += g * (dt * dt);
    const Q4<double> qy = qintegrate(q, wdt);
    const double accelZ = ((double)vf.z - (double)pv.z) / dt;
    const double sgn = g < 0 ? -1.0 : (g > 0 ? 1.0 : 0.0);
    double weight = clampd(accelZ * sgn / fabs(g), 0.0, 1.0);
    if (!isfinite(weight)) weight = 0.0;
    w.b.quatT[i] = qf;
    w.b.yLin[i] = make_float4((float)y.x, (float)y.y, (float)y.z, 0.f);
    w.b.yAng[i] = make_float4((float)qy.x, (float)qy.y, (float)qy.z, (float)qy.w);
    int fl = w.b.flags0[i];
    if (mass > 0) {
      V3<double> d{(double)vf.x * dt, (double)vf.y * dt, (double)vf.z * dt};
      d.z += g * (weight * dt * dt);
      w.b.dp[i] = make_float4((float)d.x, (float)d.y, (float)d.z, 0.f);
      w.b.dpD[i] = mkd4(d.x, d.y, d.z, 0.0);
      w.b.quat[i] = make_float4((float)qy.x, (float)qy.y, (float)qy.z, (float)qy.w);
      w.b.quatD[i] = mkd4(qy.x, qy.y, qy.z, qy.w);
    } else {
      w.b.dp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      w.b.dpD[i] = mkd4(0.0, 0.0, 0.0, 0.0);
      w.b.quatD[i] = mkd4(q.x, q.y, q.z, q.w);
    }
    {  // the iterate's qsub(q, q_t), as load_state<float> forms it
      const float4 qn = w.b.quat[i];
      const V3<float> da = qsub(Q4<float>{qn.x, qn.y, qn.z, qn.w}, Q4<float>{qf.x, qf.y, qf.z, qf.w});
      w.b.dang[i] = make_float4(da.x, da.y, da.z, 0.f);
    }
    w.b.flags[i] = fl;
    w.a.count[i] = 0;
    w.a.ccount[i] = 0;
    w.b.progress[i] = 0;
  }
}

// Live manifolds of this step: count the incident ones of every dynamic body.
__device__ inline bool precedes(const World &w, int j, int i) {
  const uint32_t pj = w.b.priority[j], pi = w.b.priority[i];
  return pj < pi || (pj == pi && j < i);
}

__global__ void adj_count_kernel(World w) {
  const int total = w.ctl->numCandidates;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
    const int n = w.cur.count[c];
    if (n <= 0) continue;
    const uint64_t k = w.cur.key[c];
    const int a = (int)(k >> 32), b = (int)(k & 0xffffffffu);
    if (w.b.flags0[a] & kBodyDynamic) {
      atomicAdd(&w.a.count[a], 1);
      atomicAdd(&w.a.ccount[a], n);
    }
    if (w.b.flags0[b] & kBodyDynamic) {
      atomicAdd(&w.a.count[b], 1);
      atomicAdd(&w.a.ccount[b], n);
    }
    atomicAdd(&w.ctl->liveManifolds, 1);
    atomicAdd(&w.ctl->liveContacts, n);
  }
}

__global__ void adj_fill_kernel(World w) {
  const int total = w.ctl->numCandidates;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
    if (w.cur.count[c] <= 0) continue;
    const uint64_t k = w.cur.key[c];
    const int a = (int)(k >> 32), b = (int)(k & 0xffffffffu);
    if (w.b.flags0[a] & kBodyDynamic) {
      const int at = atomicAdd(&w.a.cursor[a], 1);
      if (at < w.a.cap) w.a.entry[at] = ((uint32_t)c << 1) | 0u;
      else atomicOr(&w.ctl->flags, kOvfAdj);
    }
    if (w.b.flags0[b] & kBodyDynamic) {
      const int at = atomicAdd(&w.a.cursor[b], 1);
      if (at < w.a.cap) w.a.entry[at] = ((uint32_t)c << 1) | 1u;
      else atomicOr(&w.ctl->flags, kOvfAdj);
    }
  }
}

// Sort each body's manifold list (determinism) and decide its precision.
__global__ void adj_sort_kernel(World w) {
  if (step_skipped(w)) return;
  const double dt2 = w.p.dt * w.p.dt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x) {
    int fl = w.b.flags[i];
    if (!(fl & kBodyDynamic)) continue;
    int beg = w.a.start[i], end = w.a.start[i + 1];
    if (end > w.a.cap) end = w.a.cap;
    uint32_t *e = w.a.entry;
    for (int x = beg + 1; x < end; x++) {
      const uint32_t v = e[x];
      int y = x - 1;
      while (y >= beg && e[y] > v) {
        e[y + 1] = e[y];
        y--;
      }
      e[y + 1] = v;
    }
    // per-contact adjacency, in manifold order then contact order; and the
    // dynamic neighbours of higher colouring priority (the only ones a
    // colouring round reads), stored in the body's own manifold range
    {
      int at = w.a.cstart[i];
      const int cend = min(w.a.cstart[i + 1], w.a.ccap);
      int hc = 0;
      for (int x = beg; x < end; x++) {
        const uint32_t v = e[x];
        const int m = (int)(v >> 1), side = (int)(v & 1u);
        const uint64_t key = w.cur.key[m];
        const int other = side ? (int)(key >> 32) : (int)(key & 0xffffffffu);
        const int cnt = w.cur.count[m];
        for (int k = 0; k < cnt && at < cend; k++, at++)
          w.a.centry[at] = make_int2(((m * kMaxContacts + k) << 2) | side, other);  // owner bit set after colouring
        if ((w.b.flags0[other] & kBodyDynamic) && precedes(w, other, i)) w.a.hpEntry[beg + hc++] = other;
      }
      w.a.hpCount[i] = hc;
    }
    if (w.p.fp64Ratio > 0) {
      double kmax = 0;
      for (int k = w.g.cStart[i]; k < w.g.cStart[i + 1]; k++) {
        const uint32_t ref = w.g.cRef[k];
        const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu;
        if (type == kRefJoint) {
          if (w.j.state[idx]) continue;
          const float4 kl = w.j.penLin[idx];
          const double hard = isinf(w.j.stiff[idx].x) ? w.p.penaltyMax : 0.0;
          kmax = fmax(kmax, fmax(fmax((double)kl.x, (double)kl.y), fmax((double)kl.z, hard)));
        } else {
          if (w.s.state[idx]) continue;
          kmax = fmax(kmax, (double)w.s.penalty[idx]);
        }
      }
      const double inertial = w.b.massD[i].x / dt2;
      if (kmax > w.p.fp64Ratio * inertial) {
        fl |= kBodyFp64;
        atomicAdd(&w.ctl->fp64Bodies, 1);
      }
    }
    w.b.flags[i] = fl;
  }
}

// ---------------------------------------------------------------------------
// Colouring: greedy in (lowbias32(local index), index) order, computed as the
// fixed point of in-place Jacobi rounds seeded with the previous step's
// colours (the reference GPU's incremental colouring,
// src/physics/gpu/shaders.js:1558-1656, run to convergence so that the result
// is exactly the sequential greedy colouring in priority order). Then a
// stable counting sort lists each colour's bodies in index order.
// ---------------------------------------------------------------------------
// The live joint and spring partners of body i that are dynamic.
template <class F>
__device__ inline void constraint_neighbors(const World &w, int i, F &&f) {
  for (int k = w.g.cStart[i]; k < w.g.cStart[i + 1]; k++) {
    const uint32_t ref = w.g.cRef[k];
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    int2 ab;
    if (type == kRefJoint) {
      if (w.j.state[idx]) continue;
      ab = w.j.bodies[idx];
    } else {
      if (w.s.state[idx]) continue;
      ab = w.s.bodies[idx];
    }
    const int other = side ? ab.x : ab.y;
    if (other >= 0 && (w.b.flags0[other] & kBodyDynamic)) f(other);
  }
}

// log2 of the lanes of a body's group in the colour-phase solve: the fixed
// lanes parameter, else the fewest lanes (4..128) whose staging of four
// constraints per lane holds all of the body's constraints; FP64 bodies
// (register path, warp shuffles) at most 32.
__device__ __forceinline__ int lane_log2(const World &w, int4 rec) {
  int G;
  if (w.p.lanes > 0) {
    G = w.p.lanes;
  } else {
    const int i = rec.x;
    const int total = (rec.z - rec.y) + (w.g.cStart[i + 1] - w.g.cStart[i]);
    G = 4;
    while (G < kLaneMaxGroup && 4 * G < total) G <<= 1;
  }
  if ((w.b.flags[rec.x] & kBodyFp64) && G > 32) G = 32;
  return 31 - __clz(G);
}

// The lane layout of the colour-phase solve (Adjacency::laneTab), from the
// sorted colour records: groups counted per (colour, size), each colour's
// groups placed in decreasing size (so every offset is a multiple of the
// group's own size and no group crosses a chunk), chunks of all colours
// numbered in colour order. Placement within a (colour, size) class follows
// atomics and may vary between runs; a body's arithmetic depends only on its
// group size, so results do not.
__device__ void lane_layout(const World &w) {
  Control *ctl = w.ctl;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  volatile int *color = w.b.color;
  int *cnt = w.a.laneHist, *cur = w.a.laneHist + kMaxColors * kLaneBuckets;
  int *used = w.a.laneHist + 2 * kMaxColors * kLaneBuckets;
  const int nrec = w.a.colorStart[kMaxColors];
  const int numColors = *((volatile int *)&ctl->numColors);
  const int lane = threadIdx.x & 31;
  // warp-uniform loops (stride is a multiple of 32): the records of a warp
  // with equal (colour, size) share one atomic
  for (int r = tid; r - lane < nrec; r += stride) {
    int key = -1;
    if (r < nrec) {
      const int4 rec = w.a.colorRec[r];
      key = color[rec.x] * kLaneBuckets + lane_log2(w, rec);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(peers) - 1) atomicAdd(&cnt[key], __popc(peers));
  }
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  if (blockIdx.x == 0) {
    // per colour: the offsets of its size classes (largest first) and its
    // lane count; then the colours' first chunks by a block-wide scan
    __shared__ int chunkScan[256];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    int lanesTotal = 0;
    for (int c0 = 0; c0 < numColors; c0 += blockDim.x) {
      const int c = c0 + threadIdx.x;
      int chunks = 0;
      if (c < numColors) {
        int off = 0;
        for (int b = kLaneBuckets - 1; b >= 0; b--) {
          cur[c * kLaneBuckets + b] = off;
          off += cnt[c * kLaneBuckets + b] << b;
        }
        used[c] = off;
        lanesTotal += off;
        chunks = (off + kLaneMaxGroup - 1) / kLaneMaxGroup;
      }
      chunkScan[threadIdx.x] = chunks;
      __syncthreads();
      for (int d = 1; d < (int)blockDim.x; d <<= 1) {  // inclusive scan
        const int v = threadIdx.x >= d ? chunkScan[threadIdx.x - d] : 0;
        __syncthreads();
        chunkScan[threadIdx.x] += v;
        __syncthreads();
      }
      if (c < numColors) w.a.colorChunk[c] = carry + chunkScan[threadIdx.x] - chunks;
      __syncthreads();
      if (threadIdx.x == blockDim.x - 1) carry += chunkScan[threadIdx.x];
      __syncthreads();
    }
    if (threadIdx.x == 0) w.a.colorChunk[numColors] = carry;
    lanesTotal = __reduce_add_sync(0xffffffffu, lanesTotal);
    if (lane == 0 && lanesTotal) atomicAdd(&ctl->laneTotal, lanesTotal);
  }
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  for (int k = tid; k < numColors * kLaneBuckets; k += stride) cnt[k] = 0;  // for the next step
  for (int r = tid; r - lane < nrec; r += stride) {
    int key = -1, c = 0, b = 0, e = 0;
    if (r < nrec) {
      const int4 rec = w.a.colorRec[r];
      c = color[rec.x];
      b = lane_log2(w, rec);
      key = c * kLaneBuckets + b;
      e = (r << 4) | ((w.b.flags[rec.x] & kBodyFp64) ? 8 : 0) | b;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&cur[key], __popc(peers) << b);
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key < 0) continue;
    const int off = base + (__popc(peers & ((1u << lane) - 1u)) << b);
    int *dst = w.a.laneTab + (size_t)w.a.colorChunk[c] * kLaneMaxGroup + off;
    if (b >= 2) {  // off and G are multiples of 4: 16-byte stores
      const int4 e4 = make_int4(e, e, e, e);
      for (int k = 0; k < (1 << b); k += 4) *reinterpret_cast<int4 *>(dst + k) = e4;
    } else {
      for (int k = 0; k < (1 << b); k++) dst[k] = e;
    }
  }
  // the lanes past each colour's last group, up to its last chunk's end
  for (int k = tid; k < numColors * kLaneMaxGroup; k += stride) {
    const int c = k / kLaneMaxGroup;
    const size_t L = (size_t)w.a.colorChunk[c] * kLaneMaxGroup + used[c] + (k % kLaneMaxGroup);
    if (L < (size_t)w.a.colorChunk[c + 1] * kLaneMaxGroup) w.a.laneTab[L] = -1;
  }
}

// The tail of the colouring: owner bits of the contact entries, the stable
// counting sort by colour and the solve's lane layout (cooperative: grid
// barriers inside). Per-colour loops run over the colours in use only
// (Control::numColors, from the largest colour found), so a step of few
// colours pays nothing for the colour capacity.
__device__ void coloring_finish(const World &w) {
  Control *ctl = w.ctl;
  const int n = w.b.n;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  volatile int *color = w.b.color;
  // owner bit (bit 1) of every contact entry: the endpoint with the larger
  // colour owns the contact's dual update (a static endpoint has colour -1);
  // and the number of colours in use
  int maxColor = -1;
  for (int i = tid; i < n; i += stride) {
    if (!(w.b.flags0[i] & kBodyDynamic)) continue;
    const int ci = color[i];
    maxColor = max(maxColor, ci);
    const int e1 = min(w.a.cstart[i + 1], w.a.ccap);
    for (int e = w.a.cstart[i]; e < e1; e++) {
      int2 v = w.a.centry[e];
      const int oc = (w.b.flags0[v.y] & kBodyDynamic) ? color[v.y] : -1;
      v.x = (v.x & ~2) | (ci > oc ? 2 : 0);
      w.a.centry[e] = v;
    }
  }
  maxColor = __reduce_max_sync(0xffffffffu, maxColor);
  if ((threadIdx.x & 31) == 0 && maxColor >= 0) atomicMax(&ctl->numColors, maxColor + 1);
  if (tid == 0) ctl->laneTotal = 0;  // summed by lane_layout after the next barriers
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  const int numColors = *((volatile int *)&ctl->numColors);
  // --- stable counting sort by colour (per-block chunk of body indices) ---
  __shared__ int hist[kMaxColors];
  __shared__ int base[kMaxColors];
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  for (int c = threadIdx.x; c < numColors; c += blockDim.x) hist[c] = 0;
  __syncthreads();
  for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
    const int c = color[i];
    if (c >= 0) atomicAdd(&hist[c], 1);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < numColors; c += blockDim.x) w.a.blockHist[blockIdx.x * kMaxColors + c] = hist[c];
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  if (blockIdx.x == 0) {
    // per colour: the blocks' offsets (a scan over blocks), then the colours'
    // starts (a block-wide scan over colours, in rounds of blockDim colours).
    // A round's colours share the block's threads: `parts` threads a colour,
    // each summing, then offsetting, a contiguous run of blocks (the counts
    // are integers: any grouping gives the same offsets).
    __shared__ int scan[256];
    __shared__ int partSum[256];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < numColors; c0 += blockDim.x) {
      const int round = min((int)blockDim.x, numColors - c0);
      const int parts = max(1, (int)blockDim.x / round);
      const int cl = (int)threadIdx.x / parts, part = (int)threadIdx.x % parts;
      const int len = ((int)gridDim.x + parts - 1) / parts, bb = part * len, be = min((int)gridDim.x, bb + len);
      const bool mine = cl < round;
      const int cc = c0 + cl;
      int sum = 0;
      if (mine)
        for (int b = bb; b < be; b++) sum += w.a.blockHist[b * kMaxColors + cc];
      partSum[threadIdx.x] = sum;
      __syncthreads();
      if (mine) {
        int run = 0;
        for (int q = 0; q < part; q++) run += partSum[cl * parts + q];
        for (int b = bb; b < be; b++) {
          const int h = w.a.blockHist[b * kMaxColors + cc];
          w.a.blockHist[b * kMaxColors + cc] = run;
          run += h;
        }
      }
      const int c = c0 + threadIdx.x;
      int run = 0;  // colour c's total
      if (threadIdx.x < round)
        for (int q = 0; q < parts; q++) run += partSum[threadIdx.x * parts + q];
      __syncthreads();
      scan[threadIdx.x] = run;
      __syncthreads();
      for (int d = 1; d < (int)blockDim.x; d <<= 1) {  // inclusive scan
        const int v = threadIdx.x >= d ? scan[threadIdx.x - d] : 0;
        __syncthreads();
        scan[threadIdx.x] += v;
        __syncthreads();
      }
      if (c < numColors) w.a.colorStart[c] = carry + scan[threadIdx.x] - run;
      __syncthreads();
      if (threadIdx.x == blockDim.x - 1) carry += scan[threadIdx.x];
      __syncthreads();
    }
    for (int c = numColors + (int)threadIdx.x; c <= kMaxColors; c += blockDim.x) w.a.colorStart[c] = carry;
  }
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  for (int c = threadIdx.x; c < numColors; c += blockDim.x)
    base[c] = w.a.colorStart[c] + w.a.blockHist[blockIdx.x * kMaxColors + c];
  __syncthreads();
  // within a tile of blockDim bodies: rank among the tile's bodies of the same
  // colour = rank within the warp + the counts of that colour in earlier warps
  // (each warp lists its distinct colours with their counts)
  __shared__ int2 warpList[8][32];
  __shared__ int warpLen[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t0 = b0; t0 < b1; t0 += blockDim.x) {
    const int i = t0 + threadIdx.x;
    const int c = (i < b1) ? color[i] : -1;
    const unsigned m = __match_any_sync(0xffffffffu, c);
    const int rankInWarp = __popc(m & ((1u << lane) - 1u));
    const bool leader = rankInWarp == 0 && c >= 0;
    const unsigned leaders = __ballot_sync(0xffffffffu, leader);
    if (leader) warpList[warp][__popc(leaders & ((1u << lane) - 1u))] = make_int2(c, __popc(m));
    if (lane == 0) warpLen[warp] = __popc(leaders);
    __syncthreads();
    if (c >= 0) {
      int r = base[c] + rankInWarp;
      for (int q = 0; q < warp; q++)
        for (int k = 0; k < warpLen[q]; k++)
          if (warpList[q][k].x == c) r += warpList[q][k].y;
      w.a.colorBodies[r] = i;
      w.a.colorRec[r] = make_int4(i, w.a.cstart[i], min(w.a.cstart[i + 1], w.a.ccap), 0);
    }
    __syncthreads();
    for (int q = 0; q < (int)(blockDim.x >> 5); q++)  // advance the bases past this tile
      for (int k = threadIdx.x; k < warpLen[q]; k += blockDim.x) atomicAdd(&base[warpList[q][k].x], warpList[q][k].y);
    __syncthreads();
  }
  if (!grid_barrier(ctl, w.p.barrierLimit)) return;
  lane_layout(w);
}

// Smallest colour no neighbour of higher priority holds, searched in windows
// of 64 colours: one pass unless all of 0..63 are taken.
template <class F>
__device__ __forceinline__ int smallest_free_color(F &&neighbors) {
  for (int base = 0; base < kMaxColors; base += 64) {
    unsigned long long used = 0ull;
    neighbors([&](int c) {
      if (c >= base && c < base + 64) used |= 1ull << (c - base);
    });
    if (~used) return base + __ffsll((long long)~used) - 1;
  }
  return -1;
}

__global__ void __launch_bounds__(256) coloring_kernel(World w) {
  if (step_skipped(w)) return;  // every block reads the same value: none waits at a barrier
  Control *ctl = w.ctl;
  const int n = w.b.n;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  volatile int *color = w.b.color;
  // an uploaded colouring (copied and checked by the kernels before this
  // one) is used when proper; otherwise the priority colouring is computed
  if (w.a.colorOverride) {
    if (*((volatile int *)&ctl->colorBad) == 0) {
      coloring_finish(w);
      return;
    }
    if (tid == 0) atomicOr(&ctl->flags, kErrColoring);
  }
  // seed: previous colours (statics -1, new dynamic bodies 0)
  for (int i = tid; i < n; i += stride) {
    if (!(w.b.flags0[i] & kBodyDynamic)) color[i] = -1;
    else if (color[i] < 0 || color[i] >= kMaxColors) color[i] = 0;
  }
  // "changed" flags, triple-buffered: round r sets flag r % 3 and clears the
  // flag of round r + 1, which no block can still be reading (it was last
  // read in round r - 2, before the barriers of round r - 1).
  if (tid == 0) ctl->pad[1] = 0;
  int round = 0;
  for (;; round++) {
    if (tid == 0) ctl->pad[1 + (round + 1) % 3] = 0;
    if (!grid_barrier(ctl, w.p.barrierLimit)) return;
    int changed = 0;
    for (int i = tid; i < n; i += stride) {
      if (!(w.b.flags0[i] & kBodyDynamic)) continue;
      const int hb = w.a.start[i], hc = w.a.hpCount[i];
      int c = smallest_free_color([&](auto &&mark) {
        for (int k = 0; k < hc; k++) mark(color[w.a.hpEntry[hb + k]]);
        if (w.g.hasConstraints)
          constraint_neighbors(w, i, [&](int j) {
            if (precedes(w, j, i)) mark(color[j]);
          });
      });
      if (c < 0) {
        c = kMaxColors - 1;
        atomicOr(&ctl->flags, kOvfColors);
      }
      if (c != color[i]) {
        color[i] = c;
        changed = 1;
      }
    }
    if (changed) atomicOr(&ctl->pad[1 + round % 3], 1);
    if (!grid_barrier(ctl, w.p.barrierLimit)) return;
    const int any = *((volatile int *)&ctl->pad[1 + round % 3]);
    if (!any) break;
    if (round > 4096) {
      if (tid == 0) atomicOr(&ctl->flags, kOvfColors);
      break;
    }
  }
  coloring_finish(w);
}

// ---------------------------------------------------------------------------
// Per-body assembly and solve
// ---------------------------------------------------------------------------
template <class T>
struct Sys {  // lower triangles of the three 3x3 blocks + right-hand side
  T l[6];  // aLin: 00 10 11 20 21 22
  T a[6];  // aAng: same layout
  T c[9];  // aCross row-major (rows: angular dof, cols: linear dof)
  T bl[3], ba[3];
};

template <class T>
__device__ __forceinline__ void zero(Sys<T> &s) {
#pragma unroll
  for (int k = 0; k < 6; k++) s.l[k] = s.a[k] = T(0);
#pragma unroll
  for (int k = 0; k < 9; k++) s.c[k] = T(0);
#pragma unroll
  for (int k = 0; k < 3; k++) s.bl[k] = s.ba[k] = T(0);
}

template <class T>
__device__ inline T shfl_xor(T v, int m, unsigned mask, int width) {
  return __shfl_xor_sync(mask, v, m, width);
}

template <class T>
__device__ __forceinline__ void group_reduce(Sys<T> &s, unsigned mask, int G) {
  for (int m = G >> 1; m > 0; m >>= 1) {
#pragma unroll
    for (int k = 0; k < 6; k++) {
      s.l[k] += shfl_xor(s.l[k], m, mask, G);
      s.a[k] += shfl_xor(s.a[k], m, mask, G);
    }
#pragma unroll
    for (int k = 0; k < 9; k++) s.c[k] += shfl_xor(s.c[k], m, mask, G);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      s.bl[k] += shfl_xor(s.bl[k], m, mask, G);
      s.ba[k] += shfl_xor(s.ba[k], m, mask, G);
    }
  }
}

// For groups of 32 lanes: the same sums by reduce-scatter (xor distances 16,
// 8, 4, 2, 1, the butterfly's own pairing, so every total is bitwise the
// butterfly's) and an all-gather: 31 + 27 shuffles instead of 5 x 27.
// reduce_scatter32 leaves lane j with the warp's total of value j.
__device__ __forceinline__ float reduce_scatter32(const Sys<float> &s) {
  const int lane = threadIdx.x & 31;
  float v[32];
#pragma unroll
  for (int k = 0; k < 6; k++) {
    v[k] = s.l[k];
    v[6 + k] = s.a[k];
  }
#pragma unroll
  for (int k = 0; k < 9; k++) v[12 + k] = s.c[k];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    v[21 + k] = s.bl[k];
    v[24 + k] = s.ba[k];
  }
#pragma unroll
  for (int k = 27; k < 32; k++) v[k] = 0.f;
#pragma unroll
  for (int h = 16; h > 0; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int p = 0; p < h; p++) {
      const float send = up ? v[p] : v[p + h];
      const float keep = up ? v[p + h] : v[p];
      v[p] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  return v[0];
}

// Every lane gets the totals lane j holds (value j).
__device__ __forceinline__ void all_gather32(Sys<float> &s, float t) {
#pragma unroll
  for (int k = 0; k < 6; k++) {
    s.l[k] = __shfl_sync(0xffffffffu, t, k);
    s.a[k] = __shfl_sync(0xffffffffu, t, 6 + k);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) s.c[k] = __shfl_sync(0xffffffffu, t, 12 + k);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    s.bl[k] = __shfl_sync(0xffffffffu, t, 21 + k);
    s.ba[k] = __shfl_sync(0xffffffffu, t, 24 + k);
  }
}

__device__ __forceinline__ void group_reduce32(Sys<float> &s) { all_gather32(s, reduce_scatter32(s)); }

// Barriers 1..3 with immediate ids (barrier 0 is __syncthreads).
__device__ __forceinline__ void named_barrier(int id, int count) {
  if (id == 1) asm volatile("bar.sync 1, %0;" ::"r"(count) : "memory");
  else if (id == 2) asm volatile("bar.sync 2, %0;" ::"r"(count) : "memory");
  else asm volatile("bar.sync 3, %0;" ::"r"(count) : "memory");
}

// For groups of G = 64 or 128 lanes (2 or 4 whole warps of one block): each
// warp's reduce-scatter, the warps' totals added through shared memory in
// warp order (the same order in every warp, so all warps hold bitwise equal
// sums), then each warp's all-gather. Named barriers: 1 and 2 for the two
// 64-lane groups of a block, 3 for a 128-lane group, so that a warp already
// in a later group of another shape never meets one still in this group.
__device__ __forceinline__ void group_reduce_warps(Sys<float> &s, int G) {
  __shared__ float red[kSolveBlock / 32][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = G >> 5, w0 = warp & ~(nw - 1);
  const int id = nw == 2 ? 1 + (w0 >> 1) : 3;
  red[warp][lane] = reduce_scatter32(s);
  named_barrier(id, G);
  float t = red[w0][lane];
  for (int k = 1; k < nw; k++) t += red[w0 + k][lane];
  named_barrier(id, G);  // every warp has read before the next group writes
  all_gather32(s, t);
}

// sym 3x3 lower index
__device__ inline constexpr int L(int r, int c) { return r >= c ? (r * (r + 1)) / 2 + c : (c * (c + 1)) / 2 + r; }

// H_lin += k n n^T ; H_ang += k a a^T ; H_cross += k a n^T ; b += f_lin, f_ang
template <class T>
__device__ __forceinline__ void stamp_row(Sys<T> &s, T k, V3<T> n, V3<T> a) {
  const T nn[3] = {n.x, n.y, n.z}, aa[3] = {a.x, a.y, a.z};
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c <= r; c++) {
      s.l[L(r, c)] += k * nn[r] * nn[c];
      s.a[L(r, c)] += k * aa[r] * aa[c];
    }
#pragma unroll
  for (int r = 0; r < 3; r++)
#pragma unroll
    for (int c = 0; c < 3; c++) s.c[r * 3 + c] += k * aa[r] * nn[c];
}

// maths.js:660-725, unrolled LDL^T (lower storage).
template <class T>
__device__ __forceinline__ void ldlt_solve(const Sys<T> &s, T bl0, T bl1, T bl2, T ba0, T ba1, T ba2, V3<T> &xl, V3<T> &xa) {
  const T A11 = s.l[0], A21 = s.l[1], A22 = s.l[2], A31 = s.l[3], A32 = s.l[4], A33 = s.l[5];
  const T A41 = s.c[0], A42 = s.c[1], A43 = s.c[2], A44 = s.a[0];
  const T A51 = s.c[3], A52 = s.c[4], A53 = s.c[5], A54 = s.a[1], A55 = s.a[2];
  const T A61 = s.c[6], A62 = s.c[7], A63 = s.c[8], A64 = s.a[3], A65 = s.a[4], A66 = s.a[5];
  if constexpr (sizeof(T) == 4) {
    // FP32 path: one reciprocal per pivot instead of a division per entry
    const T i1 = T(1) / A11;
    const T L21 = A21 * i1, L31 = A31 * i1, L41 = A41 * i1, L51 = A51 * i1, L61 = A61 * i1;
    const T D2 = A22 - L21 * L21 * A11;
    const T i2 = T(1) / D2;
    const T L32 = (A32 - L21 * L31 * A11) * i2, L42 = (A42 - L21 * L41 * A11) * i2;
    const T L52 = (A52 - L21 * L51 * A11) * i2, L62 = (A62 - L21 * L61 * A11) * i2;
    const T D3 = A33 - (L31 * L31 * A11 + L32 * L32 * D2);
    const T i3 = T(1) / D3;
    const T L43 = (A43 - L31 * L41 * A11 - L32 * L42 * D2) * i3;
    const T L53 = (A53 - L31 * L51 * A11 - L32 * L52 * D2) * i3;
    const T L63 = (A63 - L31 * L61 * A11 - L32 * L62 * D2) * i3;
    const T D4 = A44 - (L41 * L41 * A11 + L42 * L42 * D2 + L43 * L43 * D3);
    const T i4 = T(1) / D4;
    const T L54 = (A54 - L41 * L51 * A11 - L42 * L52 * D2 - L43 * L53 * D3) * i4;
    const T L64 = (A64 - L41 * L61 * A11 - L42 * L62 * D2 - L43 * L63 * D3) * i4;
    const T D5 = A55 - (L51 * L51 * A11 + L52 * L52 * D2 + L53 * L53 * D3 + L54 * L54 * D4);
    const T i5 = T(1) / D5;
    const T L65 = (A65 - L51 * L61 * A11 - L52 * L62 * D2 - L53 * L63 * D3 - L54 * L64 * D4) * i5;
    const T D6 = A66 - (L61 * L61 * A11 + L62 * L62 * D2 + L63 * L63 * D3 + L64 * L64 * D4 + L65 * L65 * D5);
    const T i6 = T(1) / D6;
    const T y1 = bl0;
    const T y2 = bl1 - L21 * y1;
    const T y3 = bl2 - L31 * y1 - L32 * y2;
    const T y4 = ba0 - L41 * y1 - L42 * y2 - L43 * y3;
    const T y5 = ba1 - L51 * y1 - L52 * y2 - L53 * y3 - L54 * y4;
    const T y6 = ba2 - L61 * y1 - L62 * y2 - L63 * y3 - L64 * y4 - L65 * y5;
    xa.z = y6 * i6;
    xa.y = y5 * i5 - L65 * xa.z;
    xa.x = y4 * i4 - L54 * xa.y - L64 * xa.z;
    xl.z = y3 * i3 - L43 * xa.x - L53 * xa.y - L63 * xa.z;
    xl.y = y2 * i2 - L32 * xl.z - L42 * xa.x - L52 * xa.y - L62 * xa.z;
    xl.x = y1 * i1 - L21 * xl.y - L31 * xl.z - L41 * xa.x - L51 * xa.y - L61 * xa.z;
    return;
  }
  const T L21 = A21 / A11, L31 = A31 / A11, L41 = A41 / A11, L51 = A51 / A11, L61 = A61 / A11;
  const T D1 = A11;
  const T D2 = A22 - L21 * L21 * D1;
  const T L32 = (A32 - L21 * L31 * D1) / D2;
  const T L42 = (A42 - L21 * L41 * D1) / D2;
  const T L52 = (A52 - L21 * L51 * D1) / D2;
  const T L62 = (A62 - L21 * L61 * D1) / D2;
  const T D3 = A33 - (L31 * L31 * D1 + L32 * L32 * D2);
  const T L43 = (A43 - L31 * L41 * D1 - L32 * L42 * D2) / D3;
  const T L53 = (A53 - L31 * L51 * D1 - L32 * L52 * D2) / D3;
  const T L63 = (A63 - L31 * L61 * D1 - L32 * L62 * D2) / D3;
  const T D4 = A44 - (L41 * L41 * D1 + L42 * L42 * D2 + L43 * L43 * D3);
  const T L54 = (A54 - L41 * L51 * D1 - L42 * L52 * D2 - L43 * L53 * D3) / D4;
  const T L64 = (A64 - L41 * L61 * D1 - L42 * L62 * D2 - L43 * L63 * D3) / D4;
  const T D5 = A55 - (L51 * L51 * D1 + L52 * L52 * D2 + L53 * L53 * D3 + L54 * L54 * D4);
  const T L65 = (A65 - L51 * L61 * D1 - L52 * L62 * D2 - L53 * L63 * D3 - L54 * L64 * D4) / D5;
  const T D6 = A66 - (L61 * L61 * D1 + L62 * L62 * D2 + L63 * L63 * D3 + L64 * L64 * D4 + L65 * L65 * D5);
  const T y1 = bl0;
  const T y2 = bl1 - L21 * y1;
  const T y3 = bl2 - L31 * y1 - L32 * y2;
  const T y4 = ba0 - L41 * y1 - L42 * y2 - L43 * y3;
  const T y5 = ba1 - L51 * y1 - L52 * y2 - L53 * y3 - L54 * y4;
  const T y6 = ba2 - L61 * y1 - L62 * y2 - L63 * y3 - L64 * y4 - L65 * y5;
  const T z1 = y1 / D1, z2 = y2 / D2, z3 = y3 / D3, z4 = y4 / D4, z5 = y5 / D5, z6 = y6 / D6;
  xa.z = z6;
  xa.y = z5 - L65 * xa.z;
  xa.x = z4 - L54 * xa.y - L64 * xa.z;
  xl.z = z3 - L43 * xa.x - L53 * xa.y - L63 * xa.z;
  xl.y = z2 - L32 * xl.z - L42 * xa.x - L52 * xa.y - L62 * xa.z;
  xl.x = z1 - L21 * xl.y - L31 * xl.z - L41 * xa.x - L51 * xa.y - L61 * xa.z;
}

template <class T>
struct BState {
  V3<T> dp;    // p - p_t
  Q4<T> q;     // current orientation
  V3<T> dang;  // qsub(q, q_t)
};

template <class T>
__device__ __forceinline__ BState<T> load_state(const World &w, int i) {
  BState<T> s;
  const float4 qt = ld(&w.b.quatT[i]);
  const Q4<T> qT{(T)qt.x, (T)qt.y, (T)qt.z, (T)qt.w};
  // only the FP64 path consults the precision flag (FP64 bodies keep their
  // iterate in f64 shadows); the FP32 path issues its loads at once
  if (sizeof(T) == 8 && (ld(&w.b.flags[i]) & kBodyFp64)) {
    const D4 d = ldcg(&w.b.dpD[i]), q = ldcg(&w.b.quatD[i]);
    s.dp = V3<T>{(T)d.x, (T)d.y, (T)d.z};
    s.q = Q4<T>{(T)q.x, (T)q.y, (T)q.z, (T)q.w};
  } else {
    const float4 d = ldcg(&w.b.dp[i]), q = ldcg(&w.b.quat[i]);
    s.dp = V3<T>{(T)d.x, (T)d.y, (T)d.z};
    s.q = Q4<T>{(T)q.x, (T)q.y, (T)q.z, (T)q.w};
  }
  s.dang = qsub(s.q, qT);
  return s;
}

template <class T>
struct ContactEval {
  V3<T> C, F;
  bool within;
};

// The contact extensions of AVBD_CONTACT_MATERIALS (the WebGPU engine's,
// src/physics/gpu/shaders.js:1806-1845): the pair's dynamic friction, a
// positive contact skin, the contact's restitution bias, and whether this
// pass is the post-stabilisation projection (no bias there).
template <class T>
struct ContactExt {
  bool on;
  bool skin, projection;
  T mud;
  float bias;
};

// manifold.js:358-409 in delta form: C = (1 - alpha) C0 + n_r . (dx_A - dx_B),
// dx = delta + dtheta x r_world(x_t). With the extensions: a positive gap is
// kept unscaled while the skin is on, the restitution bias comes off the
// normal row, a static contact (cL.w) is bounded by the static cone and a
// force outside it is clamped to the dynamic one.
template <class T>
__device__ __forceinline__ ContactEval<T> eval_contact(const V3<T> n[3], T mu, float4 cA, float4 cB, float4 cK, float4 cL,
                                              const BState<T> &A, const BState<T> &B, T alpha,
                                              const ContactExt<T> &x = ContactExt<T>{false, false, false, T(0), 0.f}) {
  const V3<T> rA{(T)cA.x, (T)cA.y, (T)cA.z}, rB{(T)cB.x, (T)cB.y, (T)cB.z};
  const V3<T> u = (A.dp + cross(A.dang, rA)) - (B.dp + cross(B.dang, rB));
  ContactEval<T> e;
  const T om = T(1) - alpha;
  if (x.on) {
    T c0 = (x.skin && (T)cA.w > T(0)) ? (T)cA.w : om * (T)cA.w;
    if (!x.projection) c0 = c0 - (T)x.bias;
    e.C.x = c0 + dot(n[0], u);
  } else {
    e.C.x = om * (T)cA.w + dot(n[0], u);
  }
  e.C.y = om * (T)cB.w + dot(n[1], u);
  e.C.z = om * (T)cK.w + dot(n[2], u);
  e.F.x = (T)cK.x * e.C.x + (T)cL.x;
  e.F.y = (T)cK.y * e.C.y + (T)cL.y;
  e.F.z = (T)cK.z * e.C.z + (T)cL.z;
  e.F.x = e.F.x < T(0) ? e.F.x : T(0);
  const T fs = sqrt(e.F.y * e.F.y + e.F.z * e.F.z);
  if (x.on) {
    const T active = fabs(e.F.x) * (cL.w != 0.f ? mu : x.mud);
    e.within = fs <= active;
    if (!e.within && fs > T(0)) {
      const T dyn = fabs(e.F.x) * x.mud;
      e.F.y = e.F.y * dyn / fs;
      e.F.z = e.F.z * dyn / fs;
    }
    return e;
  }
  const T bounds = fabs(e.F.x) * mu;
  if (fs > bounds && fs > T(0)) {
    e.F.y *= bounds / fs;
    e.F.z *= bounds / fs;
  }
  e.within = fs <= bounds;
  return e;
}

template <class T>
__device__ __forceinline__ void manifold_rows(const World &w, int m, V3<T> n[3], T &mu, bool &sphere) {
  const float4 b0 = ld(&w.cur.basis0[m]), b1 = ld(&w.cur.basis1[m]), b2 = ld(&w.cur.basis2[m]);
  n[0] = V3<T>{(T)b0.x, (T)b0.y, (T)b0.z};
  n[1] = V3<T>{(T)b1.x, (T)b1.y, (T)b1.z};
  n[2] = V3<T>{(T)b2.x, (T)b2.y, (T)b2.z};
  mu = (T)b0.w;
  sphere = ((int)b1.w & 1) != 0;  // the narrow phase marks sphere pairs here (bit 1: a contact skin)
}

// A neighbour's state as the contact rows read it: displacement and
// qsub(q, q_t). The FP32 path reads what the neighbour published; the FP64
// path forms it from the orientation as load_state does.
template <class T>
__device__ __forceinline__ BState<T> load_other(const World &w, int i) {
  if (sizeof(T) == 8) return load_state<T>(w, i);
  BState<T> s;
  const float4 d = ldcg(&w.b.dp[i]), a = ldcg(&w.b.dang[i]);
  s.dp = V3<T>{(T)d.x, (T)d.y, (T)d.z};
  s.dang = V3<T>{(T)a.x, (T)a.y, (T)a.z};
  s.q = Q4<T>{T(0), T(0), T(0), T(1)};  // not read by the contact rows
  return s;
}

// One contact of a body's per-contact adjacency (slot = manifold * 8 + k),
// with everything its primal stamp and dual update read. Loaded once per
// body update: the dual reuses it, since no other body writes this contact's
// multiplier and stiffness between this body's primal and dual.
template <class T>
struct ContactData {
  V3<T> n[3];
  T mu;
  float4 cA, cB, cK, cL;
  BState<T> o;
  int slot, side;
  bool owned;  // this body owns the contact's dual update
  bool sphere;
  ContactExt<T> x;  // AVBD_CONTACT_MATERIALS
};

// The extension fields of a contact (AVBD_CONTACT_MATERIALS; off otherwise).
template <class T>
__device__ __forceinline__ void load_ext(const World &w, ContactData<T> &d, float b1w, float b2w, T alpha) {
  d.x.on = true;
  d.x.skin = ((int)b1w & 2) != 0;
  d.x.mud = (T)b2w;
  d.x.bias = ld(&w.cur.cX[d.slot]);
  d.x.projection = w.p.postStabilize && alpha < T(0.5);
}

template <class T, bool E>
__device__ __forceinline__ ContactData<T> load_contact(const World &w, int2 ent, T alpha) {
  ContactData<T> d;
  d.slot = ent.x >> 2;
  d.owned = (ent.x & 2) != 0;
  d.side = ent.x & 1;
  manifold_rows(w, d.slot >> 3, d.n, d.mu, d.sphere);
  d.cA = ld(&w.cur.cA[d.slot]);
  d.cB = ld(&w.cur.cB[d.slot]);
  d.cK = __ldcg(&w.cur.cK[d.slot]);
  d.cL = __ldcg(&w.cur.cL[d.slot]);
  d.o = load_other<T>(w, ent.y);
  d.x.on = false;
  if (E) load_ext<T>(w, d, ld(&w.cur.basis1[d.slot >> 3]).w, ld(&w.cur.basis2[d.slot >> 3]).w, alpha);
  return d;
}

template <class T>
__device__ __forceinline__ void contact_primal(const ContactData<T> &d, const BState<T> &self, T alpha, Sys<T> &s) {
  const BState<T> &A = d.side ? d.o : self;
  const BState<T> &B = d.side ? self : d.o;
  const T sgn = d.side ? T(-1) : T(1);
  const ContactEval<T> e = eval_contact(d.n, d.mu, d.cA, d.cB, d.cK, d.cL, A, B, alpha, d.x);
  const V3<T> r = d.side ? V3<T>{(T)d.cB.x, (T)d.cB.y, (T)d.cB.z} : V3<T>{(T)d.cA.x, (T)d.cA.y, (T)d.cA.z};
  const T kk[3] = {(T)d.cK.x, (T)d.cK.y, (T)d.cK.z};
  const T ff[3] = {e.F.x, e.F.y, e.F.z};
#pragma unroll
  for (int row = 0; row < 3; row++) {
    const V3<T> a = cross(r, d.n[row]);
    stamp_row(s, kk[row], d.n[row], a);
    const T f = sgn * ff[row];
    s.bl[0] += f * d.n[row].x; s.bl[1] += f * d.n[row].y; s.bl[2] += f * d.n[row].z;
    s.ba[0] += f * a.x; s.ba[1] += f * a.y; s.ba[2] += f * a.z;
  }
}

// manifold.js:447-491 for one contact, with the body's updated state.
template <class T>
__device__ __forceinline__ void contact_dual(const World &w, const ContactData<T> &d, const BState<T> &self, T alpha) {
  const BState<T> &A = d.side ? d.o : self;
  const BState<T> &B = d.side ? self : d.o;
  const T beta = (T)w.p.betaLin, kmax = (T)w.p.penaltyMax, thr = (T)w.p.stickThreshold;
  const ContactEval<T> e = eval_contact(d.n, d.mu, d.cA, d.cB, d.cK, d.cL, A, B, alpha, d.x);
  float4 cK = d.cK;
  float stick = d.cL.w;
  if (e.F.x < T(0)) cK.x = (float)fmin((T)cK.x + beta * fabs(e.C.x), kmax);
  if (e.within) {
    cK.y = (float)fmin((T)cK.y + beta * fabs(e.C.y), kmax);
    cK.z = (float)fmin((T)cK.z + beta * fabs(e.C.z), kmax);
    stick = sqrt(e.C.y * e.C.y + e.C.z * e.C.z) < thr ? 1.f : 0.f;
  } else if (d.sphere) {
    stick = 0.f;
  }
  if (d.x.on) stick = e.within ? 1.f : 0.f;  // static = inside the cone (shaders.js:2253-2260)
  __stcg(&w.cur.cK[d.slot], cK);
  __stcg(&w.cur.cL[d.slot], make_float4((float)e.F.x, (float)e.F.y, (float)e.F.z, stick));
}

// Joint geometry at the current iterate (joint.js:115-129), delta form.
template <class T>
struct JointGeo {
  V3<T> Clin, Cang;
  V3<T> rAw, rBw;
};

template <class T>
__device__ __forceinline__ JointGeo<T> joint_geo(const World &w, int j, int2 ab, const BState<T> &A, const BState<T> &B,
                                        bool hasA) {
  JointGeo<T> g;
  V3<T> dpt;
  if (sizeof(T) == 8) {
    const D4 d = ld(&w.j.dptD[j]);
    dpt = V3<T>{(T)d.x, (T)d.y, (T)d.z};
  } else {
    const float4 d = ld(&w.j.dpt[j]);
    dpt = V3<T>{(T)d.x, (T)d.y, (T)d.z};
  }
  const float4 ra = ld(&w.j.rAF[j]), rb = ld(&w.j.rBF[j]);
  const D4 raD = ld(&w.j.rAD[j]), rbD = ld(&w.j.rBD[j]);
  const V3<T> rAl = sizeof(T) == 8 ? V3<T>{(T)raD.x, (T)raD.y, (T)raD.z} : V3<T>{(T)ra.x, (T)ra.y, (T)ra.z};
  const V3<T> rBl = sizeof(T) == 8 ? V3<T>{(T)rbD.x, (T)rbD.y, (T)rbD.z} : V3<T>{(T)rb.x, (T)rb.y, (T)rb.z};
  g.rBw = qrotate(B.q, rBl);
  if (hasA) {
    g.rAw = qrotate(A.q, rAl);
    g.Clin = ((dpt + (A.dp - B.dp)) + g.rAw) - g.rBw;
  } else {
    g.rAw = V3<T>{0, 0, 0};
    g.Clin = (dpt - B.dp) - g.rBw;
  }
  const Q4<T> qA = hasA ? A.q : Q4<T>{0, 0, 0, 1};
  g.Cang = qsub(qA, B.q) * (T)ld(&w.j.stiff[j]).w;
  return g;
}

// The linear rows of a ball socket on one of its bodies (joint.js:162-221):
// penalties K, forces F = K C + lambda, the body's Jacobians jLin = sl I and
// jAng = S = skew(v), and the geometric stiffness of the lever arm r
// (-(F.r) I + r F^T, column-norm lumped onto the angular diagonal).
template <class T>
__device__ __forceinline__ void stamp_ball_socket(Sys<T> &s, const T K[3], const T F[3], V3<T> v, V3<T> r, T sl) {
  // skew(v) rows: [0,-vz,vy],[vz,0,-vx],[-vy,vx,0]
  const T S[9] = {T(0), -v.z, v.y, v.z, T(0), -v.x, -v.y, v.x, T(0)};
#pragma unroll
  for (int rr = 0; rr < 3; rr++) s.l[L(rr, rr)] += K[rr];
  // jAng^T K jAng  and  jAng^T K jLin = sl * (S^T K)
#pragma unroll
  for (int a = 0; a < 3; a++) {
#pragma unroll
    for (int b = 0; b <= a; b++) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < 3; q++) acc += S[q * 3 + a] * K[q] * S[q * 3 + b];
      s.a[L(a, b)] += acc;
    }
#pragma unroll
    for (int b = 0; b < 3; b++) s.c[a * 3 + b] += sl * S[b * 3 + a] * K[b];
  }
  const T fr = F[0] * r.x + F[1] * r.y + F[2] * r.z;
  const T rv[3] = {r.x, r.y, r.z};
#pragma unroll
  for (int col = 0; col < 3; col++) {
    T n2 = T(0);
#pragma unroll
    for (int row = 0; row < 3; row++) {
      const T h = (row == col ? -fr : T(0)) + rv[row] * F[col];
      n2 += h * h;
    }
    s.a[L(col, col)] += sqrt(n2);
  }
#pragma unroll
  for (int a = 0; a < 3; a++) {
    s.bl[a] += sl * F[a];
    s.ba[a] += S[0 * 3 + a] * F[0] + S[1 * 3 + a] * F[1] + S[2 * 3 + a] * F[2];
  }
}

// The grab on body i (the joint's B side, its A side the world target):
// C = target - (p + R r), F = k C (shaders.js:2119-2161).
template <class T>
__device__ __noinline__ Sys<T> grab_primal(const World &w, int i, const BState<T> self, Sys<T> s) {
  const Grab *g = w.grab;
  const D4 tg = ld(&g->target), pB = ld(&w.b.pos[i]);
  const V3<T> dpt{(T)(tg.x - pB.x), (T)(tg.y - pB.y), (T)(tg.z - pB.z)};
  V3<T> rl;
  if (sizeof(T) == 8) {
    const D4 l = ld(&g->localD);
    rl = V3<T>{(T)l.x, (T)l.y, (T)l.z};
  } else {
    const float4 l = ld(&g->local);
    rl = V3<T>{(T)l.x, (T)l.y, (T)l.z};
  }
  const V3<T> rW = qrotate(self.q, rl);
  const V3<T> C = (dpt - self.dp) - rW;
  const T k = (T)ld(&g->k);
  const T K[3] = {k, k, k}, F[3] = {k * C.x, k * C.y, k * C.z};
  stamp_ball_socket<T>(s, K, F, rW, -rW, T(-1));
  return s;
}

template <class T>
__device__ __forceinline__ void joint_primal(const World &w, int j, int side, const BState<T> &self, T alpha, Sys<T> &s) {
  if (__ldcg(&w.j.state[j])) return;
  const int2 ab = ld(&w.j.bodies[j]);
  const bool hasA = ab.x >= 0;
  BState<T> o;
  if (side == 0) o = load_state<T>(w, ab.y);
  else if (hasA) o = load_state<T>(w, ab.x);
  const BState<T> &A = side ? o : self;
  const BState<T> &B = side ? self : o;
  const JointGeo<T> g = joint_geo(w, j, ab, A, B, hasA);
  const D4 sf = ld(&w.j.stiff[j]);
  const float4 kl = __ldcg(&w.j.penLin[j]);
  if (kl.x * kl.x + kl.y * kl.y + kl.z * kl.z > 0.f) {
    const D4 lam = ldcg(&w.j.lamLin[j]);
    const float4 c0 = ld(&w.j.c0Lin[j]);
    V3<T> C = g.Clin;
    if (isinf(sf.x)) C = C - V3<T>{(T)c0.x, (T)c0.y, (T)c0.z} * alpha;
    const T K[3] = {(T)kl.x, (T)kl.y, (T)kl.z};
    const T F[3] = {K[0] * C.x + (T)lam.x, K[1] * C.y + (T)lam.y, K[2] * C.z + (T)lam.z};
    // A: jLin = I, jAng = skew(-rAw), r = rAw ; B: jLin = -I, jAng = skew(rBw), r = -rBw
    stamp_ball_socket<T>(s, K, F, side ? g.rBw : -g.rAw, side ? -g.rBw : g.rAw, side ? T(-1) : T(1));
  }
  const float4 ka = __ldcg(&w.j.penAng[j]);
  if (ka.x * ka.x + ka.y * ka.y + ka.z * ka.z > 0.f) {
    const D4 lam = ldcg(&w.j.lamAng[j]);
    const float4 c0 = ld(&w.j.c0Ang[j]);
    V3<T> C = g.Cang;
    if (isinf(sf.y)) C = C - V3<T>{(T)c0.x, (T)c0.y, (T)c0.z} * alpha;
    const T st = side ? -(T)sf.w : (T)sf.w;
    const T K[3] = {(T)ka.x, (T)ka.y, (T)ka.z};
    const T F[3] = {K[0] * C.x + (T)lam.x, K[1] * C.y + (T)lam.y, K[2] * C.z + (T)lam.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
      s.a[L(a, a)] += st * K[a] * st;
      s.ba[a] += st * F[a];
    }
  }
}

template <class T>
__device__ __forceinline__ void joint_dual(const World &w, int j, int side, const BState<T> &self, T alpha) {
  if (__ldcg(&w.j.state[j])) return;
  const int2 ab = ld(&w.j.bodies[j]);
  const bool hasA = ab.x >= 0;
  BState<T> o;
  if (side == 0) o = load_state<T>(w, ab.y);
  else if (hasA) o = load_state<T>(w, ab.x);
  const BState<T> &A = side ? o : self;
  const BState<T> &B = side ? self : o;
  const JointGeo<T> g = joint_geo(w, j, ab, A, B, hasA);
  const D4 sf = ld(&w.j.stiff[j]);
  const double kmax = w.p.penaltyMax;
  float4 kl = __ldcg(&w.j.penLin[j]);
  D4 ll = ldcg(&w.j.lamLin[j]);
  if (kl.x * kl.x + kl.y * kl.y + kl.z * kl.z > 0.f) {
    V3<T> C = g.Clin;
    if (isinf(sf.x)) {
      const float4 c0 = ld(&w.j.c0Lin[j]);
      C = C - V3<T>{(T)c0.x, (T)c0.y, (T)c0.z} * alpha;
      ll.x = (double)kl.x * (double)C.x + ll.x;
      ll.y = (double)kl.y * (double)C.y + ll.y;
      ll.z = (double)kl.z * (double)C.z + ll.z;
    }
    const double cap = fmin(sf.x, kmax);
    kl.x = (float)fmin((double)kl.x + w.p.betaLin * fabs((double)C.x), cap);
    kl.y = (float)fmin((double)kl.y + w.p.betaLin * fabs((double)C.y), cap);
    kl.z = (float)fmin((double)kl.z + w.p.betaLin * fabs((double)C.z), cap);
  }
  float4 ka = __ldcg(&w.j.penAng[j]);
  D4 la = ldcg(&w.j.lamAng[j]);
  if (ka.x * ka.x + ka.y * ka.y + ka.z * ka.z > 0.f) {
    V3<T> C = g.Cang;
    if (isinf(sf.y)) {
      const float4 c0 = ld(&w.j.c0Ang[j]);
      C = C - V3<T>{(T)c0.x, (T)c0.y, (T)c0.z} * alpha;
      la.x = (double)ka.x * (double)C.x + la.x;
      la.y = (double)ka.y * (double)C.y + la.y;
      la.z = (double)ka.z * (double)C.z + la.z;
    }
    const double cap = fmin(sf.y, kmax);
    ka.x = (float)fmin((double)ka.x + w.p.betaAng * fabs((double)C.x), cap);
    ka.y = (float)fmin((double)ka.y + w.p.betaAng * fabs((double)C.y), cap);
    ka.z = (float)fmin((double)ka.z + w.p.betaAng * fabs((double)C.z), cap);
  }
  // fracture on |lambda_ang| (joint.js:307-316)
  if (la.x * la.x + la.y * la.y + la.z * la.z > sf.z * sf.z) {
    kl = make_float4(0.f, 0.f, 0.f, 0.f);
    ka = kl;
    ll = mkd4(0, 0, 0, 0);
    la = ll;
    __stcg(&w.j.state[j], kBroken);
  }
  __stcg(&w.j.penLin[j], kl);
  __stcg(&w.j.penAng[j], ka);
  stcg(&w.j.lamLin[j], ll);
  stcg(&w.j.lamAng[j], la);
}

// spring.js:447-458: d, |d| and C at the current iterate.
template <class T>
__device__ __forceinline__ bool spring_eval(const World &w, int sIdx, const BState<T> &A, const BState<T> &B, V3<T> &d,
                                   T &len, V3<T> &rAw, V3<T> &rBw) {
  V3<T> dpt, rAl, rBl;
  if (sizeof(T) == 8) {
    const D4 x = ld(&w.s.dptD[sIdx]), a = ld(&w.s.rAD[sIdx]), b = ld(&w.s.rBD[sIdx]);
    dpt = V3<T>{(T)x.x, (T)x.y, (T)x.z};
    rAl = V3<T>{(T)a.x, (T)a.y, (T)a.z};
    rBl = V3<T>{(T)b.x, (T)b.y, (T)b.z};
  } else {
    const float4 x = ld(&w.s.dpt[sIdx]), a = ld(&w.s.rAF[sIdx]), b = ld(&w.s.rBF[sIdx]);
    dpt = V3<T>{(T)x.x, (T)x.y, (T)x.z};
    rAl = V3<T>{(T)a.x, (T)a.y, (T)a.z};
    rBl = V3<T>{(T)b.x, (T)b.y, (T)b.z};
  }
  rAw = qrotate(A.q, rAl);
  rBw = qrotate(B.q, rBl);
  d = ((dpt + (A.dp - B.dp)) + rAw) - rBw;
  len = sqrt(dot(d, d));
  return len > T(1.0e-6);
}

template <class T>
__device__ __forceinline__ void spring_primal(const World &w, int sIdx, int side, const BState<T> &self, Sys<T> &s) {
  if (__ldcg(&w.s.state[sIdx])) return;
  const int2 ab = ld(&w.s.bodies[sIdx]);
  const BState<T> o = load_state<T>(w, side ? ab.x : ab.y);
  const BState<T> &A = side ? o : self;
  const BState<T> &B = side ? self : o;
  V3<T> d, rAw, rBw;
  T len;
  if (!spring_eval(w, sIdx, A, B, d, len, rAw, rBw)) return;
  const T rest = (T)ld(&w.s.prm[sIdx]).y;
  const T k = (T)__ldcg(&w.s.penalty[sIdx]);
  const V3<T> n = d * (T(1) / len);
  const T C = len - rest;
  const T f = k * C;
  const V3<T> rW = side ? rBw : rAw;
  const V3<T> jl = side ? -n : n;
  const V3<T> ja = side ? -cross(rW, n) : cross(rW, n);
  stamp_row(s, k, jl, ja);
  s.bl[0] += f * jl.x; s.bl[1] += f * jl.y; s.bl[2] += f * jl.z;
  s.ba[0] += f * ja.x; s.ba[1] += f * ja.y; s.ba[2] += f * ja.z;
  if (w.p.springGeometric) {  // spring.js:564-616
    const T sg = side ? T(-1) : T(1);
    const T nv[3] = {n.x, n.y, n.z}, rv[3] = {rW.x, rW.y, rW.z};
    T P[9], Sk[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) P[a * 3 + b] = ((a == b ? T(1) : T(0)) - nv[a] * nv[b]) / len;
    Sk[0] = 0; Sk[1] = -rW.z; Sk[2] = rW.y;
    Sk[3] = rW.z; Sk[4] = 0; Sk[5] = -rW.x;
    Sk[6] = -rW.y; Sk[7] = rW.x; Sk[8] = 0;
    T SP[9], PS[9];
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) {
        SP[a * 3 + b] = Sk[a * 3] * P[b] + Sk[a * 3 + 1] * P[3 + b] + Sk[a * 3 + 2] * P[6 + b];
        PS[a * 3 + b] = P[a * 3] * Sk[b] + P[a * 3 + 1] * Sk[3 + b] + P[a * 3 + 2] * Sk[6 + b];
      }
    const T ndr = dot(n, rW);
    const T af = fabs(f);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      // linear column: Gll = P, Gal = S P
      T n2 = T(0);
#pragma unroll
      for (int r = 0; r < 3; r++) n2 += P[r * 3 + c] * P[r * 3 + c] + SP[r * 3 + c] * SP[r * 3 + c];
      s.l[L(c, c)] += sqrt(n2) * af;
      // angular column: Gla = -P S, Gaa = -S P S + sg(-(n.r) I + r n^T)
      T m2 = T(0);
#pragma unroll
      for (int r = 0; r < 3; r++) {
        const T gla = -PS[r * 3 + c];
        const T sps = SP[r * 3] * Sk[c] + SP[r * 3 + 1] * Sk[3 + c] + SP[r * 3 + 2] * Sk[6 + c];
        const T gaa = -sps + sg * ((r == c ? -ndr : T(0)) + rv[r] * nv[c]);
        m2 += gla * gla + gaa * gaa;
      }
      s.a[L(c, c)] += sqrt(m2) * af;
    }
  }
}

template <class T>
__device__ __forceinline__ void spring_dual(const World &w, int sIdx, int side, const BState<T> &self) {
  if (__ldcg(&w.s.state[sIdx])) return;
  const int2 ab = ld(&w.s.bodies[sIdx]);
  const BState<T> o = load_state<T>(w, side ? ab.x : ab.y);
  const BState<T> &A = side ? o : self;
  const BState<T> &B = side ? self : o;
  V3<T> d, rAw, rBw;
  T len;
  if (!spring_eval(w, sIdx, A, B, d, len, rAw, rBw)) return;
  const D4 prm = ld(&w.s.prm[sIdx]);
  const double C = (double)len - prm.y;
  if (isfinite(prm.z) && prm.y > 1.0e-6) {  // spring.js:461-470
    const double strain = fmax(0.0, C / prm.y);
    double peak = __ldcg(&w.s.peak[sIdx]);
    if (strain > peak) __stcg(&w.s.peak[sIdx], strain);
    if (strain > prm.z) {
      __stcg(&w.s.state[sIdx], kBroken);
      __stcg(&w.s.penalty[sIdx], 0.f);
      return;
    }
  }
  if (!w.p.springRamp) return;
  const double k = __ldcg(&w.s.penalty[sIdx]);
  __stcg(&w.s.penalty[sIdx], (float)fmin(k + w.p.betaLin * fabs(C), fmin(prm.x, w.p.penaltyMax)));
}

// Owner of a constraint's dual update: its endpoint with the larger colour
// (static endpoints have colour -1).
__device__ inline bool owns(int myColor, int otherColor) { return myColor > otherColor; }

// Out-of-line helpers for the less common entries of a body's update: its
// joints and springs, and contacts beyond the first one per lane. Keeping
// them out of line keeps the common path (one contact per lane, held in
// registers from the primal stamp to the dual update) within the register
// budget of two resident blocks per SM; the callee pays its own spills.
// First joint/spring entry of this lane: the smallest e >= nm with e = lane (mod G).
__device__ __forceinline__ int first_extra(int lane, int nm, int G) {
  return lane < nm ? lane + ((nm - lane + G - 1) / G) * G : lane;
}

template <class T, bool E>
__device__ __noinline__ void extra_primal(const World &w, int i, int cb, int nm, int cStart, int total, int lane,
                                          int G, const BState<T> &self, T alpha, Sys<T> &s) {
  // contacts beyond the lane's first, two at a time so that their loads overlap
  int e = lane + G;
  for (; e + G < nm; e += 2 * G) {
    const int2 ea = ld(&w.a.centry[cb + e]), eb = ld(&w.a.centry[cb + e + G]);
    const ContactData<T> da = load_contact<T, E>(w, ea, alpha);
    const ContactData<T> db = load_contact<T, E>(w, eb, alpha);
    contact_primal<T>(da, self, alpha, s);
    contact_primal<T>(db, self, alpha, s);
  }
  if (e < nm) contact_primal<T>(load_contact<T, E>(w, ld(&w.a.centry[cb + e]), alpha), self, alpha, s);
  for (e = first_extra(lane, nm, G); e < total; e += G) {
    const uint32_t ref = ld(&w.g.cRef[cStart + e - nm]);
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    if (type == kRefJoint) joint_primal<T>(w, (int)idx, (int)side, self, alpha, s);
    else spring_primal<T>(w, (int)idx, (int)side, self, s);
  }
}

// The dual updates of the extra entries this body owns; a contact's data is
// loaded only when its owner bit says so.
template <class T, bool E>
__device__ __noinline__ void extra_dual(const World &w, int i, int cb, int nm, int cStart, int total, int lane, int G,
                                        const BState<T> &self, T alpha) {
  int pending = -1;  // an owned contact waiting for a partner, so loads go two at a time
  for (int e = lane + G; e < nm; e += G) {
    const int2 ent = ld(&w.a.centry[cb + e]);
    if (!(ent.x & 2)) continue;
    if (pending < 0) {
      pending = e;
      continue;
    }
    const ContactData<T> da = load_contact<T, E>(w, ld(&w.a.centry[cb + pending]), alpha);
    const ContactData<T> db = load_contact<T, E>(w, ent, alpha);
    contact_dual<T>(w, da, self, alpha);
    contact_dual<T>(w, db, self, alpha);
    pending = -1;
  }
  if (pending >= 0) contact_dual<T>(w, load_contact<T, E>(w, ld(&w.a.centry[cb + pending]), alpha), self, alpha);
  const int myColor = total > nm ? ld(&w.b.color[i]) : 0;
  for (int e = first_extra(lane, nm, G); e < total; e += G) {
    const uint32_t ref = ld(&w.g.cRef[cStart + e - nm]);
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    const int2 ab = type == kRefJoint ? ld(&w.j.bodies[idx]) : ld(&w.s.bodies[idx]);
    const int other = side ? ab.x : ab.y;
    const int oc = other >= 0 ? ld(&w.b.color[other]) : -1;
    if (!owns(myColor, oc)) continue;
    if (type == kRefJoint) joint_dual<T>(w, (int)idx, (int)side, self, alpha);
    else spring_dual<T>(w, (int)idx, (int)side, self);
  }
}

// Inertial terms of a body's system (solver.js:425-439), added by lane 0.
template <class T>
__device__ __forceinline__ void inertial_core(const SolverParams &P, T m, T I0, T I1, T I2, float4 y, float4 qy,
                                              const BState<T> &self, bool selfSphere, Sys<T> &s) {
  const T dt2 = (T)(P.dt * P.dt);
  const T ml = m / dt2;
  s.l[0] = ml; s.l[2] = ml; s.l[5] = ml;
  const V3<T> dy = self.dp - V3<T>{(T)y.x, (T)y.y, (T)y.z};
  s.bl[0] = ml * dy.x; s.bl[1] = ml * dy.y; s.bl[2] = ml * dy.z;
  // world moment R I R^T (rigid.js:228-247), / dt^2
  T M[9];
  const bool iso = !P.rotatedInertia || selfSphere;
  if (iso) {
    M[0] = I0; M[1] = 0; M[2] = 0; M[3] = 0; M[4] = I1; M[5] = 0; M[6] = 0; M[7] = 0; M[8] = I2;
  } else {
    const Q4<T> q = self.q;
    const T xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z, xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    const T wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    const T R[9] = {T(1) - T(2) * (yy + zz), T(2) * (xy - wz), T(2) * (xz + wy),
                    T(2) * (xy + wz), T(1) - T(2) * (xx + zz), T(2) * (yz - wx),
                    T(2) * (xz - wy), T(2) * (yz + wx), T(1) - T(2) * (xx + yy)};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) M[a * 3 + b] = R[a * 3] * I0 * R[b * 3] + R[a * 3 + 1] * I1 * R[b * 3 + 1] +
                                                R[a * 3 + 2] * I2 * R[b * 3 + 2];
  }
  const V3<T> dq = qsub(self.q, Q4<T>{(T)qy.x, (T)qy.y, (T)qy.z, (T)qy.w});
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = 0; b <= a; b++) s.a[L(a, b)] = M[a * 3 + b] / dt2;
  s.ba[0] = (M[0] * dq.x + M[1] * dq.y + M[2] * dq.z) / dt2;
  s.ba[1] = (M[3] * dq.x + M[4] * dq.y + M[5] * dq.z) / dt2;
  s.ba[2] = (M[6] * dq.x + M[7] * dq.y + M[8] * dq.z) / dt2;
}

template <class T>
__device__ __forceinline__ void inertial_terms(const World &w, int i, const BState<T> &self, bool selfSphere,
                                               Sys<T> &s) {
  const D4 md = ld(&w.b.massD[i]);
  inertial_core<T>(w.p, (T)md.x, (T)md.y, (T)md.z, (T)md.w, ld(&w.b.yLin[i]), ld(&w.b.yAng[i]), self, selfSphere, s);
}

__device__ inline int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ inline void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Reduce the group's partial systems, solve the 6x6 system (maths.js:660-725),
// integrate (maths.js:568-592) and publish the new iterate; on the last main
// iteration also the BDF1 velocity (solver.js:476-488).
// publish: lane 0 releases *publish = pubValue once the body's new state is
// stored (what a later body of the tail segment reads of it), before the
// velocity and the dual updates.
template <class T>
__device__ __forceinline__ void finish_body(const World &w, int i, int lane, int G, unsigned mask, bool velocity,
                                            float4 qt, Sys<T> &s, BState<T> &self, int *publish = nullptr,
                                            int pubValue = 0) {
  const T dt = (T)w.p.dt;
  if constexpr (sizeof(T) == 4) {
    if (G == 32) group_reduce32(s);
    else if (G > 32) group_reduce_warps(s, G);
    else group_reduce(s, mask, G);
  } else {
    group_reduce(s, mask, G);
  }
  V3<T> xl, xa;
  ldlt_solve(s, -s.bl[0], -s.bl[1], -s.bl[2], -s.ba[0], -s.ba[1], -s.ba[2], xl, xa);
  self.dp = self.dp + xl;
  self.q = qintegrate(self.q, xa);
  self.dang = qsub(self.q, Q4<T>{(T)qt.x, (T)qt.y, (T)qt.z, (T)qt.w});
  if (lane != 0) return;
  __stcg(&w.b.dp[i], make_float4((float)self.dp.x, (float)self.dp.y, (float)self.dp.z, 0.f));
  __stcg(&w.b.quat[i], make_float4((float)self.q.x, (float)self.q.y, (float)self.q.z, (float)self.q.w));
  {  // what neighbours read: qsub of the f32 orientation, as load_state<float> forms it
    const V3<float> da =
        sizeof(T) == 4 ? V3<float>{(float)self.dang.x, (float)self.dang.y, (float)self.dang.z}
                       : qsub(Q4<float>{(float)self.q.x, (float)self.q.y, (float)self.q.z, (float)self.q.w},
                              Q4<float>{qt.x, qt.y, qt.z, qt.w});
    __stcg(&w.b.dang[i], make_float4(da.x, da.y, da.z, 0.f));
  }
  if (sizeof(T) == 8) {
    stcg(&w.b.dpD[i], mkd4((double)self.dp.x, (double)self.dp.y, (double)self.dp.z, 0.0));
    stcg(&w.b.quatD[i], mkd4((double)self.q.x, (double)self.q.y, (double)self.q.z, (double)self.q.w));
  }
  if (publish) st_release(publish, pubValue);
  if (velocity) {  // BDF1 (solver.js:476-488)
    w.b.prevVel[i] = ld(&w.b.vel[i]);
    w.b.vel[i] = make_float4((float)(self.dp.x / dt), (float)(self.dp.y / dt), (float)(self.dp.z / dt), 0.f);
    w.b.omega[i] = make_float4((float)(self.dang.x / dt), (float)(self.dang.y / dt), (float)(self.dang.z / dt), 0.f);
  }
}

// One body's update (solver.js:425-457) by a group of G lanes, followed by
// the dual updates (manifold.js:447, joint.js:255, spring.js:618) of the
// constraints it owns, and on the last main iteration its BDF1 velocity.
// Register form: the FP64 path.
template <class T, bool E>
__device__ void solve_body(const World &w, int4 rec, int lane, int G, unsigned mask, T alpha, bool dual, bool velocity) {
  const int i = rec.x, cb = rec.y, nm = rec.z - rec.y;
  // one round of loads: own state, constraint ranges and this lane's first contact
  BState<T> self = load_state<T>(w, i);
  const int cStart = ld(&w.g.cStart[i]), cEnd = ld(&w.g.cStart[i + 1]);
  const int total = nm + (cEnd - cStart);
  const bool selfSphere = (ld(&w.b.flags0[i]) & kBodySphere) != 0;
  const bool has0 = lane < nm;
  ContactData<T> d0;
  if (has0) d0 = load_contact<T, E>(w, ld(&w.a.centry[cb + lane]), alpha);
  const bool extra = total > nm || nm > G;  // joints, springs or more contacts than lanes
  Sys<T> s;
  zero(s);
  if (lane == 0) inertial_terms<T>(w, i, self, selfSphere, s);
  if (has0) contact_primal<T>(d0, self, alpha, s);
  if (extra) extra_primal<T, E>(w, i, cb, nm, cStart, total, lane, G, self, alpha, s);
  if (lane == 0 && ld(&w.grab->body) == i) s = grab_primal<T>(w, i, self, s);
  finish_body<T>(w, i, lane, G, mask, velocity, ld(&w.b.quatT[i]), s, self);
  if (!dual) return;
  // dual updates of the constraints this body owns (it has the larger colour)
  if (has0 && d0.owned) contact_dual<T>(w, d0, self, alpha);
  if (extra) extra_dual<T, E>(w, i, cb, nm, cStart, total, lane, G, self, alpha);
}

// ---------------------------------------------------------------------------
// Staged form (the FP32 path). Each lane copies the data of up to
// kStageSlots of its contacts - basis rows, the contact record, the other
// body's displacement and rotation - into shared memory with cp.async, all
// at once, then stamps them; a lane with no more than kStageSlots contacts
// still holds them at the dual update, which then reads no global memory but
// the writes. Slot (j, v) of thread t lives at stage[(j * kStageVecs + v) *
// kSolveBlock + t], so a warp's accesses are conflict-free.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async_ca(float4 *dst, const float4 *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_cg(float4 *dst, const float4 *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// What the solve writes during the kernel (multipliers, penalties, neighbour
// state) goes through L2 (.cg); what it only reads may also use L1 (.ca).
__device__ __forceinline__ void stage_contact(const World &w, int2 ent, float4 *st) {
  const int slot = ent.x >> 2, m = slot >> 3;
  cp_async_ca(st + 0 * kSolveBlock, &w.cur.basis0[m]);
  cp_async_ca(st + 1 * kSolveBlock, &w.cur.basis1[m]);
  cp_async_ca(st + 2 * kSolveBlock, &w.cur.basis2[m]);
  cp_async_ca(st + 3 * kSolveBlock, &w.cur.cA[slot]);
  cp_async_ca(st + 4 * kSolveBlock, &w.cur.cB[slot]);
  cp_async_cg(st + 5 * kSolveBlock, &w.cur.cK[slot]);
  cp_async_cg(st + 6 * kSolveBlock, &w.cur.cL[slot]);
  cp_async_cg(st + 7 * kSolveBlock, &w.b.dp[ent.y]);
  cp_async_cg(st + 8 * kSolveBlock, &w.b.dang[ent.y]);
}

template <bool E>
__device__ __forceinline__ ContactData<float> staged_contact(const World &w, const float4 *st, int2 ent, float alpha) {
  ContactData<float> d;
  d.slot = ent.x >> 2;
  d.owned = (ent.x & 2) != 0;
  d.side = ent.x & 1;
  const float4 b0 = st[0], b1 = st[kSolveBlock], b2 = st[2 * kSolveBlock];
  d.n[0] = V3<float>{b0.x, b0.y, b0.z};
  d.n[1] = V3<float>{b1.x, b1.y, b1.z};
  d.n[2] = V3<float>{b2.x, b2.y, b2.z};
  d.mu = b0.w;
  d.sphere = ((int)b1.w & 1) != 0;
  d.x.on = false;
  d.x.skin = ((int)b1.w & 2) != 0;
  d.x.mud = b2.w;
  d.cA = st[3 * kSolveBlock];
  d.cB = st[4 * kSolveBlock];
  d.cK = st[5 * kSolveBlock];
  d.cL = st[6 * kSolveBlock];
  const float4 dp = st[7 * kSolveBlock], da = st[8 * kSolveBlock];
  d.o.dp = V3<float>{dp.x, dp.y, dp.z};
  d.o.dang = V3<float>{da.x, da.y, da.z};
  d.o.q = Q4<float>{0.f, 0.f, 0.f, 1.f};  // not read by the contact rows
  if (E) {
    d.x.on = true;
    d.x.bias = ld(&w.cur.cX[d.slot]);
    d.x.projection = w.p.postStabilize && alpha < 0.5f;
  }
  return d;
}


// The colour-phase solve's tail: the last colours (few bodies each) run as
// one dependency-driven segment instead of one phase each. A tail body of
// colour `color` in iteration t waits, before reading a neighbour, until
// every neighbour of a lower tail colour (>= from) has published progress
// t + 1; neighbours of earlier colours finished before the segment began,
// those of higher colours finished iteration t - 1 before its last barrier.
// from < 0: no waits.
struct TailWait {
  int from, color, need;
};

// Bounded: past the limit (or once another wait gave up) the timeout flag is
// set and the caller carries on, so that no group member is left at a named
// barrier; the kernel then ends at its next grid barrier and the step
// reports the timeout.
__device__ __forceinline__ void spin_progress(const World &w, int other, int need) {
  long long polls = 0;
  while (ld_acquire(&w.b.progress[other]) < need) {
    if (++polls > w.p.waitLimit || (*((volatile unsigned *)&w.ctl->flags) & kOvfTimeout)) {
      atomicOr(&w.ctl->flags, kOvfTimeout);
      return;
    }
    __nanosleep(32);
  }
}

__device__ __forceinline__ void tail_wait_body(const World &w, int other, const TailWait &tw) {
  const int oc = ld(&w.b.color[other]);  // statics: -1
  if (oc >= tw.from && oc < tw.color) spin_progress(w, other, tw.need);
}

// Stage chunk [k0, k0 + cnt) of this lane's contacts (contact e = lane + k G),
// after the tail waits on their other bodies when `tw` is given.
__device__ __forceinline__ int stage_chunk(const World &w, int cb, int lane, int G, int k0, int cnt, int2 *ent,
                                           float4 *stage, bool ownedOnly, const TailWait *tw = nullptr) {
  int staged = 0;
#pragma unroll
  for (int j = 0; j < kStageSlots; j++)
    if (j < cnt) ent[j] = ld(&w.a.centry[cb + lane + (k0 + j) * G]);
  if (tw) {
#pragma unroll
    for (int j = 0; j < kStageSlots; j++)
      if (j < cnt) tail_wait_body(w, ent[j].y, *tw);
  }
#pragma unroll
  for (int j = 0; j < kStageSlots; j++)
    if (j < cnt && (!ownedOnly || (ent[j].x & 2))) {
      stage_contact(w, ent[j], stage + j * kStageVecs * kSolveBlock);
      staged++;
    }
  cp_async_commit();
  return staged;
}

// The joints and springs of a body (entries nm..total of its constraint list).
// Out of line, so the body state and the partial system go by value and come
// back as the return value: a reference would let their address escape and
// keep them in local memory through the whole contact loop of every body.
template <class T, bool E>
__device__ __noinline__ Sys<T> constraints_primal(const World &w, int nm, int cStart, int total, int lane, int G,
                                                  const BState<T> self, T alpha, Sys<T> s) {
  for (int e = first_extra(lane, nm, G); e < total; e += G) {
    const uint32_t ref = ld(&w.g.cRef[cStart + e - nm]);
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    if (type == kRefJoint) joint_primal<T>(w, (int)idx, (int)side, self, alpha, s);
    else spring_primal<T>(w, (int)idx, (int)side, self, s);
  }
  return s;
}

template <class T, bool E>
__device__ __noinline__ void constraints_dual(const World &w, int i, int nm, int cStart, int total, int lane, int G,
                                              const BState<T> self, T alpha) {
  const int myColor = ld(&w.b.color[i]);
  for (int e = first_extra(lane, nm, G); e < total; e += G) {
    const uint32_t ref = ld(&w.g.cRef[cStart + e - nm]);
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    const int2 ab = type == kRefJoint ? ld(&w.j.bodies[idx]) : ld(&w.s.bodies[idx]);
    const int other = side ? ab.x : ab.y;
    const int oc = other >= 0 ? ld(&w.b.color[other]) : -1;
    if (!owns(myColor, oc)) continue;
    if (type == kRefJoint) joint_dual<T>(w, (int)idx, (int)side, self, alpha);
    else spring_dual<T>(w, (int)idx, (int)side, self);
  }
}

// The joint and spring partners of a tail body (entries nm..total).
__device__ __noinline__ void tail_wait_extra(const World &w, int nm, int cStart, int total, int lane, int G,
                                             const TailWait tw) {
  for (int e = first_extra(lane, nm, G); e < total; e += G) {
    const uint32_t ref = ld(&w.g.cRef[cStart + e - nm]);
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
    const int2 ab = type == kRefJoint ? ld(&w.j.bodies[idx]) : ld(&w.s.bodies[idx]);
    const int other = side ? ab.x : ab.y;
    if (other >= 0) tail_wait_body(w, other, tw);
  }
}

// `tw`: the tail waits of this body (null outside the tail segment).
template <bool E>
__device__ void solve_body_staged(const World &w, int4 rec, int lane, int G, unsigned mask, float alpha, bool dual,
                                  bool velocity, float4 *stage, const TailWait *tw = nullptr) {
  using T = float;
  const int i = rec.x, cb = rec.y, nm = rec.z - rec.y;
  const int nk = lane < nm ? (nm - lane + G - 1) / G : 0;  // this lane's contacts
  int2 ent[kStageSlots];
  int cnt = nk < kStageSlots ? nk : kStageSlots;
  // the body's own data (state, inertial terms: massF holds massD's f32
  // conversions) is requested before the contact entries, so that one round
  // trip serves both; the contact data then follows with cp.async
  const float4 qt = ld(&w.b.quatT[i]);
  const float4 d0 = ldcg(&w.b.dp[i]), q0 = ldcg(&w.b.quat[i]);
  const float4 mf = ld(&w.b.massF[i]), y = ld(&w.b.yLin[i]), qy = ld(&w.b.yAng[i]);
  const int cStart = ld(&w.g.cStart[i]), cEnd = ld(&w.g.cStart[i + 1]);
  const bool sphere = (ld(&w.b.flags0[i]) & kBodySphere) != 0;
  const bool grabbed = lane == 0 && ld(&w.grab->body) == i;
  stage_chunk(w, cb, lane, G, 0, cnt, ent, stage, false, tw);
  BState<T> self;  // as load_state<float> forms it
  self.dp = V3<T>{d0.x, d0.y, d0.z};
  self.q = Q4<T>{q0.x, q0.y, q0.z, q0.w};
  self.dang = qsub(self.q, Q4<T>{qt.x, qt.y, qt.z, qt.w});
  const int total = nm + (cEnd - cStart);
  Sys<T> s;
  zero(s);
  if (lane == 0) inertial_core<T>(w.p, mf.x, mf.y, mf.z, mf.w, y, qy, self, sphere, s);
  for (int k0 = 0;;) {
    cp_async_wait_all();
    for (int j = 0; j < cnt; j++)
      contact_primal<T>(staged_contact<E>(w, stage + j * kStageVecs * kSolveBlock, ent[j], alpha), self, alpha, s);
    k0 += cnt;
    if (k0 >= nk) break;
    cnt = nk - k0 < kStageSlots ? nk - k0 : kStageSlots;
    stage_chunk(w, cb, lane, G, k0, cnt, ent, stage, false, tw);
  }
  if (total > nm) {
    if (tw) tail_wait_extra(w, nm, cStart, total, lane, G, *tw);
    s = constraints_primal<T, E>(w, nm, cStart, total, lane, G, self, alpha, s);
  }
  if (grabbed) s = grab_primal<T>(w, i, self, s);
  // in the tail segment the body's progress is published as soon as its state is stored: the
  // bodies waiting for it (higher colours) own every constraint they share with it, so they
  // read nothing its dual updates write
  finish_body<T>(w, i, lane, G, mask, velocity, qt, s, self, tw ? &w.b.progress[i] : nullptr, tw ? tw->need : 0);
  if (!dual) return;
  if (nk <= kStageSlots) {
    // every contact of this lane is still staged; the owner alone writes a
    // contact's multiplier and penalty, and the other body is done with
    // this iteration, so the staged values are current
    for (int j = 0; j < cnt; j++)
      if (ent[j].x & 2) contact_dual<T>(w, staged_contact<E>(w, stage + j * kStageVecs * kSolveBlock, ent[j], alpha), self, alpha);
  } else {
    for (int k0 = 0; k0 < nk; k0 += kStageSlots) {
      const int c2 = nk - k0 < kStageSlots ? nk - k0 : kStageSlots;
      stage_chunk(w, cb, lane, G, k0, c2, ent, stage, true);
      cp_async_wait_all();
      for (int j = 0; j < c2; j++)
        if (ent[j].x & 2)
          contact_dual<T>(w, staged_contact<E>(w, stage + j * kStageVecs * kSolveBlock, ent[j], alpha), self, alpha);
    }
  }
  if (total > nm) constraints_dual<T, E>(w, i, nm, cStart, total, lane, G, self, alpha);
}

// The FP64 path is kept out of line so that its register demand (and any
// spills under the 2-blocks-per-SM bound) stays in the rare FP64 bodies
// instead of lowering the occupancy of the FP32 path.
template <bool E>
__device__ __noinline__ void solve_body_f64(const World &w, int4 rec, int lane, int G, unsigned mask, double alpha,
                                            bool dual, bool velocity) {
  solve_body<double, E>(w, rec, lane, G, mask, alpha, dual, velocity);
}

// The neighbours come from the body's manifold list (one entry per touching
// body, where the per-contact list has up to eight) and its joints/springs.
// tailFrom < 0: the wavefront's rule. Otherwise the tail segment's: only
// neighbours of a lower colour >= tailFrom, for iteration it.
__device__ bool wait_neighbors(const World &w, int i, int it, int lane, int G, unsigned mask, int tailFrom = -1) {
  const int myColor = ld(&w.b.color[i]);
  const int mb = ld(&w.a.start[i]);
  int me = ld(&w.a.start[i + 1]);
  if (me > w.a.cap) me = w.a.cap;
  const int jb = ld(&w.g.cStart[i]), je = ld(&w.g.cStart[i + 1]);
  const int nm = me - mb, total = nm + (je - jb);
  long long polls = 0;
  for (int e = lane; e < total; e += G) {
    int other;
    if (e < nm) {
      const uint32_t v = ld(&w.a.entry[mb + e]);
      const unsigned long long key = __ldg(reinterpret_cast<const unsigned long long *>(w.cur.key) + (v >> 1));
      other = (v & 1u) ? (int)(key >> 32) : (int)(key & 0xffffffffu);
    } else {
      const uint32_t ref = ld(&w.g.cRef[jb + e - nm]);
      const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu, side = ref & 1u;
      const int2 ab = type == kRefJoint ? ld(&w.j.bodies[idx]) : ld(&w.s.bodies[idx]);
      other = side ? ab.x : ab.y;
      if (other < 0) continue;
    }
    if (!(ld(&w.b.flags0[other]) & kBodyDynamic)) continue;
    const int oc = ld(&w.b.color[other]);
    const int need = tailFrom < 0 ? (oc < myColor ? it + 1 : it) : (oc >= tailFrom && oc < myColor ? it + 1 : 0);
    while (ld_acquire(&w.b.progress[other]) < need) {
      if (++polls > w.p.waitLimit || (*((volatile unsigned *)&w.ctl->flags) & kOvfTimeout)) {
        atomicOr(&w.ctl->flags, kOvfTimeout);
        polls = -1;
        break;
      }
      __nanosleep(32);
    }
    if (polls < 0) break;
  }
  return __all_sync(mask, polls >= 0);
}

// Every warp of a body's lane group past this point (G > 32: the group's
// named barrier, as in group_reduce_warps).
__device__ __forceinline__ void group_sync(int G, unsigned mask) {
  if (G <= 32) {
    __syncwarp(mask);
  } else {
    const int nw = G >> 5, w0 = (threadIdx.x >> 5) & ~(nw - 1);
    named_barrier(nw == 2 ? 1 + (w0 >> 1) : 3, G);
  }
}

// Colour phases separated by grid barriers. Each block takes the colour's
// lane chunks (Adjacency::laneTab) j, j + gridDim.x, ...: one body per lane
// group, a group's G lanes working on its constraints. j transposes the
// block index (k blocks on each of S SMs: block b takes j = (b mod k) S +
// b div k), so that a colour of fewer chunks than blocks spreads over
// distinct SMs whether the launch places consecutive blocks on one SM or
// deals them round the SMs (k and S coprime).
// The tail - the last colours, each of at most gridDim / kTailDiv chunks -
// is one segment per iteration with a single barrier: its chunks, in colour
// order, taken as above; a body waits only for its lower-colour tail
// neighbours (TailWait) and publishes its progress when done. Each group
// walks its chunks in increasing colour, so the earliest unfinished tail
// body always has its inputs ready (all blocks are resident).
constexpr int kTailDiv = 8;  // default of SolverParams::tailDiv
constexpr int kTailMinColors = 16;  // automatic: steps of fewer colours have no tail segment
constexpr int kChunkCache = 64;  // colours whose chunk bounds the solve keeps in shared memory
template <bool E>
__global__ void __launch_bounds__(kSolveBlock, 3) solve_kernel(World w) {
  if (step_skipped(w)) return;
  extern __shared__ float4 stageSm[];
  float4 *stage = stageSm + threadIdx.x;
  const SolverParams &P = w.p;
  Control *ctl = w.ctl;
  const int numColors = *((volatile int *)&ctl->numColors);
  const int warpLane = threadIdx.x & 31;
  const int total = P.iterations + (P.postStabilize ? 1 : 0);
  const int kb = P.solveBlocksPerSm > 0 ? P.solveBlocksPerSm : 1, S = gridDim.x / kb;
  const int jb = S * kb == (int)gridDim.x ? ((int)blockIdx.x % kb) * S + (int)blockIdx.x / kb : (int)blockIdx.x;
  // colour chunk bounds, constant through the solve: the first kChunkCache + 1
  // in shared memory, the rest (steps of many colours) through L1
  __shared__ int chunkSm[kChunkCache + 1];
  for (int k = threadIdx.x; k <= numColors && k <= kChunkCache; k += blockDim.x) chunkSm[k] = ld(&w.a.colorChunk[k]);
  __syncthreads();
  auto chunkAt = [&](int c) { return c <= kChunkCache ? chunkSm[c] : ld(&w.a.colorChunk[c]); };
  int tail = numColors;  // first tail colour
  // tailDiv 0 (automatic): a step of few colours keeps a barrier per colour,
  // where the segment's neighbour waits cost more than the barriers they save
  // (the standing 53-layer pyramid, 4-7 colours: 1.27 ms/step without a tail,
  // 1.56 with); > 0: always; < 0: never
  if (P.tailDiv > 0 || (P.tailDiv == 0 && numColors >= kTailMinColors)) {
    const int tailDiv = P.tailDiv > 0 ? P.tailDiv : kTailDiv;
    while (tail > 0 && chunkAt(tail) - chunkAt(tail - 1) <= (int)gridDim.x / tailDiv) tail--;
  }
  for (int it = 0; it < total; it++) {
    const double alpha = P.postStabilize ? (it < P.iterations ? 1.0 : 0.0) : P.alpha;
    const bool dual = it < P.iterations;
    const bool vel = it == P.iterations - 1;
    for (int c = 0; c < tail; c++) {
      const int q0 = chunkAt(c), q1 = chunkAt(c + 1);
      for (int q = q0 + jb; q < q1; q += gridDim.x) {
        const int e = ld(&w.a.laneTab[(size_t)q * kLaneMaxGroup + threadIdx.x]);
        if (e < 0) continue;
        const int G = 1 << (e & 7);
        const int lane = threadIdx.x & (G - 1);
        const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (warpLane & ~(G - 1)));
        const int4 rec = ld(&w.a.colorRec[e >> 4]);
        if (e & 8) solve_body_f64<E>(w, rec, lane, G, mask, alpha, dual, vel);
        else solve_body_staged<E>(w, rec, lane, G, mask, (float)alpha, dual, vel, stage);
      }
      if (!grid_barrier(ctl, w.p.barrierLimit)) return;
    }
    if (tail < numColors) {  // the tail segment of iteration it
      int c = tail;
      const int qEnd = chunkAt(numColors);
      for (int q = chunkAt(tail) + jb; q < qEnd; q += gridDim.x) {
        while (chunkAt(c + 1) <= q) c++;
        const int e = ld(&w.a.laneTab[(size_t)q * kLaneMaxGroup + threadIdx.x]);
        if (e < 0) continue;
        const int G = 1 << (e & 7);
        const int lane = threadIdx.x & (G - 1);
        const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << (warpLane & ~(G - 1)));
        const int4 rec = ld(&w.a.colorRec[e >> 4]);
        if (e & 8) {
          // a wait that gave up has set the timeout flag: the body is not
          // solved on stale data, and the kernel ends at the next grid barrier
          if (wait_neighbors(w, rec.x, it, lane, G, mask, tail)) {
            __syncwarp(mask);  // every lane's reads after the others' acquires
            solve_body_f64<E>(w, rec, lane, G, mask, alpha, dual, vel);
          }
          group_sync(G, mask);  // the group's writes before lane 0's release
          if (lane == 0) st_release(&w.b.progress[rec.x], it + 1);
        } else {
          const TailWait tw{tail, c, it + 1};  // publishes the body's progress itself
          solve_body_staged<E>(w, rec, lane, G, mask, (float)alpha, dual, vel, stage, &tw);
        }
      }
      if (!grid_barrier(ctl, w.p.barrierLimit)) return;
    }
  }
}

// ---------------------------------------------------------------------------
// Dependency-driven wavefront schedule. Body i may run iteration t once every
// neighbour of lower colour has completed iteration t and every neighbour of
// higher colour has completed iteration t - 1: exactly the order of the colour
// phases, without a grid-wide barrier between them. Each group walks its
// bodies in increasing (iteration, colour) order, so the earliest unfinished
// body always has its inputs ready and the schedule cannot deadlock while all
// blocks are resident (cooperative launch). Every wait is bounded.
// ---------------------------------------------------------------------------



template <bool E>
__global__ void __launch_bounds__(kSolveBlock, 3) wave_kernel(World w, int G) {
  if (step_skipped(w)) return;
  extern __shared__ float4 stageSm[];
  float4 *stage = stageSm + threadIdx.x;
  const SolverParams &P = w.p;
  Control *ctl = w.ctl;
  const int numColors = *((volatile int *)&ctl->numColors);
  const int lane = threadIdx.x & (G - 1);
  const int warpLane = threadIdx.x & 31;
  const unsigned mask = (G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (warpLane & ~(G - 1))));
  // groups interleaved across blocks, so a thin colour still spreads over all SMs
  const int groupsPerBlock = blockDim.x / G;
  const int group = (threadIdx.x / G) * gridDim.x + blockIdx.x;
  const int groups = groupsPerBlock * gridDim.x;
  const int total = P.iterations + (P.postStabilize ? 1 : 0);
  for (int it = 0; it < total; it++) {
    const double alpha = P.postStabilize ? (it < P.iterations ? 1.0 : 0.0) : P.alpha;
    const bool dual = it < P.iterations;
    const bool vel = it == P.iterations - 1;
    for (int c = 0; c < numColors; c++) {
      const int beg = ld(&w.a.colorStart[c]), end = ld(&w.a.colorStart[c + 1]);
      for (int k = beg + group; k < end; k += groups) {
        const int4 rec = ld(&w.a.colorRec[k]);
        const int i = rec.x;
        if (!wait_neighbors(w, i, it, lane, G, mask)) return;
        __syncwarp(mask);  // orders every lane's reads after the acquires of the others
        if (ld(&w.b.flags[i]) & kBodyFp64) solve_body_f64<E>(w, rec, lane, G, mask, alpha, dual, vel);
        else solve_body_staged<E>(w, rec, lane, G, mask, (float)alpha, dual, vel, stage);
        // the warp barrier orders every lane's writes before lane 0's release,
        // which makes them visible at gpu scope to whoever acquires the flag
        __syncwarp(mask);
        if (lane == 0) st_release(&w.b.progress[i], it + 1);
      }
    }
  }
}

// x_{t+1} = x_t + delta (f64); statics: prevVel <- vel (solver.js:479).
// Also the step's bookkeeping: its candidates become the next step's previous
// manifolds, or, for a skipped step, the skip is counted and nothing moves.
__global__ void commit_kernel(World w) {
  if (step_skipped(w)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->stepsSkipped++;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->prevCandidates = w.ctl->numCandidates;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x) {
    const int fl = w.b.flags[i];
    if (!(fl & kBodyDynamic)) {
      w.b.prevVel[i] = w.b.vel[i];
      continue;
    }
    D4 p = w.b.pos[i];
    double dx, dy, dz;
    if (fl & kBodyFp64) {
      const D4 d = w.b.dpD[i];
      dx = d.x; dy = d.y; dz = d.z;
    } else {
      const float4 d = w.b.dp[i];
      dx = d.x; dy = d.y; dz = d.z;
    }
    p.x += dx; p.y += dy; p.z += dz;
    const float4 q = w.b.quat[i];
    if (!isfinite(p.x + p.y + p.z) || !isfinite(q.x + q.y + q.z + q.w)) atomicOr(&w.ctl->flags, kErrNaN);
    w.b.pos[i] = p;
  }
}

__global__ void stats_kernel(World w, double *out) {
  // out[0] max penetration, out[1] max |lambda|, out[2] max penalty (contacts + joints + springs)
  double e = 0, l = 0, k = 0;
  const int total = w.ctl->numCandidates;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
    const int n = w.cur.count[c];
    for (int s = 0; s < n; s++) {
      const float4 kk = w.cur.cK[c * kMaxContacts + s], ll = w.cur.cL[c * kMaxContacts + s];
      l = fmax(l, fmax(fabs((double)ll.x), fmax(fabs((double)ll.y), fabs((double)ll.z))));
      k = fmax(k, fmax((double)kk.x, fmax((double)kk.y, (double)kk.z)));
    }
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < w.j.n; j += gridDim.x * blockDim.x) {
    if (w.j.state[j] & kRemoved) continue;
    const D4 a = w.j.lamLin[j], b = w.j.lamAng[j];
    l = fmax(l, sqrt(fmax(a.x * a.x + a.y * a.y + a.z * a.z, b.x * b.x + b.y * b.y + b.z * b.z)));
    const float4 p = w.j.penLin[j], q = w.j.penAng[j];
    k = fmax(k, fmax(fmax((double)p.x, fmax((double)p.y, (double)p.z)), fmax((double)q.x, fmax((double)q.y, (double)q.z))));
  }
  typedef cub::BlockReduce<double, 256> R;
  __shared__ typename R::TempStorage t0, t1, t2;
  const double me = R(t0).Reduce(e, ::cuda::maximum<>{});
  const double ml = R(t1).Reduce(l, ::cuda::maximum<>{});
  const double mk = R(t2).Reduce(k, ::cuda::maximum<>{});
  if (threadIdx.x == 0) {
    // non-negative doubles order like their bit patterns
    atomicMax(reinterpret_cast<unsigned long long *>(&out[0]), __double_as_longlong(me));
    atomicMax(reinterpret_cast<unsigned long long *>(&out[1]), __double_as_longlong(ml));
    atomicMax(reinterpret_cast<unsigned long long *>(&out[2]), __double_as_longlong(mk));
  }
}

}  // namespace

size_t solver_temp_bytes(int n) {
  size_t a = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int *)nullptr, n + 1);
  return a;
}

void launch_prepare(const World &w, void *temp, size_t tempBytes, cudaStream_t st, int smCount) {
  const int blocks = smCount * 4;
  prepare_forces_kernel<<<blocks, 256, 0, st>>>(w);
  prepare_bodies_kernel<<<blocks, 256, 0, st>>>(w);
  cudaMemsetAsync(w.a.count + w.b.n, 0, sizeof(int), st);
  cudaMemsetAsync(w.a.ccount + w.b.n, 0, sizeof(int), st);
  adj_count_kernel<<<blocks, 256, 0, st>>>(w);
  size_t tb = tempBytes;
  cub::DeviceScan::ExclusiveSum(temp, tb, w.a.count, w.a.start, w.b.n + 1, st);
  tb = tempBytes;
  cub::DeviceScan::ExclusiveSum(temp, tb, w.a.ccount, w.a.cstart, w.b.n + 1, st);
  cudaMemcpyAsync(w.a.cursor, w.a.start, sizeof(int) * w.b.n, cudaMemcpyDeviceToDevice, st);
  adj_fill_kernel<<<blocks, 256, 0, st>>>(w);
  adj_sort_kernel<<<blocks, 256, 0, st>>>(w);
}

static int coloring_blocks(int smCount) {
  int perSm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, coloring_kernel, 256, 0);
  if (perSm > 2) perSm = 2;
  return perSm * smCount;
}

int coloring_grid(int smCount) { return coloring_blocks(smCount); }

// An uploaded colouring: copied, then checked against this step's graph.
__global__ void color_copy_kernel(World w) {
  if (step_skipped(w)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) w.ctl->colorBad = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x)
    w.b.color[i] = (w.b.flags0[i] & kBodyDynamic) ? w.a.colorOverride[i] : -1;
}

__global__ void color_check_kernel(World w) {
  if (step_skipped(w)) return;
  int bad = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n && !bad; i += gridDim.x * blockDim.x) {
    if (!(w.b.flags0[i] & kBodyDynamic)) continue;
    const int ci = w.b.color[i];
    if (ci < 0 || ci >= kMaxColors) {
      bad = 1;
      break;
    }
    // a conflicting edge is in the higher-priority list of one of its ends
    const int hb = w.a.start[i], hc = w.a.hpCount[i];
    for (int k = 0; k < hc && !bad; k++) bad = w.b.color[w.a.hpEntry[hb + k]] == ci;
    if (w.g.hasConstraints) constraint_neighbors(w, i, [&](int j) { bad |= w.b.color[j] == ci ? 1 : 0; });
  }
  if (bad) atomicOr(&w.ctl->colorBad, 1);
}

cudaError_t launch_coloring(const World &w, cudaStream_t st, int blocks) {
  if (w.a.colorOverride) {
    color_copy_kernel<<<blocks * 2, 256, 0, st>>>(w);
    color_check_kernel<<<blocks * 2, 256, 0, st>>>(w);
  }
  World arg = w;
  void *args[] = {&arg};
  return cudaLaunchCooperativeKernel((void *)coloring_kernel, dim3(blocks), dim3(256), args, 0,
                                     st);
}

// The grab, set between steps (avbd_set_grab); body < 0 releases it.
static __global__ void grab_kernel(Grab *g, int body, D4 local, D4 target, double k) {
  g->body = body;
  g->target = target;
  g->localD = local;
  g->local = make_float4((float)local.x, (float)local.y, (float)local.z, 0.f);
  g->k = k;
}

cudaError_t launch_set_grab(const World &w, int body, const double *local, const double *target, double k,
                            cudaStream_t st) {
  const D4 l = local ? mkd4(local[0], local[1], local[2], 0.0) : mkd4(0, 0, 0, 0);
  const D4 t = target ? mkd4(target[0], target[1], target[2], 0.0) : mkd4(0, 0, 0, 0);
  grab_kernel<<<1, 1, 0, st>>>(w.grab, body, l, t, k);
  return cudaGetLastError();
}

// A joint's anchor on body A, set between steps (avbd_update_joint_anchor).
static __global__ void joint_anchor_kernel(World w, int j, double x, double y, double z) {
  const_cast<D4 *>(w.j.rAD)[j] = mkd4(x, y, z, 0.0);
  const_cast<float4 *>(w.j.rAF)[j] = make_float4((float)x, (float)y, (float)z, 0.f);
}

cudaError_t launch_joint_anchor(const World &w, int joint, double x, double y, double z, cudaStream_t st) {
  joint_anchor_kernel<<<1, 1, 0, st>>>(w, joint, x, y, z);
  return cudaGetLastError();
}

int solve_max_blocks_per_sm(int lanesPerBody) {
  (void)lanesPerBody;
  const void *kernels[4] = {(const void *)solve_kernel<false>, (const void *)wave_kernel<false>,
                            (const void *)solve_kernel<true>, (const void *)wave_kernel<true>};
  int best = 1 << 30;
  for (const void *k : kernels) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSolveSmem);
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, kSolveBlock, kSolveSmem);
    best = a < best ? a : best;
  }
  return best;
}

// lanesPerBody: the wavefront schedule's lanes per body (the colour-phase
// schedule reads its layout from the colouring).
cudaError_t launch_solve(const World &w, int lanesPerBody, int blocksPerSm, cudaStream_t st, int smCount) {
  World arg = w;
  int G = lanesPerBody;
  void *args2[] = {&arg, &G};
  void *args1[] = {&arg};
  // the contact extensions (AVBD_CONTACT_MATERIALS) are a separate
  // instantiation, so the default kernels carry none of their registers
  const bool ext = w.p.contactModel != 0;
  if (w.p.schedule == 1)
    return cudaLaunchCooperativeKernel(ext ? (const void *)wave_kernel<true> : (const void *)wave_kernel<false>,
                                       dim3(blocksPerSm * smCount), dim3(kSolveBlock), args2, kSolveSmem, st);
  return cudaLaunchCooperativeKernel(ext ? (const void *)solve_kernel<true> : (const void *)solve_kernel<false>,
                                     dim3(blocksPerSm * smCount), dim3(kSolveBlock), args1, kSolveSmem, st);
}

void launch_commit(const World &w, cudaStream_t st, int smCount) { commit_kernel<<<smCount * 4, 256, 0, st>>>(w); }

void launch_stats(const World &w, double *out3, cudaStream_t st, int smCount) {
  cudaMemsetAsync(out3, 0, sizeof(double) * 3, st);
  stats_kernel<<<smCount * 2, 256, 0, st>>>(w, out3);
}

}  // namespace avbd
