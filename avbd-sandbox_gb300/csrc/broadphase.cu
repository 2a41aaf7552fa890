// broadphase.cu - candidate pairs of one step, in pair-key order.
//
// Semantics (src/physics/solver.js:316-336, src/physics/broadphase.js:47-215):
// a pair (A, B), A the higher body index, is a candidate when
//   |p_A - p_B|^2 <= (r_A + r_B)^2            (f64, no FMA: this unit is built
//                                              with --fmad=false)
//   and not both bodies are static
//   and no live joint or spring connects them (Rigid.constrainedTo, rigid.js:250)
// or when the pair already holds a live manifold from the previous step.
// Bodies of different scenes of a batch never pair.
//
// Structure (GB300-first rather than the reference's linked lists):
//   1. every regular body is inserted once, in the hash-grid cell of its
//      centre; the per-scene cell is at least twice the largest regular
//      bounding radius, so overlapping regular bodies sit in adjacent cells.
//      Bodies above twice the scene's 95th-percentile radius are "large" and
//      are tested against every body of their scene. Counting sort by cell
//      hash: count, exclusive scan, scatter.
//   2. per body A (one warp): its 27 neighbour cells, the scene's large
//      bodies and its old manifolds give the partners B < A; they are sorted
//      in shared memory and parked in a per-body scratch row with their count
//   3. exclusive scan of the counts; each body copies its sorted row into its
//      segment: a globally sorted candidate key array without a global sort
//   4. per candidate: index of the same pair in the previous step's manifolds
#include <cub/cub.cuh>

#include <mutex>

#include "../../include/avbd_cuda.h"
#include "avbd_device.cuh"

namespace avbd {
namespace {

__device__ __forceinline__ uint32_t cell_hash(int x, int y, int z, int scene) {
  uint32_t h = (uint32_t)x * 73856093u ^ (uint32_t)y * 19349663u ^ (uint32_t)z * 83492791u;
  h ^= (uint32_t)scene * 2654435761u;
  h ^= h >> 15;
  h *= 0x2c1b3c6du;
  h ^= h >> 12;
  return h;
}

__device__ __forceinline__ bool is_large(const World &w, int i) { return (w.b.flags0[i] & kBodyLarge) != 0; }

// The sphere test in f32 from cell indices and in-cell offsets:
// d = (cA - cB) cell + (lA - lB), so the error does not grow with the
// distance from the origin. Returns 1 when |d|^2 <= (rA + rB)^2 certainly
// holds in f64, 0 when it certainly fails, -1 when the f64 test must decide.
// Bound: per component |d_f32 - d| <= 3u (|dc| + 2) cell, giving
// |d2_f32 - d2| <= 27u Q^2 and |r2_f32 - r2| <= 7u r2, Q = (max|dc| + 2) cell;
// 64u (Q^2 + r2) covers both with a factor of two.
__device__ __forceinline__ int sphere_f32(int4 ca, float4 la, int cx, int cy, int cz, float4 lb, float cell) {
  if (ca.w < 0) return -1;
  const float ex = (float)(ca.x - cx), ey = (float)(ca.y - cy), ez = (float)(ca.z - cz);
  const float dx = ex * cell + (la.x - lb.x), dy = ey * cell + (la.y - lb.y), dz = ez * cell + (la.z - lb.z);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float rs = la.w + lb.w, r2 = rs * rs;
  const float m = fmaxf(fabsf(ex), fmaxf(fabsf(ey), fabsf(ez))) + 2.0f;
  const float E = (64.0f / 16777216.0f) * (m * m * cell * cell + r2);
  if (!(d2 == d2) || !(E < 1e30f)) return -1;
  if (d2 + E < r2) return 1;
  if (d2 - E > r2) return 0;
  return -1;
}

// The `visit` predicate of solver.js:316-329 for A = bodies[a], B = bodies[b], b < a.
__device__ bool accept(const World &w, int a, int b) {
  const double ma = w.b.massD[a].x, mb = w.b.massD[b].x;
  if (!(ma > 0 || mb > 0)) return false;
  const int4 cb = w.g.cellLo[b];
  int t = -1;
  if (cb.w >= 0) t = sphere_f32(w.g.cellLo[a], w.g.loc[a], cb.x, cb.y, cb.z, w.g.loc[b], w.g.cellF[cb.w]);
  if (t == 0) return false;
  if (t < 0) {
    const D4 pa = w.b.pos[a], pb = w.b.pos[b];
    const double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
    const double r = w.b.size[a].w + w.b.size[b].w;
    if (!(dx * dx + dy * dy + dz * dz <= r * r)) return false;
  }
  // constrainedTo: a live joint or spring between them
  for (int k = w.g.cStart[a]; k < w.g.cStart[a + 1]; k++) {
    const uint32_t ref = w.g.cRef[k];
    const uint32_t type = ref >> 30, idx = (ref >> 1) & 0x1fffffffu;
    int2 ab;
    int st;
    if (type == kRefJoint) {
      ab = w.j.bodies[idx];
      st = w.j.state[idx];
    } else {
      ab = w.s.bodies[idx];
      st = w.s.state[idx];
    }
    if (st != 0) continue;
    if ((ab.x == a && ab.y == b) || (ab.x == b && ab.y == a)) return false;
  }
  return true;
}

// Centre cell of body i. Coordinates beyond +-1e9 cells or non-finite
// positions give no cell (the body is skipped) and raise an error flag.
__device__ bool centre_cell(const World &w, int i, int4 &c) {
  const int s = w.b.scene[i];
  const double inv = w.g.invCell[s];
  const D4 p = w.b.pos[i];
  const double v[3] = {p.x * inv, p.y * inv, p.z * inv};
  bool ok = true;
  for (int k = 0; k < 3; k++) ok = ok && isfinite(v[k]) && fabs(v[k]) < 1.0e9;
  c = ok ? make_int4((int)floor(v[0]), (int)floor(v[1]), (int)floor(v[2]), s) : make_int4(0, 0, 0, s);
  if (!ok) atomicOr(&w.ctl->flags, isfinite(p.x + p.y + p.z) ? kOvfCells : kErrNaN);
  return ok;
}

__global__ void cells_kernel(World w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x) {
    int4 c;
    const bool ok = centre_cell(w, i, c);
    if (ok) {  // f32 offset from the cell corner (cell = 1 / invCell, as the f32 test's cell)
      const double cell = 1.0 / w.g.invCell[c.w];
      const D4 p = w.b.pos[i];
      w.g.loc[i] = make_float4((float)(p.x - c.x * cell), (float)(p.y - c.y * cell), (float)(p.z - c.z * cell),
                               (float)w.b.size[i].w);
    }
    c.w = ok ? c.w : -1 - c.w;  // scene, negative when the body has no cell
    w.g.cellLo[i] = c;
    if (!ok || is_large(w, i)) continue;
    atomicAdd(&w.g.tableCount[cell_hash(c.x, c.y, c.z, c.w) & w.g.tableMask], 1);
  }
}

__global__ void scatter_kernel(World w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < w.b.n; i += gridDim.x * blockDim.x) {
    const int4 c = w.g.cellLo[i];
    if (c.w < 0 || is_large(w, i)) continue;
    const int at = atomicAdd(&w.g.tableCursor[cell_hash(c.x, c.y, c.z, c.w) & w.g.tableMask], 1);
    if (at < w.g.entryCap) {
      const D4 p = w.b.pos[i];
      Entry e;
      e.x = p.x; e.y = p.y; e.z = p.z; e.r = w.b.size[i].w;
      e.loc = w.g.loc[i];
      e.b2 = (i << 1) | ((w.b.flags0[i] & kBodyDynamic) ? 1 : 0);
      e.cx = c.x; e.cy = c.y; e.cz = c.z;
      w.g.entries[at] = e;
    } else {
      atomicOr(&w.ctl->flags, kOvfCells);
    }
  }
}

// Range of body a's manifolds in the previous step (keys sorted, A-major).
__device__ void prev_range(const World &w, int a, int prevCount, int &first, int &last) {
  const uint64_t lo = (uint64_t)(uint32_t)a << 32;
  int l = 0, h = prevCount;
  while (l < h) {
    const int m = (l + h) >> 1;
    if (w.prev.key[m] < lo) l = m + 1;
    else h = m;
  }
  first = l;
  last = l;
  while (last < prevCount && (int)(w.prev.key[last] >> 32) == a) last++;
}

// Large bodies: every body b < a of the scene is tested, in chunks of
// kLargeChunk bodies, one block per (large body, chunk).
// 1. the accepted count of each chunk
__global__ void __launch_bounds__(256) large_count_kernel(World w) {
  const int li = blockIdx.y, ch = blockIdx.x;
  const int a = w.g.largeList[li];
  const int s0 = w.g.sceneStart[w.b.scene[a]];
  const int b0 = s0 + ch * kLargeChunk, b1 = min(a, b0 + kLargeChunk);
  int c = 0;
  for (int b = b0 + threadIdx.x; b < b1; b += blockDim.x) c += accept(w, a, b) ? 1 : 0;
  typedef cub::BlockReduce<int, 256> R;
  __shared__ typename R::TempStorage tmp;
  const int total = R(tmp).Sum(c);
  if (threadIdx.x == 0) w.g.largeChunk[li * w.g.maxChunks + ch] = b0 < b1 ? total : 0;
}

// 2. per large body: chunk counts -> chunk offsets, plus the old manifolds the
//    sphere test rejects (they stay candidates); the body's partner count
__global__ void large_total_kernel(World w) {
  const int li = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int a = w.g.largeList[li];
  int *cnt = w.g.largeChunk + li * w.g.maxChunks;
  int run = 0;
  for (int ch = 0; ch < w.g.maxChunks; ch++) {
    const int v = cnt[ch];
    cnt[ch] = run;
    run += v;
  }
  int first, last;
  prev_range(w, a, w.ctl->prevCandidates, first, last);
  for (int m = first; m < last; m++)
    if (w.prev.count[m] > 0 && !accept(w, a, (int)(w.prev.key[m] & 0xffffffffu))) run++;
  w.g.pairCount[a] = run;
}

__device__ void sort_segment(uint64_t *k, int n) {
  for (int i = 1; i < n; i++) {
    const uint64_t v = k[i];
    int j = i - 1;
    while (j >= 0 && k[j] > v) {
      k[j + 1] = k[j];
      j--;
    }
    k[j + 1] = v;
  }
}

// A's exact broad-phase inputs, held in registers during its walk.
struct BodyA {
  int a, s;
  int4 c;
  float4 loc;
  float cell;
  double x, y, z, r;
  bool dyn;
};

// The `visit` predicate (solver.js:316-329) against a grid entry.
__device__ __forceinline__ bool accept_entry(const World &w, const BodyA &A, const Entry &e) {
  if (!(A.dyn || (e.b2 & 1))) return false;
  const int t = sphere_f32(A.c, A.loc, e.cx, e.cy, e.cz, e.loc, A.cell);
  if (t == 0) return false;
  if (t < 0) {
    const double dx = A.x - e.x, dy = A.y - e.y, dz = A.z - e.z;
    const double r = A.r + e.r;
    if (!(dx * dx + dy * dy + dz * dz <= r * r)) return false;
  }
  return !w.g.hasConstraints || accept(w, A.a, e.b2 >> 1);
}

// Warp-cooperative enumeration of the partners b < a of a non-large body a:
// lanes take the 27 neighbour cells (and the old manifolds and the scene's
// large bodies), calling f(b) on the lane that finds b. Each partner is
// found exactly once: regular bodies live in exactly one cell; old manifolds
// are added only when the sphere test rejects them.
template <class F>
__device__ void warp_partners(const World &w, const BodyA &A, int prevCount, int lane, F &&f) {
  const int a = A.a, s = A.s;
  if (s < 0) return;
  for (int k = w.g.largeStart[s] + lane; k < w.g.largeStart[s + 1]; k += 32) {
    const int b = w.g.largeList[k];
    if (b < a && accept(w, a, b)) f(b);
  }
  if (lane < 27) {
    const int x = A.c.x + lane / 9 - 1, y = A.c.y + (lane / 3) % 3 - 1, z = A.c.z + lane % 3 - 1;
    const uint32_t bucket = cell_hash(x, y, z, s) & w.g.tableMask;
    const int beg = w.g.tableStart[bucket];
    int end = beg + w.g.tableCount[bucket];
    if (end > w.g.entryCap) end = w.g.entryCap;
    for (int k = beg; k < end; k++) {
      const Entry e = w.g.entries[k];
      const int b = e.b2 >> 1;
      // entries carry their cell: other cells hashing to this bucket are skipped
      if (b >= a || e.cx != x || e.cy != y || e.cz != z) continue;
      if (w.g.numScenes > 1 && w.b.scene[b] != s) continue;  // another scene's cell, same bucket
      if (accept_entry(w, A, e)) f(b);
    }
  }
  int first = 0, last = 0;
  if (lane == 0) prev_range(w, a, prevCount, first, last);
  first = __shfl_sync(0xffffffffu, first, 0);
  last = __shfl_sync(0xffffffffu, last, 0);
  for (int m = first + lane; m < last; m += 32) {
    if (w.prev.count[m] <= 0) continue;
    const int b = (int)(w.prev.key[m] & 0xffffffffu);
    if (!accept(w, a, b)) f(b);  // accepted ones were found above
  }
}

__device__ BodyA body_a(const World &w, int a) {
  BodyA A;
  A.a = a;
  A.c = w.g.cellLo[a];
  A.s = A.c.w;
  A.loc = w.g.loc[a];
  A.cell = A.s >= 0 ? w.g.cellF[A.s] : 0.f;
  const D4 p = w.b.pos[a];
  A.x = p.x; A.y = p.y; A.z = p.z;
  A.r = w.b.size[a].w;
  A.dyn = (w.b.flags0[a] & kBodyDynamic) != 0;
  return A;
}

constexpr int kWarpsPerBlock = 8;

// One pass per non-large body: count its partners and, when they fit, leave
// them sorted in its scratch row (kRow entries) for the copy after the scan.
template <int kRow>
__global__ void __launch_bounds__(256) pairs_kernel(World w) {
  __shared__ uint32_t buf[kWarpsPerBlock][kRow];
  __shared__ int fill[kWarpsPerBlock];
  const int prevCount = w.ctl->prevCandidates;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, warps = (gridDim.x * blockDim.x) >> 5;
  for (int a = warp; a < w.b.n; a += warps) {
    if (is_large(w, a)) continue;  // large_count_kernel
    const BodyA A = body_a(w, a);
    if (lane == 0) fill[wib] = 0;
    __syncwarp();
    warp_partners(w, A, prevCount, lane, [&](int b) {
      const int at = atomicAdd(&fill[wib], 1);
      if (at < kRow) buf[wib][at] = (uint32_t)b;
    });
    __syncwarp();
    const int n = fill[wib];
    if (lane == 0) w.g.pairCount[a] = n;
    if (n <= kRow) {
      // rank sort (partners are distinct): element i goes to #{j : b_j < b_i}
      uint32_t *row = w.g.scratch + (size_t)a * kRow;
      for (int i = lane; i < n; i += 32) {
        const uint32_t v = buf[wib][i];
        int r = 0;
        for (int j = 0; j < n; j++) r += buf[wib][j] < v ? 1 : 0;
        row[r] = v;
      }
    }
    __syncwarp();
  }
}

// Copy each body's sorted partners into its segment of the key array. The
// rare bodies with more than kRow partners are enumerated again by their
// warp straight into the segment, which the warp then sorts in place (odd-even
// transposition: n rounds of compare-exchange on alternating pairs).
template <int kRow>
__global__ void __launch_bounds__(256) copy_kernel(World w) {
  __shared__ int fill[kWarpsPerBlock];
  const int prevCount = w.ctl->prevCandidates;
  const int cap = w.g.candCap;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, warps = (gridDim.x * blockDim.x) >> 5;
  for (int a = warp; a < w.b.n; a += warps) {
    if (is_large(w, a)) continue;
    const int beg = w.g.pairStart[a];
    const int n = w.g.pairStart[a + 1] - beg;
    if (n == 0) continue;
    if (beg + n > cap) {
      if (lane == 0) atomicOr(&w.ctl->flags, kOvfPairs);
      continue;
    }
    uint64_t *seg = w.g.candKey + beg;
    const uint64_t hiKey = (uint64_t)(uint32_t)a << 32;
    if (n <= kRow) {
      const uint32_t *row = w.g.scratch + (size_t)a * kRow;
      for (int i = lane; i < n; i += 32) seg[i] = hiKey | row[i];
      continue;
    }
    if (lane == 0) fill[wib] = 0;
    __syncwarp();
    const BodyA A = body_a(w, a);
    warp_partners(w, A, prevCount, lane, [&](int b) {
      const int at = atomicAdd(&fill[wib], 1);
      if (at < n) seg[at] = hiKey | (uint32_t)b;
    });
    __syncwarp();
    for (int round = 0; round < n; round++) {
      for (int i = 2 * lane + (round & 1); i + 1 < n; i += 64) {
        const uint64_t x = seg[i], y = seg[i + 1];
        if (x > y) {
          seg[i] = y;
          seg[i + 1] = x;
        }
      }
      __syncwarp();
    }
  }
}

// 3. each chunk writes its accepted partners at its offset, in index order
__global__ void __launch_bounds__(256) large_write_kernel(World w) {
  const int li = blockIdx.y, ch = blockIdx.x;
  const int a = w.g.largeList[li];
  const int s0 = w.g.sceneStart[w.b.scene[a]];
  const int b0 = s0 + ch * kLargeChunk, b1 = min(a, b0 + kLargeChunk);
  if (b0 >= b1) return;
  const int beg = w.g.pairStart[a];
  const int n = w.g.pairStart[a + 1] - beg;
  if ((long long)beg + n > w.g.candCap) {
    if (threadIdx.x == 0) atomicOr(&w.ctl->flags, kOvfPairs);
    return;
  }
  uint64_t *seg = w.g.candKey + beg;
  const uint64_t hiKey = (uint64_t)(uint32_t)a << 32;
  typedef cub::BlockScan<int, 256> S;
  __shared__ typename S::TempStorage tmp;
  __shared__ int base;
  if (threadIdx.x == 0) base = w.g.largeChunk[li * w.g.maxChunks + ch];
  __syncthreads();
  for (int t0 = b0; t0 < b1; t0 += blockDim.x) {
    const int b = t0 + threadIdx.x;
    const int ok = (b < b1 && accept(w, a, b)) ? 1 : 0;
    int at, tot;
    S(tmp).ExclusiveSum(ok, at, tot);
    if (ok && base + at < n) seg[base + at] = hiKey | (uint32_t)b;
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
}

// 4. the old manifolds the sphere test rejected, appended, and the segment
//    sorted when there are any (rare: a large body's sphere holds its scene)
__global__ void large_extra_kernel(World w) {
  const int li = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int a = w.g.largeList[li];
  const int beg = w.g.pairStart[a];
  const int n = w.g.pairStart[a + 1] - beg;
  if ((long long)beg + n > w.g.candCap) return;
  uint64_t *seg = w.g.candKey + beg;
  const uint64_t hiKey = (uint64_t)(uint32_t)a << 32;
  int first, last;
  prev_range(w, a, w.ctl->prevCandidates, first, last);
  int c = n;
  for (int m = last - 1; m >= first; m--)  // count the extras to find where they start
    if (w.prev.count[m] > 0 && !accept(w, a, (int)(w.prev.key[m] & 0xffffffffu))) c--;
  if (c == n) return;
  for (int m = first; m < last; m++) {
    const int b = (int)(w.prev.key[m] & 0xffffffffu);
    if (w.prev.count[m] > 0 && !accept(w, a, b)) seg[c++] = hiKey | (uint32_t)b;
  }
  sort_segment(seg, n);
}

// The step's candidate count; a step whose candidates exceed the arena (or
// that follows a skipped step) is skipped: no candidate reaches the narrow
// phase and every later kernel of the step returns at once (Control::skip).
__global__ void finish_kernel(World w) {
  const int total = w.g.pairStart[w.b.n];
  w.ctl->wantCandidates = total;
  if (total > w.g.candCap) {
    atomicOr(&w.ctl->flags, kOvfPairs);
    w.ctl->skip = 1;
  }
  w.ctl->numCandidates = w.ctl->skip ? 0 : total;
}

__global__ void prev_index_kernel(World w) {
  const int total = w.ctl->numCandidates;
  const int prevCount = w.ctl->prevCandidates;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
    const uint64_t k = w.g.candKey[c];
    int l = 0, h = prevCount;
    while (l < h) {
      const int m = (l + h) >> 1;
      if (w.prev.key[m] < k) l = m + 1;
      else h = m;
    }
    w.g.candPrev[c] = (l < prevCount && w.prev.key[l] == k && w.prev.count[l] > 0) ? l : -1;
    w.cur.key[c] = k;
  }
}

}  // namespace

size_t broadphase_temp_bytes(int n, int tableSize) {
  size_t a = 0, b = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, a, (int *)nullptr, (int *)nullptr, tableSize);
  cub::DeviceScan::ExclusiveSum(nullptr, b, (int *)nullptr, (int *)nullptr, n + 1);
  return a > b ? a : b;
}

void launch_broadphase_impl(const World &w, int numLarge, void *temp, size_t tempBytes, cudaStream_t st,
                            int smCount) {
  const int T = (int)w.g.tableMask + 1;
  const int n = w.b.n;
  const int blocks = smCount * 4;
  cudaMemsetAsync(w.g.tableCount, 0, sizeof(int) * T, st);
  cells_kernel<<<blocks, 256, 0, st>>>(w);
  size_t tb = tempBytes;
  cub::DeviceScan::ExclusiveSum(temp, tb, w.g.tableCount, w.g.tableStart, T, st);
  cudaMemcpyAsync(w.g.tableCursor, w.g.tableStart, sizeof(int) * T, cudaMemcpyDeviceToDevice, st);
  scatter_kernel<<<blocks, 256, 0, st>>>(w);
  // pairCount[n] = 0 so the scan over n + 1 entries yields the total at [n]
  cudaMemsetAsync(w.g.pairCount + n, 0, sizeof(int), st);
  const int warpBlocks = (int)std::min<long long>(((long long)n + 7) / 8, (long long)smCount * 32);
  pairs_kernel<kPairScratch><<<warpBlocks, 256, 0, st>>>(w);
  if (numLarge > 0) {
    large_count_kernel<<<dim3(w.g.maxChunks, numLarge), 256, 0, st>>>(w);
    large_total_kernel<<<numLarge, 32, 0, st>>>(w);
  }
  tb = tempBytes;
  cub::DeviceScan::ExclusiveSum(temp, tb, w.g.pairCount, w.g.pairStart, n + 1, st);
  copy_kernel<kPairScratch><<<warpBlocks, 256, 0, st>>>(w);
  if (numLarge > 0) {
    large_write_kernel<<<dim3(w.g.maxChunks, numLarge), 256, 0, st>>>(w);
    large_extra_kernel<<<numLarge, 32, 0, st>>>(w);
  }
  finish_kernel<<<1, 1, 0, st>>>(w);
  prev_index_kernel<<<blocks, 256, 0, st>>>(w);
}

}  // namespace avbd

// ---------------------------------------------------------------------------
// Allocation-free overlap query (avbd_overlap_pairs_static): the kernels above
// on caller-owned inputs and outputs, with every scratch array carved out of
// one file-scope device array instead of allocated memory.
// ---------------------------------------------------------------------------
namespace avbd {

static __device__ __align__(256) unsigned char g_static_scratch[AVBD_STATIC_SCRATCH_BYTES];

namespace {

// Where the query's arrays sit in the scratch array, for n bodies.
struct StaticLayout {
  size_t pos, size, massD, flags0, scene, cStart, cellLo, loc, cellF, entries, rows, pairCount, pairStart, largeList,
      largeStart, sceneStart, invCell, tableCount, tableStart, tableCursor, ctl, temp, tempBytes, total;
  int tableSize;
};

StaticLayout static_layout(int n) {
  StaticLayout L{};
  size_t at = 0;
  auto take = [&](size_t bytes) {
    const size_t here = at;
    at = (at + bytes + 255) & ~size_t(255);
    return here;
  };
  const size_t m = (size_t)(n > 0 ? n : 1);
  int T = 1024;
  while ((size_t)T < 2 * m) T <<= 1;
  L.tableSize = T;
  L.pos = take(m * sizeof(D4));
  L.size = take(m * sizeof(D4));
  L.massD = take(m * sizeof(D4));
  L.flags0 = take(m * sizeof(int));
  L.scene = take(m * sizeof(int));
  L.cStart = take((m + 1) * sizeof(int));
  L.cellLo = take(m * sizeof(int4));
  L.loc = take(m * sizeof(float4));
  L.cellF = take(sizeof(float));
  L.entries = take(m * sizeof(Entry));
  L.rows = take(m * kStaticPairRow * sizeof(uint32_t));
  L.pairCount = take((m + 1) * sizeof(int));
  L.pairStart = take((m + 1) * sizeof(int));
  L.largeList = take(m * sizeof(int));
  L.largeStart = take(2 * sizeof(int));
  L.sceneStart = take(2 * sizeof(int));
  L.invCell = take(sizeof(double));
  L.tableCount = take((size_t)T * sizeof(int));
  L.tableStart = take((size_t)T * sizeof(int));
  L.tableCursor = take((size_t)T * sizeof(int));
  L.ctl = take(sizeof(Control));
  L.tempBytes = broadphase_temp_bytes((int)m, T);
  L.temp = take(L.tempBytes);
  L.total = at;
  return L;
}

// Caller inputs -> the step's body layout. Bodies whose diameter (padded as
// the context's pack pads its cell) exceeds the cell are "large".
__global__ void static_stage_kernel(World w, D4 *pos, D4 *size, D4 *massD, int *flags0, int *scene, int *cStart,
                                    const double *p, const double *radius, const int32_t *dynamic, double cell) {
  const int n = w.b.n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double r = radius[i];
    const bool dyn = dynamic ? dynamic[i] != 0 : true;
    const bool large = 2.0 * r * (1.0 + 1e-6) + 1e-9 > cell;
    pos[i] = mkd4(p[3 * i], p[3 * i + 1], p[3 * i + 2], 0.0);
    size[i] = mkd4(0.0, 0.0, 0.0, r);
    massD[i] = mkd4(dyn ? 1.0 : 0.0, 0.0, 0.0, 0.0);
    flags0[i] = (dyn ? kBodyDynamic : 0) | (large ? kBodyLarge : 0);
    scene[i] = 0;
    cStart[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) cStart[n] = 0;
}

// Large bodies in ascending index order (one block).
__global__ void __launch_bounds__(1024) static_large_list_kernel(World w, int *largeList, int *largeStart) {
  typedef cub::BlockScan<int, 1024> S;
  __shared__ typename S::TempStorage tmp;
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  const int n = w.b.n;
  for (int i0 = 0; i0 < n; i0 += 1024) {
    const int i = i0 + threadIdx.x;
    const int f = (i < n && is_large(w, i)) ? 1 : 0;
    int at, tot;
    S(tmp).ExclusiveSum(f, at, tot);
    if (f) largeList[base + at] = i;
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    largeStart[0] = 0;
    largeStart[1] = base;
  }
}

// large_count_kernel / large_write_kernel with the large-body count read on
// the device and no previous manifolds.
__global__ void static_large_count_kernel(World w) {
  const int numLarge = w.g.largeStart[1];
  typedef cub::BlockReduce<int, 256> R;
  __shared__ typename R::TempStorage tmp;
  for (int li = blockIdx.x; li < numLarge; li += gridDim.x) {
    const int a = w.g.largeList[li];
    int c = 0;
    for (int b = threadIdx.x; b < a; b += blockDim.x) c += accept(w, a, b) ? 1 : 0;
    const int total = R(tmp).Sum(c);
    if (threadIdx.x == 0) w.g.pairCount[a] = total;
    __syncthreads();
  }
}

__global__ void static_large_write_kernel(World w) {
  const int numLarge = w.g.largeStart[1];
  const int cap = w.g.candCap;
  typedef cub::BlockScan<int, 256> S;
  __shared__ typename S::TempStorage tmp;
  __shared__ int base;
  for (int li = blockIdx.x; li < numLarge; li += gridDim.x) {
    const int a = w.g.largeList[li];
    const int beg = w.g.pairStart[a];
    const int n = w.g.pairStart[a + 1] - beg;
    if ((long long)beg + n > cap) continue;  // count > capacity tells the caller
    uint64_t *seg = w.g.candKey + beg;
    const uint64_t hiKey = (uint64_t)(uint32_t)a << 32;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int b0 = 0; b0 < a; b0 += blockDim.x) {
      const int b = b0 + threadIdx.x;
      const int ok = (b < a && accept(w, a, b)) ? 1 : 0;
      int at, tot;
      S(tmp).ExclusiveSum(ok, at, tot);
      if (ok && base + at < n) seg[base + at] = hiKey | (uint32_t)b;
      __syncthreads();
      if (threadIdx.x == 0) base += tot;
      __syncthreads();
    }
  }
}

__global__ void static_scalars_kernel(int *sceneStart, double *invCell, float *cellF, int n, double inv) {
  sceneStart[0] = 0;
  sceneStart[1] = n;
  invCell[0] = inv;
  cellF[0] = (float)(1.0 / inv);
}

__global__ void static_finish_kernel(World w, int32_t *count) {
  count[0] = (w.ctl->flags & (kErrNaN | kOvfCells)) ? -1 : w.g.pairStart[w.b.n];
}

std::mutex g_static_mutex;
constexpr int kMaxDevices = 64;
void *g_static_ptr[kMaxDevices] = {};

}  // namespace
}  // namespace avbd

using namespace avbd;

extern "C" int avbd_overlap_pairs_static(int32_t n, const double *pos, const double *radius,
                                         const int32_t *dynamic, double cell_size, uint64_t *keys,
                                         int64_t capacity, int32_t *count, void *stream) {
  char msg[256];
  if (n < 0 || n > AVBD_STATIC_PAIRS_MAX_BODIES) {
    snprintf(msg, sizeof(msg),
             "avbd_overlap_pairs_static: %d bodies; the static scratch array (%u bytes) holds at most %d",
             (int)n, (unsigned)AVBD_STATIC_SCRATCH_BYTES, AVBD_STATIC_PAIRS_MAX_BODIES);
    return set_context_free_error(n < 0 ? AVBD_ERR_ARG : AVBD_ERR_CAPACITY, msg);
  }
  if (!count || (n > 0 && (!pos || !radius)) || (capacity > 0 && !keys) || capacity < 0 ||
      capacity > 0x7fffffff || !(cell_size > 0) || !std::isfinite(cell_size))
    return set_context_free_error(AVBD_ERR_ARG,
                                  "avbd_overlap_pairs_static: NULL buffer, capacity outside 0..2^31-1, or "
                                  "cell_size not finite and > 0");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    snprintf(msg, sizeof(msg), "avbd_overlap_pairs_static: cudaGetDevice: %s",
             e != cudaSuccess ? cudaGetErrorString(e) : "device ordinal out of range");
    return set_context_free_error(AVBD_ERR_CUDA, msg);
  }
  cudaStream_t st = (cudaStream_t)stream;
  // The array's address, looked up again on every call outside a stream
  // capture (a module reloaded after cudaDeviceReset, or another context
  // current on the device, moves it); a capture uses the last address seen.
  cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &capturing) != cudaSuccess) {
    cudaGetLastError();
    capturing = cudaStreamCaptureStatusNone;
  }
  unsigned char *base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_ptr[dev] || capturing == cudaStreamCaptureStatusNone) {
      void *p = nullptr;
      e = cudaGetSymbolAddress(&p, g_static_scratch);
      if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "avbd_overlap_pairs_static: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return set_context_free_error(AVBD_ERR_CUDA, msg);
      }
      g_static_ptr[dev] = p;
    }
    base = (unsigned char *)g_static_ptr[dev];
  }
  if (n == 0) {
    e = cudaMemsetAsync(count, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) {
      snprintf(msg, sizeof(msg), "avbd_overlap_pairs_static: %s", cudaGetErrorString(e));
      return set_context_free_error(AVBD_ERR_CUDA, msg);
    }
    return AVBD_OK;
  }
  const StaticLayout L = static_layout(n);
  if (L.total > AVBD_STATIC_SCRATCH_BYTES) {
    snprintf(msg, sizeof(msg), "avbd_overlap_pairs_static: %d bodies need %zu scratch bytes, the array holds %u",
             (int)n, L.total, (unsigned)AVBD_STATIC_SCRATCH_BYTES);
    return set_context_free_error(AVBD_ERR_CAPACITY, msg);
  }
  World w{};
  D4 *dPos = (D4 *)(base + L.pos), *dSize = (D4 *)(base + L.size), *dMass = (D4 *)(base + L.massD);
  int *dFlags = (int *)(base + L.flags0), *dScene = (int *)(base + L.scene), *dCStart = (int *)(base + L.cStart);
  w.b.n = n;
  w.b.pos = dPos;
  w.b.size = dSize;
  w.b.massD = dMass;
  w.b.flags0 = dFlags;
  w.b.scene = dScene;
  w.g.numScenes = 1;
  w.g.sceneStart = (const int *)(base + L.sceneStart);
  w.g.invCell = (const double *)(base + L.invCell);
  w.g.largeStart = (const int *)(base + L.largeStart);
  w.g.largeList = (const int *)(base + L.largeList);
  w.g.cellLo = (int4 *)(base + L.cellLo);
  w.g.loc = (float4 *)(base + L.loc);
  w.g.cellF = (const float *)(base + L.cellF);
  w.g.tableMask = (unsigned)(L.tableSize - 1);
  w.g.tableCount = (int *)(base + L.tableCount);
  w.g.tableStart = (int *)(base + L.tableStart);
  w.g.tableCursor = (int *)(base + L.tableCursor);
  w.g.entries = (Entry *)(base + L.entries);
  w.g.entryCap = n;
  w.g.scratch = (uint32_t *)(base + L.rows);
  w.g.hasConstraints = 0;
  w.g.pairCount = (int *)(base + L.pairCount);
  w.g.pairStart = (int *)(base + L.pairStart);
  w.g.candKey = keys;
  w.g.candCap = (int)capacity;
  w.g.cStart = dCStart;
  w.ctl = (Control *)(base + L.ctl);

  int smCount = 0;
  e = cudaDeviceGetAttribute(&smCount, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    // zero what the kernels accumulate into; the scene table and cell size
    const int sceneStart[2] = {0, n};
    const double inv = 1.0 / cell_size;
    cudaMemsetAsync(w.ctl, 0, sizeof(Control), st);
    cudaMemsetAsync(w.g.tableCount, 0, sizeof(int) * L.tableSize, st);
    cudaMemsetAsync(w.g.pairCount + n, 0, sizeof(int), st);
    const int blocks = smCount * 4;
    static_stage_kernel<<<blocks, 256, 0, st>>>(w, dPos, dSize, dMass, dFlags, dScene, dCStart, pos, radius,
                                                dynamic, cell_size);
    // two scalars and the inverse cell: written by a one-thread kernel so the
    // call needs no host staging buffer
    static_scalars_kernel<<<1, 1, 0, st>>>((int *)(base + L.sceneStart), (double *)(base + L.invCell),
                                           (float *)(base + L.cellF), sceneStart[1], inv);
    static_large_list_kernel<<<1, 1024, 0, st>>>(w, (int *)(base + L.largeList), (int *)(base + L.largeStart));
    cells_kernel<<<blocks, 256, 0, st>>>(w);
    size_t tb = L.tempBytes;
    cub::DeviceScan::ExclusiveSum(base + L.temp, tb, w.g.tableCount, w.g.tableStart, L.tableSize, st);
    cudaMemcpyAsync(w.g.tableCursor, w.g.tableStart, sizeof(int) * L.tableSize, cudaMemcpyDeviceToDevice, st);
    scatter_kernel<<<blocks, 256, 0, st>>>(w);
    const int warpBlocks = (int)std::min<long long>(((long long)n + 7) / 8, (long long)smCount * 32);
    pairs_kernel<kStaticPairRow><<<warpBlocks, 256, 0, st>>>(w);
    static_large_count_kernel<<<smCount, 256, 0, st>>>(w);
    tb = L.tempBytes;
    cub::DeviceScan::ExclusiveSum(base + L.temp, tb, w.g.pairCount, w.g.pairStart, n + 1, st);
    copy_kernel<kStaticPairRow><<<warpBlocks, 256, 0, st>>>(w);
    static_large_write_kernel<<<smCount, 256, 0, st>>>(w);
    static_finish_kernel<<<1, 1, 0, st>>>(w, count);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "avbd_overlap_pairs_static: %s", cudaGetErrorString(e));
    return set_context_free_error(AVBD_ERR_CUDA, msg);
  }
  return AVBD_OK;
}
