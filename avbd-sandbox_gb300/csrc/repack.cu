// repack.cu - identity-preserving repack (avbd_repack): after a topology edit
// (bodies appended or erased, joints and springs added or removed) the live
// device state follows each scene object to its new index, on the device.
//
// Reference behaviour (src/physics/gpu/backend.js:662-1301, identity runs at
// :107-145): GPU-owned body, joint and spring state is remapped by object
// identity, and contact warm-start state survives append, erase and
// order-preserving compaction because the manifolds are keyed by stable
// body identities. Here the caller names each new element's old index; the
// manifold arena is keyed by the body indices themselves, so its entries are
// renumbered: with survivors in their old relative order a pair (A > B)
// stays (A' > B') and the arena's key order is kept, so a stable compaction
// of the live entries whose two bodies survive is the new warm-start arena.
#include <cub/cub.cuh>

#include "avbd_device.cuh"

namespace avbd {
namespace {

__global__ void repack_bodies_kernel(const Bodies ob, Bodies nb, const int *oldBody) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb.n; i += gridDim.x * blockDim.x) {
    const int o = oldBody[i];
    if (o < 0) continue;
    nb.pos[i] = ob.pos[o];
    nb.quat[i] = ob.quat[o];
    nb.vel[i] = ob.vel[o];
    nb.omega[i] = ob.omega[o];
    nb.prevVel[i] = ob.prevVel[o];
  }
}

__global__ void repack_forces_kernel(const Joints oj, Joints nj, const int *oldJoint, const Springs os, Springs ns,
                                     const int *oldSpring) {
  const int stride = gridDim.x * blockDim.x;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nj.n; j += stride) {
    const int o = oldJoint[j];
    if (o < 0) continue;
    nj.penLin[j] = oj.penLin[o];
    nj.penAng[j] = oj.penAng[o];
    nj.lamLin[j] = oj.lamLin[o];
    nj.lamAng[j] = oj.lamAng[o];
    nj.state[j] = oj.state[o];  // broken / removed survive the index shift
  }
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns.n; s += stride) {
    const int o = oldSpring[s];
    if (o < 0) continue;
    ns.penalty[s] = os.penalty[o];
    ns.peak[s] = os.peak[o];
    ns.state[s] = os.state[o];  // a tear survives the index shift
  }
}

// flag[m] = 1 for a live manifold whose two bodies survive
__global__ void repack_flag_kernel(const Manifolds om, int slots, const int *newOf, int *flag) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < slots; m += gridDim.x * blockDim.x) {
    const uint64_t k = om.key[m];
    const int a = (int)(k >> 32), b = (int)(k & 0xffffffffu);
    flag[m] = (om.count[m] > 0 && newOf[a] >= 0 && newOf[b] >= 0) ? 1 : 0;
  }
}

// One thread per (manifold, contact slot) of the old arena: carried entries
// move to their compacted position with renumbered bodies. The fields are the
// ones a warm start reads (the CPU handover of avbd_write_state writes the
// same): key, count, f64 basis, and per contact the feature ID, body-local
// anchors, penalty and multiplier with the stick bit, restitution bias.
__global__ void repack_move_kernel(const Manifolds om, Manifolds nm, int slots, const int *newOf, const int *flag,
                                   const int *at) {
  const long long total = (long long)slots * kMaxContacts;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(t / kMaxContacts), c = (int)(t % kMaxContacts);
    if (!flag[m]) continue;
    const int d = at[m];
    if (c == 0) {
      const uint64_t k = om.key[m];
      const int a = newOf[(int)(k >> 32)], b = newOf[(int)(k & 0xffffffffu)];
      nm.key[d] = (uint64_t)(uint32_t)a << 32 | (uint32_t)b;
      nm.count[d] = om.count[m];
      for (int q = 0; q < 9; q++) nm.basisD[(size_t)d * 9 + q] = om.basisD[(size_t)m * 9 + q];
    }
    const size_t src = (size_t)m * kMaxContacts + c, dst = (size_t)d * kMaxContacts + c;
    const bool on = c < om.count[m];
    nm.feat[dst] = on ? om.feat[src] : 0u;
    nm.rA[dst] = on ? om.rA[src] : make_float4(0.f, 0.f, 0.f, 0.f);
    nm.rB[dst] = on ? om.rB[src] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 k = om.cK[src];
    nm.cK[dst] = on ? make_float4(k.x, k.y, k.z, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 l = om.cL[src];
    nm.cL[dst] = on ? make_float4(l.x, l.y, l.z, l.w != 0.f ? 1.f : 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    nm.cX[dst] = on ? om.cX[src] : 0.f;
    nm.cA[dst] = on ? om.cA[src] : make_float4(0.f, 0.f, 0.f, 0.f);  // .w: C0 on the normal
  }
}

__global__ void repack_finish_kernel(int slots, const int *flag, const int *at, Control *ctl) {
  ctl->prevCandidates = at[slots - 1] + flag[slots - 1];
  ctl->numCandidates = 0;
}

int grid_for(long long items) { return (int)std::max<long long>(1, std::min<long long>((items + 255) / 256, 4096)); }

}  // namespace

cudaError_t launch_repack_state(const World &oldW, const World &newW, const int *oldBody, const int *oldJoint,
                                const int *oldSpring, cudaStream_t st) {
  if (newW.b.n > 0) repack_bodies_kernel<<<grid_for(newW.b.n), 256, 0, st>>>(oldW.b, newW.b, oldBody);
  const int forces = std::max(newW.j.n, newW.s.n);
  if (forces > 0)
    repack_forces_kernel<<<grid_for(forces), 256, 0, st>>>(oldW.j, newW.j, oldJoint, oldW.s, newW.s, oldSpring);
  return cudaGetLastError();
}

cudaError_t launch_repack_manifolds(const Manifolds &oldM, const Manifolds &newM, int oldSlots, const int *newOf,
                                    int *flag, int *at, Control *ctl, cudaStream_t st) {
  if (oldSlots <= 0) return cudaSuccess;
  repack_flag_kernel<<<grid_for(oldSlots), 256, 0, st>>>(oldM, oldSlots, newOf, flag);
  size_t bytes = 0;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, bytes, flag, at, oldSlots, st);
  if (e != cudaSuccess) return e;
  void *temp = nullptr;
  if ((e = cudaMallocAsync(&temp, std::max<size_t>(bytes, 16), st)) != cudaSuccess) return e;
  e = cub::DeviceScan::ExclusiveSum(temp, bytes, flag, at, oldSlots, st);
  cudaFreeAsync(temp, st);
  if (e != cudaSuccess) return e;
  repack_move_kernel<<<grid_for((long long)oldSlots * kMaxContacts), 256, 0, st>>>(oldM, newM, oldSlots, newOf, flag,
                                                                                    at);
  repack_finish_kernel<<<1, 1, 0, st>>>(oldSlots, flag, at, ctl);
  return cudaGetLastError();
}

}  // namespace avbd
