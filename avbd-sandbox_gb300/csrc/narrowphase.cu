// narrowphase.cu - contact generation, manifold merge and warm start.
//
// One thread per candidate pair. The geometry runs in IEEE f64 with the
// reference's operation order and NO fused multiply-add (this translation
// unit is compiled with --fmad=false), so that from identical inputs the
// contact count, feature IDs and SAT/clipping decisions equal the reference
// engine's bit for bit:
//   collide.js:612-685 box-box 15-axis SAT, face clipping (:403-472),
//                      edge contact (:475-493)
//   collide.js:496-520 sphere-sphere, :526-600 sphere-OBB
//   manifold.js:214-318 feature-ID merge, sphere basis transport,
//                      C*(x_t) + margin, warm start lambda <- gamma(alpha lambda),
//                      k <- clamp(gamma k, kmin, kmax)
// Box-box SAT runs first in f32 in a frame centred on body A, each of the 15
// axis separations with a conservative bound on its distance from the f64
// value (GB300's FP64 rate is a small fraction of its FP32 rate). A bound
// that cannot settle a decision - the sign of a separation, the skip of a
// near-degenerate edge axis, the order of near-tied best axes, the edge-vs-
// face choice - sends just those axes through the exact f64 axis test, so
// every decision equals the f64 one. The winning axis's normal, the contact
// basis and the clipping stay in exact f64.
#include "avbd_device.cuh"
#include "collider.cuh"

namespace avbd {
namespace {

// The exact geometry (collider.cuh) in f64.
using geo::kFaceA;
using geo::kFaceB;
using geo::kEdge;
using geo::kPlaneEps;
using geo::kPolyCap;
using geo::kSatEps;
using geo::kMergeDistSq;
using D3 = geo::D3T<double>;
using QD = geo::QDT<double>;
using BodyD = geo::BodyT<double>;
using OBB = geo::OBBT<double>;
using NewContact = geo::NewContactT<double>;
using Collider = geo::ColliderT<double>;
using geo::add;
using geo::adds;
using geo::clampd;
using geo::conj;
using geo::crs;
using geo::dt3;
using geo::neg;
using geo::orthonormal;
using geo::rot;
using geo::scl;
using geo::sub;
__device__ __forceinline__ D3 mk(double x, double y, double z) { return D3{x, y, z}; }



struct NewContactF {
  uint32_t feature;
  float ra[3], rb[3];
};

// The two boxes in f32 in a frame centred on A: B's centre, the box axes and
// the half sizes.
struct BoxF {
  V3<float> d, ax[3], bx[3];
  float ha[3], hb[3];
};

__device__ BoxF make_boxf(const BodyD &A, const BodyD &B) {
  BoxF F;
  const Q4<float> qa{(float)A.q.x, (float)A.q.y, (float)A.q.z, (float)A.q.w};
  const Q4<float> qb{(float)B.q.x, (float)B.q.y, (float)B.q.z, (float)B.q.w};
  F.d = V3<float>{(float)(B.p.x - A.p.x), (float)(B.p.y - A.p.y), (float)(B.p.z - A.p.z)};
  F.ha[0] = (float)A.half.x; F.ha[1] = (float)A.half.y; F.ha[2] = (float)A.half.z;
  F.hb[0] = (float)B.half.x; F.hb[1] = (float)B.half.y; F.hb[2] = (float)B.half.z;
  F.ax[0] = qrotate(qa, V3<float>{1, 0, 0});
  F.ax[1] = qrotate(qa, V3<float>{0, 1, 0});
  F.ax[2] = qrotate(qa, V3<float>{0, 0, 1});
  F.bx[0] = qrotate(qb, V3<float>{1, 0, 0});
  F.bx[1] = qrotate(qb, V3<float>{0, 1, 0});
  F.bx[2] = qrotate(qb, V3<float>{0, 0, 1});
  return F;
}

// Outcome of the f32 SAT of a box pair.
constexpr int kSeparated = 0, kFaceWin = 1, kEdgeWin = 2, kUndecided = 3, kFaceTie = 4;

// f32 SAT of a box-box pair (collide.js:612-685), certified against the f64
// evaluation: every axis separation comes with a bound err >= |sep_f32 -
// sep_f64|, derived from a per-component error of the f32 box axes of at
// most ~32 ulp(1) and the 1/len amplification of normalising an edge axis,
// with a 16x margin:
//   err = 512 u S (1 + 1/len),  u = 2^-24,  S = |d|_1 + sum(hA) + sum(hB).
// kSeparated when some axis certainly separates the boxes (the f64 test then
// finds a separating axis too and returns no contact). kFaceWin / kEdgeWin
// when no axis can separate, the best face axis (largest separation, first
// on ties) and, if it can matter, the best edge axis are certain, and so is
// the choice 0.95 sepE > sepF + 0.01 between them. kFaceTie when all of that
// holds and a face wins, but which face is not certain: tieMask (bits 0-5:
// faces 0-2 of A, 0-2 of B) lists the face axes that can be the largest,
// for an exact f64 comparison of just those. kUndecided otherwise: the exact
// f64 path decides.
__device__ int classify_f32(const BoxF &F, bool &refIsA, int &axA, int &axB, int &tieMask) {
  const float S = fabsf(F.d.x) + fabsf(F.d.y) + fabsf(F.d.z) + F.ha[0] + F.ha[1] + F.ha[2] + F.hb[0] + F.hb[1] +
                  F.hb[2];
  if (!(S == S) || S > 1e30f) return kUndecided;
  constexpr float u512 = 512.0f / 16777216.0f;
  const float eBase = u512 * S;
  bool undecided = false;
  // best of each group so far, and the largest upper bound among the others
  int fBest = -1, eBest = -1;
  float fSep = 0.f, fErr = 0.f, fOther = -INFINITY, eSep = 0.f, eErr = 0.f, eOther = -INFINITY;
  float fUp[6];  // upper bound of each face axis's separation
#pragma unroll
  for (int k = 0; k < 6; k++) fUp[k] = -INFINITY;
#pragma unroll
  for (int k = 0; k < 15; k++) {
    V3<float> a;
    const bool edge = k >= 6;
    if (k < 3) a = F.ax[k];
    else if (k < 6) a = F.bx[k - 3];
    else {
      const V3<float> p = F.ax[(k - 6) / 3], q = F.bx[(k - 6) % 3];
      a = V3<float>{p.y * q.z - p.z * q.y, p.z * q.x - p.x * q.z, p.x * q.y - p.y * q.x};
    }
    const float lenSq = a.x * a.x + a.y * a.y + a.z * a.z;
    if (edge) {
      // lenSq of the f32 cross product is within 1024 u len + 1e-9 of the f64 one
      const float eLen = (1024.0f / 16777216.0f) * sqrtf(lenSq) + 1e-9f;
      if (lenSq + eLen < (float)kSatEps) continue;  // the f64 test skips this axis too
      if (lenSq - eLen < (float)kSatEps) {
        undecided = true;
        continue;
      }
    } else if (!(lenSq >= 0.25f)) {
      undecided = true;
      continue;
    }
    const float len = sqrtf(lenSq);
    const V3<float> n{a.x / len, a.y / len, a.z / len};
    const float dist = fabsf(n.x * F.d.x + n.y * F.d.y + n.z * F.d.z);
    float rA = 0.f, rB = 0.f;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      rA += F.ha[i] * fabsf(n.x * F.ax[i].x + n.y * F.ax[i].y + n.z * F.ax[i].z);
      rB += F.hb[i] * fabsf(n.x * F.bx[i].x + n.y * F.bx[i].y + n.z * F.bx[i].z);
    }
    const float sep = dist - (rA + rB);
    const float err = eBase * (1.0f + 1.0f / len);
    if (sep - err > 0.f) return kSeparated;
    if (sep + err > 0.f) {
      undecided = true;
      continue;
    }
    if (!edge) {
      fUp[k < 6 ? k : 0] = sep + err;
      if (fBest < 0 || sep > fSep) {
        if (fBest >= 0) fOther = fmaxf(fOther, fSep + fErr);
        fBest = k; fSep = sep; fErr = err;
      } else {
        fOther = fmaxf(fOther, sep + err);
      }
    } else {
      if (eBest < 0 || sep > eSep) {
        if (eBest >= 0) eOther = fmaxf(eOther, eSep + eErr);
        eBest = k; eSep = sep; eErr = err;
      } else {
        eOther = fmaxf(eOther, sep + err);
      }
    }
  }
  if (undecided || fBest < 0) return kUndecided;
  const float fLo = fSep - fErr, fHi = fmaxf(fSep + fErr, fOther);
  bool edgeWins = false;
  if (eBest >= 0) {
    const float eLo = eSep - eErr, eHi = fmaxf(eSep + eErr, eOther);
    const float slack = 1e-6f * (fabsf(eSep) + fabsf(fSep) + 0.01f);
    if (0.95f * eLo > fHi + 0.01f + slack) edgeWins = true;
    else if (!(0.95f * eHi < fLo + 0.01f - slack)) return kUndecided;
  }
  if (edgeWins) {
    if (!(eOther < eSep - eErr)) return kUndecided;  // tied edge axes
    axA = (eBest - 6) / 3;
    axB = (eBest - 6) % 3;
    return kEdgeWin;
  }
  if (!(fOther < fSep - fErr)) {  // tied face axes: the candidates for an exact comparison
    tieMask = 0;
#pragma unroll
    for (int k = 0; k < 6; k++)
      if (fUp[k] >= fLo) tieMask |= 1 << k;
    return kFaceTie;
  }
  refIsA = fBest < 3;
  axA = refIsA ? fBest : fBest - 3;
  return kFaceWin;
}

// ---- faceManifold (collide.js:403-472) in f32, in A's frame ------------------
struct FaceF {
  const BoxF &F;
  Q4<float> qaInv, qbInv;  // conjugate orientations of A and B (f32)
  NewContactF *outF;
  int count = 0;
  __device__ FaceF(const BoxF &f, const BodyD &A, const BodyD &B, NewContactF *o)
      : F(f),
        qaInv{(float)-A.q.x, (float)-A.q.y, (float)-A.q.z, (float)A.q.w},
        qbInv{(float)-B.q.x, (float)-B.q.y, (float)-B.q.z, (float)B.q.w},
        outF(o) {}
  // Every f32 point carries a bound .w on its distance from the f64 point
  // (minus A's position). Each discrete decision - clip side, intersection
  // denominator, contact depth, merge distance - is taken only when the
  // bound settles it; otherwise the function returns -1 and the caller runs
  // the f64 builder. Returns the contact count when every decision was certain.
  static constexpr float kU = 1.0f / 16777216.0f;  // unit roundoff of f32
  static constexpr float kEA = 64.0f * kU;         // error of an f32 box axis (2-norm)
  static constexpr float kFloor = 1e-9f;           // f64 rounding at world scale, and slack
  __device__ static float nrm(V3<float> v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
  __device__ static V3<float> fsub(V3<float> a, V3<float> b) { return V3<float>{a.x - b.x, a.y - b.y, a.z - b.z}; }
  __device__ static V3<float> fadds(V3<float> o, V3<float> a, float s) {
    return V3<float>{o.x + a.x * s, o.y + a.y * s, o.z + a.z * s};
  }
  __device__ static float fdot(V3<float> a, V3<float> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
  // clip side of a point at signed distance dd (bound e): 1 inside, 0 outside, -1 undecided
  __device__ static int side(float dd, float e) {
    if (dd + e <= (float)kPlaneEps) return 1;
    if (dd - e > (float)kPlaneEps) return 0;
    return -1;
  }
  // clipAgainstPlane (collide.js:202-247); -1 when a decision is undecided
  __device__ static int clipF(const float4 *in, int n, V3<float> pn, float po, float ePo, float4 *o) {
    if (n <= 0) return 0;
    auto dist = [&](float4 v, float &e) {
      const V3<float> p{v.x, v.y, v.z};
      const float np = nrm(p);
      const float dd = fdot(pn, p) - po;
      e = v.w + (kEA + 3.0f * kU) * np + ePo + kU * fabsf(dd) + kFloor;
      return dd;
    };
    int oc = 0;
    float4 a = in[n - 1];
    float ea;
    float da = dist(a, ea);
    int ai = side(da, ea);
    if (ai < 0) return -1;
    for (int i = 0; i < n; i++) {
      const float4 b = in[i];
      float eb;
      const float db = dist(b, eb);
      const int bi = side(db, eb);
      if (bi < 0) return -1;
      if (ai != bi) {
        const float denom = da - db;
        const float eDen = ea + eb + kU * fabsf(denom);
        float t = 0.f, et = 0.f;
        if (fabsf(denom) - eDen > (float)kSatEps) {
          if (fabsf(denom) < 4.0f * eDen) return -1;  // keep the first-order bound valid
          const float tr = da / denom;
          et = 1.5f * (fabsf(db) * ea + fabsf(da) * eb) / (denom * denom) + 2.0f * kU * fabsf(tr);
          t = fminf(fmaxf(tr, 0.f), 1.f);  // clamp is 1-Lipschitz: no decision to certify
        } else if (!(fabsf(denom) + eDen <= (float)kSatEps)) {
          return -1;
        }
        if (oc < kPolyCap) {
          const V3<float> pa{a.x, a.y, a.z}, pb{b.x, b.y, b.z};
          const V3<float> ab = fsub(pb, pa);
          const V3<float> q = fadds(pa, ab, t);
          const float e = a.w + t * (a.w + b.w) + nrm(ab) * et + 3.0f * kU * (nrm(pa) + nrm(ab)) + kFloor;
          o[oc++] = make_float4(q.x, q.y, q.z, e);
        }
      }
      if (bi && oc < kPolyCap) o[oc++] = b;
      a = b;
      da = db;
      ea = eb;
      ai = bi;
    }
    return oc;
  }
  // addContact (collide.js:254-285) on f32 points; 1 added, 0 merged or full,
  // -1 undecided
  __device__ int addContactF(V3<float> xA, float eA, V3<float> xB, float eB, uint32_t key, float4 *midF) {
    const V3<float> m{(xA.x + xB.x) * 0.5f, (xA.y + xB.y) * 0.5f, (xA.z + xB.z) * 0.5f};
    const float eM = 0.5f * (eA + eB) + 2.0f * kU * nrm(m) + kFloor;
    for (int i = 0; i < count; i++) {
      const V3<float> dv{m.x - midF[i].x, m.y - midF[i].y, m.z - midF[i].z};
      const float d2 = fdot(dv, dv);
      const float ee = eM + midF[i].w;
      const float e2 = 2.0f * nrm(dv) * ee + ee * ee + 4.0f * kU * d2 + kFloor;
      if (d2 + e2 < (float)kMergeDistSq) return 0;
      if (d2 - e2 < (float)kMergeDistSq) return -1;
    }
    if (count >= kMaxContacts) return 0;
    const V3<float> ra = qrotate(qaInv, xA);
    const V3<float> rb = qrotate(qbInv, fsub(xB, F.d));
    NewContactF &c = outF[count];
    c.feature = key;
    c.ra[0] = ra.x; c.ra[1] = ra.y; c.ra[2] = ra.z;
    c.rb[0] = rb.x; c.rb[1] = rb.y; c.rb[2] = rb.z;
    midF[count] = make_float4(m.x, m.y, m.z, eM);
    count++;
    return 1;
  }
  // refAx: the reference face axis in f64; ibAx: the incident box's axes in
  // f64 (the orientation decisions use the reference's own f64 expressions).
  __device__ int build(bool refIsA, int refAxis, D3 nAB, D3 refAx, const D3 *ibAx) {
    const D3 outward = refIsA ? nAB : neg(nAB);
    const double s = dt3(outward, refAx) >= 0 ? 1 : -1;
    const D3 fN64 = scl(refAx, s);
    int incAxis = 0;
    double best = -INFINITY, dots[3];
    for (int i = 0; i < 3; i++) {
      dots[i] = dt3(ibAx[i], fN64);
      const double dd = fabs(dots[i]);
      if (dd > best) {
        best = dd;
        incAxis = i;
      }
    }
    const float si = dots[incAxis] > 0 ? -1.f : 1.f;
    // the geometry in f32
    const V3<float> zero{0.f, 0.f, 0.f};
    const V3<float> *rAx = refIsA ? F.ax : F.bx;
    const V3<float> *iAx = refIsA ? F.bx : F.ax;
    const float *rH = refIsA ? F.ha : F.hb;
    const float *iH = refIsA ? F.hb : F.ha;
    const V3<float> rC = refIsA ? zero : F.d, iC = refIsA ? F.d : zero;
    const float eD = kU * nrm(F.d) + kFloor;
    const float eRC = refIsA ? 0.f : eD, eIC = refIsA ? eD : 0.f;
    const V3<float> fN{rAx[refAxis].x * (float)s, rAx[refAxis].y * (float)s, rAx[refAxis].z * (float)s};
    const float hR = rH[refAxis];
    const V3<float> fC = fadds(rC, fN, hR);
    const float eFC = eRC + kEA * hR + 3.0f * kU * (nrm(rC) + hR) + kFloor;
    const int u0 = refAxis == 0 ? 1 : 0, v0 = refAxis == 2 ? 1 : 2;
    const V3<float> fU = rAx[u0], fV = rAx[v0];
    const float fEU = rH[u0], fEV = rH[v0];
    const int u1 = incAxis == 0 ? 1 : 0, v1 = incAxis == 2 ? 1 : 2;
    const V3<float> fn{iAx[incAxis].x * si, iAx[incAxis].y * si, iAx[incAxis].z * si};
    const float hI = iH[incAxis], eU = iH[u1], eV = iH[v1];
    const V3<float> fc = fadds(iC, fn, hI);
    const float eCorner = eIC + kEA * (hI + eU + eV) + 5.0f * kU * (nrm(iC) + hI + eU + eV) + kFloor;
    float4 P[kPolyCap], Q[kPolyCap];
    for (int i = 0; i < 4; i++) {
      const float su = (i == 0 || i == 3) ? 1.f : -1.f;
      const float sv = (i == 0 || i == 1) ? 1.f : -1.f;
      const V3<float> c = fadds(fadds(fc, iAx[u1], eU * su), iAx[v1], eV * sv);
      P[i] = make_float4(c.x, c.y, c.z, eCorner);
    }
    int n = 4;
    const float nFC = nrm(fC);
    for (int k = 0; k < 4; k++) {
      const V3<float> ax = k < 2 ? fU : fV;
      const float sg = (k & 1) ? -1.f : 1.f;
      const V3<float> pn{ax.x * sg, ax.y * sg, ax.z * sg};
      const float ext = k < 2 ? fEU : fEV;
      const float po = fdot(pn, fC) + ext;
      const float ePo = kEA * nFC + eFC + 3.0f * kU * nFC + kU * (fabsf(po) + ext) + kFloor;
      n = (k & 1) ? clipF(Q, n, pn, po, ePo, P) : clipF(P, n, pn, po, ePo, Q);
      if (n < 0) return -1;
      if (n == 0) return 0;
    }
    count = 0;
    uint32_t prefix = (uint32_t)(refIsA ? kFaceA : kFaceB) << 24;
    prefix |= (uint32_t)(refAxis & 0xff) << 16;
    prefix |= (uint32_t)(incAxis & 0xff) << 8;
    float4 midF[kMaxContacts];
    count = 0;
    for (int i = 0; i < n && count < kMaxContacts; i++) {
      const V3<float> p{P[i].x, P[i].y, P[i].z};
      const V3<float> pc = fsub(p, fC);
      const float dist = fdot(pc, fN);
      const float eDist = P[i].w + eFC + kEA * nrm(pc) + 4.0f * kU * (nrm(p) + nFC) + kFloor;
      if (dist - eDist > (float)kPlaneEps) continue;
      if (dist + eDist > (float)kPlaneEps) return -1;
      const V3<float> proj = fadds(p, fN, -dist);
      const float eProj = P[i].w + kEA * fabsf(dist) + eDist + 2.0f * kU * (nrm(p) + fabsf(dist)) + kFloor;
      const int r = refIsA ? addContactF(proj, eProj, p, P[i].w, prefix | (uint32_t)(i & 0xff), midF)
                           : addContactF(p, P[i].w, proj, eProj, prefix | (uint32_t)(i & 0xff), midF);
      if (r < 0) return -1;
    }
    if (!count) return -1;  // the support-point contact is built in f64
    return count;
  }
};

__device__ BodyD load_body(const World &w, int i) {
  BodyD b;
  const D4 p = w.b.pos[i];
  const float4 q = w.b.quat[i];
  const D4 s = w.b.size[i];
  b.p = mk(p.x, p.y, p.z);
  b.q = QD{(double)q.x, (double)q.y, (double)q.z, (double)q.w};
  b.half = mk(s.x * 0.5, s.y * 0.5, s.z * 0.5);
  b.sphere = (w.b.flags0[i] & kBodySphere) != 0;
  // size.w is the broad phase's reach (the bounding radius plus the contact
  // offset under AVBD_CONTACT_MATERIALS); a sphere's own radius is half its
  // diameter (Rigid.sphere, src/physics/rigid.js:105-133)
  b.radius = (w.b.contactOffset && b.sphere) ? s.x * 0.5 : s.w;
  return b;
}

// The pair's contact skin (AVBD_CONTACT_MATERIALS: the sum of the contact
// offsets; 0 for the CPU engine's collider).
__device__ __forceinline__ double pair_skin(const World &w, int ia, int ib) {
  return w.b.contactOffset ? w.b.contactOffset[ia] + w.b.contactOffset[ib] : 0.0;
}

// transportComponents / transportPenalty (manifold.js:100-162)
__device__ void transport(double *lam, double *pen, const double *ob, const double *nb) {
  const double x = lam[0], y = lam[1], z = lam[2];
  const double kx = pen[0], ky = pen[1], kz = pen[2];
  double lo[3], po[3];
  for (int r = 0; r < 3; r++) {
    const int n = r * 3;
    const double dx = nb[n] * ob[0] + nb[n + 1] * ob[1] + nb[n + 2] * ob[2];
    const double dy = nb[n] * ob[3] + nb[n + 1] * ob[4] + nb[n + 2] * ob[5];
    const double dz = nb[n] * ob[6] + nb[n + 1] * ob[7] + nb[n + 2] * ob[8];
    lo[r] = x * dx + y * dy + z * dz;
    po[r] = kx * dx * dx + ky * dy * dy + kz * dz * dz;
  }
  for (int r = 0; r < 3; r++) {
    lam[r] = lo[r];
    pen[r] = po[r];
  }
}

// ---------------------------------------------------------------------------
// Manifold output: merge with the previous step's manifold by feature ID,
// C*(x_t) + margin, warm start (manifold.js:214-318).
// ---------------------------------------------------------------------------

// Box pairs, in f32 in A's frame (xA - xB = R_A rA - R_B rB - (pB - pA)); the
// outputs are stored in f32.
__device__ void write_manifold_materials(const World &w, int c, int ia, int ib, const BodyD &A, const BodyD &B,
                                         const D3 *ncA, const D3 *ncB, const uint32_t *feat, int num,
                                         const double *basis);

__device__ void write_box_manifold(const World &w, int c, int ia, int ib, const BodyD &A, const BodyD &B,
                                   const NewContactF *nc, int num, const double *basis) {
  const SolverParams &P = w.p;
  if (P.contactModel) {
    D3 ra[kMaxContacts], rb[kMaxContacts];
    uint32_t ft[kMaxContacts];
    for (int i = 0; i < num; i++) {
      ra[i] = mk(nc[i].ra[0], nc[i].ra[1], nc[i].ra[2]);
      rb[i] = mk(nc[i].rb[0], nc[i].rb[1], nc[i].rb[2]);
      ft[i] = nc[i].feature;
    }
    write_manifold_materials(w, c, ia, ib, A, B, ra, rb, ft, num, basis);
    return;
  }
  w.cur.count[c] = num;
  if (num == 0) return;
  const int pi = w.g.candPrev[c];
  const int oldNum = pi >= 0 ? w.prev.count[pi] : 0;
  const Q4<float> qa{(float)A.q.x, (float)A.q.y, (float)A.q.z, (float)A.q.w};
  const Q4<float> qb{(float)B.q.x, (float)B.q.y, (float)B.q.z, (float)B.q.w};
  const V3<float> dAB{(float)(B.p.x - A.p.x), (float)(B.p.y - A.p.y), (float)(B.p.z - A.p.z)};
  float bf[9];
  for (int k = 0; k < 9; k++) bf[k] = (float)basis[k];
  const float alpha = (float)P.alpha, gamma = (float)P.gamma;
  const float kmin = (float)P.penaltyMin, kmax = (float)P.penaltyMax, margin = (float)P.margin;
  for (int i = 0; i < num; i++) {
    V3<float> rA{nc[i].ra[0], nc[i].ra[1], nc[i].ra[2]};
    V3<float> rB{nc[i].rb[0], nc[i].rb[1], nc[i].rb[2]};
    float lam[3] = {0.f, 0.f, 0.f}, pen[3] = {0.f, 0.f, 0.f};
    bool stick = false;
    for (int j = 0; j < oldNum; j++) {
      const int os = pi * kMaxContacts + j;
      if (nc[i].feature == w.prev.feat[os]) {
        const float4 ok = w.prev.cK[os], ol = w.prev.cL[os];
        lam[0] = ol.x; lam[1] = ol.y; lam[2] = ol.z;
        pen[0] = ok.x; pen[1] = ok.y; pen[2] = ok.z;
        stick = ol.w != 0.0f;
        if (stick) {  // a stuck box contact keeps its anchors (manifold.js:279-282)
          const float4 oa = w.prev.rA[os], ob = w.prev.rB[os];
          rA = V3<float>{oa.x, oa.y, oa.z};
          rB = V3<float>{ob.x, ob.y, ob.z};
        }
        break;
      }
    }
    const V3<float> rAw = qrotate(qa, rA), rBw = qrotate(qb, rB);
    const V3<float> dd{rAw.x - rBw.x - dAB.x, rAw.y - rBw.y - dAB.y, rAw.z - rBw.z - dAB.z};
    float C0[3];
    for (int k = 0; k < 3; k++) C0[k] = bf[3 * k] * dd.x + bf[3 * k + 1] * dd.y + bf[3 * k + 2] * dd.z;
    C0[0] += margin;
    if (!P.postStabilize)
      for (int k = 0; k < 3; k++) lam[k] = (lam[k] * alpha) * gamma;
    for (int k = 0; k < 3; k++) {
      const float x = pen[k] * gamma;  // clamp(gamma k, kmin, kmax), NaN propagating
      pen[k] = x != x ? x : fmaxf(kmin, fminf(kmax, x));
    }
    const int s = c * kMaxContacts + i;
    w.cur.feat[s] = nc[i].feature;
    w.cur.rA[s] = make_float4(rA.x, rA.y, rA.z, 0.f);
    w.cur.rB[s] = make_float4(rB.x, rB.y, rB.z, 0.f);
    w.cur.cA[s] = make_float4(rAw.x, rAw.y, rAw.z, C0[0]);
    w.cur.cB[s] = make_float4(rBw.x, rBw.y, rBw.z, C0[1]);
    w.cur.cK[s] = make_float4(pen[0], pen[1], pen[2], C0[2]);
    w.cur.cL[s] = make_float4(lam[0], lam[1], lam[2], stick ? 1.f : 0.f);
  }
  const double friction = sqrt(w.b.friction[ia] * w.b.friction[ib]);
  for (int k = 0; k < 9; k++) w.cur.basisD[c * 9 + k] = basis[k];
  w.cur.basis0[c] = make_float4(bf[0], bf[1], bf[2], (float)friction);
  w.cur.basis1[c] = make_float4(bf[3], bf[4], bf[5], 0.f);
  w.cur.basis2[c] = make_float4(bf[6], bf[7], bf[8], 0.f);
}

// Pairs with a sphere, in f64: the basis-compatibility test and the
// transport of lambda and k into the new basis (manifold.js:222-270).
__device__ void write_sphere_manifold(const World &w, int c, int ia, int ib, const BodyD &A, const BodyD &B,
                                      const NewContact *nc, int num, const double *basis) {
  const SolverParams &P = w.p;
  if (P.contactModel) {
    D3 ra[kMaxContacts], rb[kMaxContacts];
    uint32_t ft[kMaxContacts];
    for (int i = 0; i < num; i++) {
      ra[i] = nc[i].rA;
      rb[i] = nc[i].rB;
      ft[i] = nc[i].feature;
    }
    write_manifold_materials(w, c, ia, ib, A, B, ra, rb, ft, num, basis);
    return;
  }
  w.cur.count[c] = num;
  if (num == 0) return;
  const int pi = w.g.candPrev[c];
  const int oldNum = pi >= 0 ? w.prev.count[pi] : 0;
  double oldBasis[9];
  if (oldNum > 0)
    for (int k = 0; k < 9; k++) oldBasis[k] = w.prev.basisD[pi * 9 + k];
  const double friction = sqrt(w.b.friction[ia] * w.b.friction[ib]);
  const bool compatible =
      oldNum == 0 || (oldBasis[0] * basis[0] + oldBasis[1] * basis[1] + oldBasis[2] * basis[2]) > 0.85;
  const QD qA = A.q, qB = B.q;
  for (int i = 0; i < num; i++) {
    const D3 rA = nc[i].rA, rB = nc[i].rB;
    double lam[3] = {0, 0, 0}, pen[3] = {0, 0, 0};
    bool stick = false;
    for (int j = 0; j < oldNum; j++) {
      const int os = pi * kMaxContacts + j;
      if (compatible && nc[i].feature == w.prev.feat[os]) {
        const float4 ok = w.prev.cK[os], ol = w.prev.cL[os];
        lam[0] = ol.x; lam[1] = ol.y; lam[2] = ol.z;
        pen[0] = ok.x; pen[1] = ok.y; pen[2] = ok.z;
        stick = ol.w != 0.0f;
        transport(lam, pen, oldBasis, basis);
        break;
      }
    }
    // C*(x_t) and warm start (manifold.js:292-315)
    const D3 xA = add(rot(qA, rA), A.p);
    const D3 xB = add(rot(qB, rB), B.p);
    const D3 d = sub(xA, xB);
    double C0[3];
    C0[0] = basis[0] * d.x + basis[1] * d.y + basis[2] * d.z;
    C0[1] = basis[3] * d.x + basis[4] * d.y + basis[5] * d.z;
    C0[2] = basis[6] * d.x + basis[7] * d.y + basis[8] * d.z;
    C0[0] += P.margin;
    if (!P.postStabilize) {
      for (int k = 0; k < 3; k++) {
        lam[k] = lam[k] * P.alpha;
        lam[k] = lam[k] * P.gamma;
      }
    }
    for (int k = 0; k < 3; k++) pen[k] = clampd(pen[k] * P.gamma, P.penaltyMin, P.penaltyMax);
    const D3 rAw = rot(qA, rA), rBw = rot(qB, rB);
    const int s = c * kMaxContacts + i;
    w.cur.feat[s] = nc[i].feature;
    w.cur.rA[s] = make_float4((float)rA.x, (float)rA.y, (float)rA.z, 0.f);
    w.cur.rB[s] = make_float4((float)rB.x, (float)rB.y, (float)rB.z, 0.f);
    w.cur.cA[s] = make_float4((float)rAw.x, (float)rAw.y, (float)rAw.z, (float)C0[0]);
    w.cur.cB[s] = make_float4((float)rBw.x, (float)rBw.y, (float)rBw.z, (float)C0[1]);
    w.cur.cK[s] = make_float4((float)pen[0], (float)pen[1], (float)pen[2], (float)C0[2]);
    w.cur.cL[s] = make_float4((float)lam[0], (float)lam[1], (float)lam[2], stick ? 1.f : 0.f);
  }
  for (int k = 0; k < 9; k++) w.cur.basisD[c * 9 + k] = basis[k];
  w.cur.basis0[c] = make_float4((float)basis[0], (float)basis[1], (float)basis[2], (float)friction);
  w.cur.basis1[c] = make_float4((float)basis[3], (float)basis[4], (float)basis[5], 1.f);  // .w: sphere pair
  w.cur.basis2[c] = make_float4((float)basis[6], (float)basis[7], (float)basis[8], 0.f);
}

// AVBD_CONTACT_MATERIALS: the WebGPU engine's manifold warm start with its
// contact extensions (src/physics/gpu/shaders.js:1105-1366), in f64 for box
// and sphere pairs alike (an opt-in model; the default path above keeps the
// f32 box merge). Pair materials: friction as the geometric mean of the
// static and of the dynamic coefficients, restitution as the max, contact
// and rest offsets summed. A new contact matches the old one with its
// feature ID, else the nearest old contact within the persistence distance
// (separation, tangential offset and midpoint distance within it), each old
// contact claimed once and only when the normals agree (dot > 0.85);
// multiplier and penalty are transported into the new basis; a matched
// static box contact keeps its anchors; a new contact starts static. C0 on
// the normal is measured to the rest distance; a new or re-armed impact
// (the old contact still outside rest and without a bias) faster than the
// restitution threshold gets a one-frame bias.
__device__ void write_manifold_materials(const World &w, int c, int ia, int ib, const BodyD &A, const BodyD &B,
                                         const D3 *ncA, const D3 *ncB, const uint32_t *feat, int num,
                                         const double *basis) {
  const SolverParams &P = w.p;
  w.cur.count[c] = num;
  if (num == 0) return;
  const int pi = w.g.candPrev[c];
  const int oldNum = pi >= 0 ? w.prev.count[pi] : 0;
  double ob[9];
  for (int k = 0; k < 9; k++) ob[k] = oldNum > 0 ? w.prev.basisD[pi * 9 + k] : basis[k];
  const D4 ma = w.b.mat[ia], mb = w.b.mat[ib];
  const double mus = sqrt(ma.x * mb.x), mud = sqrt(ma.y * mb.y);
  const double restitution = ma.z > mb.z ? ma.z : (mb.z > ma.z ? mb.z : ma.z);
  const double contactDistance = w.b.contactOffset[ia] + w.b.contactOffset[ib];
  const double restDistance = ma.w + mb.w;
  const D3 nN = mk(basis[0], basis[1], basis[2]);
  const bool compatible = oldNum > 0 && (ob[0] * basis[0] + ob[1] * basis[1] + ob[2] * basis[2]) > 0.85;
  const double minA = fmin(A.half.x, fmin(A.half.y, A.half.z)), minB = fmin(B.half.x, fmin(B.half.y, B.half.z));
  const double minExtent = 2.0 * fmin(minA, minB);
  const double persistence = fmax(P.contactPersistence, fmax(contactDistance, minExtent * 0.02));
  const double psq = persistence * persistence;
  const bool curved = A.sphere || B.sphere;
  const float4 vA4 = w.b.vel[ia], wA4 = w.b.omega[ia], vB4 = w.b.vel[ib], wB4 = w.b.omega[ib];
  const D3 vA = mk(vA4.x, vA4.y, vA4.z), wA = mk(wA4.x, wA4.y, wA4.z);
  const D3 vB = mk(vB4.x, vB4.y, vB4.z), wB = mk(wB4.x, wB4.y, wB4.z);
  unsigned used = 0u;
  for (int i = 0; i < num; i++) {
    D3 rA = ncA[i], rB = ncB[i];
    double lam[3] = {0, 0, 0}, pen[3] = {0, 0, 0};
    bool stick = true, priorOut = false, priorBias = false, found = false, exact = false;
    int match = -1;
    double best = psq;
    const D3 nxA = add(rot(A.q, rA), A.p), nxB = add(rot(B.q, rB), B.p);
    const D3 mid = mk((nxA.x + nxB.x) * 0.5, (nxA.y + nxB.y) * 0.5, (nxA.z + nxB.z) * 0.5);
    if (compatible) {
      for (int j = 0; j < oldNum; j++) {
        if (used & (1u << j)) continue;
        const int os = pi * kMaxContacts + j;
        const bool same = w.prev.feat[os] == feat[i];
        if (curved && same) {
          match = j;
          exact = true;
          break;
        }
        const float4 oa = w.prev.rA[os], obb = w.prev.rB[os];
        const D3 oxA = add(rot(A.q, mk(oa.x, oa.y, oa.z)), A.p);
        const D3 oxB = add(rot(B.q, mk(obb.x, obb.y, obb.z)), B.p);
        const D3 od = sub(oxA, oxB);
        const double sep = nN.x * od.x + nN.y * od.y + nN.z * od.z;
        const D3 td = mk(od.x - nN.x * sep, od.y - nN.y * sep, od.z - nN.z * sep);
        if (sep > contactDistance + persistence) continue;
        if (td.x * td.x + td.y * td.y + td.z * td.z > psq) continue;
        const D3 md = mk(mid.x - (oxA.x + oxB.x) * 0.5, mid.y - (oxA.y + oxB.y) * 0.5, mid.z - (oxA.z + oxB.z) * 0.5);
        const double mdSq = md.x * md.x + md.y * md.y + md.z * md.z;
        if (mdSq > psq) continue;
        if (same) {
          match = j;
          exact = true;
          break;
        }
        if (!found || mdSq < best) {
          found = true;
          match = j;
          best = mdSq;
        }
      }
    }
    found = found || exact;
    if (found) {
      const int os = pi * kMaxContacts + match;
      used |= 1u << match;
      const float4 ok = w.prev.cK[os], ol = w.prev.cL[os];
      for (int r = 0; r < 3; r++) {  // transport into the new basis (shaders.js:1050-1085)
        const double *nr = &basis[r * 3];
        const double a = nr[0] * ob[0] + nr[1] * ob[1] + nr[2] * ob[2];
        const double b = nr[0] * ob[3] + nr[1] * ob[4] + nr[2] * ob[5];
        const double cc = nr[0] * ob[6] + nr[1] * ob[7] + nr[2] * ob[8];
        pen[r] = (double)ok.x * (a * a) + (double)ok.y * (b * b) + (double)ok.z * (cc * cc);
        lam[r] = (double)ol.x * a + (double)ol.y * b + (double)ol.z * cc;
      }
      stick = ol.w != 0.0f;
      priorOut = w.prev.cA[os].w > 0.0f;
      priorBias = w.prev.cX[os] > 0.0f;
      if (stick && !A.sphere && !B.sphere) {
        const float4 oa = w.prev.rA[os], obb = w.prev.rB[os];
        rA = mk(oa.x, oa.y, oa.z);
        rB = mk(obb.x, obb.y, obb.z);
      }
    }
    const D3 rAw = rot(A.q, rA), rBw = rot(B.q, rB);
    const D3 d = sub(add(rAw, A.p), add(rBw, B.p));
    double C0[3];
    C0[0] = basis[0] * d.x + basis[1] * d.y + basis[2] * d.z - restDistance;
    C0[1] = basis[3] * d.x + basis[4] * d.y + basis[5] * d.z;
    C0[2] = basis[6] * d.x + basis[7] * d.y + basis[8] * d.z;
    double bias = 0.0;
    if ((!found || (priorOut && !priorBias)) && restitution > 0.0) {
      const D3 ua = add(vA, crs(wA, rAw)), ub = add(vB, crs(wB, rBw));
      const D3 rel = sub(ua, ub);
      const double vn = nN.x * rel.x + nN.y * rel.y + nN.z * rel.z;
      const double closing = fmax(0.0, -vn * P.dt), toRest = fmax(0.0, C0[0]);
      if (vn < -P.restitutionThreshold && closing > toRest) bias = restitution * (closing - toRest);
    }
    if (!P.postStabilize)
      for (int k = 0; k < 3; k++) lam[k] = lam[k] * P.alpha * P.gamma;
    for (int k = 0; k < 3; k++) pen[k] = clampd(pen[k] * P.gamma, P.penaltyMin, P.penaltyMax);
    const int s = c * kMaxContacts + i;
    w.cur.feat[s] = feat[i];
    w.cur.rA[s] = make_float4((float)rA.x, (float)rA.y, (float)rA.z, 0.f);
    w.cur.rB[s] = make_float4((float)rB.x, (float)rB.y, (float)rB.z, 0.f);
    w.cur.cA[s] = make_float4((float)rAw.x, (float)rAw.y, (float)rAw.z, (float)C0[0]);
    w.cur.cB[s] = make_float4((float)rBw.x, (float)rBw.y, (float)rBw.z, (float)C0[1]);
    w.cur.cK[s] = make_float4((float)pen[0], (float)pen[1], (float)pen[2], (float)C0[2]);
    w.cur.cL[s] = make_float4((float)lam[0], (float)lam[1], (float)lam[2], stick ? 1.f : 0.f);
    w.cur.cX[s] = (float)bias;
  }
  for (int k = 0; k < 9; k++) w.cur.basisD[c * 9 + k] = basis[k];
  const float flags = (curved ? 1.f : 0.f) + (contactDistance > 0.0 ? 2.f : 0.f);
  w.cur.basis0[c] = make_float4((float)basis[0], (float)basis[1], (float)basis[2], (float)mus);
  w.cur.basis1[c] = make_float4((float)basis[3], (float)basis[4], (float)basis[5], flags);
  w.cur.basis2[c] = make_float4((float)basis[6], (float)basis[7], (float)basis[8], (float)mud);
}

// Append to one of the work lists, one atomic per coalesced group of lanes.
__device__ __forceinline__ int push_slot(int *counter) {
  const unsigned m = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(m, base, leader);
  return base + __popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ void push_exact(const World &w, int c) {
  w.g.npExact[push_slot(&w.ctl->npCount[2])] = c;
}

// The face axis among `mask` (bits 0-5: faces of A, then of B) with the
// largest exact separation, the first on ties: the f64 expressions of
// testAxis (collide.js:291-324) for just those axes.
__device__ int exact_best_face(const BodyD &A, const BodyD &B, int mask) {
  const D3 e3[3] = {mk(1, 0, 0), mk(0, 1, 0), mk(0, 0, 1)};
  D3 ax[3], bx[3];
  for (int i = 0; i < 3; i++) {
    ax[i] = rot(A.q, e3[i]);
    bx[i] = rot(B.q, e3[i]);
  }
  const D3 delta = sub(B.p, A.p);
  int best = -1;
  double bestSep = -INFINITY;
  for (int k = 0; k < 6; k++) {
    if (!((mask >> k) & 1)) continue;
    const D3 axis = k < 3 ? ax[k] : bx[k - 3];
    const double lenSq = axis.x * axis.x + axis.y * axis.y + axis.z * axis.z;
    const double invLen = 1.0 / sqrt(lenSq);
    D3 n = scl(axis, invLen);
    if (dt3(n, delta) < 0) n = neg(n);
    const double distance = fabs(dt3(delta, n));
    const double rA = A.half.x * fabs(dt3(n, ax[0])) + A.half.y * fabs(dt3(n, ax[1])) + A.half.z * fabs(dt3(n, ax[2]));
    const double rB = B.half.x * fabs(dt3(n, bx[0])) + B.half.y * fabs(dt3(n, bx[1])) + B.half.z * fabs(dt3(n, bx[2]));
    const double separation = distance - (rA + rB);
    if (best < 0 || separation > bestSep) {
      best = k;
      bestSep = separation;
    }
  }
  return best;
}

// 1. Every candidate: the f32 SAT. Separated pairs get count 0; box pairs
//    with a certain winning axis go to the face or edge list, everything
//    else (sphere pairs, undecided box pairs) to the exact list.
__global__ void __launch_bounds__(256) classify_kernel(World w) {
  const int total = *((volatile int *)&w.ctl->numCandidates);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < total; c += gridDim.x * blockDim.x) {
    const uint64_t key = w.g.candKey[c];
    const int ia = (int)(key >> 32), ib = (int)(key & 0xffffffffu);
    const BodyD A = load_body(w, ia), B = load_body(w, ib);
    // spheres, and pairs with a contact skin (speculative contacts: the f32
    // certification covers the skin-free tests), go to the exact collider
    if (A.sphere || B.sphere || pair_skin(w, ia, ib) != 0.0) {
      push_exact(w, c);
      continue;
    }
    bool refIsA = true;
    int axA = 0, axB = 0, tieMask = 0;
    const int r = classify_f32(make_boxf(A, B), refIsA, axA, axB, tieMask);
    if (r == kSeparated) {
      w.cur.count[c] = 0;
    } else if (r == kFaceWin) {
      w.g.npFace[push_slot(&w.ctl->npCount[0])] = make_int2(c, (refIsA ? 4 : 0) | axA);
    } else if (r == kFaceTie) {
      w.g.npFace[push_slot(&w.ctl->npCount[0])] = make_int2(c, tieMask << 8);
    } else if (r == kEdgeWin) {
      w.g.npEdge[push_slot(&w.ctl->npCount[1])] = make_int2(c, axA * 3 + axB);
    } else {
      push_exact(w, c);
    }
  }
}

// 2. Face manifolds: the exact normal and basis in f64, the clipping in f32
//    with certified decisions; an undecided pair moves to the exact list.
__global__ void __launch_bounds__(128) face_kernel(World w) {
  const int total = *((volatile int *)&w.ctl->npCount[0]);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int2 e = w.g.npFace[t];
    const int c = e.x;
    bool refIsA = (e.y & 4) != 0;
    int refAxis = e.y & 3;
    const uint64_t key = w.g.candKey[c];
    const int ia = (int)(key >> 32), ib = (int)(key & 0xffffffffu);
    const BodyD A = load_body(w, ia), B = load_body(w, ib);
    if (e.y >> 8) {  // tied face axes: their exact separations decide (first largest wins)
      const int k = exact_best_face(A, B, e.y >> 8);
      refIsA = k < 3;
      refAxis = refIsA ? k : k - 3;
    }
    // f64: the reference axis, the incident box's axes, the exact normal
    const QD qRef = refIsA ? A.q : B.q, qInc = refIsA ? B.q : A.q;
    const D3 e3[3] = {mk(1, 0, 0), mk(0, 1, 0), mk(0, 0, 1)};
    const D3 refAx = rot(qRef, e3[refAxis]);
    const D3 ibAx[3] = {rot(qInc, e3[0]), rot(qInc, e3[1]), rot(qInc, e3[2])};
    const D3 n = Collider::axisNormal(refAx, sub(B.p, A.p));
    double basis[9];
    orthonormal(basis, neg(n));
    const BoxF F = make_boxf(A, B);
    NewContactF ncf[kMaxContacts];
    FaceF face(F, A, B, ncf);
    const int num = face.build(refIsA, refAxis, n, refAx, ibAx);
    if (num < 0) {
      push_exact(w, c);
      continue;
    }
    write_box_manifold(w, c, ia, ib, A, B, ncf, num, basis);
  }
}

// 3. Edge-edge contacts (collide.js:475-493), exact f64.
__global__ void __launch_bounds__(128) edge_kernel(World w) {
  const int total = *((volatile int *)&w.ctl->npCount[1]);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int2 e = w.g.npEdge[t];
    const int c = e.x, i = e.y / 3, j = e.y % 3;
    const uint64_t key = w.g.candKey[c];
    const int ia = (int)(key >> 32), ib = (int)(key & 0xffffffffu);
    const BodyD A = load_body(w, ia), B = load_body(w, ib);
    NewContact nc[2];
    Collider col(A, B, nc);
    Collider::makeOBB(col.boxA, A);
    Collider::makeOBB(col.boxB, B);
    const D3 delta = sub(col.boxB.c, col.boxA.c);
    const D3 n = Collider::axisNormal(crs(col.boxA.ax[i], col.boxB.ax[j]), delta);
    double basis[9];
    orthonormal(basis, neg(n));
    const int num = col.edgeContact(i, j, n);
    NewContactF ncf[2];
    for (int k = 0; k < num; k++) {
      ncf[k].feature = nc[k].feature;
      ncf[k].ra[0] = (float)nc[k].rA.x; ncf[k].ra[1] = (float)nc[k].rA.y; ncf[k].ra[2] = (float)nc[k].rA.z;
      ncf[k].rb[0] = (float)nc[k].rB.x; ncf[k].rb[1] = (float)nc[k].rB.y; ncf[k].rb[2] = (float)nc[k].rB.z;
    }
    write_box_manifold(w, c, ia, ib, A, B, ncf, num, basis);
  }
}

// 4. Sphere pairs and undecided box pairs: the whole f64 collider.
__global__ void __launch_bounds__(128) exact_kernel(World w) {
  const int total = *((volatile int *)&w.ctl->npCount[2]);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int c = w.g.npExact[t];
    const uint64_t key = w.g.candKey[c];
    const int ia = (int)(key >> 32), ib = (int)(key & 0xffffffffu);
    const BodyD A = load_body(w, ia), B = load_body(w, ib);
    double basis[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    NewContact nc[kMaxContacts];
    Collider col(A, B, nc);
    col.cd = pair_skin(w, ia, ib);
    const int num = col.collide(basis);
    if (A.sphere || B.sphere) {
      write_sphere_manifold(w, c, ia, ib, A, B, nc, num, basis);
      continue;
    }
    NewContactF ncf[kMaxContacts];
    for (int k = 0; k < num; k++) {
      ncf[k].feature = nc[k].feature;
      ncf[k].ra[0] = (float)nc[k].rA.x; ncf[k].ra[1] = (float)nc[k].rA.y; ncf[k].ra[2] = (float)nc[k].rA.z;
      ncf[k].rb[0] = (float)nc[k].rB.x; ncf[k].rb[1] = (float)nc[k].rB.y; ncf[k].rb[2] = (float)nc[k].rB.z;
    }
    write_box_manifold(w, c, ia, ib, A, B, ncf, num, basis);
  }
}

}  // namespace

void launch_narrowphase(const World &w, cudaStream_t st, int smCount) {
  cudaMemsetAsync(w.ctl->npCount, 0, sizeof(w.ctl->npCount), st);
  classify_kernel<<<smCount * 8, 256, 0, st>>>(w);
  face_kernel<<<smCount * 8, 128, 0, st>>>(w);
  edge_kernel<<<smCount * 4, 128, 0, st>>>(w);
  exact_kernel<<<smCount * 4, 128, 0, st>>>(w);
}

}  // namespace avbd
