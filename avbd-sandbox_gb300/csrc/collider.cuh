// collider.cuh - the exact contact geometry of the narrow phase, on a scalar
// type R: double for the narrow phase's exact path (narrowphase.cu, built
// with --fmad=false so that every operation rounds as in the reference
// engine), and the forward-mode dual number of the tangent step
// (tangent.cu), whose value part runs the very same double operations -
// hence the same SAT, clipping and merge decisions - while it carries the
// derivatives of the contact points and bases.
//
//   collide.js:612-685 box-box 15-axis SAT, face clipping (:403-472), edge
//                      contact (:475-493), merge within 1e-3 m (:254-285)
//   collide.js:496-520 sphere-sphere, :526-600 sphere-OBB
//   maths.js:389-414   orthonormal contact basis, :599-613 rotate
#pragma once

#include <cstdint>

namespace avbd {
namespace geo {

constexpr int kMaxContactsG = 8;  // collide.js:22
constexpr int kPolyCap = 8;       // a quad clipped by 4 half-planes has <= 8 vertices
constexpr int kMaxPolyVerts = 16; // collide.js:23 (never reached, see kPolyCap)
constexpr double kSatEps = 1.0e-6;
constexpr double kSphereEpsSq = 1.0e-20;
constexpr double kPlaneEps = 1.0e-5;
constexpr double kMergeDistSq = 1.0e-6;
constexpr int kFaceA = 0, kFaceB = 1, kEdge = 2;

// A parameter that takes the scalar without deducing it (literals convert).
template <class T>
struct Id {
  using type = T;
};

template <class R>
struct D3T {
  R x, y, z;
};
template <class R>
__device__ __forceinline__ D3T<R> mk3(R x, R y, R z) {
  return D3T<R>{x, y, z};
}
template <class R>
__device__ __forceinline__ D3T<R> add(D3T<R> a, D3T<R> b) {
  return D3T<R>{a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class R>
__device__ __forceinline__ D3T<R> sub(D3T<R> a, D3T<R> b) {
  return D3T<R>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class R>
__device__ __forceinline__ D3T<R> scl(D3T<R> a, typename Id<R>::type s) {
  return D3T<R>{a.x * s, a.y * s, a.z * s};
}
template <class R>
__device__ __forceinline__ D3T<R> neg(D3T<R> a) {
  return D3T<R>{-a.x, -a.y, -a.z};
}
template <class R>
__device__ __forceinline__ R dt3(D3T<R> a, D3T<R> b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
// out + a * s, the reference's vec3.addScaled
template <class R>
__device__ __forceinline__ D3T<R> adds(D3T<R> o, D3T<R> a, typename Id<R>::type s) {
  return D3T<R>{o.x + a.x * s, o.y + a.y * s, o.z + a.z * s};
}
template <class R>
__device__ __forceinline__ D3T<R> crs(D3T<R> a, D3T<R> b) {
  return D3T<R>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Math.min / Math.max: NaN propagates; on ties the first argument is kept,
// which gives Math.min(x, -0) / Math.max(+0, -0) their JavaScript results for
// every call order used here.
template <class R>
__device__ __forceinline__ R jmin(R a, typename Id<R>::type b) {
  if (a != a || b != b) return a + b;
  return a < b ? a : (b < a ? b : a);
}
template <class R>
__device__ __forceinline__ R jmax(R a, typename Id<R>::type b) {
  if (a != a || b != b) return a + b;
  return a > b ? a : (b > a ? b : a);
}
template <class R>
__device__ __forceinline__ R clampd(R x, typename Id<R>::type a, typename Id<R>::type b) {
  return jmax(a, jmin(b, x));
}

template <class R>
struct QDT {
  R x, y, z, w;
};
template <class R>
__device__ __forceinline__ D3T<R> rot(QDT<R> q, D3T<R> v) {  // maths.js:599-613
  const R tx = (q.y * v.z - q.z * v.y) * 2;
  const R ty = (q.z * v.x - q.x * v.z) * 2;
  const R tz = (q.x * v.y - q.y * v.x) * 2;
  return D3T<R>{v.x + tx * q.w + (q.y * tz - q.z * ty), v.y + ty * q.w + (q.z * tx - q.x * tz),
                v.z + tz * q.w + (q.x * ty - q.y * tx)};
}
template <class R>
__device__ __forceinline__ QDT<R> conj(QDT<R> q) {
  return QDT<R>{-q.x, -q.y, -q.z, q.w};
}

// mat3.orthonormal (maths.js:389-414): rows n, t1, t2.
template <class R>
__device__ void orthonormal(R *o, D3T<R> n) {
  R t1x, t1y, t1z;
  if (fabs(n.x) > fabs(n.z)) {
    t1x = -n.y; t1y = n.x; t1z = 0;
  } else {
    t1x = 0; t1y = -n.z; t1z = n.y;
  }
  const R len = sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
  t1x /= len; t1y /= len; t1z /= len;
  o[0] = n.x; o[1] = n.y; o[2] = n.z;
  o[3] = t1x; o[4] = t1y; o[5] = t1z;
  o[6] = n.y * t1z - n.z * t1y;
  o[7] = n.z * t1x - n.x * t1z;
  o[8] = n.x * t1y - n.y * t1x;
}

template <class R>
struct BodyT {
  D3T<R> p;
  QDT<R> q;
  D3T<R> half;
  R radius;
  bool sphere;
};

template <class R>
struct OBBT {
  D3T<R> c, h, ax[3];
};

template <class R>
struct NewContactT {
  uint32_t feature;
  D3T<R> rA, rB;
};

template <class R>
struct ColliderT {
  using D3 = D3T<R>;
  using QD = QDT<R>;
  using OBB = OBBT<R>;
  using BodyD = BodyT<R>;
  using NewContact = NewContactT<R>;
  const BodyD &A, &B;
  OBB boxA, boxB;
  D3 fN, fC, fU, fV;
  R fEU, fEV;
  R faceExtU, faceExtV;
  D3 mid[kMaxContactsG];
  int count = 0;
  NewContact *out;
  // the pair's contact skin: contacts are generated up to this separation
  // (AVBD_CONTACT_MATERIALS, the WGSL collider's contactDistance,
  // src/physics/gpu/shaders.js:716-886, 1039); 0 for the CPU engine's collider
  double cd = 0.0;

  __device__ ColliderT(const BodyD &a, const BodyD &b, NewContact *o) : A(a), B(b), out(o) {}

  __device__ static D3 unit(int i) { return D3{R(i == 0 ? 1 : 0), R(i == 1 ? 1 : 0), R(i == 2 ? 1 : 0)}; }
  __device__ static void makeOBB(OBB &box, const BodyD &b) {
    box.c = b.p;
    box.h = b.half;
    box.ax[0] = rot(b.q, unit(0));
    box.ax[1] = rot(b.q, unit(1));
    box.ax[2] = rot(b.q, unit(2));
  }
  __device__ static R hcomp(D3 h, int i) { return i == 0 ? h.x : (i == 1 ? h.y : h.z); }
  __device__ static D3 support(const OBB &b, D3 dir) {
    const R sx = dt3(dir, b.ax[0]) >= 0 ? R(1) : R(-1);
    const R sy = dt3(dir, b.ax[1]) >= 0 ? R(1) : R(-1);
    const R sz = dt3(dir, b.ax[2]) >= 0 ? R(1) : R(-1);
    D3 o = b.c;
    o = adds(o, b.ax[0], b.h.x * sx);
    o = adds(o, b.ax[1], b.h.y * sy);
    o = adds(o, b.ax[2], b.h.z * sz);
    return o;
  }
  __device__ void faceAxes(const OBB &b, int axis, D3 &u, D3 &v) {
    if (axis == 0) {
      u = b.ax[1]; v = b.ax[2]; faceExtU = b.h.y; faceExtV = b.h.z;
    } else if (axis == 1) {
      u = b.ax[0]; v = b.ax[2]; faceExtU = b.h.x; faceExtV = b.h.z;
    } else {
      u = b.ax[0]; v = b.ax[1]; faceExtU = b.h.x; faceExtV = b.h.y;
    }
  }
  // collide.js:254-285
  __device__ bool addContact(D3 xA, D3 xB, uint32_t key) {
    const D3 m{(xA.x + xB.x) * 0.5, (xA.y + xB.y) * 0.5, (xA.z + xB.z) * 0.5};
    for (int i = 0; i < count; i++) {
      const R dx = m.x - mid[i].x, dy = m.y - mid[i].y, dz = m.z - mid[i].z;
      if (dx * dx + dy * dy + dz * dz < kMergeDistSq) return false;
    }
    if (count >= kMaxContactsG) return false;
    NewContact &c = out[count];
    c.feature = key;
    c.rA = rot(conj(A.q), sub(xA, A.p));
    c.rB = rot(conj(B.q), sub(xB, B.p));
    mid[count] = m;
    count++;
    return true;
  }
  // collide.js:202-247; returns the new count
  __device__ static int clipPlane(const D3 *in, int n, D3 pn, R po, D3 *o) {
    if (n <= 0) return 0;
    int oc = 0;
    D3 a = in[n - 1];
    R da = pn.x * a.x + pn.y * a.y + pn.z * a.z - po;
    for (int i = 0; i < n; i++) {
      const D3 b = in[i];
      const R db = pn.x * b.x + pn.y * b.y + pn.z * b.z - po;
      const bool ai = da <= kPlaneEps, bi = db <= kPlaneEps;
      if (ai != bi) {
        R t = 0;
        const R denom = da - db;
        if (fabs(denom) > kSatEps) t = clampd(da / denom, 0, 1);
        if (oc < kMaxPolyVerts && oc < kPolyCap) {
          o[oc] = D3{a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t};
          oc++;
        }
      }
      if (bi && oc < kMaxPolyVerts && oc < kPolyCap) {
        o[oc] = b;
        oc++;
      }
      a = b;
      da = db;
    }
    return oc;
  }
  struct Sat {
    int type, ia, ib;
    R sep;
    D3 n;
    bool valid;
  };
  // collide.js:291-324
  __device__ bool testAxis(D3 delta, D3 axis, int type, int ia, int ib, Sat &t) {
    const R lenSq = axis.x * axis.x + axis.y * axis.y + axis.z * axis.z;
    if (lenSq < kSatEps) return true;
    const R invLen = 1.0 / sqrt(lenSq);
    D3 n = scl(axis, invLen);
    if (dt3(n, delta) < 0) n = neg(n);
    const R distance = fabs(dt3(delta, n));
    const R rA = boxA.h.x * fabs(dt3(n, boxA.ax[0])) + boxA.h.y * fabs(dt3(n, boxA.ax[1])) +
                 boxA.h.z * fabs(dt3(n, boxA.ax[2]));
    const R rB = boxB.h.x * fabs(dt3(n, boxB.ax[0])) + boxB.h.y * fabs(dt3(n, boxB.ax[1])) +
                 boxB.h.z * fabs(dt3(n, boxB.ax[2]));
    const R separation = distance - (rA + rB);
    if (separation > cd) return false;
    if (!t.valid || separation > t.sep) {
      t.valid = true; t.type = type; t.ia = ia; t.ib = ib; t.sep = separation; t.n = n;
    }
    return true;
  }
  __device__ static void supportEdge(const OBB &b, int axis, D3 dir, D3 &e0, D3 &e1) {
    const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
    const R s1 = dt3(dir, b.ax[a1]) >= 0 ? R(1) : R(-1);
    const R s2 = dt3(dir, b.ax[a2]) >= 0 ? R(1) : R(-1);
    D3 t = b.c;
    t = adds(t, b.ax[a1], hcomp(b.h, a1) * s1);
    t = adds(t, b.ax[a2], hcomp(b.h, a2) * s2);
    e0 = adds(t, b.ax[axis], -hcomp(b.h, axis));
    e1 = adds(t, b.ax[axis], hcomp(b.h, axis));
  }
  // collide.js:345-393
  __device__ static void closestSeg(D3 p0, D3 p1, D3 q0, D3 q1, D3 &c0, D3 &c1) {
    const R d1x = p1.x - p0.x, d1y = p1.y - p0.y, d1z = p1.z - p0.z;
    const R d2x = q1.x - q0.x, d2y = q1.y - q0.y, d2z = q1.z - q0.z;
    const R rx = p0.x - q0.x, ry = p0.y - q0.y, rz = p0.z - q0.z;
    const R a = d1x * d1x + d1y * d1y + d1z * d1z;
    const R e = d2x * d2x + d2y * d2y + d2z * d2z;
    const R f = d2x * rx + d2y * ry + d2z * rz;
    R s = 0, t = 0;
    if (a <= kSatEps && e <= kSatEps) {
      c0 = p0; c1 = q0;
      return;
    }
    if (a <= kSatEps) {
      t = clampd(f / e, 0, 1);
    } else {
      const R c = d1x * rx + d1y * ry + d1z * rz;
      if (e <= kSatEps) {
        s = clampd(-c / a, 0, 1);
      } else {
        const R b = d1x * d2x + d1y * d2y + d1z * d2z;
        const R denom = a * e - b * b;
        if (fabs(denom) > kSatEps) s = clampd((b * f - c * e) / denom, 0, 1);
        t = (b * s + f) / e;
        if (t < 0) {
          t = 0; s = clampd(-c / a, 0, 1);
        } else if (t > 1) {
          t = 1; s = clampd((b - c) / a, 0, 1);
        }
      }
    }
    c0 = D3{p0.x + d1x * s, p0.y + d1y * s, p0.z + d1z * s};
    c1 = D3{q0.x + d2x * t, q0.y + d2y * t, q0.z + d2z * t};
  }
  // collide.js:403-472
  __device__ int faceManifold(bool refIsA, int refAxis, D3 nAB) {
    D3 clip0[kPolyCap], clip1[kPolyCap];
    const OBB &rb = refIsA ? boxA : boxB;
    const OBB &ib = refIsA ? boxB : boxA;
    const D3 outward = refIsA ? nAB : neg(nAB);
    {  // buildFaceFrame
      const R s = dt3(outward, rb.ax[refAxis]) >= 0 ? R(1) : R(-1);
      fN = scl(rb.ax[refAxis], s);
      fC = adds(rb.c, fN, hcomp(rb.h, refAxis));
      faceAxes(rb, refAxis, fU, fV);
      fEU = faceExtU;
      fEV = faceExtV;
    }
    int incAxis = 0;
    {  // chooseIncidentFaceAxis
      R best = -INFINITY;
      for (int i = 0; i < 3; i++) {
        const R d = fabs(dt3(ib.ax[i], fN));
        if (d > best) { best = d; incAxis = i; }
      }
    }
    {  // buildIncidentFace
      const R s = dt3(ib.ax[incAxis], fN) > 0 ? R(-1) : R(1);
      const D3 fn = scl(ib.ax[incAxis], s);
      const D3 fc = adds(ib.c, fn, hcomp(ib.h, incAxis));
      D3 u, v;
      faceAxes(ib, incAxis, u, v);
      const R eU = faceExtU, eV = faceExtV;
      for (int i = 0; i < 4; i++) {
        const R su = (i == 0 || i == 3) ? R(1) : R(-1);
        const R sv = (i == 0 || i == 1) ? R(1) : R(-1);
        clip0[i] = D3{fc.x + u.x * (eU * su) + v.x * (eV * sv), fc.y + u.y * (eU * su) + v.y * (eV * sv),
                      fc.z + u.z * (eU * su) + v.z * (eV * sv)};
      }
    }
    int n = 4;
    D3 pn = fU;
    n = clipPlane(clip0, n, pn, dt3(pn, fC) + fEU, clip1);
    if (!n) return 0;
    pn = neg(fU);
    n = clipPlane(clip1, n, pn, dt3(pn, fC) + fEU, clip0);
    if (!n) return 0;
    pn = fV;
    n = clipPlane(clip0, n, pn, dt3(pn, fC) + fEV, clip1);
    if (!n) return 0;
    pn = neg(fV);
    n = clipPlane(clip1, n, pn, dt3(pn, fC) + fEV, clip0);
    if (!n) return 0;
    count = 0;
    uint32_t prefix = (uint32_t)(refIsA ? kFaceA : kFaceB) << 24;
    prefix |= (uint32_t)(refAxis & 0xff) << 16;
    prefix |= (uint32_t)(incAxis & 0xff) << 8;
    for (int i = 0; i < n && count < kMaxContactsG; i++) {
      const D3 p = clip0[i];
      const R distance = dt3(sub(p, fC), fN);
      if (distance > cd + kPlaneEps) continue;
      const D3 proj = adds(p, fN, -distance);
      if (refIsA) addContact(proj, p, prefix | (uint32_t)(i & 0xff));
      else addContact(p, proj, prefix | (uint32_t)(i & 0xff));
    }
    if (!count) addContact(support(boxA, nAB), support(boxB, neg(nAB)), prefix);
    return count;
  }
  // collide.js:475-493
  __device__ int edgeContact(int axA, int axB, D3 nAB) {
    const D3 nn = neg(nAB);
    D3 a0, a1, b0, b1, xA, xB;
    supportEdge(boxA, axA, nAB, a0, a1);
    supportEdge(boxB, axB, nn, b0, b1);
    closestSeg(a0, a1, b0, b1, xA, xB);
    count = 0;
    const uint32_t key = ((uint32_t)kEdge << 24) | ((uint32_t)(axA & 0xff) << 8) | (uint32_t)(axB & 0xff);
    addContact(xA, xB, key);
    if (!count) addContact(support(boxA, nAB), support(boxB, nn), key);
    return count;
  }
  // collide.js:496-520
  __device__ int sphereSphere(R *basis) {
    const D3 delta = sub(B.p, A.p);
    const R d2 = delta.x * delta.x + delta.y * delta.y + delta.z * delta.z;
    const R rs = A.radius + B.radius + cd;
    if (d2 > rs * rs) return 0;
    D3 n = d2 > kSphereEpsSq ? scl(delta, 1 / sqrt(d2)) : unit(0);
    orthonormal(basis, neg(n));
    const D3 xA = adds(A.p, n, A.radius);
    const D3 xB = adds(B.p, n, -B.radius);
    count = 0;
    addContact(xA, xB, 0x31000001u);
    return count;
  }
  // collide.js:526-600
  __device__ int sphereBox(R *basis, bool sphereIsA) {
    const BodyD &sp = sphereIsA ? A : B;
    const BodyD &bx = sphereIsA ? B : A;
    makeOBB(boxA, bx);
    const D3 delta = sub(sp.p, boxA.c);
    const R lx = dt3(delta, boxA.ax[0]), ly = dt3(delta, boxA.ax[1]), lz = dt3(delta, boxA.ax[2]);
    const R cx = clampd(lx, -boxA.h.x, boxA.h.x);
    const R cy = clampd(ly, -boxA.h.y, boxA.h.y);
    const R cz = clampd(lz, -boxA.h.z, boxA.h.z);
    D3 closest = boxA.c;
    closest = adds(closest, boxA.ax[0], cx);
    closest = adds(closest, boxA.ax[1], cy);
    closest = adds(closest, boxA.ax[2], cz);
    const D3 t3 = sub(sp.p, closest);
    const R d2 = t3.x * t3.x + t3.y * t3.y + t3.z * t3.z;
    int fa = 0;
    D3 n;
    if (d2 > kSphereEpsSq) {
      const R d = sqrt(d2);
      if (d - sp.radius > cd) return 0;
      n = scl(t3, 1 / d);
    } else {
      const R gx = boxA.h.x - fabs(lx), gy = boxA.h.y - fabs(ly), gz = boxA.h.z - fabs(lz);
      fa = gx < gy ? (gx < gz ? 0 : 2) : (gy < gz ? 1 : 2);
      const R local = fa == 0 ? lx : fa == 1 ? ly : lz;
      const R sg = local >= 0 ? R(1) : R(-1);
      n = scl(boxA.ax[fa], sg);
      const R gap = fa == 0 ? gx : fa == 1 ? gy : gz;
      closest = adds(sp.p, n, gap);
    }
    const D3 pole = adds(sp.p, n, -sp.radius);
    D3 xA, xB;
    if (sphereIsA) {
      xA = pole; xB = closest;
      orthonormal(basis, n);
    } else {
      xA = closest; xB = pole;
      orthonormal(basis, neg(n));
    }
    count = 0;
    int sx = lx < -boxA.h.x ? 1 : lx > boxA.h.x ? 2 : 0;
    int sy = ly < -boxA.h.y ? 1 : ly > boxA.h.y ? 2 : 0;
    int sz = lz < -boxA.h.z ? 1 : lz > boxA.h.z ? 2 : 0;
    if ((sx | sy | sz) == 0) {
      const R local = fa == 0 ? lx : fa == 1 ? ly : lz;
      const int side = local >= 0 ? 2 : 1;
      if (fa == 0) sx = side;
      else if (fa == 1) sy = side;
      else sz = side;
    }
    const uint32_t region = (uint32_t)(sx | (sy << 2) | (sz << 4));
    addContact(xA, xB, 0x32000000u | (region << 2) | (sphereIsA ? 1u : 2u));
    return count;
  }
  // The exact unit normal of an SAT axis, oriented from A to B, with the
  // operations of testAxis (collide.js:291-324).
  __device__ static D3 axisNormal(D3 axis, D3 delta) {
    const R lenSq = axis.x * axis.x + axis.y * axis.y + axis.z * axis.z;
    const R invLen = 1.0 / sqrt(lenSq);
    D3 n = scl(axis, invLen);
    if (dt3(n, delta) < 0) n = neg(n);
    return n;
  }
  // collide.js:612-685
  __device__ int collide(R *basis) {
    if (A.sphere && B.sphere) return sphereSphere(basis);
    if (A.sphere || B.sphere) return sphereBox(basis, A.sphere);
    makeOBB(boxA, A);
    makeOBB(boxB, B);
    const D3 delta = sub(boxB.c, boxA.c);
    Sat bf, be;
    bf.sep = -INFINITY; bf.valid = false; bf.type = 0; bf.ia = bf.ib = -1; bf.n = D3{R(0), R(0), R(0)};
    be = bf;
    for (int i = 0; i < 3; i++)
      if (!testAxis(delta, boxA.ax[i], kFaceA, i, -1, bf)) return 0;
    for (int i = 0; i < 3; i++)
      if (!testAxis(delta, boxB.ax[i], kFaceB, -1, i, bf)) return 0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        if (!testAxis(delta, crs(boxA.ax[i], boxB.ax[j]), kEdge, i, j, be)) return 0;
    if (!bf.valid) return 0;
    Sat best = bf;
    if (be.valid && 0.95 * be.sep > bf.sep + 0.01) best = be;
    orthonormal(basis, neg(best.n));
    if (best.type == kEdge) return edgeContact(best.ia, best.ib, best.n);
    if (best.type == kFaceA) return faceManifold(true, best.ia, best.n);
    return faceManifold(false, best.ib, best.n);
  }
};

}  // namespace geo
}  // namespace avbd
