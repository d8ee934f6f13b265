// clip.cuh — per-element-pair contact polygons (device).
//
// The three contact-surface queries of the reference (Drake's
// ComputeContactSurfaceFromSoftVolumeRigidSurface, ...RigidHalfSpace and
// ...CompliantVolumes, called at mujoco_contact_surfaces_plugin.cpp:284-303)
// restated for one element pair at a time, from the published hydroelastic
// method (Elandt et al. 2019; Masterjohn et al. 2021):
//   soft-rigid : polygon = rigid triangle ∩ soft tet.  Computed as the tet's
//                section by the triangle's plane, clipped by the triangle's
//                three in-plane edge planes.
//   half-space : polygon = the tet's section by the plane z = 0 of the
//                plane geom.
//   soft-soft  : polygon = equal-pressure plane ∩ tet A ∩ tet B: tet A's
//                section by p_A - p_B = 0, clipped by tet B's four faces.
// Faces whose normal makes an angle above 5*pi/8 with the soft pressure
// gradient are culled (the method's back-face test).
//
// Precision: every sign decision is first taken in FP32 with a conservative
// error margin.  When any FP32 value falls inside its margin the whole
// element pair is recomputed in FP64 from the stored FP32 inputs and the
// FP64 frames, so decisions equal an FP64 evaluation.  In FP64 a value
// within 1e-12 (metres, or cosine units for the normal test) of its
// threshold marks the pair near-degenerate.
#pragma once
#include "geom_math.cuh"
#include "hc_internal.h"

namespace hc {

constexpr float kFilt = 3.0e-6f;            // FP32 margin factor (~50 ulp)
constexpr double kNearTol = 1.0e-12;        // near-degenerate threshold
constexpr float kCosAlphaF = -0.38268343236508978f;   // cos(5*pi/8)
constexpr double kCosAlphaD = -0.38268343236508978;

// Polygon vertex: position, pressure, and a bound on its position error
// (metres; FP32 pass only).
template <class R>
struct PVx {
  R x, y, z, p, e;
};

template <class R>
__device__ __forceinline__ PVx<R> pv_lerp(const PVx<R>& a, const PVx<R>& b, R t) {
  PVx<R> o;
  o.x = a.x + t * (b.x - a.x);
  o.y = a.y + t * (b.y - a.y);
  o.z = a.z + t * (b.z - a.z);
  o.p = a.p + t * (b.p - a.p);
  o.e = a.e > b.e ? a.e : b.e;
  return o;
}

template <class R>
__device__ __forceinline__ V3<R> pv_pos(const PVx<R>& a) { return mk(a.x, a.y, a.z); }

// Uncertainty bookkeeping: FP32 passes set `unc` when a decision is inside
// its margin; FP64 passes set `near` when a value is within kNearTol.
struct Decide {
  bool unc = false;
  bool near = false;
};

template <class R>
__device__ __forceinline__ void check(Decide& dc, R v, R tol) {
  if (sizeof(R) == 4) {
    if (abs_r(v) <= tol) dc.unc = true;
  } else {
    if (abs_r(v) < (R)kNearTol) dc.near = true;
  }
}

// Section of tet (vertices tv[0..3], values s[0..3]) by s = 0.  Output is a
// triangle or quad in cyclic order (marching-tetrahedron pattern).
// tol_s: margin of the s values (FP32 only).
template <class R>
__device__ __forceinline__ int tet_section(const PVx<R> tv[4], const R s[4], R tol_s, Decide& dc,
                                           PVx<R> out[kMaxPolyV]) {
  int pos = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    check(dc, s[k], tol_s);
    pos |= (s[k] > (R)0) << k;
  }
  int np = __popc(pos);
  if (np == 0 || np == 4) return 0;
  int ea[4], eb[4], n;
  if (np == 1 || np == 3) {
    int single = np == 1 ? __ffs(pos) - 1 : __ffs(~pos & 0xF) - 1;
    n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k != single) { ea[n] = single; eb[n] = k; ++n; }
    n = 3;
  } else {
    int a = __ffs(pos) - 1, b = __ffs(pos & ~(1 << a)) - 1;
    int neg = ~pos & 0xF;
    int c = __ffs(neg) - 1, d = __ffs(neg & ~(1 << c)) - 1;
    ea[0] = a; eb[0] = c;
    ea[1] = a; eb[1] = d;
    ea[2] = b; eb[2] = d;
    ea[3] = b; eb[3] = c;
    n = 4;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i < n) {
      const int a = ea[i], b = eb[i];
      R sa = s[a], sb = s[b];
      R t = sa / (sa - sb);
      out[i] = pv_lerp(tv[a], tv[b], t);
      if (sizeof(R) == 4) {
        V3<R> d = pv_pos(tv[b]) - pv_pos(tv[a]);
        out[i].e = amax(d) * ((R)2 * tol_s / abs_r(sa - sb) + (R)4e-7) + (tv[a].e > tv[b].e ? tv[a].e : tv[b].e);
      }
    }
  }
  return n;
}

// Sutherland-Hodgman clip of a convex polygon by n.x - o >= 0.
// tol_p: margin of the plane evaluation itself (FP32 only).
template <class R>
__device__ __forceinline__ int clip_plane(const PVx<R>* in, int n, V3<R> pn, R po, R tol_p, Decide& dc,
                                          PVx<R>* out) {
  R d[kMaxPolyV];
  bool all_in = true;
  for (int i = 0; i < n; ++i) {
    d[i] = dot(pn, pv_pos(in[i])) - po;
    R tol = tol_p + (R)2 * in[i].e;
    check(dc, d[i], tol);
    all_in &= d[i] >= (R)0;
  }
  if (all_in) {
    for (int i = 0; i < n; ++i) out[i] = in[i];
    return n;
  }
  int m = 0;
  for (int i = 0; i < n; ++i) {
    int j = i + 1 == n ? 0 : i + 1;
    bool ii = d[i] >= (R)0, ij = d[j] >= (R)0;
    if (ii && m < kMaxPolyV) out[m++] = in[i];
    if (ii != ij && m < kMaxPolyV) {
      R t = d[i] / (d[i] - d[j]);
      PVx<R> v = pv_lerp(in[i], in[j], t);
      if (sizeof(R) == 4) {
        V3<R> dd = pv_pos(in[j]) - pv_pos(in[i]);
        R ti = tol_p + (R)2 * in[i].e, tj = tol_p + (R)2 * in[j].e;
        v.e = (in[i].e > in[j].e ? in[i].e : in[j].e) + amax(dd) * ((ti + tj) / abs_r(d[i] - d[j]) + (R)4e-7);
      }
      out[m++] = v;
    }
  }
  return m;
}

// Linear field of a tet from its vertex values: p(x) = g.x + c.  Also the
// tet's minimum height (for conditioning-based margins).
template <class R>
__device__ __forceinline__ void tet_field(const V3<R> X[4], const R P[4], V3<R>& g, R& c, R& hmin) {
  V3<R> e1 = X[1] - X[0], e2 = X[2] - X[0], e3 = X[3] - X[0];
  V3<R> c23 = cross(e2, e3), c31 = cross(e3, e1), c12 = cross(e1, e2);
  R det = dot(e1, c23);
  R d1 = P[1] - P[0], d2 = P[2] - P[0], d3 = P[3] - P[0];
  if (det == (R)0) {
    g = mk<R>(0, 0, 0);
    c = P[0];
    hmin = 0;
    return;
  }
  R inv = (R)1 / det;
  g = (c23 * d1 + c31 * d2 + c12 * d3) * inv;
  c = P[0] - dot(g, X[0]);
  // face areas*2: |c23| (face opposite 0), |c31|, |c12|, |(e2-e1)x(e3-e1)|
  V3<R> f0 = cross(e2 - e1, e3 - e1);
  R amax_ = norm(c23);
  R t1 = norm(c31), t2 = norm(c12), t3 = norm(f0);
  amax_ = amax_ > t1 ? amax_ : t1;
  amax_ = amax_ > t2 ? amax_ : t2;
  amax_ = amax_ > t3 ? amax_ : t3;
  hmin = abs_r(det) / amax_;
}

// Inward unit face planes of a tet; face k is opposite vertex k.
template <class R>
__device__ __forceinline__ void tet_planes(const V3<R> X[4], V3<R> n[4], R o[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i0 = k == 0 ? 1 : 0;
    const int i1 = k <= 1 ? 2 : 1;
    const int i2 = k <= 2 ? 3 : 2;
    V3<R> nn = cross(X[i1] - X[i0], X[i2] - X[i0]);
    if (dot(nn, X[k] - X[i0]) < (R)0) nn = nn * (R)-1;
    R l = norm(nn);
    nn = l > (R)0 ? nn * ((R)1 / l) : nn;
    n[k] = nn;
    o[k] = dot(nn, X[i0]);
  }
}

}  // namespace hc
