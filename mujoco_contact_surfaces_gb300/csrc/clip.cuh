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
// Precision.  The section function values s_k of the four tet vertices
// (signed distance to the triangle plane / plane, or p_A - p_B) are
// evaluated in FP64: they set the penetration, to which area and force are
// most sensitive.  Section vertices are interpolated from the edge endpoint
// nearest the plane and kept in coordinates relative to the tet vertex
// nearest the plane, so FP32 carries only the small offsets.  Clip-plane
// distances are carried per vertex and interpolated with the positions.
// Every FP32 sign decision has a conservative margin; when a value falls
// inside it the element pair is recomputed in FP64 from the stored FP32
// inputs and the FP64 frames, so decisions equal an FP64 evaluation.  In
// FP64 a value within 1e-12 (metres, or cosine units for the normal test)
// of its threshold marks the pair near-degenerate.
#pragma once
#include "geom_math.cuh"
#include "hc_internal.h"

namespace hc {

constexpr float kFilt = 3.0e-6f;            // FP32 margin factor (~50 ulp)
constexpr float kFiltRel = 1.0e-6f;         // margin of interpolated values
constexpr double kNearTol = 1.0e-12;        // near-degenerate threshold
constexpr double kCosAlphaD = -0.38268343236508978;   // cos(5*pi/8)

// Polygon vertex: position (relative to an anchor), pressure, the
// distances to up to ND clip planes, and the two constraints the vertex lies
// on besides the section plane (lab = c0 | c1 << 4; 0-3: the tet face
// opposite vertex k, 4 + j: clip plane j).  The adjoint differentiates each
// vertex as the intersection of those three planes.
template <class R, int ND>
struct PV {
  R x, y, z, p;
  R d[ND];
  int lab;
};
// A vertex without carried distances (the FP32 soft-rigid polygon: each
// clip plane's distance is evaluated from the position when it is needed).
template <class R>
struct PV<R, 0> {
  R x, y, z, p;
  int lab;
};

template <class R, int ND>
__device__ __forceinline__ PV<R, ND> pv_lerp(const PV<R, ND>& a, const PV<R, ND>& b, R t) {
  PV<R, ND> o;
  o.x = a.x + t * (b.x - a.x);
  o.y = a.y + t * (b.y - a.y);
  o.z = a.z + t * (b.z - a.z);
  o.p = a.p + t * (b.p - a.p);
  if constexpr (ND > 0) {
#pragma unroll
    for (int j = 0; j < ND; ++j) o.d[j] = a.d[j] + t * (b.d[j] - a.d[j]);
  }
  o.lab = a.lab;
  return o;
}

// The constraint shared by two consecutive vertices (the polygon edge's).
__device__ __forceinline__ int shared_label(int la, int lb) {
  const int a0 = la & 15, a1 = la >> 4, b0 = lb & 15, b1 = lb >> 4;
  return (a0 == b0 || a0 == b1) ? a0 : a1;
}

template <class R, int ND>
__device__ __forceinline__ V3<R> pv_pos(const PV<R, ND>& a) { return mk(a.x, a.y, a.z); }

// v[i] for a lane-varying i in 0..3 with static indices only, so that a
// four-entry array stays in registers (the values are those of v[i]).
template <class T>
__device__ __forceinline__ T sel4(const T v[4], int i) {
  T r = v[0];
  r = i == 1 ? v[1] : r;
  r = i == 2 ? v[2] : r;
  r = i == 3 ? v[3] : r;
  return r;
}

// FP32 passes set `unc` when a decision is inside its margin; FP64 passes
// set `near` when a value is within kNearTol.
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

// a - b and (a x b) . u with every product and sum rounded on its own.
__device__ __forceinline__ V3<float> sub_rn(V3<float> a, V3<float> b) {
  return mk(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float winding_rn(V3<float> a, V3<float> b, V3<float> u) {
  const float cx = __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y));
  const float cy = __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z));
  const float cz = __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x));
  return __fadd_rn(__fadd_rn(__fmul_rn(cx, u.x), __fmul_rn(cy, u.y)), __fmul_rn(cz, u.z));
}

// Sign patterns (bit k: s_k > 0) whose marching-tetrahedron section below
// winds clockwise about grad s in a positively oriented tet, whose
// (X1 - X0) . ((X2 - X0) x (X3 - X0)) > 0; a negatively oriented tet winds
// every pattern the other way.
constexpr unsigned kSectionCw = 0x32DAu;   // patterns 1, 3, 4, 6, 7, 9, 12, 13

// Section of a tet by s = 0 (s for the four vertices: FP64, or the FP32 head
// of a double-float value, whose sign it has whenever it is not near zero).
// Output: triangle or quad in cyclic order (marching-tetrahedron pattern),
// each vertex interpolated from the endpoint with the smaller |s|.  In FP32
// the order is counter-clockwise about grad s (the contact plane's normal),
// as the reference's contact polygons wind: the pattern's winding, from
// kSectionCw and the tet's parity, decides whether the vertices after the
// first are stored in reverse, and clipping keeps the winding.  The FP64
// fallbacks leave the marching order; orient_ccw winds their results.
template <class R, int ND, class S>
__device__ __forceinline__ int tet_section(const PV<R, ND> tv[4], const S s[4], Decide& dc, PV<R, ND> out[4]) {
  int pos = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (abs_r(s[k]) < (S)kNearTol) {
      if (sizeof(R) == 4) dc.unc = true;
      else dc.near = true;
    }
    pos |= (s[k] > (S)0) << k;
  }
  const int np = __popc(pos);
  if (np == 0 || np == 4) return 0;
  bool rev = false;
  if constexpr (sizeof(R) == 4) {
    // the tet's parity from its anchored vertices, each operation rounded
    // on its own so that every kernel decides alike
    const V3<float> x0 = pv_pos(tv[0]);
    const float det = winding_rn(sub_rn(pv_pos(tv[2]), x0), sub_rn(pv_pos(tv[3]), x0), sub_rn(pv_pos(tv[1]), x0));
    rev = (((kSectionCw >> pos) & 1u) != 0u) != (det < 0.f);
  }
  int ea[4], eb[4], n;
  if (np == 1 || np == 3) {
    const int single = np == 1 ? __ffs(pos) - 1 : __ffs(~pos & 0xF) - 1;
    n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k != single) { ea[n] = single; eb[n] = k; ++n; }
  } else {
    const int a = __ffs(pos) - 1, b = __ffs(pos & ~(1 << a)) - 1;
    const int neg = ~pos & 0xF;
    const int c = __ffs(neg) - 1, d = __ffs(neg & ~(1 << c)) - 1;
    ea[0] = a; eb[0] = c;
    ea[1] = a; eb[1] = d;
    ea[2] = b; eb[2] = d;
    ea[3] = b; eb[3] = c;
    n = 4;
  }
  // (loops here are not unrolled: the narrow kernels inline this code in
  // several places and are bound by instruction fetch, not arithmetic)
#pragma unroll 1
  for (int i = 0; i < 4; ++i) {
    if (i < n) {
      int a = ea[i], b = eb[i];
      // the tet edge (a, b) lies on the faces opposite the two other vertices
      const int other = 0xF & ~((1 << a) | (1 << b));
      const int c = __ffs(other) - 1, d = __ffs(other & ~(1 << c)) - 1;
      S s_a = sel4(s, a), s_b = sel4(s, b);
      if (abs_r(s_a) > abs_r(s_b)) {
        int t = a; a = b; b = t;
        S u = s_a; s_a = s_b; s_b = u;
      }
      const PV<R, ND> va = sel4(tv, a), vb = sel4(tv, b);
      const R sa = (R)s_a, sb = (R)s_b;
      PV<R, ND>& o = out[rev && i > 0 ? n - i : i];
      o = pv_lerp(va, vb, sa / (sa - sb));
      if (sizeof(S) == 8 && sizeof(R) == 4) {
        // FP64 section values: the pressure there in FP64 too.  The tet's
        // vertex pressures are of the order of E while a contact near first
        // touch sees pressures thousands of times smaller; interpolated in
        // FP32 those would keep only a few digits.
        const double ta = (double)s_a / ((double)s_a - (double)s_b);
        o.p = (R)((double)va.p + ta * ((double)vb.p - (double)va.p));
      }
      o.lab = c | (d << 4);
    }
  }
  return n;
}

// Sutherland-Hodgman clip of a convex polygon by d_j >= 0 (carried
// distances), in place.  A convex polygon crosses a plane at most twice, so
// the output never runs more than one vertex ahead of the input: the write
// index m stays at most i + 1 while vertex i is processed, and at m = i + 1
// vertex i is outside (writes only the crossing, at i + 1).  Each next
// vertex is read before the writes of its turn, and the first vertex is kept
// aside for the closing edge, so no vertex is overwritten before it is read.
// The arithmetic is that of a clip into a second array.  Rounding can give
// a sign pattern with more than two changes (every vertex within noise of
// the plane); that polygon is clipped through a copy.  n >= 1.  tol: FP32
// margin of the plane distances.
template <class R, int ND>
__device__ __forceinline__ int clip_step(const PV<R, ND>& a, const PV<R, ND>& b, int j, PV<R, ND>* out, int m) {
  const R di = a.d[j], dk = b.d[j];
  const bool ii = di >= (R)0, ik = dk >= (R)0;
  if (ii && m < kMaxPolyV) out[m++] = a;
  if (ii != ik && m < kMaxPolyV) {
    out[m] = abs_r(di) <= abs_r(dk) ? pv_lerp(a, b, di / (di - dk)) : pv_lerp(b, a, dk / (dk - di));
    out[m].lab = shared_label(a.lab, b.lab) | ((4 + j) << 4);
    ++m;
  }
  return m;
}

// The same clip through a copy of the input: for sign patterns with more
// than two changes around the polygon (rounding, every vertex within noise
// of the plane), where clipping in place could overwrite an unread vertex.
template <class R, int ND>
__device__ __noinline__ int clip_dist_copy(PV<R, ND>* p, int n, int j) {
  PV<R, ND> in[kMaxPolyV];
  for (int i = 0; i < n; ++i) in[i] = p[i];
  int m = 0;
  for (int i = 0; i < n; ++i) m = clip_step(in[i], in[i + 1 == n ? 0 : i + 1], j, p, m);
  return m;
}

template <class R, int ND>
__device__ __forceinline__ int clip_dist(PV<R, ND>* p, int n, int j, R tol, Decide& dc) {
  bool all_in = true;
  int changes = 0;
  bool prev = p[n - 1].d[j] >= (R)0;
  for (int i = 0; i < n; ++i) {
    check(dc, p[i].d[j], tol);
    const bool in = p[i].d[j] >= (R)0;
    all_in &= in;
    changes += in != prev;
    prev = in;
  }
  if (all_in) return n;
  if (changes > 2) return clip_dist_copy(p, n, j);
  const PV<R, ND> first = p[0];
  PV<R, ND> cur = first;
  int m = 0;
  for (int i = 0; i < n; ++i) {
    const PV<R, ND> nxt = i + 1 < n ? p[i + 1] : first;
    m = clip_step(cur, nxt, j, p, m);
    cur = nxt;
  }
  return m;
}

// Signed distance of a vertex to the plane e.x + c = 0 (x relative to the
// polygon's anchor; c: the plane's value at the anchor).
__device__ __forceinline__ float pos_dist(const PV<float, 0>& v, const float* e, float c) {
  return fmaf(e[2], v.z, fmaf(e[1], v.y, fmaf(e[0], v.x, c)));
}

__device__ __forceinline__ int clip_step_pos(const PV<float, 0>& a, const PV<float, 0>& b, float da, float db, int j,
                                             PV<float, 0>* out, int m) {
  const bool ii = da >= 0.f, ik = db >= 0.f;
  if (ii && m < kMaxPolyV) out[m++] = a;
  if (ii != ik && m < kMaxPolyV) {
    out[m] = fabsf(da) <= fabsf(db) ? pv_lerp(a, b, da / (da - db)) : pv_lerp(b, a, db / (db - da));
    out[m].lab = shared_label(a.lab, b.lab) | ((4 + j) << 4);
    ++m;
  }
  return m;
}

__device__ __noinline__ int clip_pos_copy(PV<float, 0>* p, int n, int j, const float* e, float c) {
  PV<float, 0> in[kMaxPolyV];
  for (int i = 0; i < n; ++i) in[i] = p[i];
  int m = 0;
  for (int i = 0; i < n; ++i) {
    const PV<float, 0>& b = in[i + 1 == n ? 0 : i + 1];
    m = clip_step_pos(in[i], b, pos_dist(in[i], e, c), pos_dist(b, e, c), j, p, m);
  }
  return m;
}

// clip_dist for vertices without carried distances: the distance to clip
// plane j is e.x + c from each vertex's position, in place as clip_dist.
__device__ __forceinline__ int clip_pos(PV<float, 0>* p, int n, int j, const float* e, float c, float tol,
                                        Decide& dc) {
  bool all_in = true;
  int changes = 0;
  bool prev = pos_dist(p[n - 1], e, c) >= 0.f;
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    const float d = pos_dist(p[i], e, c);
    check(dc, d, tol);
    const bool in = d >= 0.f;
    all_in &= in;
    changes += in != prev;
    prev = in;
  }
  if (all_in) return n;
  if (changes > 2) return clip_pos_copy(p, n, j, e, c);
  const PV<float, 0> first = p[0];
  const float d_first = pos_dist(first, e, c);
  PV<float, 0> cur = first;
  float d_cur = d_first;
  int m = 0;
#pragma unroll 1
  for (int i = 0; i < n; ++i) {
    const PV<float, 0> nxt = i + 1 < n ? p[i + 1] : first;
    const float d_nxt = i + 1 < n ? pos_dist(nxt, e, c) : d_first;
    m = clip_step_pos(cur, nxt, d_cur, d_nxt, j, p, m);
    cur = nxt;
    d_cur = d_nxt;
  }
  return m;
}

// Winds a finished polygon counter-clockwise about `up` (the direction in
// which the section value grows: the contact plane's normal), as the
// reference's contact polygons are wound: when the fan area vector from the
// first vertex points against up, the order is reversed (first vertex
// kept).  Applied to the FP64 fallbacks' polygons (the FP32 section is
// wound by tet_section).  Each product and sum is rounded on its own, so
// every kernel that builds the polygon decides the same way on a sliver
// whose area is near zero.
template <int ND>
__device__ __forceinline__ void orient_ccw(PV<float, ND>* p, int nv, V3<float> up) {
  if (nv < 3) return;
  float w = 0.f;
  const float x0 = p[0].x, y0 = p[0].y, z0 = p[0].z;
  float ax = __fsub_rn(p[1].x, x0), ay = __fsub_rn(p[1].y, y0), az = __fsub_rn(p[1].z, z0);
  for (int i = 2; i < nv; ++i) {
    const float bx = __fsub_rn(p[i].x, x0), by = __fsub_rn(p[i].y, y0), bz = __fsub_rn(p[i].z, z0);
    const float cx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    const float cy = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    const float cz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    w = __fadd_rn(w, __fadd_rn(__fadd_rn(__fmul_rn(cx, up.x), __fmul_rn(cy, up.y)), __fmul_rn(cz, up.z)));
    ax = bx; ay = by; az = bz;
  }
  if (w < 0.f) {
    for (int i = 1, k = nv - 1; i < k; ++i, --k) {
      const PV<float, ND> tmp = p[i];
      p[i] = p[k];
      p[k] = tmp;
    }
  }
}

// Linear field of a tet from its vertex values: p(x) = g.x + c; also the
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

// FP64 signed value n.x - o of a float point.
__device__ __forceinline__ double plane64(const double* n, double o, float x, float y, float z) {
  return fma(n[2], (double)z, fma(n[1], (double)y, n[0] * (double)x)) - o;
}

}  // namespace hc
