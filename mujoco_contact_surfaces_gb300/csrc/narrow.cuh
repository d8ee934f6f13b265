// narrow.cuh — the narrow-phase kernel (included by contact.cu inside
// namespace hc).
//
// One warp per work item (soft leaf cluster x other cluster), items taken
// from a global counter.  The other cluster's 32 elements are staged in
// shared memory in the soft frame (with FP64 planes / fields); each lane
// owns one soft tet and walks the staged elements.  Per non-empty polygon:
// centroid quadrature (mujoco_contact_surfaces_plugin.cpp:320-409),
// Hunt-Crossley damping and regularised friction, and the
// flat-sensor ray binning (flat_tactile_sensor.cpp:316-392).  The warp's
// sums are reduced in FP64 in a fixed order.

struct Acc {
  float F[3], T[3], area, fn0;
  int n_poly, n_faces, n_near;
};

struct PairCtx {
  const PairDev* P;
  const FrameDev* F;
  int pair;
};

// One quadrature point and the force law, soft frame.
__device__ __forceinline__ void point_force(Acc& ac, const FrameDev& F, float damping, float mu, int apply, float A,
                                            V3<float> p, V3<float> n, float gM, float gN, float p0) {
  if (!(A > 1.0e-14f)) return;
  if (gM < 1.0e-14f || gN < 1.0e-14f) return;
  const float g = 1.0f / (1.0f / gM + 1.0f / gN);
  const float fn0 = A * p0;
  const float k = A * g;
  ac.area += A;
  ac.fn0 += fn0;
  ac.n_faces += 1;
  const V3<float> lin = mk(F.lin[0], F.lin[1], F.lin[2]), ang = mk(F.ang[0], F.ang[1], F.ang[2]);
  const V3<float> v = lin + cross(ang, p);
  const float vn = dot(v, n);
  const float fn = fmaxf(0.f, 1.f - damping * vn) * (fn0 - 0.001f * k * vn);
  if (!apply) return;
  const V3<float> vt = v - n * vn;
  const float eps = (1.0e-4f * 1.0e-2f) * (1.0e-4f * 1.0e-2f);
  const float v_slip = sqrtf(dot(vt, vt) + eps);
  const float s = v_slip / 1.0e-4f;
  const float mu_reg = s < 1.f ? mu * s * (2.f - s) : mu;
  const V3<float> f = vt * (-mu_reg * fn / v_slip) + n * fn;
  const V3<float> tq = cross(p, f);
  ac.F[0] += f.x; ac.F[1] += f.y; ac.F[2] += f.z;
  ac.T[0] += tq.x; ac.T[1] += tq.y; ac.T[2] += tq.z;
}

// Ray hits of one fan triangle (soft frame) on a sensor's sample grid.  The
// sensor's rays are parallel to its -z axis, start 1.5*zs (+1e-8) above its
// centre and accept 0 < t < 1.5*zs (flat_tactile_sensor.cpp:324-346); the
// triangle test follows the acceptance rules of the Moeller-Trumbore test in
// bvh.cpp:49-74 (|det| < 1e-10 rejects, u in [0,1], v >= 0, u+v <= 1), here
// in the sensor frame.  Each sample keeps the smallest t, packed with the
// pressure at the hit, by a 64-bit atomicMin (order independent).
__device__ void raster_tri(const StepArgs& a, int sid, const float* Rl, const float* tl, V3<float> A, V3<float> B,
                           V3<float> C, float pa, float pb, float pc) {
  const SensorDev S = a.sensors[sid];
  const V3<float> T = mk(tl[0], tl[1], tl[2]);
  const V3<float> la = mat_mul<float>(Rl, A) + T, lb = mat_mul<float>(Rl, B) + T, lc = mat_mul<float>(Rl, C) + T;
  const float e1x = lb.x - la.x, e1y = lb.y - la.y, e2x = lc.x - la.x, e2y = lc.y - la.y;
  const float det = e1x * e2y - e1y * e2x;
  if (fabsf(det) < 1e-10f) return;
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  const float x0 = sx[0], dx = S.nx > 1 ? sx[1] - sx[0] : 1.f;
  const float y0 = sy[0], dy = S.ny > 1 ? sy[1] - sy[0] : 1.f;
  const float mnx = fminf(la.x, fminf(lb.x, lc.x)), mxx = fmaxf(la.x, fmaxf(lb.x, lc.x));
  const float mny = fminf(la.y, fminf(lb.y, lc.y)), mxy = fmaxf(la.y, fmaxf(lb.y, lc.y));
  const float fx0 = floorf((mnx - x0) / dx) - 1.f, fx1 = ceilf((mxx - x0) / dx) + 1.f;
  const float fy0 = floorf((mny - y0) / dy) - 1.f, fy1 = ceilf((mxy - y0) / dy) + 1.f;
  if (!(fx1 >= 0.f && fy1 >= 0.f && fx0 <= (float)(S.nx - 1) && fy0 <= (float)(S.ny - 1))) return;
  const int X0 = max(0, (int)fx0), X1 = min(S.nx - 1, (int)fx1);
  const int Y0 = max(0, (int)fy0), Y1 = min(S.ny - 1, (int)fy1);
  const float inv = 1.f / det;
  unsigned long long* smp = a.samples + S.sample_off;
  for (int X = X0; X <= X1; ++X) {
    const float wx = sx[X] - la.x;
    for (int Y = Y0; Y <= Y1; ++Y) {
      const float wy = sy[Y] - la.y;
      const float u = (wx * e2y - wy * e2x) * inv;
      if (u < 0.f || u > 1.f) continue;
      const float v = (e1x * wy - e1y * wx) * inv;
      if (v < 0.f || u + v > 1.f) continue;
      const float z = la.z + u * (lb.z - la.z) + v * (lc.z - la.z);
      const float t = (S.zs15 + 1e-8f) - z;
      if (!(t > 0.f && t < S.zs15)) continue;
      const float pr = (1.f - u - v) * pa + u * pb + v * pc;
      const unsigned long long key =
          ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)__float_as_uint(pr);
      atomicMin(&smp[(size_t)X * S.ny + Y], key);
    }
  }
}

// Quadrature of one polygon (vertices relative to `anc`, soft frame) and its
// contribution to forces and sensors.  n: contact normal out of N into M.
template <int ND>
__device__ void integrate_polygon(const StepArgs& a, const PairCtx& pc, Acc& ac, const PV<float, ND>* v, int nv,
                                  V3<float> anc, V3<float> n, float gM, float gN) {
  const FrameDev& F = *pc.F;
  const PairDev& P = *pc.P;
  // area-weighted centroid by a fan from vertex 0 (local coordinates)
  float A = 0.f, pcen = 0.f;
  V3<float> c = mk(0.f, 0.f, 0.f);
  const V3<float> v0 = pv_pos(v[0]);
  for (int i = 1; i + 1 < nv; ++i) {
    const V3<float> vi = pv_pos(v[i]), vj = pv_pos(v[i + 1]);
    const float ai = 0.5f * dot(cross(vi - v0, vj - v0), n);
    A += ai;
    c = c + (v0 + vi + vj) * (ai * (1.f / 3.f));
    pcen += ai * (v[0].p + v[i].p + v[i + 1].p) * (1.f / 3.f);
  }
  if (A != 0.f) {
    c = c * (1.f / A);
    pcen /= A;
  } else {
    c = mk(0.f, 0.f, 0.f);
    pcen = 0.f;
    for (int i = 0; i < nv; ++i) {
      c = c + pv_pos(v[i]) * (1.f / nv);
      pcen += v[i].p / nv;
    }
  }
  if (a.repr == 1) {
    point_force(ac, F, P.damping, P.mu, a.apply_forces, fabsf(A), anc + c, n, gM, gN, pcen);
  } else {
    for (int i = 0; i < nv; ++i) {
      const int j = i + 1 == nv ? 0 : i + 1;
      const V3<float> vi = pv_pos(v[i]), vj = pv_pos(v[j]);
      const float Ai = 0.5f * norm(cross(vi - c, vj - c));
      const V3<float> cen = anc + (c + vi + vj) * (1.f / 3.f);
      const float p0 = pcen / 3.f + v[i].p / 3.f + v[j].p / 3.f;
      point_force(ac, F, P.damping, P.mu, a.apply_forces, Ai, cen, n, gM, gN, p0);
    }
  }
  for (int q = 0; q < 2; ++q) {
    const int sid = q == 0 ? P.sensor0 : P.sensor1;
    if (sid < 0) continue;
    const float* Rl = q == 0 ? F.Rl : F.Rl1;
    const float* tl = q == 0 ? F.tl : F.tl1;
    const V3<float> ca = anc + c;
    for (int i = 0; i < nv; ++i) {
      const int j = i + 1 == nv ? 0 : i + 1;
      raster_tri(a, sid, Rl, tl, anc + pv_pos(v[i]), anc + pv_pos(v[j]), ca, v[i].p, v[j].p, pcen);
    }
  }
}

template <int ND>
__device__ void record(const StepArgs& a, const PairCtx& pc, const PV<float, ND>* v, int nv, V3<float> anc,
                       V3<float> n, int ea, int eb, int flags) {
  if (a.debug & 1) {
    const int k = atomicAdd(a.cand_count, 1);
    if (k < a.cand_cap) {
      CandRec r;
      r.pair = pc.pair; r.elem_a = ea; r.elem_b = eb; r.n_vert = nv; r.flags = flags;
      a.cand[k] = r;
    } else {
      atomicOr(a.status, 2);
    }
  }
  if (a.want_polys && (a.want_pair < 0 || a.want_pair == pc.pair)) {
    const int k = atomicAdd(a.poly_count, 1);
    if (k < a.poly_cap) {
      PolyRec& r = a.polys[k];
      r.pair = pc.pair; r.elem_a = ea; r.elem_b = eb; r.nv = nv;
      r.n[0] = n.x; r.n[1] = n.y; r.n[2] = n.z; r.n[3] = 0.f;
      for (int i = 0; i < kMaxPolyV; ++i) {
        const bool in = i < nv;
        r.v[i][0] = in ? anc.x + v[i].x : 0.f;
        r.v[i][1] = in ? anc.y + v[i].y : 0.f;
        r.v[i][2] = in ? anc.z + v[i].z : 0.f;
        r.v[i][3] = in ? v[i].p : 0.f;
      }
    } else {
      atomicOr(a.status, 4);
    }
  }
}

// ---- element data -----------------------------------------------------------
template <class R>
struct TetIn {
  V3<R> X[4];
  R P[4];
  V3<R> g;
  R c, gl, hmin, kappa, xmax, pmax;
};

template <class R>
__device__ __forceinline__ void tet_prepare(TetIn<R>& t) {
  tet_field(t.X, t.P, t.g, t.c, t.hmin);
  t.gl = norm(t.g);
  R lmax = 0, xm = 0, pm = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    xm = fmax(xm, amax(t.X[i]));
    pm = fmax(pm, abs_r(t.P[i]));
#pragma unroll
    for (int j = i + 1; j < 4; ++j) lmax = fmax(lmax, norm(t.X[j] - t.X[i]));
  }
  t.xmax = xm;
  t.pmax = pm;
  t.kappa = t.hmin > (R)0 ? lmax / t.hmin : (R)1e30;
}

template <class R>
__device__ __forceinline__ void load_tet(const float4* tets, int idx, TetIn<R>& t) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 v = tets[4 * (size_t)idx + k];
    t.X[k] = mk<R>(v.x, v.y, v.z);
    t.P[k] = v.w;
  }
}

// Index of the tet vertex nearest the section plane.
__device__ __forceinline__ int nearest_vertex(const double s[4]) {
  int k = 0;
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (fabs(s[i]) < fabs(s[k])) k = i;
  return k;
}

template <class R, int ND>
__device__ __forceinline__ void tet_local(const TetIn<R>& t, int anc, PV<R, ND> tv[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    tv[k].x = t.X[k].x - t.X[anc].x;
    tv[k].y = t.X[k].y - t.X[anc].y;
    tv[k].z = t.X[k].z - t.X[anc].z;
    tv[k].p = t.P[k];
  }
}

// Rigid triangle in the soft frame.
struct TriData {
  double n64[3], o64;  // FP64 plane (unit normal, offset)
  float Y[3][3];       // vertices
  float n[3];          // unit normal (out of the rigid body)
  float en[3][3];      // in-plane inward edge normals
  float eo[3];
  float lo[3], hi[3];
  float M, h, Lt;      // coordinate magnitude, min altitude, max edge
  int orig;
  int valid;
};

template <class R>
__device__ __forceinline__ void tri_planes(const V3<R> Y[3], V3<R>& n, R& o, V3<R> en[3], R eo[3], R& h, R& Lt,
                                           bool& valid) {
  const V3<R> N = cross(Y[1] - Y[0], Y[2] - Y[0]);
  const R ln = norm(N);
  valid = ln > (R)0;
  n = valid ? N * ((R)1 / ln) : mk<R>(0, 0, 1);
  o = dot(n, Y[0]);
  R le = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const V3<R> e = Y[j == 2 ? 0 : j + 1] - Y[j];
    le = fmax(le, norm(e));
    const V3<R> m = cross(n, e);
    const R lm = norm(m);
    en[j] = lm > (R)0 ? m * ((R)1 / lm) : m;
    eo[j] = dot(en[j], Y[j]);
  }
  Lt = le;
  h = le > (R)0 ? ln / le : (R)0;
}

// FP64 triangle in the soft frame from its stored rigid-frame vertices.
__device__ __forceinline__ void tri_fp64(const StepArgs& a, const FrameDev& F, int idx, V3<double> Y[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 r = a.tris[3 * (size_t)idx + k];
    Y[k] = mat_mul<double>(F.R, mk<double>(r.x, r.y, r.z)) + mk(F.t[0], F.t[1], F.t[2]);
  }
}

// Soft-rigid polygon: tet section by the triangle plane (FP64 values s),
// clipped by the three edge planes.
template <class R>
__device__ int sr_polygon(const TetIn<R>& t, const double s[4], V3<R> n, const V3<R> en[3], const R eo[3], R M,
                          R h, R Lt, Decide& dc, int& anc, PV<R, 3>* out, PV<R, 3>* tmp) {
  if (!(t.gl > (R)0)) return 0;
  const R cg = dot(n, t.g) / t.gl;
  check(dc, cg - (R)kCosAlphaD, (R)kFilt * ((R)1 + M / h + t.kappa));
  if (!dc.unc && !(cg > (R)kCosAlphaD)) return 0;
  anc = nearest_vertex(s);
  PV<R, 3> tv[4];
  tet_local(t, anc, tv);
  R dmax[3] = {0, 0, 0}, D = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    D = fmax(D, amax(t.X[k]));
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      tv[k].d[j] = dot(en[j], t.X[k]) - eo[j];
      dmax[j] = fmax(dmax[j], abs_r(tv[k].d[j]));
    }
  }
  int nv = tet_section(tv, s, dc, out);
  if (nv == 0) return 0;
  const R tol_p = (R)kFilt * (M * ((R)1 + (D + Lt) / h) + D + Lt);
  PV<R, 3>* src = out;
  PV<R, 3>* dst = tmp;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    nv = clip_dist(src, nv, j, tol_p + (R)kFiltRel * dmax[j], dc, dst);
    PV<R, 3>* sw = src; src = dst; dst = sw;
    if (nv == 0) return 0;
  }
  if (src != out)
    for (int i = 0; i < nv; ++i) out[i] = src[i];
  return nv;
}

// Half-space polygon: tet section by the plane (FP64 values s).
template <class R>
__device__ int hs_polygon(const TetIn<R>& t, const double s[4], V3<R> n, Decide& dc, int& anc, PV<R, 1>* out) {
  if (!(t.gl > (R)0)) return 0;
  const R cg = dot(n, t.g) / t.gl;
  check(dc, cg - (R)kCosAlphaD, (R)kFilt * ((R)1 + t.kappa));
  if (!dc.unc && !(cg > (R)kCosAlphaD)) return 0;
  anc = nearest_vertex(s);
  PV<R, 1> tv[4];
  tet_local(t, anc, tv);
#pragma unroll
  for (int k = 0; k < 4; ++k) tv[k].d[0] = 0;
  return tet_section(tv, s, dc, out);
}

// Soft tet of body B in A's frame.
struct TetB {
  double g64[3], c64;  // FP64 field in A's frame
  float Y[4][3];
  float g[3], gl;
  float pn[4][3], po[4];
  float lo[3], hi[3];
  float M, h, kappa;
  int orig;
  int valid;
};

// FP64 tet of B in A's frame with its field.
__device__ __forceinline__ void tetb_fp64(const StepArgs& a, const FrameDev& F, int idx, TetIn<double>& t) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 r = a.tets[4 * (size_t)idx + k];
    t.X[k] = mat_mul<double>(F.R, mk<double>(r.x, r.y, r.z)) + mk(F.t[0], F.t[1], F.t[2]);
    t.P[k] = r.w;
  }
  tet_prepare(t);
}

// Soft-soft polygon: tet A's section by p_A - p_B = 0 (FP64 values s),
// clipped by tet B's faces.
template <class R>
__device__ int ss_polygon(const TetIn<R>& ta, const double s[4], V3<R> gb, R glb, V3<R> nrm, R lm,
                          const V3<R> pn[4], const R po[4], R Mb, R hb, R kb, Decide& dc, int& anc, PV<R, 4>* out,
                          PV<R, 4>* tmp) {
  const R cond = (((R)1 + ta.kappa) * ta.gl + ((R)1 + kb + Mb / hb) * glb) / lm;
  const R tol_c = (R)kFilt * cond;
  const R ca = dot(nrm, ta.g) / ta.gl;
  const R cbb = -dot(nrm, gb) / glb;
  check(dc, ca - (R)kCosAlphaD, tol_c);
  check(dc, cbb - (R)kCosAlphaD, tol_c);
  if (!dc.unc && !(ca > (R)kCosAlphaD && cbb > (R)kCosAlphaD)) return 0;
  anc = nearest_vertex(s);
  PV<R, 4> tv[4];
  tet_local(ta, anc, tv);
  R dmax[4] = {0, 0, 0, 0};
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      tv[k].d[j] = dot(pn[j], ta.X[k]) - po[j];
      dmax[j] = fmax(dmax[j], abs_r(tv[k].d[j]));
    }
  int nv = tet_section(tv, s, dc, out);
  if (nv == 0) return 0;
  const R D = ta.xmax + Mb;
  const R tol_p = (R)kFilt * (Mb * ((R)1 + D / hb) + D);
  PV<R, 4>* src = out;
  PV<R, 4>* dst = tmp;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    nv = clip_dist(src, nv, j, tol_p + (R)kFiltRel * dmax[j], dc, dst);
    PV<R, 4>* sw = src; src = dst; dst = sw;
    if (nv == 0) return 0;
  }
  if (src != out)
    for (int i = 0; i < nv; ++i) out[i] = src[i];
  return nv;
}

// Gradient component along a face normal.  A component below
// 1e-9 of |g| is rounding noise of a gradient perpendicular to the face and
// counts as zero, so the face is skipped deterministically; an
// FP32 value within 1e-5 |g| of zero is re-evaluated in FP64 for that test.
__device__ __forceinline__ float grad_noise_rule(double gi, double gl) {
  return fabs(gi) < 1e-9 * gl ? 0.f : (float)gi;
}

__device__ __forceinline__ float grad_along(const StepArgs& a, int tet_idx, float g32, float gl32, const double* n64) {
  if (fabsf(g32) > 1e-5f * gl32) return g32;
  TetIn<double> td;
  load_tet(a.tets, tet_idx, td);
  tet_prepare(td);
  return grad_noise_rule(td.g.x * n64[0] + td.g.y * n64[1] + td.g.z * n64[2], td.gl);
}

__device__ __forceinline__ bool aabb_overlap(const float* alo, const float* ahi, const float* blo, const float* bhi) {
  return alo[0] <= bhi[0] && ahi[0] >= blo[0] && alo[1] <= bhi[1] && ahi[1] >= blo[1] && alo[2] <= bhi[2] &&
         ahi[2] >= blo[2];
}

template <int ND>
__device__ __forceinline__ void to_f(const PV<double, ND>* in, int n, PV<float, ND>* out) {
  for (int i = 0; i < n; ++i) {
    out[i].x = (float)in[i].x; out[i].y = (float)in[i].y; out[i].z = (float)in[i].z; out[i].p = (float)in[i].p;
#pragma unroll
    for (int j = 0; j < ND; ++j) out[i].d[j] = (float)in[i].d[j];
  }
}

constexpr int kNarrowWarps = 4;

__global__ void __launch_bounds__(128) narrow_kernel(StepArgs a) {
  __shared__ union Stage {
    TriData tri[kCluster];
    TetB tetb[kCluster];
  } s_stage[kNarrowWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n_items = *a.item_total;
  while (true) {
    int item = 0;
    if (lane == 0) item = atomicAdd(a.item_next, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= n_items) break;
    const int4 it = a.items[item];
    PairCtx pc;
    pc.pair = it.x;
    pc.P = &a.pairs[it.x];
    pc.F = &a.frames[it.x];
    const PairDev& P = *pc.P;
    const FrameDev& F = *pc.F;
    Acc ac;
    for (int i = 0; i < 3; ++i) ac.F[i] = ac.T[i] = 0.f;
    ac.area = ac.fn0 = 0.f;
    ac.n_poly = ac.n_faces = ac.n_near = 0;
    const int sl = it.y, oc = it.z;
    const int ti = sl * kCluster + lane;
    const bool tvalid = ti < P.s_n_elem && F.valid;
    TetIn<float> t;
    float tlo[3], thi[3];
    if (tvalid) {
      load_tet(a.tets, P.s_elem_off + ti, t);
      tet_prepare(t);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float lo = fminf(fminf((&t.X[0].x)[i], (&t.X[1].x)[i]), fminf((&t.X[2].x)[i], (&t.X[3].x)[i]));
        const float hi = fmaxf(fmaxf((&t.X[0].x)[i], (&t.X[1].x)[i]), fmaxf((&t.X[2].x)[i], (&t.X[3].x)[i]));
        const float pad = 1e-5f * (fabsf(lo) + fabsf(hi)) + 1e-7f;
        tlo[i] = lo - pad;
        thi[i] = hi + pad;
      }
    }
    const int torig = tvalid ? a.tet_orig[P.s_elem_off + ti] : -1;
    const float sgn = P.s_is_m ? 1.f : -1.f;
    if (P.query == 1) {
      PV<float, 3> poly[kMaxPolyV], tmp[kMaxPolyV];
      // ---- stage the rigid triangles of cluster oc in the soft frame ----
      const int tj = oc * kCluster + lane;
      TriData& S = s_stage[wid].tri[lane];
      S.valid = 0;
      if (tj < P.o_n_elem && F.valid) {
        V3<double> Yd[3], nd, end[3];
        double od, eod[3], hd, Ltd;
        bool okd;
        tri_fp64(a, F, P.o_elem_off + tj, Yd);
        tri_planes(Yd, nd, od, end, eod, hd, Ltd, okd);
        V3<float> Y[3], n, en[3];
        float o, eo[3], h, Lt, M = 0.f;
        bool ok;
        for (int k = 0; k < 3; ++k) {
          const float4 r = a.tris[3 * (size_t)(P.o_elem_off + tj) + k];
          M = fmaxf(M, amax(mk(r.x, r.y, r.z)));
          Y[k] = mk((float)Yd[k].x, (float)Yd[k].y, (float)Yd[k].z);
        }
        M = fmaxf(M, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
        tri_planes(Y, n, o, en, eo, h, Lt, ok);
        S.n64[0] = nd.x; S.n64[1] = nd.y; S.n64[2] = nd.z; S.o64 = od;
        for (int k = 0; k < 3; ++k) {
          S.Y[k][0] = Y[k].x; S.Y[k][1] = Y[k].y; S.Y[k][2] = Y[k].z;
          S.en[k][0] = en[k].x; S.en[k][1] = en[k].y; S.en[k][2] = en[k].z;
          S.eo[k] = eo[k];
        }
        S.n[0] = n.x; S.n[1] = n.y; S.n[2] = n.z;
        const float pad = 1e-5f * (M + Lt) + 1e-7f;
        for (int i = 0; i < 3; ++i) {
          S.lo[i] = fminf(fminf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]) - pad;
          S.hi[i] = fmaxf(fmaxf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]) + pad;
        }
        S.M = M; S.h = h; S.Lt = Lt;
        S.orig = a.tri_orig[P.o_elem_off + tj];
        S.valid = okd && ok && h > 0.f ? 1 : 0;
      }
      __syncwarp();
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TriData& T = s_stage[wid].tri[j];
        if (!tvalid || !T.valid || !aabb_overlap(tlo, thi, T.lo, T.hi)) continue;
        double s[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) s[k] = plane64(T.n64, T.o64, t.X[k].x, t.X[k].y, t.X[k].z);
        // all four vertices strictly on one side: no section
        const bool allp = s[0] > kNearTol && s[1] > kNearTol && s[2] > kNearTol && s[3] > kNearTol;
        const bool alln = s[0] < -kNearTol && s[1] < -kNearTol && s[2] < -kNearTol && s[3] < -kNearTol;
        if (allp || alln) continue;
        const V3<float> n = mk(T.n[0], T.n[1], T.n[2]);
        const V3<float> en[3] = {mk(T.en[0][0], T.en[0][1], T.en[0][2]), mk(T.en[1][0], T.en[1][1], T.en[1][2]),
                                 mk(T.en[2][0], T.en[2][1], T.en[2][2])};
        Decide dc;
        int anc = 0;
        int nv = sr_polygon<float>(t, s, n, en, T.eo, fmaxf(T.M, t.xmax), T.h, T.Lt, dc, anc, poly, tmp);
        float gint = nv >= 3 ? grad_along(a, P.s_elem_off + ti, dot(t.g, n), t.gl, T.n64) : 0.f;
        int flags = 0;
        if (dc.unc) {
          // exact-decision fallback in FP64 from the stored inputs
          TetIn<double> td;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          V3<double> Yd[3], nd, end[3];
          double od, eod[3], hd, Ltd;
          bool okd;
          tri_fp64(a, F, P.o_elem_off + oc * kCluster + j, Yd);
          tri_planes(Yd, nd, od, end, eod, hd, Ltd, okd);
          Decide dd;
          PV<double, 3> pd[kMaxPolyV], td2[kMaxPolyV];
          nv = okd ? sr_polygon<double>(td, s, nd, end, eod, 0.0, 1.0, 0.0, dd, anc, pd, td2) : 0;
          to_f(pd, nv, poly);
          if (dd.near) flags |= 1;
          gint = grad_noise_rule(dot(td.g, nd), td.gl);
        }
        if (nv >= 3) {
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          const V3<float> nc = n * sgn;
          const float gM = P.s_is_m ? gint : INFINITY;
          const float gN = P.s_is_m ? INFINITY : gint;
          integrate_polygon<3>(a, pc, ac, poly, nv, t.X[anc], nc, gM, gN);
          record<3>(a, pc, poly, nv, t.X[anc], nc, torig, T.orig, flags);
        }
      }
      __syncwarp();
    } else if (P.query == 2) {
      if (tvalid) {
        PV<float, 1> poly[kMaxPolyV];
        const double n64[3] = {F.R[2], F.R[5], F.R[8]};
        const double o64 = F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2];
        double s[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) s[k] = plane64(n64, o64, t.X[k].x, t.X[k].y, t.X[k].z);
        const V3<float> n = mk(F.Rf[2], F.Rf[5], F.Rf[8]);
        Decide dc;
        int anc = 0;
        int nv = hs_polygon<float>(t, s, n, dc, anc, poly);
        float gint = nv >= 3 ? grad_along(a, P.s_elem_off + ti, dot(t.g, n), t.gl, n64) : 0.f;
        int flags = 0;
        if (dc.unc) {
          TetIn<double> td;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          const V3<double> nd = mk(F.R[2], F.R[5], F.R[8]);
          Decide dd;
          PV<double, 1> pd[kMaxPolyV];
          nv = hs_polygon<double>(td, s, nd, dd, anc, pd);
          to_f(pd, nv, poly);
          if (dd.near) flags |= 1;
          gint = grad_noise_rule(dot(td.g, nd), td.gl);
        }
        if (nv >= 3) {
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          const V3<float> nc = n * sgn;
          const float gM = P.s_is_m ? gint : INFINITY;
          const float gN = P.s_is_m ? INFINITY : gint;
          integrate_polygon<1>(a, pc, ac, poly, nv, t.X[anc], nc, gM, gN);
          record<1>(a, pc, poly, nv, t.X[anc], nc, torig, -1, flags);
        }
      }
    } else if (P.query == 3) {
      PV<float, 4> poly[kMaxPolyV], tmp[kMaxPolyV];
      // ---- stage the B tets of cluster oc in A's (soft) frame ----
      const int tj = oc * kCluster + lane;
      TetB& S = s_stage[wid].tetb[lane];
      S.valid = 0;
      if (tj < P.o_n_elem && F.valid) {
        TetIn<double> bd;
        tetb_fp64(a, F, P.o_elem_off + tj, bd);
        TetIn<float> tb;
        float M = 0.f;
        for (int k = 0; k < 4; ++k) {
          const float4 r = a.tets[4 * (size_t)(P.o_elem_off + tj) + k];
          M = fmaxf(M, amax(mk(r.x, r.y, r.z)));
          tb.X[k] = mk((float)bd.X[k].x, (float)bd.X[k].y, (float)bd.X[k].z);
          tb.P[k] = r.w;
        }
        M = fmaxf(M, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
        tet_prepare(tb);
        V3<float> pn[4];
        float po[4];
        tet_planes(tb.X, pn, po);
        S.g64[0] = bd.g.x; S.g64[1] = bd.g.y; S.g64[2] = bd.g.z; S.c64 = bd.c;
        for (int k = 0; k < 4; ++k) {
          S.Y[k][0] = tb.X[k].x; S.Y[k][1] = tb.X[k].y; S.Y[k][2] = tb.X[k].z;
          S.pn[k][0] = pn[k].x; S.pn[k][1] = pn[k].y; S.pn[k][2] = pn[k].z;
          S.po[k] = po[k];
        }
        S.g[0] = tb.g.x; S.g[1] = tb.g.y; S.g[2] = tb.g.z; S.gl = tb.gl;
        const float pad = 1e-5f * M + 1e-7f;
        for (int i = 0; i < 3; ++i) {
          S.lo[i] = fminf(fminf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fminf((&tb.X[2].x)[i], (&tb.X[3].x)[i])) - pad;
          S.hi[i] = fmaxf(fmaxf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fmaxf((&tb.X[2].x)[i], (&tb.X[3].x)[i])) + pad;
        }
        S.M = M; S.h = tb.hmin; S.kappa = tb.kappa;
        S.orig = a.tet_orig[P.o_elem_off + tj];
        S.valid = tb.hmin > 0.f && bd.hmin > 0.0 ? 1 : 0;
      }
      __syncwarp();
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TetB& B = s_stage[wid].tetb[j];
        if (!tvalid || !B.valid || !aabb_overlap(tlo, thi, B.lo, B.hi)) continue;
        const V3<float> gb = mk(B.g[0], B.g[1], B.g[2]);
        const V3<float> m = t.g - gb;
        const float lm = norm(m);
        if (!(lm > 0.f) || !(t.gl > 0.f) || !(B.gl > 0.f)) continue;
        double s[4];
        const double il = 1.0 / (double)lm;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          s[k] = ((double)t.P[k] - (fma(B.g64[2], (double)t.X[k].z, fma(B.g64[1], (double)t.X[k].y,
                                                                          B.g64[0] * (double)t.X[k].x)) +
                                    B.c64)) * il;
        const bool allp = s[0] > kNearTol && s[1] > kNearTol && s[2] > kNearTol && s[3] > kNearTol;
        const bool alln = s[0] < -kNearTol && s[1] < -kNearTol && s[2] < -kNearTol && s[3] < -kNearTol;
        if (allp || alln) continue;
        const V3<float> pn[4] = {mk(B.pn[0][0], B.pn[0][1], B.pn[0][2]), mk(B.pn[1][0], B.pn[1][1], B.pn[1][2]),
                                 mk(B.pn[2][0], B.pn[2][1], B.pn[2][2]), mk(B.pn[3][0], B.pn[3][1], B.pn[3][2])};
        V3<float> nrm = m * (1.f / lm);
        Decide dc;
        int anc = 0;
        int nv = ss_polygon<float>(t, s, gb, B.gl, nrm, lm, pn, B.po, B.M, B.h, B.kappa, dc, anc, poly, tmp);
        float gM = dot(t.g, nrm), gN = -dot(gb, nrm);
        int flags = 0;
        if (!dc.unc && nv >= 3 && (fabsf(gM) <= 1e-5f * t.gl || fabsf(gN) <= 1e-5f * B.gl)) {
          TetIn<double> td, tbd;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          tetb_fp64(a, F, P.o_elem_off + oc * kCluster + j, tbd);
          const V3<double> md = td.g - tbd.g;
          const V3<double> nrmd = md * (1.0 / norm(md));
          gM = grad_noise_rule(dot(td.g, nrmd), td.gl);
          gN = grad_noise_rule(-dot(tbd.g, nrmd), tbd.gl);
        }
        if (dc.unc) {
          TetIn<double> td, tbd;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          tetb_fp64(a, F, P.o_elem_off + oc * kCluster + j, tbd);
          V3<double> pnd[4];
          double pod[4];
          tet_planes(tbd.X, pnd, pod);
          const V3<double> md = td.g - tbd.g;
          const double lmd = norm(md);
          Decide dd;
          PV<double, 4> pd[kMaxPolyV], td2[kMaxPolyV];
          nv = 0;
          if (lmd > 0.0) {
            const V3<double> nrmd = md * (1.0 / lmd);
            nv = ss_polygon<double>(td, s, tbd.g, tbd.gl, nrmd, lmd, pnd, pod, 0.0, 1.0, 0.0, dd, anc, pd, td2);
            if (nv >= 3) {
              nrm = mk((float)nrmd.x, (float)nrmd.y, (float)nrmd.z);
              gM = grad_noise_rule(dot(td.g, nrmd), td.gl);
              gN = grad_noise_rule(-dot(tbd.g, nrmd), tbd.gl);
            }
          }
          to_f(pd, nv, poly);
          if (dd.near) flags |= 1;
        }
        if (nv >= 3) {
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          integrate_polygon<4>(a, pc, ac, poly, nv, t.X[anc], nrm, gM, gN);
          record<4>(a, pc, poly, nv, t.X[anc], nrm, torig, B.orig, flags);
        }
      }
      __syncwarp();
    }
    // ---- deterministic warp reduction (FP64 butterfly) ----
    double v[8] = {ac.F[0], ac.F[1], ac.F[2], ac.T[0], ac.T[1], ac.T[2], ac.area, ac.fn0};
    int c3[3] = {ac.n_poly, ac.n_faces, ac.n_near};
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
#pragma unroll
      for (int i = 0; i < 3; ++i) c3[i] += __shfl_xor_sync(0xffffffffu, c3[i], o);
    }
    if (lane == 0) {
      ItemOut r;
      for (int i = 0; i < 8; ++i) r.v[i] = v[i];
      r.n_poly = c3[0]; r.n_faces = c3[1]; r.n_near = c3[2]; r.pad = 0;
      a.item_out[item] = r;
    }
  }
}
