// narrow.cuh — the narrow-phase kernels (included by contact.cu inside
// namespace hc).
//
// One kernel per query type, each over the contiguous range of work items
// of its type (units are ordered by query type).  One warp per item (soft
// leaf cluster x other cluster); items are taken from a per-type counter.
// Per item the warp stages the soft tets and the other elements in shared
// memory (soft frame), builds a queue of candidate element pairs with cheap
// conservative tests (AABB overlap and an FP32 plane test with an error
// margin), and then works the queue with all 32 lanes.  Per non-empty
// polygon: centroid quadrature (mujoco_contact_surfaces_plugin.cpp:320-409),
// Hunt-Crossley damping and regularised friction, and flat-sensor
// ray binning (flat_tactile_sensor.cpp:316-392).  The warp's sums are reduced
// in FP64 in a fixed order.

struct Acc {
  float F[3], T[3], area, fn0;
  int n_poly, n_faces, n_near;
};

__device__ __forceinline__ void acc_zero(Acc& ac) {
#pragma unroll
  for (int i = 0; i < 3; ++i) ac.F[i] = ac.T[i] = 0.f;
  ac.area = ac.fn0 = 0.f;
  ac.n_poly = ac.n_faces = ac.n_near = 0;
}

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

// Ray samples of a flat sensor hit by one contact polygon.  The sensor's
// rays are parallel to its -z axis, start 1.5*zs (+1e-8) above its centre and
// accept 0 < t < 1.5*zs (flat_tactile_sensor.cpp:324-346).  The reference
// casts them against the polygon's fan triangles (Moeller-Trumbore,
// bvh.cpp:49-74) and evaluates the pressure barycentrically; a ray through
// the convex polygon hits exactly one fan triangle and, the field being
// linear on the polygon, the pressure at the hit is the polygon's linear
// field there.  Polygons whose projection is degenerate (|2A| < 1e-10, the
// test's parallel threshold) are skipped.  Each sample keeps the smallest t
// packed with the pressure by a 64-bit atomicMin (order independent).
//
// The same compiled function serves the adjoint (G != null): a sample this
// polygon won in the forward pass (bit-identical key) is claimed with a CAS
// that also clears it, and dL/dp at the hit is added to G.
struct AdjAcc {
  float gx[6];     // dL/dxi: twist (w, v) of the other body in the soft frame
  float glin[3];   // dL/dlin of the velocity field v = lin + ang x p
  float gang[3];   // dL/dang
  float gE;        // sum of dL/dp * p over won samples (taxel part of dL/dE * E);
                   // soft-soft: dL/dE_M itself
};

// Soft-soft terms of the adjoint.  The section plane p_M = p_N moves with
// N's field and with both moduli, so the adjoint needs both gradients (soft
// frame, M's), |g_M - g_N|, 1/E of both geoms; it sums dL/dE_N and
// dL/d(damping) here (the combined dissipation depends on E_M / E_N).
struct SsAdj {
  V3<float> ga, gb;
  float lm, iEa, iEb;
  float gEb, gD;
};

// One polygon prepared for ray binning on one sensor (sensor frame): vertex
// x, y, edge vectors, the plane z(x, y) and the linear pressure p(x, y), and
// the range of sample indices its bounding box covers.  All arithmetic uses
// explicitly rounded intrinsics, so every kernel that inlines these
// functions computes bit-identical keys (the adjoint re-identifies the
// forward's winning samples by their keys).
struct RasterPoly {
  float lx[kMaxPolyV], ly[kMaxPolyV], ex[kMaxPolyV], ey[kMaxPolyV];
  float lz0, zx, zy, px, py, p0;
  bool pos;           // orientation of the projected polygon
  int nv, X0, X1, Y0, Y1;
};

__device__ __forceinline__ float dot3_rn(const float* r, float x, float y, float z) {
  return __fadd_rn(__fadd_rn(__fmul_rn(r[0], x), __fmul_rn(r[1], y)), __fmul_rn(r[2], z));
}

// vtx(i) -> float4 (x, y, z relative to anc, pressure).  Returns false when
// the polygon projects degenerately (|2A| < 1e-10, the ray test's parallel
// threshold) or misses the sample grid.
template <class Vtx>
__device__ __forceinline__ bool raster_prepare(const StepArgs& a, const SensorDev& S, const float* Rl,
                                               const float* tl, int nv, V3<float> anc, V3<float> g_soft, Vtx vtx,
                                               RasterPoly& rp) {
  float lz[kMaxPolyV];
  float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
#pragma unroll
  for (int i = 0; i < kMaxPolyV; ++i) {
    rp.lx[i] = rp.ly[i] = lz[i] = 0.f;
    if (i < nv) {
      const float4 v = vtx(i);
      const float X = __fadd_rn(anc.x, v.x), Y = __fadd_rn(anc.y, v.y), Z = __fadd_rn(anc.z, v.z);
      rp.lx[i] = __fadd_rn(dot3_rn(Rl, X, Y, Z), tl[0]);
      rp.ly[i] = __fadd_rn(dot3_rn(Rl + 3, X, Y, Z), tl[1]);
      lz[i] = __fadd_rn(dot3_rn(Rl + 6, X, Y, Z), tl[2]);
      mnx = fminf(mnx, rp.lx[i]); mxx = fmaxf(mxx, rp.lx[i]);
      mny = fminf(mny, rp.ly[i]); mxy = fmaxf(mxy, rp.ly[i]);
      if (i == 0) rp.p0 = v.w;
    }
  }
  float A2 = 0.f;
#pragma unroll
  for (int i = 1; i + 1 < kMaxPolyV; ++i)
    if (i + 1 < nv)
      A2 = __fadd_rn(A2, __fsub_rn(__fmul_rn(__fsub_rn(rp.lx[i], rp.lx[0]), __fsub_rn(rp.ly[i + 1], rp.ly[0])),
                                   __fmul_rn(__fsub_rn(rp.ly[i], rp.ly[0]), __fsub_rn(rp.lx[i + 1], rp.lx[0]))));
  if (!(fabsf(A2) >= 1e-10f)) return false;
  rp.pos = A2 > 0.f;
  // plane of the polygon and the pressure gradient, sensor frame
  const float e1x = __fsub_rn(rp.lx[1], rp.lx[0]), e1y = __fsub_rn(rp.ly[1], rp.ly[0]), e1z = __fsub_rn(lz[1], lz[0]);
  float nx = 0.f, ny = 0.f, nz = 0.f;
#pragma unroll
  for (int i = 2; i < kMaxPolyV; ++i) {
    if (i < nv) {
      const float fx = __fsub_rn(rp.lx[i], rp.lx[0]), fy = __fsub_rn(rp.ly[i], rp.ly[0]), fz = __fsub_rn(lz[i], lz[0]);
      nx = __fadd_rn(nx, __fsub_rn(__fmul_rn(e1y, fz), __fmul_rn(e1z, fy)));
      ny = __fadd_rn(ny, __fsub_rn(__fmul_rn(e1z, fx), __fmul_rn(e1x, fz)));
      nz = __fadd_rn(nz, __fsub_rn(__fmul_rn(e1x, fy), __fmul_rn(e1y, fx)));
    }
  }
  if (!(fabsf(nz) > 0.f)) return false;
  rp.zx = __fdiv_rn(-nx, nz);   // dz/dx, dz/dy on the plane
  rp.zy = __fdiv_rn(-ny, nz);
  const float glx = dot3_rn(Rl, g_soft.x, g_soft.y, g_soft.z);
  const float gly = dot3_rn(Rl + 3, g_soft.x, g_soft.y, g_soft.z);
  const float glz = dot3_rn(Rl + 6, g_soft.x, g_soft.y, g_soft.z);
  rp.px = __fadd_rn(glx, __fmul_rn(glz, rp.zx));   // dp/dx, dp/dy on the plane
  rp.py = __fadd_rn(gly, __fmul_rn(glz, rp.zy));
  rp.lz0 = lz[0];
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  const float x0 = sx[0], dx = S.nx > 1 ? __fsub_rn(sx[1], sx[0]) : 1.f;
  const float y0 = sy[0], dy = S.ny > 1 ? __fsub_rn(sy[1], sy[0]) : 1.f;
  const float fx0 = ceilf(__fsub_rn(__fdiv_rn(__fsub_rn(mnx, x0), dx), 1e-3f));
  const float fx1 = floorf(__fadd_rn(__fdiv_rn(__fsub_rn(mxx, x0), dx), 1e-3f));
  const float fy0 = ceilf(__fsub_rn(__fdiv_rn(__fsub_rn(mny, y0), dy), 1e-3f));
  const float fy1 = floorf(__fadd_rn(__fdiv_rn(__fsub_rn(mxy, y0), dy), 1e-3f));
  if (!(fx1 >= 0.f && fy1 >= 0.f && fx0 <= (float)(S.nx - 1) && fy0 <= (float)(S.ny - 1))) return false;
  rp.X0 = max(0, (int)fx0); rp.X1 = min(S.nx - 1, (int)fx1);
  rp.Y0 = max(0, (int)fy0); rp.Y1 = min(S.ny - 1, (int)fy1);
  rp.nv = nv;
#pragma unroll
  for (int i = 0; i < kMaxPolyV; ++i) {
    const bool last = i + 1 >= nv;
    const float nxv = last ? rp.lx[0] : rp.lx[i + 1 < kMaxPolyV ? i + 1 : 0];
    const float nyv = last ? rp.ly[0] : rp.ly[i + 1 < kMaxPolyV ? i + 1 : 0];
    rp.ex[i] = __fsub_rn(nxv, rp.lx[i]);
    rp.ey[i] = __fsub_rn(nyv, rp.ly[i]);
  }
  return true;
}

// Sample keys (64-bit, smallest wins): the ray parameter t in the high word
// (positive floats order as their bits), a tie-break in the low word: the
// hit pressure (clamped to +0, so bit 31 is clear) when the polygon is cast
// inline, or, when it is cast from the kept records, bit 31 set, the sensor
// side of its pair in bit 30 and its pair-ordered record slot below (the
// taxel pass then evaluates the winner's pressure from its stored linear
// model, and the adjoint recognises its samples by the key alone).
constexpr unsigned kSlotTag = 0x80000000u, kSideBit = 0x40000000u;
__device__ __forceinline__ unsigned long long key_pressure(float t, float pr) {
  return ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)__float_as_uint(pr > 0.f ? pr : 0.f);
}
__device__ __forceinline__ unsigned long long key_slot(float t, int slot, int side) {
  return ((unsigned long long)__float_as_uint(t) << 32) |
         (unsigned long long)(kSlotTag | (side ? kSideBit : 0u) | (unsigned)slot);
}

// Height of a prepared polygon's plane at (qx, qy).
__device__ __forceinline__ float raster_height(float lx0, float ly0, float lz0, float zx, float zy, float qx,
                                               float qy) {
  const float ddx = __fsub_rn(qx, lx0), ddy = __fsub_rn(qy, ly0);
  return __fadd_rn(__fadd_rn(lz0, __fmul_rn(zx, ddx)), __fmul_rn(zy, ddy));
}

// Pressure of a prepared polygon's linear model at (qx, qy).
__device__ __forceinline__ float raster_pressure(float lx0, float ly0, float p0, float px, float py, float qx,
                                                 float qy) {
  const float ddx = __fsub_rn(qx, lx0), ddy = __fsub_rn(qy, ly0);
  return __fadd_rn(__fadd_rn(p0, __fmul_rn(px, ddx)), __fmul_rn(py, ddy));
}

// Sample (qx, qy) against a prepared polygon: false when the ray misses the
// polygon or its hit lies outside 0 < t < 1.5 zs; else t, the hit height z
// and the pressure there.
// MV: the most vertices the polygon can have (the loop's bound).
template <int MV = kMaxPolyV>
__device__ __forceinline__ bool raster_probe(const RasterPoly& rp, const SensorDev& S, float qx, float qy,
                                             float& t, float& z, float& pr) {
#pragma unroll
  for (int i = 0; i < MV; ++i) {
    if (i >= rp.nv) break;
    const float e = __fsub_rn(__fmul_rn(rp.ex[i], __fsub_rn(qy, rp.ly[i])),
                              __fmul_rn(rp.ey[i], __fsub_rn(qx, rp.lx[i])));
    if (rp.pos ? e < 0.f : e > 0.f) return false;   // outside this edge
  }
  z = raster_height(rp.lx[0], rp.ly[0], rp.lz0, rp.zx, rp.zy, qx, qy);
  t = __fsub_rn(__fadd_rn(S.zs15, 1e-8f), z);
  if (!(t > 0.f && t < S.zs15)) return false;
  pr = raster_pressure(rp.lx[0], rp.ly[0], rp.p0, rp.px, rp.py, qx, qy);
  return true;
}

// Adjoint of one won sample: dL/dp = pbar at the hit (qx, qy, z) of the
// sensor frame.
template <bool kSS>
__device__ __forceinline__ void sample_adjoint(const StepArgs& a, const SensorDev& S, const float* Rl,
                                               const float* tl, float qx, float qy, float z, float pr, int X, int Y,
                                               V3<float> g_soft, V3<float> n_tri, int soft_is_sensor, AdjAcc& G,
                                               SsAdj* ss) {
  // dL/dp at this sample: cell (X / sr, Y / sr), window weight of (X % sr, Y % sr)
  const float w = a.weights[S.weight_off + (X % S.sr) * S.sr + (Y % S.sr)];
  const float pbar = a.adj_taxel[S.taxel_off + X / S.sr + S.cy * (Y / S.sr)] * w * S.rmean;
  if (pbar == 0.f) return;
  const V3<float> xs = mat_tmul<float>(Rl, mk(qx, qy, z) - mk(tl[0], tl[1], tl[2]));   // hit point, soft frame
  if (kSS) {
    // hit x = o + t D on p_M - p_N = 0 (m = g_M - g_N), reading p = p_M(x).
    // Rays on N (move with it): dp = kb g_M . (w x x + v); rays on M:
    // dp = -ka g_N . (w x x + v), with ka = g_M.D / m.D, kb = -g_N.D / m.D
    // (ka + kb = 1).  Moduli: dp/dE_M = kb p / E_M, dp/dE_N = ka p / E_N.
    const V3<float> D = mk(-Rl[6], -Rl[7], -Rl[8]);
    const float mD = dot(ss->ga - ss->gb, D);
    if (!(fabsf(mD) > 0.f)) return;
    const float ka = dot(ss->ga, D) / mD, kb = -dot(ss->gb, D) / mD;
    G.gE += pbar * pr * kb * ss->iEa;
    ss->gEb += pbar * pr * ka * ss->iEb;
    const V3<float> gv = soft_is_sensor ? ss->gb * (-ka) : ss->ga * kb;
    const V3<float> wx = cross(xs, gv);
    G.gx[0] += pbar * wx.x; G.gx[1] += pbar * wx.y; G.gx[2] += pbar * wx.z;
    G.gx[3] += pbar * gv.x; G.gx[4] += pbar * gv.y; G.gx[5] += pbar * gv.z;
    return;
  }
  G.gE += pbar * pr;
  if (!soft_is_sensor) {
    // rays and plane move with the other body: dp = g . (w x x + v)
    const V3<float> wx = cross(xs, g_soft);
    G.gx[0] += pbar * wx.x; G.gx[1] += pbar * wx.y; G.gx[2] += pbar * wx.z;
    G.gx[3] += pbar * g_soft.x; G.gx[4] += pbar * g_soft.y; G.gx[5] += pbar * g_soft.z;
  } else {
    // rays fixed in the soft frame, plane n.x = o moving: dx = dt D,
    // dt = -(w.(n x x) - n.v) / (n.D), D = -(sensor z) in the soft frame
    const V3<float> D = mk(-Rl[6], -Rl[7], -Rl[8]);
    const float nD = dot(n_tri, D);
    if (!(fabsf(nD) > 0.f)) return;
    const float r = -dot(g_soft, D) / nD;
    const V3<float> nx = cross(n_tri, xs);
    G.gx[0] += pbar * r * nx.x; G.gx[1] += pbar * r * nx.y; G.gx[2] += pbar * r * nx.z;
    G.gx[3] -= pbar * r * n_tri.x; G.gx[4] -= pbar * r * n_tri.y; G.gx[5] -= pbar * r * n_tri.z;
  }
}

// Grow a sensor's touched sample box to hold (X0..X1, Y0..Y1).  The box is
// read from L2 first (it changes only during the step, and a stale value
// can only be looser), so most polygons issue no atomic at all.
__device__ __forceinline__ void grow_box(int4* b, int X0, int X1, int Y0, int Y1) {
  const int4 c = __ldcg(b);
  if (X0 < c.x) atomicMin(&b->x, X0);
  if (X1 > c.y) atomicMax(&b->y, X1);
  if (Y0 < c.z) atomicMin(&b->z, Y0);
  if (Y1 > c.w) atomicMax(&b->w, Y1);
}

template <int ND, bool kSS = false>
__device__ __noinline__ void raster_keys(const StepArgs& a, int sid, const float* Rl, const float* tl,
                                         const PV<float, ND>* v, int nv, V3<float> anc, V3<float> g_soft,
                                         V3<float> n_tri, int soft_is_sensor, AdjAcc* G, SsAdj* ss = nullptr) {
  const SensorDev S = a.sensors[sid];
  RasterPoly rp;
  if (!raster_prepare(a, S, Rl, tl, nv, anc, g_soft,
                      [&](int i) { return make_float4(v[i].x, v[i].y, v[i].z, v[i].p); }, rp))
    return;
  unsigned long long* smp = a.samples + S.sample_off;
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  if (!G && a.sens_box && rp.X0 <= rp.X1 && rp.Y0 <= rp.Y1) grow_box(a.sens_box + sid, rp.X0, rp.X1, rp.Y0, rp.Y1);
  for (int X = rp.X0; X <= rp.X1; ++X) {
    const float qx = sx[X];
    for (int Y = rp.Y0; Y <= rp.Y1; ++Y) {
      float t, z, pr;
      if (!raster_probe(rp, S, qx, sy[Y], t, z, pr)) continue;
      const unsigned long long key = key_pressure(t, pr);
      const size_t si = (size_t)X * S.ny + Y;
      if (!G) {
        atomicMin(&smp[si], key);
        continue;
      }
      if (atomicCAS(&smp[si], key, ~0ull) != key) continue;
      sample_adjoint<kSS>(a, S, Rl, tl, qx, sy[Y], z, pr, X, Y, g_soft, n_tri, soft_is_sensor, *G, ss);
    }
  }
}

// Quadrature of one polygon (vertices relative to `anc`, soft frame) and its
// forces.  n: contact normal out of N into M.
template <int ND>
__device__ void integrate_forces(const StepArgs& a, const PairDev& P, const FrameDev& F, Acc& ac,
                                 const PV<float, ND>* v, int nv, V3<float> anc, V3<float> n, float gM, float gN) {
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
}

// Ray binning of one polygon for the flat sensors of the pair.  g: the soft
// (M-side for soft-soft) pressure gradient, soft frame.
template <int ND>
__device__ __forceinline__ void raster_polygon(const StepArgs& a, const PairDev& P, const FrameDev& F,
                                               const PV<float, ND>* v, int nv, V3<float> anc, V3<float> n,
                                               V3<float> g) {
  if (P.sensor0 >= 0) raster_keys<ND>(a, P.sensor0, F.Rl, F.tl, v, nv, anc, g, n, 0, nullptr);
  if (P.sensor1 >= 0) raster_keys<ND>(a, P.sensor1, F.Rl1, F.tl1, v, nv, anc, g, n, 0, nullptr);
}

template <int ND>
__device__ void integrate_polygon(const StepArgs& a, const PairDev& P, const FrameDev& F, Acc& ac,
                                  const PV<float, ND>* v, int nv, V3<float> anc, V3<float> n, float gM, float gN,
                                  V3<float> g) {
  integrate_forces<ND>(a, P, F, ac, v, nv, anc, n, gM, gN);
  raster_polygon<ND>(a, P, F, v, nv, anc, n, g);
}

template <int ND>
__device__ void record(const StepArgs& a, int pair, const PV<float, ND>* v, int nv, V3<float> anc, V3<float> n,
                       int ea, int eb, int flags) {
  if (a.debug & 1) {
    const int k = atomicAdd(a.cand_count, 1);
    if (k < a.cand_cap) {
      CandRec r;
      r.pair = pair; r.elem_a = ea; r.elem_b = eb; r.n_vert = nv; r.flags = flags;
      a.cand[k] = r;
    } else {
      atomicOr(a.status, 2);
    }
  }
  if (a.want_polys && (a.want_pair < 0 || a.want_pair == pair)) {
    const int k = atomicAdd(a.poly_count, 1);
    if (k < a.poly_cap) {
      PolyRec& r = a.polys[k];
      r.pair = pair; r.elem_a = ea; r.elem_b = eb; r.nv = nv;
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

// Soft tet staged in shared memory (soft frame).
struct TetStage {
  float X[4][3];
  float P[4];
  float g[3];
  float gl, kappa, xmax, pmax;
  int orig, valid;
};

// The padded box of a staged tet (computed where it is needed, by the lane
// that staged the tet, rather than kept in shared memory).
__device__ __forceinline__ void tet_box(const TetStage& S, float lo[3], float hi[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float l = fminf(fminf(S.X[0][i], S.X[1][i]), fminf(S.X[2][i], S.X[3][i]));
    const float h = fmaxf(fmaxf(S.X[0][i], S.X[1][i]), fmaxf(S.X[2][i], S.X[3][i]));
    const float pad = 1e-5f * (fabsf(l) + fabsf(h)) + 1e-7f;
    lo[i] = l - pad;
    hi[i] = h + pad;
  }
}

// (not inlined: the forward and adjoint kernels share one compiled body, so
// the staged values are bit-identical in both)
__device__ __noinline__ void stage_tet(const StepArgs& a, const PairDev& P, int ti, TetStage& S) {
  S.valid = 0;
  if (ti >= P.s_n_elem) return;
  const int idx = P.s_elem_off + ti;
  TetIn<float> t;
  load_tet(a.tets, idx, t);
  // the field's constants, computed when the pool was built (tet_props_kernel)
  const float4 p0 = a.tet_props[2 * (size_t)idx], p1 = a.tet_props[2 * (size_t)idx + 1];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    S.X[k][0] = t.X[k].x; S.X[k][1] = t.X[k].y; S.X[k][2] = t.X[k].z;
    S.P[k] = t.P[k];
  }
  S.g[0] = p0.x; S.g[1] = p0.y; S.g[2] = p0.z;
  S.gl = p0.w; S.kappa = p1.x; S.xmax = p1.y; S.pmax = p1.z;
  S.orig = a.tet_orig[idx];
  S.valid = p1.w > 0.f ? 1 : 0;
}

// The constants of each soft tet's field (what tet_prepare derives), once
// per pool build.
__global__ void tet_props_kernel(const float4* tets, float4* props, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  TetIn<float> t;
  load_tet(tets, i, t);
  tet_prepare(t);
  props[2 * (size_t)i] = make_float4(t.g.x, t.g.y, t.g.z, t.gl);
  props[2 * (size_t)i + 1] = make_float4(t.kappa, t.xmax, t.pmax, t.hmin);
}

__device__ __forceinline__ void unstage_tet(const TetStage& S, TetIn<float>& t) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    t.X[k] = mk(S.X[k][0], S.X[k][1], S.X[k][2]);
    t.P[k] = S.P[k];
  }
  t.g = mk(S.g[0], S.g[1], S.g[2]);
  t.gl = S.gl; t.kappa = S.kappa; t.xmax = S.xmax; t.pmax = S.pmax;
  t.c = 0.f; t.hmin = 0.f;
}

// Index of the tet vertex nearest the section plane.
template <class S>
__device__ __forceinline__ int nearest_vertex(const S s[4]) {
  int k = 0;
  S best = abs_r(s[0]);
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (abs_r(s[i]) < best) {
      best = abs_r(s[i]);
      k = i;
    }
  return k;
}

template <class R, int ND>
__device__ __forceinline__ void tet_local(const TetIn<R>& t, int anc, PV<R, ND> tv[4]) {
  const V3<R> xa = sel4(t.X, anc);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    tv[k].x = t.X[k].x - xa.x;
    tv[k].y = t.X[k].y - xa.y;
    tv[k].z = t.X[k].z - xa.z;
    tv[k].p = t.P[k];
  }
}

// Conservative FP32 test: all four vertices certainly on one side of
// n.x = o (margin covers float rounding of n, o and the dot products).
__device__ __forceinline__ bool one_sided32(const float X[4][3], const float* n, float o, float margin) {
  int pos = 0, neg = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float s = n[0] * X[k][0] + n[1] * X[k][1] + n[2] * X[k][2] - o;
    pos += s > margin;
    neg += s < -margin;
  }
  return pos == 4 || neg == 4;
}

// Gradient component along a face normal.  A component below
// 1e-9 of |g| is rounding noise of a gradient perpendicular to the face and
// counts as zero, so the face is skipped deterministically; an
// FP32 value within 1e-5 |g| of zero is re-evaluated in FP64 for that test.
__device__ __forceinline__ float grad_noise_rule(double gi, double gl) {
  return fabs(gi) < 1e-9 * gl ? 0.f : (float)gi;
}

__device__ __noinline__ float grad_along64(const StepArgs& a, int tet_idx, double n0, double n1, double n2) {
  TetIn<double> td;
  load_tet(a.tets, tet_idx, td);
  tet_prepare(td);
  return grad_noise_rule(td.g.x * n0 + td.g.y * n1 + td.g.z * n2, td.gl);
}

__device__ __forceinline__ bool aabb_overlap(const float* alo, const float* ahi, const float* blo, const float* bhi) {
  return alo[0] <= bhi[0] && ahi[0] >= blo[0] && alo[1] <= bhi[1] && ahi[1] >= blo[1] && alo[2] <= bhi[2] &&
         ahi[2] >= blo[2];
}

template <int ND, int MD>
__device__ __forceinline__ void to_f(const PV<double, ND>* in, int n, PV<float, MD>* out) {
  for (int i = 0; i < n; ++i) {
    out[i].x = (float)in[i].x; out[i].y = (float)in[i].y; out[i].z = (float)in[i].z; out[i].p = (float)in[i].p;
    out[i].lab = in[i].lab;
    if constexpr (MD > 0) {
#pragma unroll
      for (int j = 0; j < MD; ++j) out[i].d[j] = (float)in[i].d[j];
    }
  }
}

// Error-free float addition (Knuth's TwoSum) and double-float accumulation;
// the _rn intrinsics keep the compiler from contracting or reassociating.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void df_add(float& hi, float& lo, float h2, float l2) {
  float s, e;
  two_sum(hi, h2, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, l2));
  hi = __fadd_rn(s, e);
  lo = __fsub_rn(e, __fsub_rn(hi, s));
}

// Fixed-order butterfly of the lanes' sums in double-float arithmetic (on
// the FP32 pipe; FP64 runs at 1/64 of the FP32 rate on this part); lane 0
// stores the item's (hi, lo) pairs.
// kKeep: the item's polygons were kept as records (their forces come from
// the records later), so only the counts are summed; the force sums stored
// are zero.
template <bool kKeep = false>
__device__ __forceinline__ void warp_reduce_store(const StepArgs& a, const Acc& ac, int item, int lane) {
  if constexpr (kKeep) {
    const int n_poly = __reduce_add_sync(0xffffffffu, ac.n_poly);
    const int n_near = __reduce_add_sync(0xffffffffu, ac.n_near);
    if (lane == 0) {
      ItemOut r;
#pragma unroll
      for (int i = 0; i < 8; ++i) r.hi[i] = r.lo[i] = 0.f;
      r.n_poly = n_poly; r.n_faces = 0; r.n_near = n_near; r.pad = 0;
      a.item_out[item] = r;
    }
    return;
  }
  float hi[8] = {ac.F[0], ac.F[1], ac.F[2], ac.T[0], ac.T[1], ac.T[2], ac.area, ac.fn0};
  float lo[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int c3[3] = {ac.n_poly, ac.n_faces, ac.n_near};
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const float h2 = __shfl_xor_sync(0xffffffffu, hi[i], o);
      const float l2 = __shfl_xor_sync(0xffffffffu, lo[i], o);
      df_add(hi[i], lo[i], h2, l2);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) c3[i] += __shfl_xor_sync(0xffffffffu, c3[i], o);
  }
  if (lane == 0) {
    ItemOut r;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      r.hi[i] = hi[i];
      r.lo[i] = lo[i];
    }
    r.n_poly = c3[0]; r.n_faces = c3[1]; r.n_near = c3[2]; r.pad = 0;
    a.item_out[item] = r;
  }
}

// Item range of query type q and the next item for this warp.
__device__ __forceinline__ int next_item(const StepArgs& a, int q, int lane, int& ie) {
  const int total = *a.item_total;
  const int ib = min(a.unit_off[a.type_unit_begin[q]], total);
  ie = min(a.unit_off[a.type_unit_end[q]], total);
  int item = 0;
  if (lane == 0) item = atomicAdd(a.item_next + q, 1);
  return ib + __shfl_sync(0xffffffffu, item, 0);
}

// The next chunk of a.chunk consecutive items of query type q for this warp
// (consecutive items usually share their pair and other cluster, whose
// staged elements the warp then keeps).
__device__ __forceinline__ int next_chunk(const StepArgs& a, int q, int lane, int& ie) {
  const int total = *a.item_total;
  const int ib = min(a.unit_off[a.type_unit_begin[q]], total);
  ie = min(a.unit_off[a.type_unit_end[q]], total);
  int c = 0;
  if (lane == 0) c = atomicAdd(a.item_next + q, a.chunk);
  return ib + __shfl_sync(0xffffffffu, c, 0);
}

// Candidate queue entries held per warp at once.  A warp's item has up to
// 32 x 32 candidates but typically a few dozen; the queue is a window of the
// lane-major order, refilled from the lanes' masks when the rounds reach its
// end (kQCap is a multiple of 32, so a round never straddles two windows).
// Holding 256 instead of 1024 entries leaves 6 KB more of each SM's L1 to the
// narrow kernels' per-lane polygon arrays.
constexpr int kQCap = 256;

// Compact the warp's candidate masks (bit j of lane i: element pair (i, j))
// into queue entries (i | j << 5) in lane-major order; the entries at
// positions [from, from + kQCap) go to q.  Returns the total count.
__device__ __forceinline__ int build_queue(unsigned mask, unsigned short* q, int lane, int from = 0) {
  const int cnt = __popc(mask);
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  int w = incl - cnt;
  const int end = from + kQCap;
  if (w < end && incl > from) {
    while (mask) {
      const int j = __ffs(mask) - 1;
      mask &= mask - 1;
      if (w >= from && w < end) q[w - from] = (unsigned short)(lane | (j << 5));
      ++w;
    }
  }
  return __shfl_sync(0xffffffffu, incl, 31);
}

// Queue entry k of the warp's candidates: the round starting at `base`
// (a multiple of 32) first refills the window when it starts a new one.
__device__ __forceinline__ void queue_window(unsigned mask, unsigned short* q, int lane, int base) {
  if (base > 0 && base % kQCap == 0) {
    __syncwarp();
    build_queue(mask, q, lane, base);
    __syncwarp();
  }
}

// Unnormalised normals of the four faces of a tet (face k opposite vertex k).
__device__ __forceinline__ void tet_face_normals(const V3<float> X[4], V3<float> face[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int i0 = k == 0 ? 1 : 0;
    const int i1 = k <= 1 ? 2 : 1;
    const int i2 = k <= 2 ? 3 : 2;
    face[k] = cross(X[i1] - X[i0], X[i2] - X[i0]);
  }
}

// Writes record r of a kept polygon, keyed (item, seq).
template <int ND>
__device__ __forceinline__ void write_record(const StepArgs& a, int r, int item, int seq, int pair, int kind,
                                             const PV<float, ND>* poly, int nv, V3<float> anc, V3<float> n,
                                             V3<float> g, float gint, const V3<float>* X, const float (*clip)[3],
                                             int elem_a, int elem_b) {
  a.rec_key[r] = make_int2(item, seq);
  AdjPoly& R = a.recs[r];
  int l0 = 0, l1 = 0;
#pragma unroll 1
  for (int i = 0; i < kMaxPolyV; ++i) {
    const bool in = i < nv;
    *reinterpret_cast<float4*>(R.v[i]) =
        in ? make_float4(poly[i].x, poly[i].y, poly[i].z, poly[i].p) : make_float4(0.f, 0.f, 0.f, 0.f);
    const int lb = in ? (poly[i].lab & 0xFF) : 0;
    if (i < 4) l0 |= lb << (8 * i);
    else l1 |= lb << (8 * (i - 4));
  }
  R.anc[0] = anc.x; R.anc[1] = anc.y; R.anc[2] = anc.z; R.gint = gint;
  R.n[0] = n.x; R.n[1] = n.y; R.n[2] = n.z; R.lab0 = l0;
  R.g[0] = g.x; R.g[1] = g.y; R.g[2] = g.z; R.lab1 = l1;
  V3<float> face[4];
  tet_face_normals(X, face);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    R.face[k][0] = face[k].x; R.face[k][1] = face[k].y; R.face[k][2] = face[k].z;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int c = 0; c < 3; ++c) R.clip[j][c] = clip ? clip[j][c] : 0.f;
  R.pair = pair;
  R.nv = nv;
  R.kind = kind;
  R.elem_a = elem_a;
  R.elem_b = elem_b;
}

// Keeps this lane's polygon as an adjoint record.  All lanes of the warp
// call it together once per round (`have` marks a polygon); the record's key
// is (item, seq), seq being the polygon's rank among the item's polygons in
// processing order (rounds, then lanes), so the keys do not depend on the
// order in which warps reach the counter.
template <int ND>
__device__ __forceinline__ void keep_polygon(const StepArgs& a, bool have, int item, int& seq, int lane, int pair,
                                             int kind, const PV<float, ND>* poly, int nv, V3<float> anc,
                                             V3<float> n, V3<float> g, float gint, const V3<float>* X,
                                             const float (*clip)[3], int elem_a, int elem_b) {
  const unsigned b = __ballot_sync(0xffffffffu, have);
  if (!b) return;
  int base = 0;
  if (lane == 0) base = atomicAdd(a.rec_count, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  const int rank = __popc(b & ((1u << lane) - 1u));
  const int seq0 = seq;
  seq += __popc(b);
  if (!have) return;
  const int r = base + rank;
  if (r >= a.rec_cap) {
    atomicOr(a.status, 8);
    return;
  }
  write_record<ND>(a, r, item, seq0 + rank, pair, kind, poly, nv, anc, n, g, gint, X, clip, elem_a, elem_b);
}

constexpr int kNarrowWarps = 4;

// ============================================================================
// soft-rigid
// ============================================================================
struct TriStage {
  float n[3], o;       // plane (unit normal out of the rigid body, offset): FP32 head
  float en[3][3];      // in-plane inward edge planes: FP32 head
  float eo[3];
  float nl[3], ol;     // FP32 tails: head + tail is the FP64 plane to 2^-48
  float enl[3][3];
  float eol[3];
  float lo[3], hi[3];
  float M, h, Lt;      // coordinate magnitude, min altitude, max edge
  int orig, valid;
};

// True when the tet lies beyond one of the triangle's edge planes by more
// than the FP32 margin (all four vertices outside): its section would be
// clipped away whole.  sr_polygon makes the same test with the same values;
// here it keeps such pairs out of the candidate queue.
__device__ __forceinline__ bool edge_outside32(const float X[4][3], const TriStage& T, float xmax) {
  bool out = false;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float tol = 4e-6f * (xmax + fabsf(T.eo[j]));
    bool all_out = true;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float d = T.en[j][0] * X[k][0] + T.en[j][1] * X[k][1] + T.en[j][2] * X[k][2] - T.eo[j];
      all_out &= d < -tol;
    }
    out |= all_out;
  }
  return out;
}

// Double-float product of two (head, tail) values (the tail-tail product,
// below 2^-48 of the result, is dropped; unnormalised) and sum (normalised).
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  h = __fmul_rn(ah, bh);
  l = __fadd_rn(__fmaf_rn(ah, bh, -h), __fadd_rn(__fmul_rn(ah, bl), __fmul_rn(al, bh)));
}
__device__ __forceinline__ void df_sum(float ah, float al, float bh, float bl, float& h, float& l) {
  float s, e;
  two_sum(ah, bh, s, e);
  e = __fadd_rn(e, __fadd_rn(al, bl));
  h = __fadd_rn(s, e);
  l = __fsub_rn(e, __fsub_rn(h, s));
}

// A body-frame plane of the other body moved into the soft frame with the
// pair's transform: n = R n_b, o = o_b + n . t, in double-float arithmetic
// on the FP32 pipe (head and tail out).
__device__ __forceinline__ void df_plane_rotate(const FrameDev& F, const DfPlane& pb, float nh[3], float nl[3],
                                                float& oh, float& ol) {
  const float bh[3] = {pb.hi.x, pb.hi.y, pb.hi.z}, bl[3] = {pb.lo.x, pb.lo.y, pb.lo.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float h, l, h2, l2;
    df_mul(F.Rf[3 * k], F.Rlo[3 * k], bh[0], bl[0], h, l);
    df_mul(F.Rf[3 * k + 1], F.Rlo[3 * k + 1], bh[1], bl[1], h2, l2);
    df_sum(h, l, h2, l2, h, l);
    df_mul(F.Rf[3 * k + 2], F.Rlo[3 * k + 2], bh[2], bl[2], h2, l2);
    df_sum(h, l, h2, l2, nh[k], nl[k]);
  }
  float h = pb.hi.w, l = pb.lo.w;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float h2, l2;
    df_mul(nh[k], nl[k], F.tf[k], F.tlo[k], h2, l2);
    df_sum(h, l, h2, l2, h, l);
  }
  oh = h;
  ol = l;
}

__device__ __noinline__ void stage_tri(const StepArgs& a, const PairDev& P, const FrameDev& F, int tj,
                                          TriStage& S) {
  S.valid = 0;
  if (tj >= P.o_n_elem) return;
  const int idx = P.o_elem_off + tj;
  const float4 meta = a.tri_meta[idx];
  // plane: n = R n_body, o = o_body + n . t, in double-float (FP32 pipe)
  df_plane_rotate(F, a.tri_plane[idx], S.n, S.nl, S.o, S.ol);
  const V3<float> n = mk(S.n[0], S.n[1], S.n[2]);
  V3<float> Y[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 r = a.tris[3 * (size_t)idx + k];
    Y[k] = mat_mul<float>(F.Rf, mk(r.x, r.y, r.z)) + mk(F.tf[0], F.tf[1], F.tf[2]);
  }
  // edge planes: en = R en_body, eo = eo_body + en . t, in double-float
#pragma unroll
  for (int j = 0; j < 3; ++j) df_plane_rotate(F, a.tri_edges[3 * (size_t)idx + j], S.en[j], S.enl[j], S.eo[j], S.eol[j]);
  const float M = fmaxf(meta.z, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
  const float pad = 1e-5f * (M + meta.y) + 1e-7f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.lo[i] = fminf(fminf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]) - pad;
    S.hi[i] = fmaxf(fmaxf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]) + pad;
  }
  S.M = M; S.h = meta.x; S.Lt = meta.y;
  S.orig = a.tri_orig[idx];
  S.valid = meta.x > 0.f ? 1 : 0;
}

// The staged FP64 planes, head + tail.
__device__ __forceinline__ void tri_plane64(const TriStage& T, double n[3], double& o) {
#pragma unroll
  for (int k = 0; k < 3; ++k) n[k] = (double)T.n[k] + (double)T.nl[k];
  o = (double)T.o + (double)T.ol;
}
__device__ __forceinline__ void tri_edge64(const TriStage& T, int j, double m[3], double& o) {
#pragma unroll
  for (int k = 0; k < 3; ++k) m[k] = (double)T.en[j][k] + (double)T.enl[j][k];
  o = (double)T.eo[j] + (double)T.eol[j];
}

// n.x - o for a float point x and a double-float plane (heads nh, oh; tails
// nl, ol), on the FP32 pipe: the head products are split exactly by FMA and
// the sums carried by TwoSum, so the result (returned rounded to float) is
// within 2^-44 of the terms' magnitude of the FP64 value; a head within
// 1e-12 of zero sends the element pair to the FP64 path.
__device__ __forceinline__ float plane_df(const float* nh, const float* nl, float oh, float ol, float x, float y,
                                          float z) {
  const float p0 = __fmul_rn(nh[0], x), p1 = __fmul_rn(nh[1], y), p2 = __fmul_rn(nh[2], z);
  const float e0 = __fmaf_rn(nh[0], x, -p0), e1 = __fmaf_rn(nh[1], y, -p1), e2 = __fmaf_rn(nh[2], z, -p2);
  float s, t1, t2, t3;
  two_sum(p0, p1, s, t1);
  two_sum(s, p2, s, t2);
  two_sum(s, -oh, s, t3);
  const float tl = __fadd_rn(__fadd_rn(__fmul_rn(nl[0], x), __fmul_rn(nl[1], y)), __fmul_rn(nl[2], z));
  const float lo = __fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(e0, e1), e2), __fadd_rn(__fadd_rn(t1, t2), t3)),
                             __fsub_rn(ol, tl));
  return __fadd_rn(s, lo);
}

// Soft-rigid polygon: tet section by the triangle plane (FP64 values s),
// clipped by the three edge planes.  In FP32 an edge plane whose four tet
// distances are all certainly positive is inactive (no clip); an active
// plane's distances are evaluated in FP64 (its position matters to the
// area), then carried in FP32 and interpolated with the vertices.
template <class R, class S>
__device__ int sr_polygon(const TetIn<R>& t, const S s[4], const TriStage& T, V3<R> n, R M, Decide& dc,
                          int& anc, PV<R, 3>* out) {
  if (!(t.gl > (R)0)) return 0;
  const R cg = dot(n, t.g) / t.gl;
  check(dc, cg - (R)kCosAlphaD, (R)kFilt * ((R)1 + M / (R)T.h + t.kappa));
  if (!dc.unc && !(cg > (R)kCosAlphaD)) return 0;
  anc = nearest_vertex(s);
  PV<R, 3> tv[4];
  tet_local(t, anc, tv);
  bool active[3];
  R dmax[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    active[j] = true;
    if (sizeof(R) == 4) {
      const float tol = 4e-6f * ((float)t.xmax + fabsf(T.eo[j]));
      bool all_in = true, all_out = true;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float d = T.en[j][0] * (float)t.X[k].x + T.en[j][1] * (float)t.X[k].y + T.en[j][2] * (float)t.X[k].z -
                        T.eo[j];
        tv[k].d[j] = (R)d;
        all_in &= d > tol;
        all_out &= d < -tol;
      }
      if (all_out) return 0;
      active[j] = !all_in;
    }
    dmax[j] = 0;
    if (active[j]) {
      if (sizeof(R) == 4) {
        // double-float: the plane's position matters to the area
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          tv[k].d[j] = (R)plane_df(T.en[j], T.enl[j], T.eo[j], T.eol[j], (float)t.X[k].x, (float)t.X[k].y,
                                   (float)t.X[k].z);
          dmax[j] = fmax(dmax[j], abs_r(tv[k].d[j]));
        }
      } else {
        double m[3], eo;
        tri_edge64(T, j, m, eo);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          tv[k].d[j] = (R)(fma(m[2], (double)t.X[k].z, fma(m[1], (double)t.X[k].y, m[0] * (double)t.X[k].x)) - eo);
          dmax[j] = fmax(dmax[j], abs_r(tv[k].d[j]));
        }
      }
    }
  }
  int nv = tet_section(tv, s, dc, out);
  if (nv == 0) return 0;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    if (!active[j]) continue;
    nv = clip_dist(out, nv, j, (R)kFiltRel * dmax[j], dc);
    if (nv == 0) return 0;
  }
  return nv;
}

// Edge plane j of the staged triangle against the tet (FP32 with margins):
// -1 when all four vertices are certainly outside (no polygon), 0 when all
// are certainly inside (the plane clips nothing), 1 when it is active; then
// c is its double-float value at the anchor vertex (the plane's offset for
// the clip) and tol the clip margin.
__device__ __forceinline__ int edge_plane_f(const TetIn<float>& t, const TriStage& T, int j, int anc, float xr,
                                            float& c, float& tol) {
  const float tj = 4e-6f * (t.xmax + fabsf(T.eo[j]));
  bool all_in = true, all_out = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float d = T.en[j][0] * t.X[k].x + T.en[j][1] * t.X[k].y + T.en[j][2] * t.X[k].z - T.eo[j];
    all_in &= d > tj;
    all_out &= d < -tj;
  }
  c = 0.f;
  tol = 0.f;
  if (all_out) return -1;
  if (all_in) return 0;
  // double-float at the four vertices: the plane's position matters to the
  // area; the anchor's value is the plane's offset for the clip
  float dmax = 0.f;
#pragma unroll 1   // one copy of the evaluation (code size; sel4 keeps t.X in registers)
  for (int k = 0; k < 4; ++k) {
    const V3<float> x = sel4(t.X, k);
    const float d = plane_df(T.en[j], T.enl[j], T.eo[j], T.eol[j], x.x, x.y, x.z);
    dmax = fmaxf(dmax, fabsf(d));
    if (k == anc) c = d;
  }
  tol = (float)kFiltRel * (dmax + xr);
  return 1;
}

// The FP32 soft-rigid polygon: as sr_polygon, with vertices that carry no
// clip distances.  An active edge plane's distance is its double-float value
// at the anchor vertex plus the FP32 plane normal times the vertex's offset
// from the anchor; its margin covers that product's rounding (relative to
// the anchored tet's extent) as well as the distances' own, so every
// decision inside it still goes to the FP64 fallback.
__device__ __forceinline__ int sr_polygon_f(const TetIn<float>& t, const float s[4], const TriStage& T, V3<float> n,
                                            float M, Decide& dc, int& anc, PV<float, 0>* out) {
  if (!(t.gl > 0.f)) return 0;
  const float cg = dot(n, t.g) / t.gl;
  check(dc, cg - (float)kCosAlphaD, kFilt * (1.f + M / T.h + t.kappa));
  if (!dc.unc && !(cg > (float)kCosAlphaD)) return 0;
  anc = nearest_vertex(s);
  PV<float, 0> tv[4];
  tet_local(t, anc, tv);
  float xr = 0.f;   // the anchored tet's extent
#pragma unroll
  for (int k = 0; k < 4; ++k) xr = fmaxf(xr, fmaxf(fabsf(tv[k].x), fmaxf(fabsf(tv[k].y), fabsf(tv[k].z))));
  // the three edge planes in a loop that is not unrolled (one copy of the
  // double-float evaluation: the kernel's code, not its arithmetic, limits
  // it through instruction fetch); the per-plane results in scalars
  int act_mask = 0;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f, t0 = 0.f, t1 = 0.f, t2 = 0.f;
#pragma unroll 1
  for (int j = 0; j < 3; ++j) {
    float cj, tolj;
    const int r = edge_plane_f(t, T, j, anc, xr, cj, tolj);
    if (r < 0) return 0;
    if (r > 0) {
      act_mask |= 1 << j;
      if (j == 0) { c0 = cj; t0 = tolj; }
      else if (j == 1) { c1 = cj; t1 = tolj; }
      else { c2 = cj; t2 = tolj; }
    }
  }
  int nv = tet_section(tv, s, dc, out);
  if (nv == 0) return 0;
#pragma unroll 1
  for (int j = 0; j < 3; ++j) {
    if (!((act_mask >> j) & 1)) continue;
    const float cj = j == 0 ? c0 : (j == 1 ? c1 : c2);
    const float tj = j == 0 ? t0 : (j == 1 ? t1 : t2);
    nv = clip_pos(out, nv, j, T.en[j], cj, tj, dc);
    if (nv == 0) return 0;
  }
  return nv;
}

// Exact-decision fallback of one soft-rigid element pair in FP64 from the
// stored inputs (the section values too); returns the vertex count and sets
// near/gint.
__device__ __noinline__ int sr_fp64(const StepArgs& a, const TriStage& T, int tet_idx, int& anc,
                                    PV<float, 0>* poly, bool& near, float& gint) {
  TetIn<double> td;
  load_tet(a.tets, tet_idx, td);
  tet_prepare(td);
  double n64[3], o64;
  tri_plane64(T, n64, o64);
  double s[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) s[q] = fma(n64[2], td.X[q].z, fma(n64[1], td.X[q].y, n64[0] * td.X[q].x)) - o64;
  const V3<double> n = mk(n64[0], n64[1], n64[2]);
  Decide dd;
  PV<double, 3> pd[kMaxPolyV];
  const int nv = sr_polygon<double>(td, s, T, n, 0.0, dd, anc, pd);
  to_f(pd, nv, poly);
  near = dd.near;
  gint = grad_noise_rule(dot(td.g, n), td.gl);
  return nv;
}

// FP32 soft-rigid polygon (inlined: its inputs and outputs stay out of
// local memory where the compiler can keep them in registers).
__device__ __forceinline__ int sr_poly_f(const TetIn<float>& t, const float* s, const TriStage& T, V3<float> n,
                                      float M, Decide& dc, int& anc, PV<float, 0>* out) {
  return sr_polygon_f(t, s, T, n, M, dc, anc, out);
}

// shared memory of one warp of the soft-rigid kernel
struct SrWarpSmem {
  TriStage tri[kCluster];
  TetStage tet[kCluster];
  unsigned short q[kQCap];
};

// kKeep: polygons are kept as records (forces and rays come later from the
// records) rather than integrated and cast inline; kDiag: candidate or
// surface recording is on (hc_get_surface, debug).  Each launch carries only
// its own output paths.
template <bool kKeep, bool kDiag>
__global__ void __launch_bounds__(128, 5) narrow_sr_kernel(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SrWarpSmem& W = reinterpret_cast<SrWarpSmem*>(smem_raw)[wid];
  int staged_pair = -1, staged_oc = -1;   // other cluster held in W.tri
  while (true) {
    int ie;
    const int c0 = next_chunk(a, 0, lane, ie);
    if (c0 >= ie) break;
    const int c1 = min(c0 + a.chunk, ie);
  for (int item = c0; item < c1; ++item) {
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    Acc ac;
    acc_zero(ac);
    const int sl = it.y, oc = it.z;
    __syncwarp();
    if (F.valid) {
      if (it.x != staged_pair || oc != staged_oc) {
        stage_tri(a, P, F, oc * kCluster + lane, W.tri[lane]);
        staged_pair = it.x;
        staged_oc = oc;
      }
      stage_tet(a, P, sl * kCluster + lane, W.tet[lane]);
    } else {
      W.tri[lane].valid = 0;
      W.tet[lane].valid = 0;
      staged_pair = -1;
    }
    __syncwarp();
    // candidate queue
    unsigned mask = 0;
    const TetStage& me = W.tet[lane];
    if (me.valid) {
      float mlo[3], mhi[3];
      tet_box(me, mlo, mhi);
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TriStage& T = W.tri[j];
        if (!T.valid || !aabb_overlap(mlo, mhi, T.lo, T.hi)) continue;
        const float margin = 4e-6f * (me.xmax + fabsf(T.o) + T.Lt);
        if (one_sided32(me.X, T.n, T.o, margin) || edge_outside32(me.X, T, me.xmax)) continue;
        mask |= 1u << j;
      }
    }
    const int total = build_queue(mask, W.q, lane);
    __syncwarp();
    const float sgn = P.s_is_m ? 1.f : -1.f;
    int seq = 0;
    for (int base = 0; base < total; base += 32) {
      queue_window(mask, W.q, lane, base);
      const int k = base + lane;
      bool have = false;
      PV<float, 0> poly[kMaxPolyV];
      TetIn<float> t;
      V3<float> n = mk(0.f, 0.f, 0.f);
      int nv = 0, anc = 0, jt = 0, orig_a = 0, orig_b = 0, flags = 0;
      float gint = 0.f;
      do {
        if (k >= total) break;
        const int e = W.q[k % kQCap];
        const int i = e & 31, j = e >> 5;
        jt = j;
        const TetStage& TS = W.tet[i];
        const TriStage& T = W.tri[j];
        float s[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) s[q] = plane_df(T.n, T.nl, T.o, T.ol, TS.X[q][0], TS.X[q][1], TS.X[q][2]);
        constexpr float tol = (float)kNearTol;
        const bool allp = s[0] > tol && s[1] > tol && s[2] > tol && s[3] > tol;
        const bool alln = s[0] < -tol && s[1] < -tol && s[2] < -tol && s[3] < -tol;
        if (allp || alln) break;
        unstage_tet(TS, t);
        n = mk(T.n[0], T.n[1], T.n[2]);
        Decide dc;
        nv = sr_poly_f(t, s, T, n, fmaxf(T.M, t.xmax), dc, anc, poly);
        const int tet_idx = P.s_elem_off + sl * kCluster + i;
        if (dc.unc) {
          bool near;
          nv = sr_fp64(a, T, tet_idx, anc, poly, near, gint);
          orient_ccw(poly, nv, n);
          flags = near ? 1 : 0;
        } else if (nv >= 3) {
          gint = dot(t.g, n);
          if (fabsf(gint) <= 1e-5f * t.gl) {
            double n64[3], o64;
            tri_plane64(T, n64, o64);
            gint = grad_along64(a, tet_idx, n64[0], n64[1], n64[2]);
          }
        }
        if (nv < 3) break;
        ac.n_poly += 1;
        ac.n_near += flags;
        orig_a = TS.orig;
        orig_b = T.orig;
        have = true;
      } while (0);
      // forces, records and rays as separate phases the warp enters together
      __syncwarp();
      const V3<float> nc = n * sgn;
      if (have) {
        const float gM = P.s_is_m ? gint : INFINITY;
        const float gN = P.s_is_m ? INFINITY : gint;
        // with kept polygons the forces are integrated by rec_forward_kernel
        if constexpr (!kKeep) integrate_forces<0>(a, P, F, ac, poly, nv, sel4(t.X, anc), nc, gM, gN);
        if constexpr (kDiag) record<0>(a, it.x, poly, nv, sel4(t.X, anc), nc, orig_a, orig_b, flags);
      }
      __syncwarp();
      // with kept polygons the rays are cast by rec_forward_kernel
      if constexpr (!kKeep) {
        if (have) raster_polygon<0>(a, P, F, poly, nv, sel4(t.X, anc), nc, t.g);
      }
      __syncwarp();
      if constexpr (kKeep)
        keep_polygon<0>(a, have, item, seq, lane, it.x, 0, poly, nv, sel4(t.X, have ? anc : 0), n, t.g, gint, t.X,
                        W.tri[jt].en, orig_a, orig_b);
    }
    __syncwarp();
    warp_reduce_store<kKeep>(a, ac, item, lane);
  }
  }
}

constexpr size_t kSrSmemBytes = sizeof(SrWarpSmem) * kNarrowWarps;

// ---- soft-rigid, polygons kept as records: rounds across items ------------
//
// The adjoint step's forward soft-rigid narrow phase.  An item (32 tets of
// the soft body against a staged cluster of 32 triangles) typically holds
// well under 32 candidate element pairs, so a round per item leaves most
// lanes idle.  Here the candidates of consecutive items that share a pair
// and a triangle cluster go into one circular queue per warp, and a round
// takes the next 32 of them whatever their item.  A lane loads its
// candidate's tet from global memory (the filter phase has just read it, so
// the lines are in L1 or L2); nothing but the triangles is staged.  A record
// is keyed (item, rank of the polygon among its item's polygons in
// candidate order), the key narrow_sr_kernel gives it, so both kernels keep
// the same records in the same slots.

constexpr int kRing = 32;     // items with candidates pending in a warp's queue
constexpr int kRQCap = 256;   // queue entries per warp (a power of two)

// An item whose candidates are in the queue: its tets' base index, the
// polygons and near-degenerate polygons it has so far, the candidates left.
struct RingItem {
  int item, tet_base, seq, near, left;
};

// A lane's polygon in shared memory (in local memory the 24 warps' arrays
// outgrew the L1 beside the staging: 0.42 -> 0.39 ms at 4 CTAs per SM instead
// of 6), padded to an odd number of words so that lanes at the same vertex
// hit different banks.
struct LanePoly {
  PV<float, 0> v[kMaxPolyV];
  int pad;
};

struct SrKeepWarpSmem {
  TriStage tri[kCluster];
  RingItem ring[kRing];
  unsigned short q[kRQCap];   // ring slot | tet lane << 5 | triangle << 10
  LanePoly lp[32];            // each lane's polygon of the round
};

constexpr size_t kSrKeepSmemBytes = sizeof(SrKeepWarpSmem) * kNarrowWarps;

// CTAs per SM narrow_sr_keep_kernel is compiled for (its register budget;
// its shared memory, 47.6 KB per CTA, allows 4).
constexpr int kSrKeepCtas = 4;

// The item's counts (its forces come from the records later).
__device__ __forceinline__ void store_item_counts(const StepArgs& a, int item, int n_poly, int n_near) {
  ItemOut r;
#pragma unroll
  for (int i = 0; i < 8; ++i) r.hi[i] = r.lo[i] = 0.f;
  r.n_poly = n_poly; r.n_faces = 0; r.n_near = n_near; r.pad = 0;
  a.item_out[item] = r;
}

// One round of up to 32 queued candidates (nr of them, from queue position
// head): polygon, record, then the item bookkeeping.  Every lane calls it.
__device__ __forceinline__ void sr_keep_round(const StepArgs& a, SrKeepWarpSmem& W, int pair, int head, int nr,
                                              int lane) {
  const bool on = lane < nr;
  const int e = on ? W.q[(head + lane) & (kRQCap - 1)] : 0;
  const int slot = e & 31, i = (e >> 5) & 31, j = e >> 10;
  const int item = W.ring[slot].item, seq0 = W.ring[slot].seq;
  const int tet_idx = W.ring[slot].tet_base + i;
  bool have = false;
  PV<float, 0>* poly = W.lp[lane].v;
  TetIn<float> t;
  V3<float> n = mk(0.f, 0.f, 0.f);
  int nv = 0, anc = 0, orig_a = 0, orig_b = 0, flags = 0;
  float gint = 0.f;
  do {
    if (!on) break;
    const TriStage& T = W.tri[j];
    load_tet(a.tets, tet_idx, t);
    const float4 p0 = a.tet_props[2 * (size_t)tet_idx], p1 = a.tet_props[2 * (size_t)tet_idx + 1];
    t.g = mk(p0.x, p0.y, p0.z);
    t.gl = p0.w; t.kappa = p1.x; t.xmax = p1.y; t.pmax = p1.z;
    t.c = 0.f; t.hmin = 0.f;
    float s[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) s[q] = plane_df(T.n, T.nl, T.o, T.ol, t.X[q].x, t.X[q].y, t.X[q].z);
    constexpr float tol = (float)kNearTol;
    const bool allp = s[0] > tol && s[1] > tol && s[2] > tol && s[3] > tol;
    const bool alln = s[0] < -tol && s[1] < -tol && s[2] < -tol && s[3] < -tol;
    if (allp || alln) break;
    n = mk(T.n[0], T.n[1], T.n[2]);
    Decide dc;
    nv = sr_poly_f(t, s, T, n, fmaxf(T.M, t.xmax), dc, anc, poly);
    if (dc.unc) {
      bool near;
      nv = sr_fp64(a, T, tet_idx, anc, poly, near, gint);
      orient_ccw(poly, nv, n);
      flags = near ? 1 : 0;
    } else if (nv >= 3) {
      gint = dot(t.g, n);
      if (fabsf(gint) <= 1e-5f * t.gl) {
        double n64[3], o64;
        tri_plane64(T, n64, o64);
        gint = grad_along64(a, tet_idx, n64[0], n64[1], n64[2]);
      }
    }
    if (nv < 3) break;
    orig_a = a.tet_orig[tet_idx];
    orig_b = T.orig;
    have = true;
  } while (0);
  __syncwarp();
  // the polygon's rank among its item's: the item's earlier polygons plus
  // this round's on lower lanes of the same item
  const unsigned hv = __ballot_sync(0xffffffffu, have);
  const unsigned nm = __ballot_sync(0xffffffffu, have && flags);
  const unsigned same = __match_any_sync(0xffffffffu, on ? slot : 32 + lane);
  const unsigned lt = (1u << lane) - 1u;
  if (hv) {
    int base = 0;
    if (lane == 0) base = atomicAdd(a.rec_count, __popc(hv));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (have) {
      const int r = base + __popc(hv & lt);
      if (r >= a.rec_cap) atomicOr(a.status, 8);
      else
        write_record<0>(a, r, item, seq0 + __popc(same & hv & lt), pair, 0, poly, nv, sel4(t.X, anc), n, t.g, gint,
                        t.X, W.tri[j].en, orig_a, orig_b);
    }
  }
  // the highest lane of each item's run updates the item; an item whose
  // last candidate this was stores its counts
  if (on && (same >> lane) == 1u) {
    RingItem& R = W.ring[slot];
    R.seq += __popc(same & hv);
    R.near += __popc(same & nm);
    R.left -= __popc(same);
    if (R.left == 0) store_item_counts(a, R.item, R.seq, R.near);
  }
  __syncwarp();
}

// A float's bits as an int of the same order (for warp min/max reductions).
__device__ __forceinline__ int ordered_bits(float f) {
  const int i = __float_as_int(f);
  return i ^ ((i >> 31) & 0x7fffffff);
}

// The tet at idx against the staged triangles that can reach the warp's
// tets (tmask, from the union of their boxes): narrow_sr_kernel's per-pair
// tests on the same values.  Returns the candidate mask.
__device__ __forceinline__ unsigned sr_filter(const StepArgs& a, const SrKeepWarpSmem& W, int idx, bool in,
                                              int n_o, int lane) {
  float X[4][3];
  float mlo[3], mhi[3], xmax = 0.f;
  bool tv = false;
  if (in) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 v = a.tets[4 * (size_t)idx + k];
      X[k][0] = v.x; X[k][1] = v.y; X[k][2] = v.z;
    }
    const float4 p1 = a.tet_props[2 * (size_t)idx + 1];
    tv = p1.w > 0.f;
    xmax = p1.y;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    mlo[c] = INFINITY;
    mhi[c] = -INFINITY;
    if (tv) {
      const float l = fminf(fminf(X[0][c], X[1][c]), fminf(X[2][c], X[3][c]));
      const float h = fmaxf(fmaxf(X[0][c], X[1][c]), fmaxf(X[2][c], X[3][c]));
      const float pad = 1e-5f * (fabsf(l) + fabsf(h)) + 1e-7f;
      mlo[c] = l - pad;
      mhi[c] = h + pad;
    }
  }
  // the triangles whose box meets the union of the tets' boxes (a triangle
  // that misses the union misses every tet's box): lane j tests triangle j
  float clo[3], chi[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int lo = __reduce_min_sync(0xffffffffu, ordered_bits(mlo[c]));
    const int hi = __reduce_max_sync(0xffffffffu, ordered_bits(mhi[c]));
    clo[c] = __int_as_float(lo ^ ((lo >> 31) & 0x7fffffff));
    chi[c] = __int_as_float(hi ^ ((hi >> 31) & 0x7fffffff));
  }
  bool reach = false;
  if (lane < n_o) {
    const TriStage& T = W.tri[lane];
    reach = T.valid && aabb_overlap(clo, chi, T.lo, T.hi);
  }
  unsigned tmask = __ballot_sync(0xffffffffu, reach);
  unsigned mask = 0;
  if (!tv) return 0;
  while (tmask) {
    const int jj = __ffs(tmask) - 1;
    tmask &= tmask - 1;
    const TriStage& T = W.tri[jj];
    if (!aabb_overlap(mlo, mhi, T.lo, T.hi)) continue;
    const float margin = 4e-6f * (xmax + fabsf(T.o) + T.Lt);
    if (one_sided32(X, T.n, T.o, margin) || edge_outside32(X, T, xmax)) continue;
    mask |= 1u << jj;
  }
  return mask;
}

// One loop step does one of: a round of queued candidates, a window of the
// current item's candidates into the queue, or the next item (staging its
// triangles, filtering its tets).  The round has one call site.
template <int kMinCtas>
__global__ void __launch_bounds__(128, kMinCtas) narrow_sr_keep_kernel(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SrKeepWarpSmem& W = reinterpret_cast<SrKeepWarpSmem*>(smem_raw)[wid];
  int staged_pair = -1, staged_oc = -1;
  int head = 0, pending = 0, ring_ctr = 0;   // queue state, the same on every lane
  int nxt = 0, end = 0;                      // the warp's chunk of items
  int held = -1;                             // an item waiting for the queue to drain
  bool drain = false, finished = false;
  int from = 0, total = 0, slot = 0, w0 = 0; // the item being appended
  unsigned mask = 0;
  while (true) {
    if (pending >= 32 || (pending > 0 && drain)) {
      const int nr = min(32, pending);
      sr_keep_round(a, W, staged_pair, head, nr, lane);
      head += nr;
      pending -= nr;
      continue;
    }
    if (from < total) {
      // the next window of the item's lane-major candidates
      const int nput = min(total - from, kRQCap - pending);
      const int tail = head + pending;
      int w = w0;
      const int incl = w0 + __popc(mask);
      if (w < from + nput && incl > from) {
        unsigned m = mask;
        while (m) {
          const int jj = __ffs(m) - 1;
          m &= m - 1;
          if (w >= from && w < from + nput)
            W.q[(tail + w - from) & (kRQCap - 1)] = (unsigned short)(slot | (lane << 5) | (jj << 10));
          ++w;
        }
      }
      from += nput;
      pending += nput;
      __syncwarp();
      continue;
    }
    drain = false;
    int item = held;
    if (item < 0) {
      if (nxt >= end) {
        if (finished) break;
        int ie;
        const int c0 = next_chunk(a, 0, lane, ie);
        if (c0 >= ie) {
          finished = true;
          drain = true;
          continue;
        }
        nxt = c0;
        end = min(c0 + a.chunk, ie);
      }
      item = nxt++;
    }
    held = -1;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    const int sl = it.y, oc = it.z;
    if (!F.valid) {
      if (lane == 0) store_item_counts(a, item, 0, 0);
      continue;
    }
    if (it.x != staged_pair || oc != staged_oc) {
      if (pending > 0) {
        // the queued candidates read the staged triangles: finish them first
        held = item;
        drain = true;
        continue;
      }
      __syncwarp();
      stage_tri(a, P, F, oc * kCluster + lane, W.tri[lane]);
      staged_pair = it.x;
      staged_oc = oc;
      __syncwarp();
    }
    const int ti = sl * kCluster + lane;
    mask = sr_filter(a, W, P.s_elem_off + ti, ti < P.s_n_elem, min(kCluster, P.o_n_elem - oc * kCluster), lane);
    // lane-major positions of this lane's candidates
    const int cnt = __popc(mask);
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    w0 = incl - cnt;
    total = __shfl_sync(0xffffffffu, incl, 31);
    from = 0;
    if (total == 0) {
      if (lane == 0) store_item_counts(a, item, 0, 0);
      continue;
    }
    slot = ring_ctr & (kRing - 1);
    ++ring_ctr;
    if (lane == 0) {
      RingItem& R = W.ring[slot];
      R.item = item; R.tet_base = P.s_elem_off + sl * kCluster; R.seq = 0; R.near = 0; R.left = total;
    }
  }
}

// ============================================================================
// soft vs rigid half-space
// ============================================================================
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

__device__ __noinline__ int hs_poly_f(const TetIn<float>& t, const double* s, V3<float> n, Decide& dc, int& anc,
                                      PV<float, 1>* out) {
  return hs_polygon<float>(t, s, n, dc, anc, out);
}

__device__ __noinline__ int hs_fp64(const StepArgs& a, const FrameDev& F, int tet_idx, const double s[4], int& anc,
                                    PV<float, 1>* poly, bool& near, float& gint) {
  TetIn<double> td;
  load_tet(a.tets, tet_idx, td);
  tet_prepare(td);
  const V3<double> nd = mk(F.R[2], F.R[5], F.R[8]);
  Decide dd;
  PV<double, 1> pd[kMaxPolyV];
  const int nv = hs_polygon<double>(td, s, nd, dd, anc, pd);
  to_f(pd, nv, poly);
  near = dd.near;
  gint = grad_noise_rule(dot(td.g, nd), td.gl);
  return nv;
}

template <bool kKeep, bool kDiag>
__global__ void __launch_bounds__(128, 4) narrow_hs_kernel(StepArgs a) {
  __shared__ TetStage s_tet[kNarrowWarps][kCluster];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  while (true) {
    int ie;
    const int item = next_item(a, 1, lane, ie);
    if (item >= ie) break;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    Acc ac;
    acc_zero(ac);
    const int sl = it.y;
    if (F.valid) stage_tet(a, P, sl * kCluster + lane, s_tet[wid][lane]);
    else s_tet[wid][lane].valid = 0;
    const double n64[3] = {F.R[2], F.R[5], F.R[8]};
    const double o64 = F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2];
    const float nf[3] = {F.Rf[2], F.Rf[5], F.Rf[8]};
    const float of = (float)o64;
    // crossing tets, compacted
    bool cand = false;
    {
      const TetStage& me = s_tet[wid][lane];
      cand = me.valid && !one_sided32(me.X, nf, of, 4e-6f * (me.xmax + fabsf(of)));
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, cand);
    const int total = __popc(ballot);
    const float sgn = P.s_is_m ? 1.f : -1.f;
    bool have = false;
    PV<float, 1> poly[kMaxPolyV];
    TetIn<float> t;
    const V3<float> n = mk(nf[0], nf[1], nf[2]);
    int nv = 0, anc = 0, orig_a = 0, flags = 0;
    float gint = 0.f;
    if (lane < total) {
      // the lane-th set bit of the ballot
      unsigned m = ballot;
      for (int r = 0; r < lane; ++r) m &= m - 1;
      const int i = __ffs(m) - 1;
      const TetStage& TS = s_tet[wid][i];
      double s[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q] = plane64(n64, o64, TS.X[q][0], TS.X[q][1], TS.X[q][2]);
      unstage_tet(TS, t);
      Decide dc;
      nv = hs_poly_f(t, s, n, dc, anc, poly);
      const int tet_idx = P.s_elem_off + sl * kCluster + i;
      if (dc.unc) {
        bool near;
        nv = hs_fp64(a, F, tet_idx, s, anc, poly, near, gint);
        orient_ccw(poly, nv, n);
        flags = near ? 1 : 0;
      } else if (nv >= 3) {
        gint = dot(t.g, n);
        if (fabsf(gint) <= 1e-5f * t.gl) gint = grad_along64(a, tet_idx, n64[0], n64[1], n64[2]);
      }
      if (nv >= 3) {
        ac.n_poly += 1;
        ac.n_near += flags;
        orig_a = TS.orig;
        have = true;
      }
    }
    // forces, records and rays as separate phases the warp enters together
    __syncwarp();
    const V3<float> nc = n * sgn;
    if (have) {
      const float gM = P.s_is_m ? gint : INFINITY;
      const float gN = P.s_is_m ? INFINITY : gint;
      if constexpr (!kKeep) integrate_forces<1>(a, P, F, ac, poly, nv, t.X[anc], nc, gM, gN);
      if constexpr (kDiag) record<1>(a, it.x, poly, nv, t.X[anc], nc, orig_a, -1, flags);
    }
    __syncwarp();
    if constexpr (!kKeep) {
      if (have) raster_polygon<1>(a, P, F, poly, nv, t.X[anc], nc, t.g);
    }
    __syncwarp();
    if constexpr (kKeep) {
      int seq = 0;
      keep_polygon<1>(a, have, item, seq, lane, it.x, 1, poly, nv, t.X[have ? anc : 0], n, t.g, gint, t.X, nullptr,
                      orig_a, -1);
    }
    __syncwarp();
    warp_reduce_store<kKeep>(a, ac, item, lane);
  }
}

// ============================================================================
// soft-soft
// ============================================================================
struct TetBStage {
  double g64[3], c64;  // FP64 field of the B tet in A's frame
  float g[3], gl;
  float pn[4][3], po[4];     // face planes (inward unit normal, offset) in A's frame, from
                             // the FP64 vertices, rounded to FP32
  float lo[3], hi[3];
  float M, h, kappa;
  int orig, valid;
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

__device__ __forceinline__ void stage_tetb(const StepArgs& a, const PairDev& P, const FrameDev& F, int tj,
                                           TetBStage& S) {
  S.valid = 0;
  if (tj >= P.o_n_elem) return;
  const int idx = P.o_elem_off + tj;
  TetIn<double> bd;
  tetb_fp64(a, F, idx, bd);
  TetIn<float> tb;
  float M = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 r = a.tets[4 * (size_t)idx + k];
    M = fmaxf(M, amax(mk(r.x, r.y, r.z)));
    tb.X[k] = mk((float)bd.X[k].x, (float)bd.X[k].y, (float)bd.X[k].z);
    tb.P[k] = r.w;
  }
  M = fmaxf(M, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
  tet_prepare(tb);
  // the face planes in FP64 from the FP64 vertices (not from the vertices
  // rounded to FP32), then rounded
  V3<double> pn[4];
  double po[4];
  tet_planes(bd.X, pn, po);
  S.g64[0] = bd.g.x; S.g64[1] = bd.g.y; S.g64[2] = bd.g.z; S.c64 = bd.c;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    S.pn[k][0] = (float)pn[k].x; S.pn[k][1] = (float)pn[k].y; S.pn[k][2] = (float)pn[k].z;
    S.po[k] = (float)po[k];
  }
  S.g[0] = tb.g.x; S.g[1] = tb.g.y; S.g[2] = tb.g.z; S.gl = tb.gl;
  const float pad = 1e-5f * M + 1e-7f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    S.lo[i] = fminf(fminf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fminf((&tb.X[2].x)[i], (&tb.X[3].x)[i])) - pad;
    S.hi[i] = fmaxf(fmaxf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fmaxf((&tb.X[2].x)[i], (&tb.X[3].x)[i])) + pad;
  }
  S.M = M; S.h = tb.hmin; S.kappa = tb.kappa;
  S.orig = a.tet_orig[idx];
  S.valid = tb.hmin > 0.f && bd.hmin > 0.0 ? 1 : 0;
}

// Soft-soft polygon: tet A's section by p_A - p_B = 0 (FP64 values s),
// clipped by tet B's faces.
template <class R>
__device__ int ss_polygon(const TetIn<R>& ta, const double s[4], V3<R> gb, R glb, V3<R> nrm, R lm,
                          const V3<R> pn[4], const R po[4], R Mb, R hb, R kb, Decide& dc, int& anc, PV<R, 4>* out) {
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
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    nv = clip_dist(out, nv, j, tol_p + (R)kFiltRel * dmax[j], dc);
    if (nv == 0) return 0;
  }
  return nv;
}

// FP64 pass of one soft-soft element pair: the exact-decision fallback
// (`full`) or only the gradient components near zero.
__device__ __noinline__ int ss_fp64(const StepArgs& a, const FrameDev& F, int ta_idx, int tb_idx, const double s[4],
                                    bool full, int& anc, PV<float, 4>* poly, bool& near, V3<float>& nrm, float& gM,
                                    float& gN, int nv_in) {
  TetIn<double> td, tbd;
  load_tet(a.tets, ta_idx, td);
  tet_prepare(td);
  tetb_fp64(a, F, tb_idx, tbd);
  const V3<double> md = td.g - tbd.g;
  const double lmd = norm(md);
  near = false;
  if (!(lmd > 0.0)) return 0;
  const V3<double> nrmd = md * (1.0 / lmd);
  int nv = nv_in;
  if (full) {
    V3<double> pnd[4];
    double pod[4];
    tet_planes(tbd.X, pnd, pod);
    Decide dd;
    PV<double, 4> pd[kMaxPolyV];
    nv = ss_polygon<double>(td, s, tbd.g, tbd.gl, nrmd, lmd, pnd, pod, 0.0, 1.0, 0.0, dd, anc, pd);
    to_f(pd, nv, poly);
    near = dd.near;
    nrm = mk((float)nrmd.x, (float)nrmd.y, (float)nrmd.z);
  }
  gM = grad_noise_rule(dot(td.g, nrmd), td.gl);
  gN = grad_noise_rule(-dot(tbd.g, nrmd), tbd.gl);
  return nv;
}

// One soft-soft element pair: tet A (soft frame) against the staged tet B.
// Its polygon relative to A's vertex `anc`, the unit normal (g_A - g_B) / |.|
// (out of N into M), gM = g_A . n and gN = -g_B . n, with the FP64 pass where
// the FP32 decisions or gradient terms are uncertain (`flags` 1: a value
// was near zero in FP64).  The adjoint recomputes the forward's polygons
// (and so its ray keys) with this same code.  Returns the vertex count.
__device__ __forceinline__ int ss_element_pair(const StepArgs& a, const FrameDev& F, const TetIn<float>& t,
                                               const TetBStage& B, int ta_idx, int tb_idx, PV<float, 4>* poly,
                                               int& anc, V3<float>& nrm, float& gM, float& gN, int& flags) {
  const V3<float> gb = mk(B.g[0], B.g[1], B.g[2]);
  const V3<float> m = t.g - gb;
  const float lm = norm(m);
  if (!(lm > 0.f) || !(t.gl > 0.f) || !(B.gl > 0.f)) return 0;
  double s[4];
  const double il = 1.0 / (double)lm;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    s[q] = ((double)t.P[q] - (fma(B.g64[2], (double)t.X[q].z, fma(B.g64[1], (double)t.X[q].y, B.g64[0] * (double)t.X[q].x)) +
                              B.c64)) * il;
  const bool allp = s[0] > kNearTol && s[1] > kNearTol && s[2] > kNearTol && s[3] > kNearTol;
  const bool alln = s[0] < -kNearTol && s[1] < -kNearTol && s[2] < -kNearTol && s[3] < -kNearTol;
  if (allp || alln) return 0;
  const V3<float> pn[4] = {mk(B.pn[0][0], B.pn[0][1], B.pn[0][2]), mk(B.pn[1][0], B.pn[1][1], B.pn[1][2]),
                           mk(B.pn[2][0], B.pn[2][1], B.pn[2][2]), mk(B.pn[3][0], B.pn[3][1], B.pn[3][2])};
  nrm = m * (1.f / lm);
  Decide dc;
  anc = 0;
  int nv = ss_polygon<float>(t, s, gb, B.gl, nrm, lm, pn, B.po, B.M, B.h, B.kappa, dc, anc, poly);
  gM = dot(t.g, nrm);
  gN = -dot(gb, nrm);
  flags = 0;
  if (dc.unc || (nv >= 3 && (fabsf(gM) <= 1e-5f * t.gl || fabsf(gN) <= 1e-5f * B.gl))) {
    bool near;
    nv = ss_fp64(a, F, ta_idx, tb_idx, s, dc.unc, anc, poly, near, nrm, gM, gN, nv);
    if (dc.unc) orient_ccw(poly, nv, nrm);
    flags = near ? 1 : 0;
  }
  return nv;
}

// Stages one soft-soft item in the warp's shared memory (its 32 A tets and,
// in A's frame, 32 B tets) and queues the element pairs whose boxes
// overlap.  Returns the queue length (the warp is synchronised).
__device__ __forceinline__ int ss_stage_item(const StepArgs& a, const PairDev& P, const FrameDev& F, int sl, int oc,
                                             TetBStage* tb, TetStage* tet, unsigned short* q, int lane,
                                             unsigned& mask) {
  if (F.valid) {
    stage_tetb(a, P, F, oc * kCluster + lane, tb[lane]);
    stage_tet(a, P, sl * kCluster + lane, tet[lane]);
  } else {
    tb[lane].valid = 0;
    tet[lane].valid = 0;
  }
  __syncwarp();
  mask = 0;
  const TetStage& me = tet[lane];
  if (me.valid) {
    float mlo[3], mhi[3];
    tet_box(me, mlo, mhi);
    const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
    for (int j = 0; j < n_o; ++j) {
      const TetBStage& B = tb[j];
      if (B.valid && aabb_overlap(mlo, mhi, B.lo, B.hi)) mask |= 1u << j;
    }
  }
  const int total = build_queue(mask, q, lane);
  __syncwarp();
  return total;
}

__global__ void __launch_bounds__(128, 4) narrow_ss_kernel(StepArgs a) {
  __shared__ TetBStage s_tb[kNarrowWarps][kCluster];
  __shared__ TetStage s_tet[kNarrowWarps][kCluster];
  __shared__ unsigned short s_q[kNarrowWarps][kQCap];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  while (true) {
    int ie;
    const int item = next_item(a, 2, lane, ie);
    if (item >= ie) break;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    Acc ac;
    acc_zero(ac);
    const int sl = it.y, oc = it.z;
    unsigned mask;
    const int total = ss_stage_item(a, P, F, sl, oc, s_tb[wid], s_tet[wid], s_q[wid], lane, mask);
    for (int base = 0; base < total; base += 32) {
      queue_window(mask, s_q[wid], lane, base);
      const int k = base + lane;
      if (k >= total) continue;
      const int e = s_q[wid][k % kQCap];
      const int i = e & 31, j = e >> 5;
      const TetStage& TS = s_tet[wid][i];
      const TetBStage& B = s_tb[wid][j];
      TetIn<float> t;
      unstage_tet(TS, t);
      PV<float, 4> poly[kMaxPolyV];
      int anc = 0, flags = 0;
      V3<float> nrm;
      float gM, gN;
      const int ta_idx = P.s_elem_off + sl * kCluster + i, tb_idx = P.o_elem_off + oc * kCluster + j;
      const int nv = ss_element_pair(a, F, t, B, ta_idx, tb_idx, poly, anc, nrm, gM, gN, flags);
      if (nv < 3) continue;
      ac.n_poly += 1;
      ac.n_near += flags;
      integrate_polygon<4>(a, P, F, ac, poly, nv, t.X[anc], nrm, gM, gN, t.g);
      record<4>(a, it.x, poly, nv, t.X[anc], nrm, TS.orig, B.orig, flags);
    }
    __syncwarp();
    warp_reduce_store(a, ac, item, lane);
  }
}
