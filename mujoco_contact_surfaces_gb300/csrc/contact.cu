// contact.cu — the per-step device pipeline of the hydroelastic contact path.
//
//   frames_kernel     pair setup: relative transforms (FP64), velocity field,
//                     sensor frames (the pose/velocity fetches of
//                     passiveCallback, mujoco_contact_surfaces_plugin.cpp:435-451)
//   bp_count_kernel   cluster-level broadphase over the LBVH, counts
//   bp_scan_kernel    exclusive scan of the per-block counts
//   bp_emit_kernel    block prefix-scan compaction of work items
//   narrow_kernel     per item: element tests, clipping, quadrature
//                     (P:320-409), Hunt-Crossley + friction,
//                     taxel binning (flat_tactile_sensor.cpp:262-402)
//   reduce_kernel     deterministic FP64 per-pair wrench
//   taxel_kernel      per-cell sums of the binned samples
#include <cuda_runtime.h>
#include <stdint.h>

#include "clip.cuh"
#include "kernels.h"

namespace hc {

// ---------------------------------------------------------------------------
// LBVH build / refit
// ---------------------------------------------------------------------------
// One CTA per geom: leaf boxes from the 32 elements of each cluster, then the
// internal nodes level by level.  Elements are float4 vertices (x, y, z, *),
// `vpe` per element.
__global__ void refit_kernel(const float4* __restrict__ elems, int vpe, float4* __restrict__ nodes,
                             const int* __restrict__ geom_elem_off, const int* __restrict__ geom_n_elem,
                             const int* __restrict__ geom_node_off, const int* __restrict__ geom_leaves) {
  const int g = blockIdx.x;
  const int eoff = geom_elem_off[g], ne = geom_n_elem[g], L = geom_leaves[g];
  float4* nd = nodes + 2 * (size_t)geom_node_off[g];
  const int ncl = (ne + kCluster - 1) / kCluster;
  for (int c = threadIdx.x; c < L; c += blockDim.x) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (c < ncl) {
      int e0 = c * kCluster, e1 = min(ne, e0 + kCluster);
      for (int e = e0; e < e1; ++e)
        for (int k = 0; k < vpe; ++k) {
          float4 v = elems[(size_t)(eoff + e) * vpe + k];
          lo[0] = fminf(lo[0], v.x); lo[1] = fminf(lo[1], v.y); lo[2] = fminf(lo[2], v.z);
          hi[0] = fmaxf(hi[0], v.x); hi[1] = fmaxf(hi[1], v.y); hi[2] = fmaxf(hi[2], v.z);
        }
    }
    nd[2 * (L + c)] = make_float4(lo[0], lo[1], lo[2], 0.f);
    nd[2 * (L + c) + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
  }
  __syncthreads();
  for (int w = L >> 1; w >= 1; w >>= 1) {
    for (int k = w + threadIdx.x; k < 2 * w; k += blockDim.x) {
      float4 a = nd[2 * (2 * k)], b = nd[2 * (2 * k + 1)];
      float4 c = nd[2 * (2 * k) + 1], d = nd[2 * (2 * k + 1) + 1];
      nd[2 * k] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.f);
      nd[2 * k + 1] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.f);
    }
    __syncthreads();
  }
}

void launch_refit(const float4* elems, int vpe, float4* nodes, const int* geom_elem_off, const int* geom_n_elem,
                  const int* geom_node_off, const int* geom_leaves, int n_geoms, cudaStream_t s) {
  if (n_geoms <= 0) return;
  refit_kernel<<<n_geoms, 256, 0, s>>>(elems, vpe, nodes, geom_elem_off, geom_n_elem, geom_node_off, geom_leaves);
}

// ---------------------------------------------------------------------------
// pair frames
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool finite_d(double x) { return isfinite(x); }

__global__ void frames_kernel(StepArgs a) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n_pair) return;
  const PairDev P = a.pairs[p];
  FrameDev F;
  if (P.query == 0) {   // unsupported pair: no poses are read
    memset(&F, 0, sizeof(F));
    a.frames[p] = F;
    return;
  }
  const double* RS = a.xmat + 9 * (size_t)P.gs;
  const double* RO = a.xmat + 9 * (size_t)P.go;
  V3<double> xS = mk(a.xpos[3 * P.gs], a.xpos[3 * P.gs + 1], a.xpos[3 * P.gs + 2]);
  V3<double> xO = mk(a.xpos[3 * P.go], a.xpos[3 * P.go + 1], a.xpos[3 * P.go + 2]);
  bool ok = true;
  for (int i = 0; i < 9; ++i) {
    F.RS[i] = RS[i];
    ok &= finite_d(RS[i]) && finite_d(RO[i]);
  }
  ok &= finite_d(xS.x) && finite_d(xS.y) && finite_d(xS.z) && finite_d(xO.x) && finite_d(xO.y) && finite_d(xO.z);
  // R = RS^T RO, t = RS^T (xO - xS)
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      F.R[3 * i + j] = RS[i] * RO[j] + RS[3 + i] * RO[3 + j] + RS[6 + i] * RO[6 + j];
  V3<double> t = mat_tmul<double>(RS, xO - xS);
  F.t[0] = t.x; F.t[1] = t.y; F.t[2] = t.z;
  F.xS[0] = xS.x; F.xS[1] = xS.y; F.xS[2] = xS.z;
  for (int i = 0; i < 3; ++i) {
    F.xM[i] = a.xpos[3 * P.gm + i];
    F.xN[i] = a.xpos[3 * P.gn + i];
  }
  for (int i = 0; i < 9; ++i) F.Rf[i] = (float)F.R[i];
  for (int i = 0; i < 3; ++i) F.tf[i] = (float)F.t[i];
  // velocity field v_M - v_N = c + w x p (world), in the soft frame
  V3<double> wM = mk(0.0, 0.0, 0.0), vM = wM, wN = wM, vN = wM;
  if (a.vel) {
    const double* VM = a.vel + 6 * (size_t)P.gm;
    const double* VN = a.vel + 6 * (size_t)P.gn;
    wM = mk(VM[0], VM[1], VM[2]); vM = mk(VM[3], VM[4], VM[5]);
    wN = mk(VN[0], VN[1], VN[2]); vN = mk(VN[3], VN[4], VN[5]);
    for (int i = 0; i < 6; ++i) ok &= finite_d(VM[i]) && finite_d(VN[i]);
  }
  V3<double> xM = mk(F.xM[0], F.xM[1], F.xM[2]), xN = mk(F.xN[0], F.xN[1], F.xN[2]);
  V3<double> c = vM - vN - cross(wM, xM) + cross(wN, xN);
  V3<double> w = wM - wN;
  V3<double> lin = mat_tmul<double>(RS, c + cross(w, xS));
  V3<double> ang = mat_tmul<double>(RS, w);
  F.lin[0] = (float)lin.x; F.lin[1] = (float)lin.y; F.lin[2] = (float)lin.z;
  F.ang[0] = (float)ang.x; F.ang[1] = (float)ang.y; F.ang[2] = (float)ang.z;
  // soft -> sensor local frames
  for (int q = 0; q < 2; ++q) {
    int sid = q == 0 ? P.sensor0 : P.sensor1;
    float* Rl = q == 0 ? F.Rl : F.Rl1;
    float* tl = q == 0 ? F.tl : F.tl1;
    if (sid < 0) {
      for (int i = 0; i < 9; ++i) Rl[i] = 0.f;
      for (int i = 0; i < 3; ++i) tl[i] = 0.f;
      continue;
    }
    int gq = a.sensors[sid].geom;
    const double* RQ = a.xmat + 9 * (size_t)gq;
    V3<double> xQ = mk(a.xpos[3 * gq], a.xpos[3 * gq + 1], a.xpos[3 * gq + 2]);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        Rl[3 * i + j] = (float)(RQ[i] * RS[j] + RQ[3 + i] * RS[3 + j] + RQ[6 + i] * RS[6 + j]);
    V3<double> tq = mat_tmul<double>(RQ, xS - xQ);
    tl[0] = (float)tq.x; tl[1] = (float)tq.y; tl[2] = (float)tq.z;
  }
  F.valid = ok ? 1 : 0;
  F.pad = 0;
  a.frames[p] = F;
}

// ---------------------------------------------------------------------------
// broadphase over the implicit cluster trees
// ---------------------------------------------------------------------------
struct QueryBox {
  float c[3], h[3];   // centre and half extents in the soft frame (padded)
  int plane;          // 1: straddle test against n.x = o instead
  float n[3], o, r;   // plane (plane query), r = pad
};

__device__ __forceinline__ bool box_test(const QueryBox& q, float4 lo, float4 hi) {
  if (q.plane) {
    float cx = 0.5f * (lo.x + hi.x), cy = 0.5f * (lo.y + hi.y), cz = 0.5f * (lo.z + hi.z);
    float hx = 0.5f * (hi.x - lo.x), hy = 0.5f * (hi.y - lo.y), hz = 0.5f * (hi.z - lo.z);
    if (!(hx >= 0.f)) return false;   // empty (inverted) node
    float d = q.n[0] * cx + q.n[1] * cy + q.n[2] * cz - q.o;
    float r = fabsf(q.n[0]) * hx + fabsf(q.n[1]) * hy + fabsf(q.n[2]) * hz;
    return fabsf(d) <= r + q.r;
  }
  return lo.x <= q.c[0] + q.h[0] && hi.x >= q.c[0] - q.h[0] && lo.y <= q.c[1] + q.h[1] &&
         hi.y >= q.c[1] - q.h[1] && lo.z <= q.c[2] + q.h[2] && hi.z >= q.c[2] - q.h[2];
}

__device__ QueryBox make_query(const StepArgs& a, const PairDev& P, const FrameDev& F, int cl) {
  QueryBox q;
  if (P.query == 2) {
    q.plane = 1;
    q.n[0] = F.Rf[2]; q.n[1] = F.Rf[5]; q.n[2] = F.Rf[8];
    q.o = (float)(F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2]);
    q.r = 1e-5f * (fabsf(q.o) + 1e-3f) + 1e-7f;
    return q;
  }
  q.plane = 0;
  const float4* nd = a.nodes + 2 * (size_t)P.o_node_off;
  float4 lo = nd[2 * (P.o_leaves + cl)], hi = nd[2 * (P.o_leaves + cl) + 1];
  float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
  float h[3] = {0.5f * (hi.x - lo.x), 0.5f * (hi.y - lo.y), 0.5f * (hi.z - lo.z)};
  float mag = 0.f;
  for (int i = 0; i < 3; ++i) {
    q.c[i] = F.Rf[3 * i] * c[0] + F.Rf[3 * i + 1] * c[1] + F.Rf[3 * i + 2] * c[2] + F.tf[i];
    q.h[i] = fabsf(F.Rf[3 * i]) * h[0] + fabsf(F.Rf[3 * i + 1]) * h[1] + fabsf(F.Rf[3 * i + 2]) * h[2];
    mag = fmaxf(mag, fabsf(c[i]) + h[i]);
    mag = fmaxf(mag, fabsf(F.tf[i]));
  }
  float pad = 1e-5f * mag + 1e-7f;
  for (int i = 0; i < 3; ++i) q.h[i] += pad;
  return q;
}

// Stackless pre-order walk of the heap-numbered tree; calls emit(leaf).
template <class Emit>
__device__ __forceinline__ void walk(const float4* nd, int L, int ncl, const QueryBox& q, Emit emit) {
  int k = 1;
  while (true) {
    if (box_test(q, nd[2 * k], nd[2 * k + 1])) {
      if (k >= L) {
        if (k - L < ncl) emit(k - L);
      } else {
        k = 2 * k;
        continue;
      }
    }
    while (k & 1) k >>= 1;
    if (k == 0) break;
    k += 1;
  }
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  return v;
}

// Block exclusive scan (blockDim = kBpBlock); returns the exclusive prefix
// and the block total.
__device__ __forceinline__ int block_excl_scan(int v, int* total) {
  __shared__ int wsum[kBpBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int s = lane < kBpBlock / 32 ? wsum[lane] : 0;
    int si = warp_incl_scan(s);
    if (lane < kBpBlock / 32) wsum[lane] = si - s;
    if (lane == kBpBlock / 32 - 1) *total = si;
  }
  __syncthreads();
  int r = incl - v + wsum[wid];
  __syncthreads();
  return r;
}

__global__ void bp_count_kernel(StepArgs a) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  int cnt = 0;
  if (u < a.n_units) {
    const int p = a.unit_pair[u];
    const PairDev& P = a.pairs[p];
    const FrameDev& F = a.frames[p];
    if (F.valid) {
      QueryBox q = make_query(a, P, F, a.unit_cl[u]);
      const float4* nd = a.nodes + 2 * (size_t)P.s_node_off;
      int ncl = (P.s_n_elem + kCluster - 1) / kCluster;
      walk(nd, P.s_leaves, ncl, q, [&](int) { ++cnt; });
    }
    a.unit_count[u] = cnt;
  }
  __shared__ int total;
  int dummy = block_excl_scan(cnt, &total);
  (void)dummy;
  if (threadIdx.x == 0) a.block_sum[blockIdx.x] = total;
}

// Single CTA: exclusive scan of the block sums, total item count, overflow
// flag, and the work counter reset for the narrow phase.
__global__ void bp_scan_kernel(StepArgs a) {
  __shared__ int carry;
  __shared__ int tot;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < a.n_bp_blocks; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = (i < a.n_bp_blocks && a.n_units > 0) ? a.block_sum[i] : 0;
    int ex = block_excl_scan(v, &tot);
    if (i < a.n_bp_blocks) a.block_sum[i] = ex + carry;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int total = carry;
    if (total > a.item_cap) {
      atomicOr(a.status, 1);
      total = a.item_cap;
    }
    *a.item_total = total;
    *a.item_next = 0;
    a.unit_off[a.n_units] = carry;
  }
}

__global__ void bp_emit_kernel(StepArgs a) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  int cnt = u < a.n_units ? a.unit_count[u] : 0;
  __shared__ int total;
  int off = block_excl_scan(cnt, &total) + a.block_sum[blockIdx.x];
  if (u >= a.n_units) return;
  a.unit_off[u] = off;
  if (!cnt) return;
  const int p = a.unit_pair[u];
  const PairDev& P = a.pairs[p];
  const FrameDev& F = a.frames[p];
  const int cl = a.unit_cl[u];
  QueryBox q = make_query(a, P, F, cl);
  const float4* nd = a.nodes + 2 * (size_t)P.s_node_off;
  int ncl = (P.s_n_elem + kCluster - 1) / kCluster;
  int k = off;
  walk(nd, P.s_leaves, ncl, q, [&](int leaf) {
    if (k < a.item_cap) a.items[k] = make_int4(p, leaf, cl, 0);
    ++k;
  });
}

// ---------------------------------------------------------------------------
// narrow phase
// ---------------------------------------------------------------------------
struct Acc {
  float F[3], T[3], area, fn0;
  int n_poly, n_faces, n_near;
};

struct PairCtx {
  const PairDev* P;
  const FrameDev* F;
  int pair;
};

// One quadrature point (mujoco_contact_surfaces_plugin.cpp:345-404) and the
// force law in the soft frame.
__device__ __forceinline__ void point_force(Acc& ac, const FrameDev& F, float damping, float mu, int apply, float A,
                                            V3<float> p, V3<float> n, float gM, float gN, float p0) {
  if (!(A > 1.0e-14f)) return;
  if (gM < 1.0e-14f || gN < 1.0e-14f) return;
  float g = 1.0f / (1.0f / gM + 1.0f / gN);
  float fn0 = A * p0;
  float k = A * g;
  ac.area += A;
  ac.fn0 += fn0;
  ac.n_faces += 1;
  V3<float> lin = mk(F.lin[0], F.lin[1], F.lin[2]), ang = mk(F.ang[0], F.ang[1], F.ang[2]);
  V3<float> v = lin + cross(ang, p);
  float vn = dot(v, n);
  float fn = fmaxf(0.f, 1.f - damping * vn) * (fn0 - 0.001f * k * vn);
  if (!apply) return;
  V3<float> vt = v - n * vn;
  const float eps = (1.0e-4f * 1.0e-2f) * (1.0e-4f * 1.0e-2f);
  float v_slip = sqrtf(dot(vt, vt) + eps);
  float s = v_slip / 1.0e-4f;
  float mu_reg = s < 1.f ? mu * s * (2.f - s) : mu;
  V3<float> f = vt * (-mu_reg * fn / v_slip) + n * fn;
  V3<float> tq = cross(p, f);
  ac.F[0] += f.x; ac.F[1] += f.y; ac.F[2] += f.z;
  ac.T[0] += tq.x; ac.T[1] += tq.y; ac.T[2] += tq.z;
}

// Ray hits of one fan triangle (soft frame) on a sensor's sample grid: the
// sensor's rays are parallel to its -z axis, start 1.5*zs above its centre
// (+1e-8) and accept 0 < t < 1.5*zs (flat_tactile_sensor.cpp:324-346); the
// triangle test follows the Moeller-Trumbore acceptance rules of
// bvh.cpp:49-74 in the sensor frame.  Each sample keeps the smallest t,
// packed with the pressure at the hit, by a 64-bit atomicMin.
__device__ void raster_tri(const StepArgs& a, int sid, const float* Rl, const float* tl, V3<float> A, V3<float> B,
                           V3<float> C, float pa, float pb, float pc) {
  const SensorDev S = a.sensors[sid];
  V3<float> la = mat_mul<float>(Rl, A) + mk(tl[0], tl[1], tl[2]);
  V3<float> lb = mat_mul<float>(Rl, B) + mk(tl[0], tl[1], tl[2]);
  V3<float> lc = mat_mul<float>(Rl, C) + mk(tl[0], tl[1], tl[2]);
  float e1x = lb.x - la.x, e1y = lb.y - la.y, e2x = lc.x - la.x, e2y = lc.y - la.y;
  float det = e1x * e2y - e1y * e2x;
  if (fabsf(det) < 1e-10f) return;
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  float x0 = sx[0], dx = S.nx > 1 ? sx[1] - sx[0] : 1.f;
  float y0 = sy[0], dy = S.ny > 1 ? sy[1] - sy[0] : 1.f;
  float mnx = fminf(la.x, fminf(lb.x, lc.x)), mxx = fmaxf(la.x, fmaxf(lb.x, lc.x));
  float mny = fminf(la.y, fminf(lb.y, lc.y)), mxy = fmaxf(la.y, fmaxf(lb.y, lc.y));
  int X0 = max(0, (int)floorf((mnx - x0) / dx) - 1), X1 = min(S.nx - 1, (int)ceilf((mxx - x0) / dx) + 1);
  int Y0 = max(0, (int)floorf((mny - y0) / dy) - 1), Y1 = min(S.ny - 1, (int)ceilf((mxy - y0) / dy) + 1);
  if (X0 > X1 || Y0 > Y1) return;
  float inv = 1.f / det;
  unsigned long long* smp = a.samples + S.sample_off;
  for (int X = X0; X <= X1; ++X) {
    float wx = sx[X] - la.x;
    for (int Y = Y0; Y <= Y1; ++Y) {
      float wy = sy[Y] - la.y;
      float u = (wx * e2y - wy * e2x) * inv;
      if (u < 0.f || u > 1.f) continue;
      float v = (e1x * wy - e1y * wx) * inv;
      if (v < 0.f || u + v > 1.f) continue;
      float z = la.z + u * (lb.z - la.z) + v * (lc.z - la.z);
      float t = (S.zs15 + 1e-8f) - z;
      if (!(t > 0.f && t < S.zs15)) continue;
      float pr = (1.f - u - v) * pa + u * pb + v * pc;
      unsigned long long key =
          ((unsigned long long)__float_as_uint(t) << 32) | (unsigned long long)__float_as_uint(pr);
      atomicMin(&smp[(size_t)X * S.ny + Y], key);
    }
  }
}

// Quadrature of one polygon (float, soft frame) and its contribution to the
// forces and to the sensors.  n: contact normal out of N into M.
__device__ void integrate_polygon(const StepArgs& a, const PairCtx& pc, Acc& ac, const PVx<float>* v, int nv,
                                  V3<float> n, float gM, float gN) {
  const FrameDev& F = *pc.F;
  const PairDev& P = *pc.P;
  // area-weighted centroid by a fan from vertex 0
  float A = 0.f, pcen = 0.f;
  V3<float> c = mk(0.f, 0.f, 0.f);
  V3<float> v0 = pv_pos(v[0]);
  for (int i = 1; i + 1 < nv; ++i) {
    V3<float> vi = pv_pos(v[i]), vj = pv_pos(v[i + 1]);
    float ai = 0.5f * dot(cross(vi - v0, vj - v0), n);
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
    point_force(ac, F, P.damping, P.mu, a.apply_forces, fabsf(A), c, n, gM, gN, pcen);
  } else {
    for (int i = 0; i < nv; ++i) {
      int j = i + 1 == nv ? 0 : i + 1;
      V3<float> vi = pv_pos(v[i]), vj = pv_pos(v[j]);
      float Ai = 0.5f * norm(cross(vi - c, vj - c));
      V3<float> cen = (c + vi + vj) * (1.f / 3.f);
      float p0 = pcen / 3.f + v[i].p / 3.f + v[j].p / 3.f;
      point_force(ac, F, P.damping, P.mu, a.apply_forces, Ai, cen, n, gM, gN, p0);
    }
  }
  for (int q = 0; q < 2; ++q) {
    int sid = q == 0 ? P.sensor0 : P.sensor1;
    if (sid < 0) continue;
    const float* Rl = q == 0 ? F.Rl : F.Rl1;
    const float* tl = q == 0 ? F.tl : F.tl1;
    for (int i = 0; i < nv; ++i) {
      int j = i + 1 == nv ? 0 : i + 1;
      raster_tri(a, sid, Rl, tl, pv_pos(v[i]), pv_pos(v[j]), c, v[i].p, v[j].p, pcen);
    }
  }
}

__device__ void record(const StepArgs& a, const PairCtx& pc, const PVx<float>* v, int nv, V3<float> n, int ea,
                       int eb, int flags) {
  if (a.debug & 1) {
    int k = atomicAdd(a.cand_count, 1);
    if (k < a.cand_cap) {
      CandRec r;
      r.pair = pc.pair; r.elem_a = ea; r.elem_b = eb; r.n_vert = nv; r.flags = flags;
      a.cand[k] = r;
    } else {
      atomicOr(a.status, 2);
    }
  }
  if (a.want_polys && (a.want_pair < 0 || a.want_pair == pc.pair)) {
    int k = atomicAdd(a.poly_count, 1);
    if (k < a.poly_cap) {
      PolyRec& r = a.polys[k];
      r.pair = pc.pair; r.elem_a = ea; r.elem_b = eb; r.nv = nv;
      r.n[0] = n.x; r.n[1] = n.y; r.n[2] = n.z; r.n[3] = 0.f;
      for (int i = 0; i < kMaxPolyV; ++i) {
        bool in = i < nv;
        r.v[i][0] = in ? v[i].x : 0.f;
        r.v[i][1] = in ? v[i].y : 0.f;
        r.v[i][2] = in ? v[i].z : 0.f;
        r.v[i][3] = in ? v[i].p : 0.f;
      }
    } else {
      atomicOr(a.status, 4);
    }
  }
}

// --- soft-rigid element pair ------------------------------------------------
struct TriData {
  float Y[3][3];     // vertices, soft frame
  float n[3];        // unit normal (out of the rigid body)
  float o;           // n . Y0
  float en[3][3];    // in-plane inward edge normals
  float eo[3];
  float lo[3], hi[3];
  float M, h, Lt;    // magnitude, min altitude, max edge
  int orig;
  int valid;
};

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

// Soft-rigid polygon of tet `t` and triangle (Y, n, o, en, eo).
// Returns vertex count (0 when empty or culled).
template <class R>
__device__ int sr_polygon(const TetIn<R>& t, const V3<R> Y[3], V3<R> n, R o, const V3<R> en[3], const R eo[3], R M,
                          R h, R Lt, Decide& dc, PVx<R>* out, PVx<R>* tmp) {
  if (!(t.gl > (R)0)) return 0;
  R cg = dot(n, t.g) / t.gl;
  R tol_c = (R)kFilt * ((R)1 + M / h + t.kappa);
  check(dc, cg - (R)kCosAlphaD, tol_c);
  if (!dc.unc && !(cg > (R)kCosAlphaD)) return 0;
  R D = 0;
  R s[4];
  PVx<R> tv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    s[k] = dot(n, t.X[k]) - o;
    D = fmax(D, amax(t.X[k] - Y[0]));
    tv[k].x = t.X[k].x; tv[k].y = t.X[k].y; tv[k].z = t.X[k].z; tv[k].p = t.P[k]; tv[k].e = 0;
  }
  R tol_s = (R)kFilt * (M * ((R)1 + D / h) + D);
  int nv = tet_section(tv, s, tol_s, dc, out);
  if (nv == 0) return 0;
  R tol_p = (R)kFilt * (M * ((R)1 + (D + Lt) / h) + D + Lt);
  PVx<R>* src = out;
  PVx<R>* dst = tmp;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    nv = clip_plane(src, nv, en[j], eo[j], tol_p, dc, dst);
    PVx<R>* sw = src; src = dst; dst = sw;
    if (nv == 0) return 0;
  }
  if (src != out)
    for (int i = 0; i < nv; ++i) out[i] = src[i];
  return nv;
}

template <class R>
__device__ __forceinline__ void tri_prepare(const V3<R> Yin[3], V3<R> Y[3], V3<R>& n, R& o, V3<R> en[3], R eo[3],
                                            R& h, R& Lt, bool& valid) {
  for (int k = 0; k < 3; ++k) Y[k] = Yin[k];
  V3<R> N = cross(Y[1] - Y[0], Y[2] - Y[0]);
  R ln = norm(N);
  valid = ln > (R)0;
  n = valid ? N * ((R)1 / ln) : mk<R>(0, 0, 1);
  o = dot(n, Y[0]);
  R le = 0;
  for (int j = 0; j < 3; ++j) {
    V3<R> e = Y[j == 2 ? 0 : j + 1] - Y[j];
    le = fmax(le, norm(e));
    V3<R> m = cross(n, e);
    R lm = norm(m);
    en[j] = lm > (R)0 ? m * ((R)1 / lm) : m;
    eo[j] = dot(en[j], Y[j]);
  }
  Lt = le;
  h = le > (R)0 ? ln / le : (R)0;
}

// --- half-space element --------------------------------------------------------
template <class R>
__device__ int hs_polygon(const TetIn<R>& t, V3<R> n, R o, Decide& dc, PVx<R>* out) {
  if (!(t.gl > (R)0)) return 0;
  R cg = dot(n, t.g) / t.gl;
  R tol_c = (R)kFilt * ((R)1 + t.kappa);
  check(dc, cg - (R)kCosAlphaD, tol_c);
  if (!dc.unc && !(cg > (R)kCosAlphaD)) return 0;
  R s[4];
  PVx<R> tv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    s[k] = dot(n, t.X[k]) - o;
    tv[k].x = t.X[k].x; tv[k].y = t.X[k].y; tv[k].z = t.X[k].z; tv[k].p = t.P[k]; tv[k].e = 0;
  }
  R tol_s = (R)kFilt * (t.xmax + abs_r(o));
  return tet_section(tv, s, tol_s, dc, out);
}

// --- soft-soft element pair -----------------------------------------------------
struct TetB {
  float Y[4][3];
  float P[4];
  float g[3], c, gl;
  float pn[4][3], po[4];
  float lo[3], hi[3];
  float M, h, kappa;
  int orig;
  int valid;
};

template <class R>
__device__ int ss_polygon(const TetIn<R>& ta, V3<R> gb, R cb, R glb, const V3<R> pn[4], const R po[4], R Mb, R hb,
                          R kb, Decide& dc, PVx<R>* out, PVx<R>* tmp, V3<R>& nrm) {
  V3<R> m = ta.g - gb;
  R lm = norm(m);
  if (!(lm > (R)0) || !(ta.gl > (R)0) || !(glb > (R)0)) return 0;
  nrm = m * ((R)1 / lm);
  R cond = (((R)1 + ta.kappa) * ta.gl + ((R)1 + kb + Mb / hb) * glb) / lm;
  R tol_c = (R)kFilt * cond;
  R ca = dot(nrm, ta.g) / ta.gl;
  R cbb = -dot(nrm, gb) / glb;
  check(dc, ca - (R)kCosAlphaD, tol_c);
  check(dc, cbb - (R)kCosAlphaD, tol_c);
  if (!dc.unc && !(ca > (R)kCosAlphaD && cbb > (R)kCosAlphaD)) return 0;
  R s[4];
  PVx<R> tv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    s[k] = (ta.P[k] - (dot(gb, ta.X[k]) + cb)) / lm;
    tv[k].x = ta.X[k].x; tv[k].y = ta.X[k].y; tv[k].z = ta.X[k].z; tv[k].p = ta.P[k]; tv[k].e = 0;
  }
  R tol_s = (R)kFilt * (ta.pmax + glb * (ta.xmax + Mb) * ((R)1 + Mb / hb) + abs_r(cb)) / lm;
  int nv = tet_section(tv, s, tol_s, dc, out);
  if (nv == 0) return 0;
  R D = ta.xmax + Mb;
  R tol_p = (R)kFilt * (Mb * ((R)1 + D / hb) + D);
  PVx<R>* src = out;
  PVx<R>* dst = tmp;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    nv = clip_plane(src, nv, pn[j], po[j], tol_p, dc, dst);
    PVx<R>* sw = src; src = dst; dst = sw;
    if (nv == 0) return 0;
  }
  if (src != out)
    for (int i = 0; i < nv; ++i) out[i] = src[i];
  return nv;
}

__device__ __forceinline__ bool aabb_overlap(const float* alo, const float* ahi, const float* blo, const float* bhi) {
  return alo[0] <= bhi[0] && ahi[0] >= blo[0] && alo[1] <= bhi[1] && ahi[1] >= blo[1] && alo[2] <= bhi[2] &&
         ahi[2] >= blo[2];
}

template <class R>
__device__ __forceinline__ void load_tet(const float4* tets, int idx, TetIn<R>& t) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float4 v = tets[4 * (size_t)idx + k];
    t.X[k] = mk<R>(v.x, v.y, v.z);
    t.P[k] = v.w;
  }
}

template <class R>
__device__ __forceinline__ PVx<float> to_f(const PVx<R>& v) {
  PVx<float> o;
  o.x = (float)v.x; o.y = (float)v.y; o.z = (float)v.z; o.p = (float)v.p; o.e = 0.f;
  return o;
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
    const bool tvalid = ti < P.s_n_elem;
    TetIn<float> t;
    float tlo[3], thi[3];
    if (tvalid) {
      load_tet(a.tets, P.s_elem_off + ti, t);
      tet_prepare(t);
      for (int i = 0; i < 3; ++i) {
        float lo = fminf(fminf((&t.X[0].x)[i], (&t.X[1].x)[i]), fminf((&t.X[2].x)[i], (&t.X[3].x)[i]));
        float hi = fmaxf(fmaxf((&t.X[0].x)[i], (&t.X[1].x)[i]), fmaxf((&t.X[2].x)[i], (&t.X[3].x)[i]));
        float pad = 1e-5f * (fabsf(lo) + fabsf(hi)) + 1e-7f;
        tlo[i] = lo - pad;
        thi[i] = hi + pad;
      }
    }
    const int torig = tvalid ? a.tet_orig[P.s_elem_off + ti] : -1;
    const float sgn = P.s_is_m ? 1.f : -1.f;
    PVx<float> poly[kMaxPolyV], tmp[kMaxPolyV];
    if (P.query == 1) {
      // ---- stage the rigid triangles of cluster oc (soft frame) ----
      const int tj = oc * kCluster + lane;
      TriData& S = s_stage[wid].tri[lane];
      S.valid = 0;
      if (tj < P.o_n_elem && F.valid) {
        V3<float> Yin[3], Y[3], n, en[3];
        float o, eo[3], h, Lt, M = 0.f;
        bool ok;
        for (int k = 0; k < 3; ++k) {
          float4 r = a.tris[3 * (size_t)(P.o_elem_off + tj) + k];
          V3<float> rv = mk(r.x, r.y, r.z);
          M = fmaxf(M, amax(rv));
          Yin[k] = mat_mul<float>(F.Rf, rv) + mk(F.tf[0], F.tf[1], F.tf[2]);
        }
        M = fmaxf(M, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
        tri_prepare(Yin, Y, n, o, en, eo, h, Lt, ok);
        for (int k = 0; k < 3; ++k) {
          S.Y[k][0] = Y[k].x; S.Y[k][1] = Y[k].y; S.Y[k][2] = Y[k].z;
          S.en[k][0] = en[k].x; S.en[k][1] = en[k].y; S.en[k][2] = en[k].z;
          S.eo[k] = eo[k];
        }
        S.n[0] = n.x; S.n[1] = n.y; S.n[2] = n.z; S.o = o;
        for (int i = 0; i < 3; ++i) {
          float lo = fminf(fminf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]);
          float hi = fmaxf(fmaxf((&Y[0].x)[i], (&Y[1].x)[i]), (&Y[2].x)[i]);
          float pad = 1e-5f * (M + Lt) + 1e-7f;
          S.lo[i] = lo - pad;
          S.hi[i] = hi + pad;
        }
        S.M = M; S.h = h; S.Lt = Lt;
        S.orig = a.tri_orig[P.o_elem_off + tj];
        S.valid = ok && h > 0.f ? 1 : 0;
      }
      __syncwarp();
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TriData& T = s_stage[wid].tri[j];
        if (!tvalid || !T.valid || !aabb_overlap(tlo, thi, T.lo, T.hi)) continue;
        V3<float> Y[3] = {mk(T.Y[0][0], T.Y[0][1], T.Y[0][2]), mk(T.Y[1][0], T.Y[1][1], T.Y[1][2]),
                          mk(T.Y[2][0], T.Y[2][1], T.Y[2][2])};
        V3<float> en[3] = {mk(T.en[0][0], T.en[0][1], T.en[0][2]), mk(T.en[1][0], T.en[1][1], T.en[1][2]),
                           mk(T.en[2][0], T.en[2][1], T.en[2][2])};
        V3<float> n = mk(T.n[0], T.n[1], T.n[2]);
        float M = fmaxf(T.M, t.xmax);
        Decide dc;
        int nv = sr_polygon<float>(t, Y, n, T.o, en, T.eo, M, T.h, T.Lt, dc, poly, tmp);
        float gint = dot(t.g, n);
        int flags = 0;
        if (dc.unc) {
          // exact-decision fallback in FP64 from the stored inputs
          TetIn<double> td;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          V3<double> Yd[3], Ydp[3], nd, end[3];
          double od, eod[3], hd, Ltd;
          bool okd;
          for (int k = 0; k < 3; ++k) {
            float4 r = a.tris[3 * (size_t)(P.o_elem_off + oc * kCluster + j) + k];
            Yd[k] = mat_mul<double>(F.R, mk<double>(r.x, r.y, r.z)) + mk(F.t[0], F.t[1], F.t[2]);
          }
          tri_prepare(Yd, Ydp, nd, od, end, eod, hd, Ltd, okd);
          Decide dd;
          PVx<double> pd[kMaxPolyV], td2[kMaxPolyV];
          nv = okd ? sr_polygon<double>(td, Ydp, nd, od, end, eod, 0.0, 1.0, 0.0, dd, pd, td2) : 0;
          for (int i = 0; i < nv; ++i) poly[i] = to_f(pd[i]);
          if (dd.near) flags |= 1;
          gint = (float)dot(td.g, nd);
        }
        if (nv >= 3) {
          V3<float> nc = n * sgn;
          float gM = P.s_is_m ? gint : INFINITY;
          float gN = P.s_is_m ? INFINITY : gint;
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          integrate_polygon(a, pc, ac, poly, nv, nc, gM, gN);
          record(a, pc, poly, nv, nc, torig, T.orig, flags);
        }
      }
      __syncwarp();
    } else if (P.query == 2) {
      if (tvalid && F.valid) {
        V3<float> n = mk(F.Rf[2], F.Rf[5], F.Rf[8]);
        float o = (float)(F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2]);
        Decide dc;
        int nv = hs_polygon<float>(t, n, o, dc, poly);
        float gint = dot(t.g, n);
        int flags = 0;
        if (dc.unc) {
          TetIn<double> td;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          V3<double> nd = mk(F.R[2], F.R[5], F.R[8]);
          double od = F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2];
          Decide dd;
          PVx<double> pd[kMaxPolyV];
          nv = hs_polygon<double>(td, nd, od, dd, pd);
          for (int i = 0; i < nv; ++i) poly[i] = to_f(pd[i]);
          if (dd.near) flags |= 1;
          gint = (float)dot(td.g, nd);
        }
        if (nv >= 3) {
          V3<float> nc = n * sgn;
          float gM = P.s_is_m ? gint : INFINITY;
          float gN = P.s_is_m ? INFINITY : gint;
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          integrate_polygon(a, pc, ac, poly, nv, nc, gM, gN);
          record(a, pc, poly, nv, nc, torig, -1, flags);
        }
      }
    } else if (P.query == 3) {
      // ---- stage the B tets of cluster oc in A's (soft) frame ----
      const int tj = oc * kCluster + lane;
      TetB& S = s_stage[wid].tetb[lane];
      S.valid = 0;
      if (tj < P.o_n_elem && F.valid) {
        TetIn<float> tb;
        float M = 0.f;
        for (int k = 0; k < 4; ++k) {
          float4 r = a.tets[4 * (size_t)(P.o_elem_off + tj) + k];
          V3<float> rv = mk(r.x, r.y, r.z);
          M = fmaxf(M, amax(rv));
          tb.X[k] = mat_mul<float>(F.Rf, rv) + mk(F.tf[0], F.tf[1], F.tf[2]);
          tb.P[k] = r.w;
        }
        M = fmaxf(M, fmaxf(fabsf(F.tf[0]), fmaxf(fabsf(F.tf[1]), fabsf(F.tf[2]))));
        tet_prepare(tb);
        V3<float> pn[4];
        float po[4];
        tet_planes(tb.X, pn, po);
        for (int k = 0; k < 4; ++k) {
          S.Y[k][0] = tb.X[k].x; S.Y[k][1] = tb.X[k].y; S.Y[k][2] = tb.X[k].z;
          S.P[k] = tb.P[k];
          S.pn[k][0] = pn[k].x; S.pn[k][1] = pn[k].y; S.pn[k][2] = pn[k].z;
          S.po[k] = po[k];
        }
        S.g[0] = tb.g.x; S.g[1] = tb.g.y; S.g[2] = tb.g.z; S.c = tb.c; S.gl = tb.gl;
        for (int i = 0; i < 3; ++i) {
          float lo = fminf(fminf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fminf((&tb.X[2].x)[i], (&tb.X[3].x)[i]));
          float hi = fmaxf(fmaxf((&tb.X[0].x)[i], (&tb.X[1].x)[i]), fmaxf((&tb.X[2].x)[i], (&tb.X[3].x)[i]));
          float pad = 1e-5f * M + 1e-7f;
          S.lo[i] = lo - pad;
          S.hi[i] = hi + pad;
        }
        S.M = M; S.h = tb.hmin; S.kappa = tb.kappa;
        S.orig = a.tet_orig[P.o_elem_off + tj];
        S.valid = tb.hmin > 0.f ? 1 : 0;
      }
      __syncwarp();
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TetB& B = s_stage[wid].tetb[j];
        if (!tvalid || !B.valid || !aabb_overlap(tlo, thi, B.lo, B.hi)) continue;
        V3<float> pn[4] = {mk(B.pn[0][0], B.pn[0][1], B.pn[0][2]), mk(B.pn[1][0], B.pn[1][1], B.pn[1][2]),
                           mk(B.pn[2][0], B.pn[2][1], B.pn[2][2]), mk(B.pn[3][0], B.pn[3][1], B.pn[3][2])};
        V3<float> gb = mk(B.g[0], B.g[1], B.g[2]);
        Decide dc;
        V3<float> nrm;
        int nv = ss_polygon<float>(t, gb, B.c, B.gl, pn, B.po, B.M, B.h, B.kappa, dc, poly, tmp, nrm);
        float gM = dot(t.g, nrm), gN = -dot(gb, nrm);
        int flags = 0;
        if (dc.unc) {
          TetIn<double> td, tbd;
          load_tet(a.tets, P.s_elem_off + ti, td);
          tet_prepare(td);
          for (int k = 0; k < 4; ++k) {
            float4 r = a.tets[4 * (size_t)(P.o_elem_off + oc * kCluster + j) + k];
            tbd.X[k] = mat_mul<double>(F.R, mk<double>(r.x, r.y, r.z)) + mk(F.t[0], F.t[1], F.t[2]);
            tbd.P[k] = r.w;
          }
          tet_prepare(tbd);
          V3<double> pnd[4];
          double pod[4];
          tet_planes(tbd.X, pnd, pod);
          Decide dd;
          PVx<double> pd[kMaxPolyV], td2[kMaxPolyV];
          V3<double> nrmd;
          nv = tbd.hmin > 0.0 ? ss_polygon<double>(td, tbd.g, tbd.c, tbd.gl, pnd, pod, 0.0, 1.0, 0.0, dd, pd, td2, nrmd)
                              : 0;
          for (int i = 0; i < nv; ++i) poly[i] = to_f(pd[i]);
          if (dd.near) flags |= 1;
          if (nv >= 3) {
            nrm = mk((float)nrmd.x, (float)nrmd.y, (float)nrmd.z);
            gM = (float)dot(td.g, nrmd);
            gN = (float)-dot(tbd.g, nrmd);
          }
        }
        if (nv >= 3) {
          ac.n_poly += 1;
          ac.n_near += flags & 1;
          integrate_polygon(a, pc, ac, poly, nv, nrm, gM, gN);
          record(a, pc, poly, nv, nrm, torig, B.orig, flags);
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

// ---------------------------------------------------------------------------
// per-pair reduction (fixed order, FP64) and the world-frame wrench
// ---------------------------------------------------------------------------
__global__ void reduce_kernel(StepArgs a) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n_pair) return;
  const PairDev& P = a.pairs[p];
  const int total = *a.item_total;
  int b = min(a.unit_off[P.unit_begin], total), e = min(a.unit_off[P.unit_end], total);
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int c[3] = {0, 0, 0};
  for (int i = b + lane; i < e; i += 32) {
    const ItemOut& r = a.item_out[i];
    for (int k = 0; k < 8; ++k) v[k] += r.v[k];
    c[0] += r.n_poly; c[1] += r.n_faces; c[2] += r.n_near;
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k] += __shfl_xor_sync(0xffffffffu, c[k], o);
  }
  if (lane) return;
  const FrameDev& F = a.frames[p];
  PairOut o;
  V3<double> Fs = mk(v[0], v[1], v[2]), Ts = mk(v[3], v[4], v[5]);
  V3<double> Fw = mat_mul<double>(F.RS, Fs), Tw = mat_mul<double>(F.RS, Ts);
  V3<double> xS = mk(F.xS[0], F.xS[1], F.xS[2]), xM = mk(F.xM[0], F.xM[1], F.xM[2]);
  Tw = Tw + cross(xS - xM, Fw);
  bool on = a.apply_forces && F.valid;
  o.wrench[0] = on ? Fw.x : 0.0; o.wrench[1] = on ? Fw.y : 0.0; o.wrench[2] = on ? Fw.z : 0.0;
  o.wrench[3] = on ? Tw.x : 0.0; o.wrench[4] = on ? Tw.y : 0.0; o.wrench[5] = on ? Tw.z : 0.0;
  o.area = v[6];
  o.total_fn0 = v[7];
  o.n_poly = c[0]; o.n_faces = c[1]; o.n_near = c[2];
  o.n_items = e - b;
  a.pair_out[p] = o;
}

// ---------------------------------------------------------------------------
// taxel sums (flat_tactile_sensor.cpp:316-397): per cell, the samples in the
// reference's i-major, j-minor order, weight * pressure * (1/s^2); the
// sample slots are reset for the next step.
// ---------------------------------------------------------------------------
__global__ void taxel_kernel(StepArgs a) {
  const int gc = blockIdx.x * blockDim.x + threadIdx.x;
  if (gc >= a.n_cells_total) return;
  const int sid = a.cell_sensor[gc];
  const SensorDev S = a.sensors[sid];
  const int cell = gc - a.cell_first[sid];
  const int x = cell / S.cy, y = cell % S.cy;
  unsigned long long* smp = a.samples + S.sample_off;
  const float* w = a.weights + S.weight_off;
  float avg = 0.f;
  for (int i = 0; i < S.sr; ++i) {
    const int X = x * S.sr + i;
    for (int j = 0; j < S.sr; ++j) {
      const int Y = y * S.sr + j;
      unsigned long long k = smp[(size_t)X * S.ny + Y];
      if (k != ~0ull) {
        float pr = __uint_as_float((unsigned)(k & 0xffffffffu));
        float raw = pr * S.rmean;
        avg += w[i * S.sr + j] * raw;
        smp[(size_t)X * S.ny + Y] = ~0ull;
      }
    }
  }
  a.taxels[S.taxel_off + x + S.cy * y] = avg;
}

// ---------------------------------------------------------------------------
int launch_step(const StepArgs& a, cudaStream_t s, cudaEvent_t* ev) {
  int n = 0;
  if (ev) cudaEventRecord(ev[0], s);
  if (a.n_pair > 0) {
    frames_kernel<<<(a.n_pair + 127) / 128, 128, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecord(ev[1], s);
  if (a.n_units > 0) {
    bp_count_kernel<<<a.n_bp_blocks, kBpBlock, 0, s>>>(a); ++n;
  }
  bp_scan_kernel<<<1, kBpBlock, 0, s>>>(a); ++n;
  if (a.n_units > 0) {
    bp_emit_kernel<<<a.n_bp_blocks, kBpBlock, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecord(ev[2], s);
  if (a.n_pair > 0) {
    narrow_kernel<<<a.narrow_grid, a.narrow_block, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecord(ev[3], s);
  if (a.n_pair > 0) {
    reduce_kernel<<<(a.n_pair * 32 + 127) / 128, 128, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecord(ev[4], s);
  if (a.n_cells_total > 0) {
    taxel_kernel<<<(a.n_cells_total + 127) / 128, 128, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecord(ev[5], s);
  return n;
}

}  // namespace hc
