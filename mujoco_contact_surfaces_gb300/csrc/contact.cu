// contact.cu — the per-step device pipeline of the hydroelastic contact path.
//
//   step_begin_kernel  counters and scan tiles zeroed; pair setup: relative
//                      transforms (FP64), velocity field, sensor frames (the
//                      pose/velocity fetches of passiveCallback,
//                      mujoco_contact_surfaces_plugin.cpp:435-451); the last
//                      step's touched samples cleared
//   bp_kernel          cluster-level broadphase over the LBVH and the
//                      compaction of its work items in one pass (decoupled
//                      look-back scan)
//   narrow kernels     per item: element tests, clipping, quadrature
//                      (P:320-409), Hunt-Crossley + friction,
//                      taxel binning (flat_tactile_sensor.cpp:262-402), or the
//                      polygons kept for rec_forward_kernel and the adjoint
//   reduce_kernel      deterministic FP64 per-pair wrench
//   taxel_kernel       per-cell sums of the binned samples
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

__device__ __forceinline__ void pair_frame(const StepArgs& a, int p) {
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
  for (int i = 0; i < 9; ++i) {
    F.Rf[i] = (float)F.R[i];
    F.Rlo[i] = (float)(F.R[i] - (double)F.Rf[i]);
  }
  for (int i = 0; i < 3; ++i) {
    F.tf[i] = (float)F.t[i];
    F.tlo[i] = (float)(F.t[i] - (double)F.tf[i]);
  }
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

// Every flat sensor's samples inside the box the last step touched go back
// to "no hit" (the taxel pass clears what it reads unless the samples are
// kept for the adjoint), and the box is emptied.  One block, rows of the box
// across its threads.
__device__ __forceinline__ void clear_box(const StepArgs& a, int sid) {
  const SensorDev S = a.sensors[sid];
  const int4 b = a.sens_box[sid];
  if (b.x <= b.y && b.z <= b.w) {
    unsigned long long* smp = a.samples + S.sample_off;
    const int nY = b.w - b.z + 1, cnt = (b.y - b.x + 1) * nY;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x)
      smp[(size_t)(b.x + i / nY) * S.ny + b.z + i % nY] = ~0ull;
  }
  __syncthreads();
  if (threadIdx.x == 0) a.sens_box[sid] = make_int4(0x7fffffff, -1, 0x7fffffff, -1);
}

// The step's first kernel: the step counters and the scans' tile states
// zeroed, the pair frames (a thread per pair in the first n_frame_blocks
// blocks) and, in the
// blocks after them, one block per flat sensor clearing the last step's
// touched samples.  The three are independent.
__global__ void step_begin_kernel(StepArgs a, int n_frame_blocks) {
  if ((int)blockIdx.x < n_frame_blocks) {
    if (blockIdx.x == 0 && a.reset_words && threadIdx.x < kResetWords) a.reset_words[threadIdx.x] = 0;
    // the single-pass scans' tile states
    const int g = blockIdx.x * blockDim.x + threadIdx.x, stride = n_frame_blocks * blockDim.x;
    if (a.bp_tiles)
      for (int i = g; i < a.n_bp_blocks; i += stride) a.bp_tiles[i] = 0;
    if (a.poly_tiles)
      for (int i = g; i < a.n_item_blocks; i += stride) a.poly_tiles[i] = 0;
    const int p = g;
    if (p < a.n_pair) pair_frame(a, p);
  } else {
    clear_box(a, blockIdx.x - n_frame_blocks);
  }
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

// Stackless pre-order walk of the subtree rooted at r (heap numbering);
// calls emit(leaf) for the leaves whose boxes pass, left to right.
template <class Emit>
__device__ __forceinline__ void walk_sub(const float4* nd, int L, int ncl, const QueryBox& q, int r, Emit emit) {
  int k = r;
  while (true) {
    if (box_test(q, nd[2 * k], nd[2 * k + 1])) {
      if (k >= L) {
        if (k - L < ncl) emit(k - L);
      } else {
        k = 2 * k;
        continue;
      }
    }
    while (k != r && (k & 1)) k >>= 1;
    if (k == r) break;
    k += 1;
  }
}

// A unit's tree is walked by a warp: lane i takes the i-th subtree of the
// level with min(32, L) nodes (L, the leaf count, is a power of two); the
// lanes' leaves in lane order are the leaves of a whole pre-order walk.
__device__ __forceinline__ int lane_root(int L, int lane) {
  const int w = L < 32 ? L : 32;
  return lane < w ? w + lane : 0;
}

constexpr int kBpUnits = kBpBlock / 32;   // units per broadphase block (a warp each)

// ---- single-pass prefix scans (decoupled look-back) ------------------------
// A block takes the next tile from an atomic counter, so every tile it waits
// on belongs to a block that started before it and is running; each tile
// publishes its aggregate, then its inclusive prefix, as one 64-bit word
// (state in the top two bits).  A wait is bounded: past the bound the
// status word gets bit 32 and the host reports the step as failed.
constexpr unsigned long long kTileAggregate = 1ull << 62;
constexpr unsigned long long kTileInclusive = 2ull << 62;
constexpr unsigned long long kTileValue = (1ull << 62) - 1;
constexpr int kTileWaitRounds = 1 << 22;   // about 0.3 s of 64 ns sleeps
constexpr int kStatusScanWait = 32;

// The exclusive prefix of tile t given its aggregate (one thread calls it).
__device__ __forceinline__ int tile_lookback(unsigned long long* st, int t, int agg, int* status) {
  if (t == 0) {
    atomicExch(st, kTileInclusive | (unsigned long long)agg);
    return 0;
  }
  atomicExch(st + t, kTileAggregate | (unsigned long long)agg);
  const volatile unsigned long long* vs = st;
  unsigned long long excl = 0;
  for (int k = t - 1; k >= 0; --k) {
    unsigned long long v = vs[k];
    for (int w = 0; v == 0; ++w) {
      if (w == kTileWaitRounds) {
        atomicOr(status, kStatusScanWait);
        return 0;
      }
      __nanosleep(64);
      v = vs[k];
    }
    excl += v & kTileValue;
    if ((v >> 62) == 2) break;
  }
  atomicExch(st + t, kTileInclusive | (excl + (unsigned long long)agg));
  return (int)excl;
}

// Broadphase in one pass: a warp per (pair, other cluster) unit walks the
// soft tree with the cluster's box (or the plane) and counts the leaves that
// pass; the block's units get their item offsets from the tile scan; the
// walk is repeated to write the items (pair, soft leaf, other cluster) in
// pre-order.  The last tile writes the item total (clamped to the capacity;
// an overflow sets status bit 1 and leaves the full total in
// unit_off[n_units]).
__global__ void bp_kernel(StepArgs a) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __shared__ int tile_s, excl_s;
  __shared__ int ucnt[kBpUnits];
  if (threadIdx.x == 0) tile_s = atomicAdd(a.tile_ctr, 1);
  __syncthreads();
  const int tile = tile_s;
  const int u = tile * kBpUnits + wid;
  int p = 0, r = 0, cnt = 0, cl = 0, ncl = 0;
  // the passing leaves of the lane's subtree as bits (leaf0 + bit), when
  // the subtree has at most 32 leaves (trees of up to 1024 leaf clusters):
  // the items are then written from the bits instead of a second walk
  unsigned lmask = 0;
  int leaf0 = 0;
  bool masked = false;
  QueryBox q;
  const float4* nd = nullptr;
  const PairDev* P = nullptr;
  if (u < a.n_units) {
    p = a.unit_pair[u];
    P = &a.pairs[p];
    const FrameDev& F = a.frames[p];
    if (F.valid) {
      cl = a.unit_cl[u];
      q = make_query(a, *P, F, cl);
      nd = a.nodes + 2 * (size_t)P->s_node_off;
      ncl = (P->s_n_elem + kCluster - 1) / kCluster;
      r = lane_root(P->s_leaves, lane);
      const int w = P->s_leaves < 32 ? P->s_leaves : 32, per = P->s_leaves / w;
      masked = per <= 32;
      leaf0 = r ? (r - w) * per : 0;
      if (r)
        walk_sub(nd, P->s_leaves, ncl, q, r, [&](int leaf) {
          ++cnt;
          if (masked) lmask |= 1u << (leaf - leaf0);
        });
    }
  }
  const int lane_first = warp_incl_scan(cnt) - cnt;   // this lane's leaves follow the lanes' before it
  const int total_u = __shfl_sync(0xffffffffu, lane_first + cnt, 31);
  if (lane == 0) ucnt[wid] = u < a.n_units ? total_u : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    int agg = 0;
    for (int w = 0; w < kBpUnits; ++w) agg += ucnt[w];
    excl_s = tile_lookback(a.bp_tiles, tile, agg, a.status);
    if (tile == (int)gridDim.x - 1) {
      int total = excl_s + agg;
      a.unit_off[a.n_units] = total;
      if (total > a.item_cap) {
        atomicOr(a.status, 1);
        total = a.item_cap;
      }
      *a.item_total = total;
    }
  }
  __syncthreads();
  if (u >= a.n_units) return;
  int off = excl_s;
  for (int w = 0; w < wid; ++w) off += ucnt[w];
  if (lane == 0) a.unit_off[u] = off;
  if (!ucnt[wid]) return;
  int k = off + lane_first;
  if (r && masked) {
    // ascending bits: the walk's left-to-right order
    for (unsigned m = lmask; m; m &= m - 1) {
      if (k < a.item_cap) a.items[k] = make_int4(p, leaf0 + __ffs(m) - 1, cl, 0);
      ++k;
    }
  } else if (r) {
    walk_sub(nd, P->s_leaves, ncl, q, r, [&](int leaf) {
      if (k < a.item_cap) a.items[k] = make_int4(p, leaf, cl, 0);
      ++k;
    });
  }
}

#include "narrow.cuh"
#include "adjoint.cuh"
#include "taxel_sensor.cuh"
#include "curved_sensor.cuh"

// ---------------------------------------------------------------------------
// per-pair reduction (fixed order, FP64) and the world-frame wrench
// ---------------------------------------------------------------------------
// kReducePairs pairs per block: warp w sums pair w of the block in
// double-float on the FP32 pipe (FP64 runs at 1/64 of its rate) in a fixed
// order, lane-strided, then a fixed butterfly; then the first kReducePairs
// threads turn the pairs' sums into world wrenches side by side in FP64 (one
// FP64 tail per warp would cost the FP64 pipe a full warp instruction per
// operation).
__global__ void __launch_bounds__(kReducePairs * 32) reduce_kernel(StepArgs a) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ float sh[kReducePairs][8], sl[kReducePairs][8];
  __shared__ int sc[kReducePairs][3];
  const int total = *a.item_total;
  const int pw = blockIdx.x * kReducePairs + w;
  if (pw < a.n_pair) {
    const PairDev& P = a.pairs[pw];
    const int b = min(a.unit_off[P.unit_begin], total), e = min(a.unit_off[P.unit_end], total);
    float vh[8] = {0, 0, 0, 0, 0, 0, 0, 0}, vl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int c[3] = {0, 0, 0};
    for (int i = b + lane; i < e; i += 32) {
      const ItemOut& r = a.item_out[i];
#pragma unroll
      for (int k = 0; k < 8; ++k) df_add(vh[k], vl[k], r.hi[k], r.lo[k]);
      c[0] += r.n_poly; c[1] += r.n_faces; c[2] += r.n_near;
    }
    if (rec_ok(a) && P.query != 3) {
      // forces of the kept polygons, in pair order (soft-soft pairs keep none,
      // and a step of soft-soft pairs alone runs no record scan)
      const int rb = a.item_poly_off[b], re = a.item_poly_off[e];
      // four records per lane in flight, then summed in the same order
      // (the loads of a plain lane-strided loop waited one by one)
      int i = rb + lane;
      for (; i + 96 < re; i += 128) {
        float4 q0[4], q1[4];
        int nf[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float4* s = reinterpret_cast<const float4*>(a.rec_out + i + 32 * u);
          q0[u] = s[0];
          q1[u] = s[1];
          nf[u] = reinterpret_cast<const int*>(s + 2)[0];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float x[8] = {q0[u].x, q0[u].y, q0[u].z, q0[u].w, q1[u].x, q1[u].y, q1[u].z, q1[u].w};
#pragma unroll
          for (int k = 0; k < 8; ++k) df_add(vh[k], vl[k], x[k], 0.f);
          c[1] += nf[u];
        }
      }
      for (; i < re; i += 32) {
        const RecOut& r = a.rec_out[i];
        const float x[8] = {r.F[0], r.F[1], r.F[2], r.T[0], r.T[1], r.T[2], r.area, r.fn0};
#pragma unroll
        for (int k = 0; k < 8; ++k) df_add(vh[k], vl[k], x[k], 0.f);
        c[1] += r.n_faces;
      }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float h2 = __shfl_xor_sync(0xffffffffu, vh[k], o), l2 = __shfl_xor_sync(0xffffffffu, vl[k], o);
        df_add(vh[k], vl[k], h2, l2);
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) c[k] += __shfl_xor_sync(0xffffffffu, c[k], o);
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < 8; ++k) { sh[w][k] = vh[k]; sl[w][k] = vl[k]; }
#pragma unroll
      for (int k = 0; k < 3; ++k) sc[w][k] = c[k];
    }
  }
  __syncthreads();
  const int p = blockIdx.x * kReducePairs + threadIdx.x;
  if (threadIdx.x >= kReducePairs || p >= a.n_pair) return;
  const PairDev& P = a.pairs[p];
  const int b = min(a.unit_off[P.unit_begin], total), e = min(a.unit_off[P.unit_end], total);
  double v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = (double)sh[threadIdx.x][k] + (double)sl[threadIdx.x][k];
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
  o.n_poly = sc[threadIdx.x][0]; o.n_faces = sc[threadIdx.x][1]; o.n_near = sc[threadIdx.x][2];
  o.n_items = e - b;
  a.pair_out[p] = o;
}

// ---------------------------------------------------------------------------
// taxel sums (flat_tactile_sensor.cpp:316-397): per cell, the samples in the
// reference's i-major, j-minor order, weight * pressure * (1/s^2); the
// sample slots are reset for the next step.
// ---------------------------------------------------------------------------
// The pressure a sample holds (0 when no ray hit it): the value itself, or
// for a sample won by a kept polygon that polygon's pressure model at the
// sample, times the sensor's 1/s^2.
__device__ __forceinline__ float sample_pressure(const StepArgs& a, const SensorDev& S, unsigned long long k, int X,
                                                 int Y) {
  if (k == ~0ull) return 0.f;
  const unsigned lo = (unsigned)(k & 0xffffffffu);
  float pr = __uint_as_float(lo);
  if (lo & kSlotTag) {
    const int slot = (int)(lo & ~(kSlotTag | kSideBit));
    const int side = (lo & kSideBit) ? 1 : 0;
    const float4 m0 = a.slot_press[6 * (size_t)slot + 3 * side];
    const float4 m1 = a.slot_press[6 * (size_t)slot + 3 * side + 1];
    pr = raster_pressure(m0.x, m0.y, m0.z, m0.w, m1.x, a.samp_coord[S.samp_off_x + X], a.samp_coord[S.samp_off_y + Y]);
  }
  return pr * S.rmean;
}

// Samples of a touched box resolved in shared memory at once.
constexpr int kTaxBoxSamples = 8192;
// Threads per sensor block: 512 resolve a touched box (about 1500 samples
// on the bench) in fewer steps than 256 (step 1.360 -> 1.352 ms).
constexpr int kTaxelBlock = 512;

// A block per sensor.  Its touched box's samples are resolved first, each by
// its own thread (the sample, then the winning polygon's pressure model: two
// dependent loads, issued for many samples at once), into shared memory;
// then each cell sums its samples from there in the reference's i-major,
// j-minor order.  Cells outside the box hold no hit (value 0).  A box larger
// than the shared array is summed cell by cell from global memory.
__global__ void __launch_bounds__(kTaxelBlock) taxel_kernel(StepArgs a) {
  __shared__ SensorDev S;
  __shared__ int4 box;
  __shared__ float val[kTaxBoxSamples];
  const int sid = blockIdx.x;
  if (threadIdx.x == 0) {
    S = a.sensors[sid];
    // without boxes every sample is read (the no-alloc step clears them all)
    box = a.sens_box ? a.sens_box[sid] : make_int4(0, S.nx - 1, 0, S.ny - 1);
    box.x = max(box.x, 0); box.y = min(box.y, S.nx - 1);
    box.z = max(box.z, 0); box.w = min(box.w, S.ny - 1);
  }
  __syncthreads();
  const int n = S.cx * S.cy;
  float* out = a.taxels + S.taxel_off;
  if (box.x > box.y || box.z > box.w) {
    // no ray of this step touched the sensor: every value is 0 and its
    // samples are already clear
    for (int cell = threadIdx.x; cell < n; cell += blockDim.x) out[cell / S.cy + S.cy * (cell % S.cy)] = 0.f;
    return;
  }
  unsigned long long* smp = a.samples + S.sample_off;
  const float* w = a.weights + S.weight_off;
  const int bw = box.w - box.z + 1, nb = (box.y - box.x + 1) * bw;
  const bool staged = nb <= kTaxBoxSamples;
  if (staged) {
    // two samples per thread in flight: their keys, then the winning
    // polygons' pressure models and the sample coordinates, then the values
    // as sample_pressure forms them (one sample at a time waited out both
    // loads; four at a time took 57 registers, two fewer blocks per SM)
    const int nt = blockDim.x;
    for (int i0 = threadIdx.x; i0 < nb; i0 += 2 * nt) {
      unsigned long long k[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + u * nt;
        k[u] = i < nb ? smp[(size_t)(box.x + i / bw) * S.ny + (box.z + i % bw)] : ~0ull;
      }
      float4 m0[2], m1[2];
      float sx[2], sy[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + u * nt;
        const unsigned lo = (unsigned)(k[u] & 0xffffffffu);
        m0[u] = m1[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        sx[u] = sy[u] = 0.f;
        if (k[u] != ~0ull && (lo & kSlotTag)) {
          const size_t b6 = 6 * (size_t)(lo & ~(kSlotTag | kSideBit)) + ((lo & kSideBit) ? 3 : 0);
          m0[u] = a.slot_press[b6];
          m1[u] = a.slot_press[b6 + 1];
          sx[u] = a.samp_coord[S.samp_off_x + box.x + i / bw];
          sy[u] = a.samp_coord[S.samp_off_y + box.z + i % bw];
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + u * nt;
        if (i >= nb) break;
        const unsigned lo = (unsigned)(k[u] & 0xffffffffu);
        const float pr = (lo & kSlotTag) ? raster_pressure(m0[u].x, m0[u].y, m0[u].z, m0[u].w, m1[u].x, sx[u], sy[u])
                                         : __uint_as_float(lo);
        val[i] = k[u] == ~0ull ? 0.f : pr * S.rmean;
        if (!a.keep_samples && k[u] != ~0ull) smp[(size_t)(box.x + i / bw) * S.ny + (box.z + i % bw)] = ~0ull;
      }
    }
    __syncthreads();
  }
  for (int cell = threadIdx.x; cell < n; cell += blockDim.x) {
    const int x = cell / S.cy, y = cell % S.cy;
    // a cell whose samples lie outside the box this step's rays touched
    // holds no hit: its value is 0 and its samples are already clear
    if (x * S.sr > box.y || x * S.sr + S.sr - 1 < box.x || y * S.sr > box.w || y * S.sr + S.sr - 1 < box.z) {
      out[x + S.cy * y] = 0.f;
      continue;
    }
    float avg = 0.f;
    for (int i = 0; i < S.sr; ++i) {
      const int X = x * S.sr + i;
      for (int j = 0; j < S.sr; ++j) {
        const int Y = y * S.sr + j;
        if (X < box.x || X > box.y || Y < box.z || Y > box.w) continue;   // no hit there
        float raw;
        if (staged) {
          raw = val[(X - box.x) * bw + (Y - box.z)];
        } else {
          unsigned long long* q = smp + (size_t)X * S.ny + Y;
          const unsigned long long k = *q;
          raw = sample_pressure(a, S, k, X, Y);
          if (!a.keep_samples && k != ~0ull) *q = ~0ull;
        }
        avg = __fadd_rn(avg, __fmul_rn(w[i * S.sr + j], raw));
      }
    }
    out[x + S.cy * y] = avg;
  }
}

void launch_tet_props(const float4* tets, float4* props, int n_tets, cudaStream_t s) {
  if (n_tets > 0) tet_props_kernel<<<(n_tets + 255) / 256, 256, 0, s>>>(tets, props, n_tets);
}

// ---------------------------------------------------------------------------
cudaError_t init_kernel_attributes() {
  cudaError_t e = cudaSuccess;
  for (const void* k : {(const void*)narrow_sr_kernel<false, false>, (const void*)narrow_sr_kernel<true, true>,
                        (const void*)narrow_sr_kernel<false, true>}) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSrSmemBytes);
    if (e != cudaSuccess) return e;
  }
  e = cudaFuncSetAttribute((const void*)narrow_sr_keep_kernel<kSrKeepCtas>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kSrKeepSmemBytes);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(taxel_sensor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTaxelSmemBytes);
  if (e != cudaSuccess) return e;
  // the taxel sensors' grid-count table (a pure function of the step count)
  grid_table_kernel<<<(kTaxMaxSt + 256) / 256, 256>>>();
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(adjoint_sr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSrSmemBytes);
}

void record_ctas_per_sm(int* fwd, int* adj) {
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(fwd, rec_forward_kernel<0>, 128, 0) != cudaSuccess || *fwd < 1)
    *fwd = 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(adj, adjoint_rec_kernel<0>, 128, 0) != cudaSuccess || *adj < 1)
    *adj = 1;
}

int launch_adjoint(const StepArgs& a, cudaStream_t s) {
  int n = 0;
  if (a.n_pair <= 0) return 0;
  adjoint_setup_kernel<<<(a.n_pair + 127) / 128, 128, 0, s>>>(a); ++n;
  if (a.use_recs) {
    // kept polygons, in the slots the forward assigned (returns at once if
    // the records overflowed)
    if (a.repr == 1) adjoint_rec_kernel<1><<<a.rec_adj_grid, 128, 0, s>>>(a);
    else adjoint_rec_kernel<0><<<a.rec_adj_grid, 128, 0, s>>>(a);
    ++n;
  }
  // the recomputing soft-rigid and half-space adjoints (they return at once
  // when the kept polygons are valid; a fused step re-runs on an overflow)
  const bool recompute = !(a.use_recs && a.fused);
  if (recompute && a.type_unit_end[0] > a.type_unit_begin[0]) {
    adjoint_sr_kernel<<<a.narrow_grid, 128, kSrSmemBytes, s>>>(a); ++n;
  }
  if (recompute && a.type_unit_end[1] > a.type_unit_begin[1]) {
    adjoint_hs_kernel<<<a.narrow_grid, 128, 0, s>>>(a); ++n;
  }
  if (a.type_unit_end[2] > a.type_unit_begin[2]) {
    adjoint_ss_kernel<<<a.narrow_grid, 128, 0, s>>>(a); ++n;
  }
  adjoint_reduce_kernel<<<(a.n_pair + kReducePairs - 1) / kReducePairs, kReducePairs * 32, 0, s>>>(a); ++n;
  return n;
}

int launch_step(const StepArgs& a, cudaStream_t s, cudaEvent_t* ev) {
  int n = 0;
  if (ev) cudaEventRecordWithFlags(ev[0], s, cudaEventRecordExternal);
  {
    const int nfb = a.n_pair > 0 ? (a.n_pair + 127) / 128 : 1;
    const int nsb = a.sens_box ? a.n_sensor : 0;
    step_begin_kernel<<<nfb + nsb, 128, 0, s>>>(a, nfb); ++n;
  }
  if (ev) cudaEventRecordWithFlags(ev[1], s, cudaEventRecordExternal);
  // (also with no units: the last tile writes the item total)
  bp_kernel<<<a.n_bp_blocks > 0 ? a.n_bp_blocks : 1, kBpBlock, 0, s>>>(a); ++n;
  if (ev) cudaEventRecordWithFlags(ev[2], s, cudaEventRecordExternal);
  if (a.type_unit_end[0] > a.type_unit_begin[0]) {
    const bool diag = (a.debug & 1) || a.want_polys;
    if (a.recs) {
      if (diag) narrow_sr_kernel<true, true><<<a.narrow_grid, 128, kSrSmemBytes, s>>>(a);
      else narrow_sr_keep_kernel<kSrKeepCtas><<<a.narrow_grid, 128, kSrKeepSmemBytes, s>>>(a);
    } else {
      if (diag) narrow_sr_kernel<false, true><<<a.narrow_grid, 128, kSrSmemBytes, s>>>(a);
      else narrow_sr_kernel<false, false><<<a.narrow_grid, 128, kSrSmemBytes, s>>>(a);
    }
    ++n;
  }
  if (a.type_unit_end[1] > a.type_unit_begin[1]) {
    const bool diag = (a.debug & 1) || a.want_polys;
    if (a.recs) {
      if (diag) narrow_hs_kernel<true, true><<<a.narrow_grid, 128, 0, s>>>(a);
      else narrow_hs_kernel<true, false><<<a.narrow_grid, 128, 0, s>>>(a);
    } else {
      if (diag) narrow_hs_kernel<false, true><<<a.narrow_grid, 128, 0, s>>>(a);
      else narrow_hs_kernel<false, false><<<a.narrow_grid, 128, 0, s>>>(a);
    }
    ++n;
  }
  if (a.type_unit_end[2] > a.type_unit_begin[2]) {
    narrow_ss_kernel<<<a.narrow_grid, 128, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecordWithFlags(ev[6], s, cudaEventRecordExternal);
  if (a.recs && a.type_unit_end[1] > a.type_unit_begin[0]) {
    // kept polygons: pair-ordered slots, then forces and rays per polygon
    poly_slots_kernel<<<(a.n_item_blocks + kSlotItems - 1) / kSlotItems, kBpBlock, 0, s>>>(a); ++n;
    if (a.repr == 1) rec_forward_kernel<1><<<a.rec_fwd_grid, 128, 0, s>>>(a);
    else rec_forward_kernel<0><<<a.rec_fwd_grid, 128, 0, s>>>(a);
    ++n;
    if (a.n_tsens > 0) {
      if (a.n_tpairs > 0) {
        taxel_order_kernel<<<a.n_tpairs, kTaxThreads, 0, s>>>(a); ++n;
      }
      taxel_sensor_kernel<<<a.n_tsens, kTaxThreads, kTaxelSmemBytes, s>>>(a); ++n;
    }
    if (a.n_csens > 0) {
      curved_sensor_kernel<<<a.n_csens, kCurvThreads, 0, s>>>(a); ++n;
    }
  }
  if (ev) cudaEventRecordWithFlags(ev[3], s, cudaEventRecordExternal);
  if (a.n_pair > 0) {
    reduce_kernel<<<(a.n_pair + kReducePairs - 1) / kReducePairs, kReducePairs * 32, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecordWithFlags(ev[4], s, cudaEventRecordExternal);
  if (a.n_cells_total > 0) {
    taxel_kernel<<<a.n_sensor, kTaxelBlock, 0, s>>>(a); ++n;
  }
  if (ev) cudaEventRecordWithFlags(ev[5], s, cudaEventRecordExternal);
  return n;
}

}  // namespace hc
