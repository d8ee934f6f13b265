// lbvh.cu — the LBVH build on the device: each geom's elements ordered along
// a Morton curve of their centroids, then gathered into the element pools the
// broadphase and narrow phase read (the node boxes follow by refit_kernel).
//
// Replaces Drake's per-geom Bvh<Obb> build at load (the reference builds one
// per soft and rigid geometry while parsing cs:: properties,
// mujoco_contact_surfaces_plugin.cpp:650-790) and runs again on every
// geometry change (onGeomChanged).
//
// Order: the key of element i of a geom is (Morton code << 32) | i, the code
// interleaving 10 bits per axis of the centroid's place in the bounding box
// of the geom's vertices, in FP64 exactly as a host restatement computes it;
// keys are unique, so the order is that of a stable sort by code.  Sorting:
// chunks of kSortChunk keys are sorted in shared memory (bitonic), then each
// key's place in its geom is its place in its chunk plus, for every other
// chunk of the geom, the number of keys below it (binary search).
#include <cuda_runtime.h>

#include "hc_internal.h"
#include "kernels.h"

namespace hc {

namespace {

constexpr int kSortChunk = 2048;
constexpr int kSortThreads = 1024;

__device__ __forceinline__ uint32_t expand_bits3(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

// Keys of every element of geom blockIdx.x, at its pool positions.
__global__ void morton_kernel(const float4* __restrict__ raw, int npe, const LbvhSeg* __restrict__ segs,
                              unsigned long long* __restrict__ keys) {
  const LbvhSeg S = segs[blockIdx.x];
  double ext[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ext[a] = S.hi[a] - S.lo[a];
  for (int i = threadIdx.x; i < S.n; i += blockDim.x) {
    const float4* e = raw + (size_t)npe * ((size_t)S.off + i);
    double c[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < npe; ++k) {
      const float4 v = e[k];
      c[0] = __dadd_rn(c[0], __ddiv_rn((double)v.x, (double)npe));
      c[1] = __dadd_rn(c[1], __ddiv_rn((double)v.y, (double)npe));
      c[2] = __dadd_rn(c[2], __ddiv_rn((double)v.z, (double)npe));
    }
    uint32_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double f = ext[a] > 0.0 ? __ddiv_rn(__dsub_rn(c[a], S.lo[a]), ext[a]) : 0.5;
      q[a] = (uint32_t)fmin(1023.0, fmax(0.0, __dmul_rn(f, 1024.0)));
    }
    const uint32_t code = (expand_bits3(q[0]) << 2) | (expand_bits3(q[1]) << 1) | expand_bits3(q[2]);
    keys[(size_t)S.off + i] = ((unsigned long long)code << 32) | (unsigned)i;
  }
}

// The keys of one chunk of one geom, sorted in place (bitonic, in shared
// memory; short chunks are padded with keys above every real one).
__global__ void __launch_bounds__(kSortThreads) sort_chunks_kernel(unsigned long long* __restrict__ keys,
                                                                   const LbvhSeg* __restrict__ segs,
                                                                   const int* __restrict__ chunk_seg) {
  __shared__ unsigned long long s[kSortChunk];
  const LbvhSeg S = segs[chunk_seg[blockIdx.x]];
  const int c = blockIdx.x - S.chunk_off;
  const size_t base = (size_t)S.off + (size_t)c * kSortChunk;
  const int n = min(kSortChunk, S.n - c * kSortChunk);
  for (int i = threadIdx.x; i < kSortChunk; i += blockDim.x) s[i] = i < n ? keys[base + i] : ~0ull;
  __syncthreads();
  for (int k = 2; k <= kSortChunk; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < kSortChunk; i += blockDim.x) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long x = s[i], y = s[l];
          if ((x > y) == ((i & k) == 0)) {
            s[i] = y;
            s[l] = x;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) keys[base + i] = s[i];
}

// Each key's place in its geom: its place in its sorted chunk plus the keys
// below it in the geom's other chunks.  perm[place] = element index in the
// geom.
__global__ void rank_kernel(const unsigned long long* __restrict__ keys, const LbvhSeg* __restrict__ segs,
                            const int* __restrict__ chunk_seg, int* __restrict__ perm) {
  const LbvhSeg S = segs[chunk_seg[blockIdx.x]];
  const int c = blockIdx.x - S.chunk_off;
  const int nc = (S.n + kSortChunk - 1) / kSortChunk;
  const size_t base = (size_t)S.off + (size_t)c * kSortChunk;
  const int n = min(kSortChunk, S.n - c * kSortChunk);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const unsigned long long key = keys[base + i];
    int r = i;
    for (int o = 0; o < nc; ++o) {
      if (o == c) continue;
      const unsigned long long* ck = keys + (size_t)S.off + (size_t)o * kSortChunk;
      int lo = 0, hi = min(kSortChunk, S.n - o * kSortChunk);
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ck[mid] < key) lo = mid + 1;
        else hi = mid;
      }
      r += lo;
    }
    if (r < S.n) perm[(size_t)S.off + r] = (int)(key & 0xffffffffull);   // unique keys: r < n
  }
}

// Elements of `npe` float4 each, and the per-element side arrays, into pool
// order; orig = the element's index in its geom.
__global__ void gather_kernel(const float4* __restrict__ raw, int npe, const LbvhSeg* __restrict__ segs,
                              const int* __restrict__ perm, float4* __restrict__ out, int* __restrict__ orig,
                              const DfPlane* __restrict__ plane_raw, DfPlane* __restrict__ plane,
                              const DfPlane* __restrict__ edge_raw, DfPlane* __restrict__ edge,
                              const float4* __restrict__ meta_raw, float4* __restrict__ meta) {
  const LbvhSeg S = segs[blockIdx.x];
  for (int i = threadIdx.x; i < S.n; i += blockDim.x) {
    const size_t dst = (size_t)S.off + i;
    int t = perm[dst];
    if (t < 0 || t >= S.n) t = i;   // unreachable with unique keys; keeps every read in the geom
    const size_t src = (size_t)S.off + t;
    for (int k = 0; k < npe; ++k) out[npe * dst + k] = raw[npe * src + k];
    orig[dst] = t;
    if (plane) {
      plane[dst] = plane_raw[src];
      for (int j = 0; j < 3; ++j) edge[3 * dst + j] = edge_raw[3 * src + j];
      meta[dst] = meta_raw[src];
    }
  }
}

}  // namespace

void launch_lbvh_order(const float4* raw, int npe, const LbvhSeg* segs, int n_segs, const int* chunk_seg,
                       int n_chunks, unsigned long long* keys, int* perm, float4* out, int* orig,
                       const DfPlane* plane_raw, DfPlane* plane, const DfPlane* edge_raw, DfPlane* edge,
                       const float4* meta_raw, float4* meta, cudaStream_t s) {
  if (n_segs <= 0) return;
  morton_kernel<<<n_segs, 256, 0, s>>>(raw, npe, segs, keys);
  if (n_chunks > 0) {
    sort_chunks_kernel<<<n_chunks, kSortThreads, 0, s>>>(keys, segs, chunk_seg);
    rank_kernel<<<n_chunks, 256, 0, s>>>(keys, segs, chunk_seg, perm);
  }
  gather_kernel<<<n_segs, 256, 0, s>>>(raw, npe, segs, perm, out, orig, plane_raw, plane, edge_raw, edge, meta_raw,
                                       meta);
}

int lbvh_sort_chunk() { return kSortChunk; }

}  // namespace hc
