// noalloc.cu — hc_step_noalloc: the forward contact step with all of its
// working memory in one static device array, for callers that cannot have
// device memory allocated while they run (include/hc/hc.h states who and
// why).  The kernels are the ones hc_step launches (contact.cu); only the
// buffers they work in differ.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/hc/hc.h"
#include "hc_internal.h"
#include "kernels.h"
#include "noalloc.h"

namespace {

constexpr size_t kScratchBytes = HC_NOALLOC_SCRATCH_BYTES;

// The working memory of every hc_step_noalloc call on a device.  Static
// device memory: the module loader reserves it once per device, nothing
// allocates it per call.
__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_scratch on `dev` (which must be current); looked up
// on the first call for each device and remembered.
hc_status scratch_on(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return hc::set_last_error(HC_ERR_INVALID_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) {
      char msg[160];
      snprintf(msg, sizeof(msg), "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
      return hc::set_last_error(HC_ERR_CUDA, msg);
    }
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return HC_OK;
}

// 256-byte aligned pieces of the array, in order.
struct Carve {
  unsigned char* base;
  size_t used;
  template <class T>
  T* take(size_t n) {
    const size_t off = (used + 255) & ~size_t(255);
    if (off > kScratchBytes || n > (kScratchBytes - off) / sizeof(T)) return nullptr;
    used = off + n * sizeof(T);
    return reinterpret_cast<T*>(base + off);
  }
  size_t left() const {
    const size_t off = (used + 255) & ~size_t(255);
    return off >= kScratchBytes ? 0 : kScratchBytes - off;
  }
};

// Word layout of the counter block (the same meaning as hc_step's).
constexpr int kWTotal = 0, kWStatus = 1, kWCand = 2, kWPoly = 3, kWNext = 4, kWRec = 7, kWTile = 8, kWords = 10;

// The wrench part of the per-pair records, to the caller's n_pair x 6 array.
__global__ void wrench_out_kernel(const hc::PairOut* __restrict__ po, int n_pair, double* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 6 * n_pair) w[i] = po[i / 6].wrench[i % 6];
}

hc_status cuda_fail(const char* what, cudaError_t e) {
  char msg[200];
  snprintf(msg, sizeof(msg), "%s: %s", what, cudaGetErrorString(e));
  return hc::set_last_error(HC_ERR_CUDA, msg);
}

}  // namespace

extern "C" HC_API hc_status hc_step_noalloc(hc_context* ctx, int n_geom, const double* d_xpos,
                                            const double* d_xmat, const double* d_vel, double* d_wrench,
                                            float* d_taxels, void* stream) {
  hc::NoallocView v;
  if (hc_status st = hc::noalloc_view(ctx, &v)) return st;
  hc::StepArgs a = v.args;
  const int n_pair = a.n_pair;
  if (n_pair > 0) {
    if (n_geom <= v.max_geom_id) return hc::set_last_error(HC_ERR_INVALID_ARG, "n_geom must cover every registered geom id");
    if (!d_xpos || !d_xmat) return hc::set_last_error(HC_ERR_INVALID_ARG, "d_xpos and d_xmat are required");
    if (!d_wrench) return hc::set_last_error(HC_ERR_INVALID_ARG, "d_wrench is required");
  }
  // Taxel-point and curved sensors read the polygons a step keeps, which
  // this step does not keep: refuse rather than leave their values stale.
  if (a.n_tsens > 0 || a.n_csens > 0)
    return hc::set_last_error(HC_ERR_UNSUPPORTED,
                              "hc_step_noalloc evaluates flat sensors only; the context has taxel-point or curved "
                              "sensors (use hc_step)");
  if (a.n_cells_total > 0 && !d_taxels) return hc::set_last_error(HC_ERR_INVALID_ARG, "d_taxels is required (the context has sensors)");
  if (n_pair == 0 && a.n_cells_total == 0) return HC_OK;

  cudaError_t e = cudaSetDevice(v.device);
  if (e != cudaSuccess) return cuda_fail("cudaSetDevice", e);
  unsigned char* base = nullptr;
  if (hc_status st = scratch_on(v.device, &base)) return st;

  // Carve the array: fixed-size pieces first, the rest for work items.
  Carve cv{base, 0};
  int* words = cv.take<int>(kWords);
  a.frames = cv.take<hc::FrameDev>(n_pair > 0 ? n_pair : 1);
  a.pair_out = cv.take<hc::PairOut>(n_pair > 0 ? n_pair : 1);
  a.unit_off = cv.take<int>((size_t)a.n_units + 1);
  a.bp_tiles = cv.take<unsigned long long>(a.n_bp_blocks > 0 ? a.n_bp_blocks : 1);   // zeroed by the first kernel
  a.poly_tiles = nullptr;
  a.samples = cv.take<unsigned long long>(v.n_samples > 0 ? v.n_samples : 1);
  a.sens_box = nullptr;   // the whole sample array is cleared below and read
  if (!words || !a.frames || !a.pair_out || !a.unit_off || !a.bp_tiles || !a.samples) {
    char msg[240];
    snprintf(msg, sizeof(msg),
             "no-alloc scratch (%zu bytes) too small for %d pairs, %d broadphase units and %zu ray samples",
             kScratchBytes, n_pair, a.n_units, v.n_samples);
    return hc::set_last_error(HC_ERR_OVERFLOW, msg);
  }
  // items and their per-item sums, two aligned arrays of equal length
  const size_t per_item = sizeof(int4) + sizeof(hc::ItemOut);
  const size_t left = cv.left();
  const size_t cap = left > 512 ? (left - 512) / per_item : 0;
  const int item_cap = (int)(cap < (size_t)0x7fffffff ? cap : (size_t)0x7fffffff);
  a.items = item_cap > 0 ? cv.take<int4>((size_t)item_cap) : nullptr;
  a.item_out = item_cap > 0 ? cv.take<hc::ItemOut>((size_t)item_cap) : nullptr;
  if (!a.items || !a.item_out) {
    char msg[200];
    snprintf(msg, sizeof(msg), "no-alloc scratch (%zu bytes) leaves no room for work items", kScratchBytes);
    return hc::set_last_error(HC_ERR_OVERFLOW, msg);
  }
  a.item_cap = item_cap;
  a.reset_words = nullptr;   // zeroed below, with the samples
  a.out_stage = nullptr;
  a.fused = 0;
  a.item_total = words + kWTotal;
  a.status = words + kWStatus;
  a.cand_count = words + kWCand;
  a.poly_count = words + kWPoly;
  a.item_next = words + kWNext;
  a.tile_ctr = words + kWTile;
  // inputs and outputs of the caller
  a.xpos = d_xpos;
  a.xmat = d_xmat;
  a.vel = d_vel;
  a.taxels = d_taxels;
  // no debug records, no surface records, no kept samples
  a.debug = 0;
  a.cand = nullptr;
  a.cand_cap = 0;
  a.polys = nullptr;
  a.poly_cap = 0;
  a.want_polys = 0;
  a.want_pair = -1;
  a.keep_samples = 0;
  a.recs = nullptr;
  a.rec_key = nullptr;
  a.rec_cap = 0;
  a.rec_count = words + kWRec;

  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : v.stream;
  // The array keeps the previous call's contents: the counter words must
  // start at zero and every ray-sample key at "no hit" (all ones).  The
  // other pieces are fully written by the step before they are read.
  if ((e = cudaMemsetAsync(words, 0, kWords * sizeof(int), s)) != cudaSuccess) return cuda_fail("cudaMemsetAsync", e);
  if (v.n_samples > 0 &&
      (e = cudaMemsetAsync(a.samples, 0xFF, v.n_samples * sizeof(unsigned long long), s)) != cudaSuccess)
    return cuda_fail("cudaMemsetAsync", e);
  hc::launch_step(a, s, nullptr);
  if (n_pair > 0) wrench_out_kernel<<<(6 * n_pair + 255) / 256, 256, 0, s>>>(a.pair_out, n_pair, d_wrench);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail("step launch", e);
  int w[kWords];
  int needed = 0;
  if ((e = cudaMemcpyAsync(w, words, sizeof(w), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return cuda_fail("cudaMemcpyAsync", e);
  if ((e = cudaMemcpyAsync(&needed, a.unit_off + a.n_units, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
    return cuda_fail("cudaMemcpyAsync", e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail("cudaStreamSynchronize", e);
  if (w[kWStatus] & 32) return hc::set_last_error(HC_ERR_CUDA, "a single-pass scan waited past its bound for an earlier tile");
  if (w[kWStatus] & 1) {
    char msg[200];
    snprintf(msg, sizeof(msg), "the step needs %d work items; the no-alloc scratch (%zu bytes) holds %d", needed,
             kScratchBytes, item_cap);
    return hc::set_last_error(HC_ERR_OVERFLOW, msg);
  }
  return HC_OK;
}
