// hc_api.cu — host implementation of the C ABI (include/hc/hc.h).
//
// Owns the device pools and per-step buffers of one context, performs the
// pair dispatch of collision_cb (mujoco_contact_surfaces_plugin.cpp:255-318)
// on the host once per pair list, and launches the device pipeline.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/hc/hc.h"
#include "hc_internal.h"
#include "kernels.h"
#include "meshgen.h"
#include <nvtx3/nvToolsExt.h>
#include "noalloc.h"

namespace {
// A named range on the profiler timeline (NVTX) for the span of a host call;
// without a profiler attached it costs a call and a branch.
struct HostRange {
  explicit HostRange(const char* name) { nvtxRangePushA(name); }
  ~HostRange() { nvtxRangePop(); }
  HostRange(const HostRange&) = delete;
  HostRange& operator=(const HostRange&) = delete;
};
}  // namespace

namespace {

thread_local std::string g_last_error;

hc_status fail(hc_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

#define HC_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(HC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// A device array owned by the context (freed with it).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;  // capacity in elements
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  cudaError_t reserve(size_t want) {
    if (want <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    size_t cap = std::max<size_t>(want, 1);
    cudaError_t e = cudaMalloc(&p, cap * sizeof(T));
    if (e == cudaSuccess) n = cap;
    return e;
  }
  cudaError_t upload(const std::vector<T>& v, cudaStream_t s) {
    cudaError_t e = reserve(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

struct GeomHost {
  int id = -1, type = 0, kind = -1, order = 0;
  double size[3] = {0, 0, 0}, cs5[5] = {0, 0, 0, 0, 0};
  bool is_plane = false;
  hc::SoftMesh soft;
  hc::RigidMesh rigid;
  std::vector<double> mesh_v;  // user mesh for HC_GEOM_MESH (regeneration)
  std::vector<int> mesh_f;
  // device placement
  int elem_off = 0, n_elem = 0, node_off = 0, leaves = 1;
};

struct TaxelHost {
  int geom;
  int method, sample_method, visualize;
  double margin, res;
  std::vector<float4> taxels;   // geom frame
};

struct CurvedHost {
  int geom;
  double margin;
  int n_taxels;
  std::vector<float4> points, normals;   // the surface points some taxel uses (geom frame)
  std::vector<int> off, pt;              // per taxel: its points (local index) in point order
  std::vector<float> w;                  // and their weights
};

struct SensorHost {
  int geom;
  double resolution;
  int sr, window;
  double sigma;
  int cx, cy;
  hc::SensorDev dev;
};

// Device counter words of a context.
constexpr int kCntTotal = 0;   // work items of the step (clamped to capacity)
constexpr int kCntStatus = 1;  // bit 0 item overflow, 1 candidate, 2 polygon
constexpr int kCntCand = 2;    // candidate records written
constexpr int kCntPoly = 3;    // polygon records written
constexpr int kCntNext = 4;    // three work counters, one per query type
constexpr int kCntRec = 7;     // adjoint records kept (may exceed the capacity)
constexpr int kCntAdjSkip = 8; // two words: adjoint vertices left out, smallest |det| (debug)
constexpr int kCntTile = 10;   // two words: the next tile of the broadphase and slot scans
constexpr int kCntWords = 16;
constexpr int kStatusScanWaitBit = 32;   // status: a look-back wait ran out (contact.cu)
static_assert(kCntTile + 1 < hc::kResetWords, "the step's first kernel zeroes the counters up to kCntTile + 1");

int next_pow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

double combined_E(double a, double b) {
  if (std::isinf(a)) return b;
  if (std::isinf(b)) return a;
  return a * b / (a + b);
}

}  // namespace

struct hc_context {
  hc_config cfg;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::map<int, GeomHost> geoms;
  int n_registered = 0;
  bool pools_dirty = true;
  int max_geom_id = -1;
  // pools
  DevBuf<float4> tets, tris, nodes;
  DevBuf<float4> tet_props;   // two per tet: the constants of its field
  DevBuf<int> tet_orig, tri_orig;
  // inputs
  DevBuf<double> xpos, xmat, vel;
  int n_pose = 0;
  bool have_vel = false;
  bool poses_set = false;
  // pairs
  std::vector<hc::PairDev> pairs_h;
  std::vector<int> g1_h, g2_h;
  DevBuf<hc::PairDev> pairs;
  DevBuf<hc::FrameDev> frames;
  DevBuf<int> unit_pair, unit_cl, unit_off;
  DevBuf<unsigned long long> bp_tiles;   // the broadphase scan's look-back state, one per block
  int n_units = 0, n_bp_blocks = 0;
  DevBuf<int4> items;
  DevBuf<hc::ItemOut> item_out;
  int item_cap = 0;
  DevBuf<int> counters;  // see kCnt* below
  int type_units[3][2] = {{0, 0}, {0, 0}, {0, 0}};  // unit ranges per query type
  DevBuf<hc::DfPlane> tri_plane, tri_edges;
  DevBuf<float4> tri_meta;
  DevBuf<hc::PairOut> pair_out;
  // sensors
  std::vector<SensorHost> sensors;
  DevBuf<hc::SensorDev> sensors_d;
  DevBuf<unsigned long long> samples;
  DevBuf<int4> sens_box;   // per flat sensor: the sample box the last step touched
  DevBuf<float> taxels, weights, samp_coord;
  DevBuf<int> cell_sensor, cell_first;
  int n_cells = 0;
  bool sensors_dirty = false;
  // debug
  int debug = 0;
  DevBuf<hc::CandRec> cand;
  int cand_cap = 0;
  DevBuf<hc::PolyRec> polys;
  int poly_cap = 0;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_valid = false;
  bool stepped = false;
  bool timing = false;
  cudaEvent_t ev[8] = {};   // stage boundaries; ev[6]: narrow kernels | kept polygons;
                            // ev[7]: end of the adjoint (fused step)
  // forward step and adjoint captured as one graph (hc_step_adjoint*)
  cudaGraph_t fused_graph = nullptr;
  cudaGraphExec_t fused_exec = nullptr;
  // host copies beside the fused graph (hc_step_adjoint): the upstream
  // gradients go in and the taxel maps come out on copy_stream while the
  // graph computes; xev[0] upstream in (the graph's adjoint waits on it),
  // xev[1] forward done (recorded by the graph), xev[2] taxel maps out
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t xev[3] = {};
  bool fused_valid = false;
  const void* fused_key[6] = {};   // upstream, adjoint and result buffers it was captured with
  DevBuf<double> out_stage;        // fused step's results back to back: wrenches n x 6,
                                   // pose gradients n x 12, moduli gradients n x 2
  bool last_fused = false;         // the last step ran as the fused graph
  hc_timings last_timings = {};
  int launches_per_step = 0;
  int narrow_block = 128, narrow_ctas_per_sm = 8, narrow_chunk = 4;
  int rec_fwd_ctas = 4, rec_adj_ctas = 4;   // resident CTAs per SM of the kept-polygon kernels
  int n_sm = 0;
  // adjoint
  bool adjoint_mode = false;   // steps keep the won taxel samples
  bool samples_dirty = false;  // the sample buffer holds a kept step's hits
  bool step_checked = false;  // the last step's status word was read and clean
  bool samples_used = false;   // a taxel adjoint consumed some of them (recomputed
                               // polygons take their samples once: exact ties)
  DevBuf<float> adj_pair, adj_taxel;
  DevBuf<double> adj_item, adj_out, adj_wrench;
  int adj_launches = 0;
  // adjoint records (polygons kept by steps in adjoint mode)
  DevBuf<hc::AdjPoly> recs;
  DevBuf<int2> rec_key;
  DevBuf<hc::RecOut> rec_out;
  DevBuf<float4> slot_press;
  DevBuf<int> rec_perm;
  DevBuf<int> rec_dst;
  // taxel-point sensors
  std::vector<TaxelHost> tsens_h;
  std::vector<int> tsens_enabled_h;
  DevBuf<hc::TaxelSensorDev> tsens;
  DevBuf<int> tsens_pairs, tsens_enabled;
  DevBuf<float4> taxel_pos;
  DevBuf<float> taxel_val;
  DevBuf<int> tpairs, tpair_ai, tsort, tidx;   // taxel-sensor pairs; polygon order per record slot
  DevBuf<unsigned long long> tkey;
  DevBuf<double> tat;                           // running fan areas (area-importance sensors)
  int n_tpairs = 0;
  // curved sensors
  std::vector<CurvedHost> csens_h;
  std::vector<int> csens_enabled_h;
  DevBuf<hc::CurvedSensorDev> csens;
  DevBuf<int> csens_pairs, csens_enabled, clist_off, clist_pt;
  DevBuf<float4> cpoints, cnormals;
  DevBuf<float> clist_w, chit, cvalues;
  bool tsens_ai = false;
  int n_taxel_total = 0;
  DevBuf<float> rec_grad;
  DevBuf<int> item_poly_off;
  DevBuf<unsigned long long> poly_tiles;   // the slot scan's look-back state, one per kBpBlock items
  int rec_cap = 0;
  bool recs_step = false;  // the last step kept its polygons
};

namespace {

void invalidate_graph(hc_context* c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
  c->graph_valid = false;
  if (c->fused_exec) cudaGraphExecDestroy(c->fused_exec);
  if (c->fused_graph) cudaGraphDestroy(c->fused_graph);
  c->fused_exec = nullptr;
  c->fused_graph = nullptr;
  c->fused_valid = false;
}

hc_status build_pools(hc_context* c) {
  if (!c->pools_dirty) return HC_OK;
  std::vector<GeomHost*> order;
  for (auto& kv : c->geoms) order.push_back(&kv.second);
  std::sort(order.begin(), order.end(), [](GeomHost* a, GeomHost* b) { return a->order < b->order; });
  // every element in its geom's original order; the device orders each geom
  // along its Morton curve (launch_lbvh_order)
  std::vector<float4> tets, tris, tri_meta;
  std::vector<hc::Dbl4> tri_plane, tri_edges;
  std::vector<hc::LbvhSeg> sseg, rseg;
  std::vector<int> s_chunk_seg, r_chunk_seg;
  const int chunk = hc::lbvh_sort_chunk();
  auto segment = [&](std::vector<hc::LbvhSeg>& segs, std::vector<int>& chunk_seg, const std::vector<double>& v,
                     int off, int n) {
    hc::LbvhSeg g{};
    g.off = off;
    g.n = n;
    g.chunk_off = (int)chunk_seg.size();
    for (int a = 0; a < 3; ++a) g.lo[a] = 1e300, g.hi[a] = -1e300;
    for (size_t i = 0; i < v.size(); i += 3)
      for (int a = 0; a < 3; ++a) g.lo[a] = std::min(g.lo[a], v[i + a]), g.hi[a] = std::max(g.hi[a], v[i + a]);
    for (int k = 0; k < (n + chunk - 1) / chunk; ++k) chunk_seg.push_back((int)segs.size());
    segs.push_back(g);
  };
  int node_total = 0;
  std::vector<int> s_eoff, s_ne, s_noff, s_L, r_eoff, r_ne, r_noff, r_L;
  for (GeomHost* g : order) {
    g->n_elem = 0;
    g->leaves = 1;
    if (g->kind == HC_SOFT) {
      const auto& m = g->soft;
      int ne = (int)(m.t.size() / 4);
      g->elem_off = (int)(tets.size() / 4);
      g->n_elem = ne;
      for (int t = 0; t < ne; ++t) {
        for (int k = 0; k < 4; ++k) {
          int vi = m.t[4 * t + k];
          tets.push_back(make_float4((float)m.v[3 * vi], (float)m.v[3 * vi + 1], (float)m.v[3 * vi + 2], (float)m.p[vi]));
        }
      }
      segment(sseg, s_chunk_seg, m.v, g->elem_off, ne);
      s_eoff.push_back(g->elem_off); s_ne.push_back(ne);
    } else if (g->kind == HC_RIGID && !g->is_plane) {
      const auto& m = g->rigid;
      int ne = (int)(m.f.size() / 3);
      g->elem_off = (int)(tris.size() / 3);
      g->n_elem = ne;
      for (int t = 0; t < ne; ++t) {
        const double* r[3];
        for (int k = 0; k < 3; ++k) {
          int vi = m.f[3 * t + k];
          r[k] = &m.v[3 * vi];
          tris.push_back(make_float4((float)m.v[3 * vi], (float)m.v[3 * vi + 1], (float)m.v[3 * vi + 2], 0.f));
        }
        // FP64 plane of the triangle in its body frame (from the stored
        // float vertices), min altitude, max edge and coordinate magnitude
        double e1[3], e2[3], N[3];
        for (int a = 0; a < 3; ++a) e1[a] = r[1][a] - r[0][a], e2[a] = r[2][a] - r[0][a];
        N[0] = e1[1] * e2[2] - e1[2] * e2[1];
        N[1] = e1[2] * e2[0] - e1[0] * e2[2];
        N[2] = e1[0] * e2[1] - e1[1] * e2[0];
        double ln = std::sqrt(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
        double le = 0, mag = 0;
        for (int k = 0; k < 3; ++k) {
          const double* p0 = r[k];
          const double* p1 = r[(k + 1) % 3];
          double d2 = 0;
          for (int a = 0; a < 3; ++a) d2 += (p1[a] - p0[a]) * (p1[a] - p0[a]), mag = std::max(mag, std::fabs(p0[a]));
          le = std::max(le, std::sqrt(d2));
        }
        double n[3] = {0, 0, 1};
        if (ln > 0) n[0] = N[0] / ln, n[1] = N[1] / ln, n[2] = N[2] / ln;
        tri_plane.push_back(hc::Dbl4{n[0], n[1], n[2], n[0] * r[0][0] + n[1] * r[0][1] + n[2] * r[0][2]});
        // in-plane inward edge planes: unit n x (r_{j+1} - r_j), offset at r_j
        for (int j = 0; j < 3; ++j) {
          const double* a0 = r[j];
          const double* a1 = r[(j + 1) % 3];
          double e[3] = {a1[0] - a0[0], a1[1] - a0[1], a1[2] - a0[2]};
          double m[3] = {n[1] * e[2] - n[2] * e[1], n[2] * e[0] - n[0] * e[2], n[0] * e[1] - n[1] * e[0]};
          double lm = std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
          if (lm > 0) m[0] /= lm, m[1] /= lm, m[2] /= lm;
          tri_edges.push_back(hc::Dbl4{m[0], m[1], m[2], m[0] * a0[0] + m[1] * a0[1] + m[2] * a0[2]});
        }
        tri_meta.push_back(make_float4(ln > 0 && le > 0 ? (float)(ln / le) : 0.f, (float)le, (float)mag, 0.f));
      }
      segment(rseg, r_chunk_seg, m.v, g->elem_off, ne);
      r_eoff.push_back(g->elem_off); r_ne.push_back(ne);
    } else {
      continue;
    }
    int ncl = std::max(1, (g->n_elem + hc::kCluster - 1) / hc::kCluster);
    g->leaves = next_pow2(ncl);
    g->node_off = node_total;
    node_total += 2 * g->leaves;
    if (g->kind == HC_SOFT) { s_noff.push_back(g->node_off); s_L.push_back(g->leaves); }
    else { r_noff.push_back(g->node_off); r_L.push_back(g->leaves); }
  }
  cudaStream_t s = c->stream;
  const size_t n_tet = tets.size() / 4, n_tri = tris.size() / 3;
  HC_CUDA(c->tets.reserve(std::max<size_t>(4, tets.size())));
  HC_CUDA(c->tris.reserve(std::max<size_t>(3, tris.size())));
  HC_CUDA(c->tet_orig.reserve(std::max<size_t>(1, n_tet)));
  HC_CUDA(c->tri_orig.reserve(std::max<size_t>(1, n_tri)));
  // planes as FP32 head and tail (the device rotates them in double-float)
  auto split = [](const std::vector<hc::Dbl4>& in) {
    std::vector<hc::DfPlane> out(in.size());
    for (size_t i = 0; i < in.size(); ++i) {
      const double d[4] = {in[i].x, in[i].y, in[i].z, in[i].w};
      float h[4], l[4];
      for (int k = 0; k < 4; ++k) {
        h[k] = (float)d[k];
        l[k] = (float)(d[k] - (double)h[k]);
      }
      out[i].hi = make_float4(h[0], h[1], h[2], h[3]);
      out[i].lo = make_float4(l[0], l[1], l[2], l[3]);
    }
    return out;
  };
  HC_CUDA(c->tri_plane.reserve(std::max<size_t>(1, n_tri)));
  HC_CUDA(c->tri_edges.reserve(std::max<size_t>(3, 3 * n_tri)));
  HC_CUDA(c->tri_meta.reserve(std::max<size_t>(1, n_tri)));
  {
    // the LBVH element order on the device: Morton keys, sort, gather
    DevBuf<float4> raw, meta_raw;
    DevBuf<hc::DfPlane> plane_raw, edge_raw;
    DevBuf<hc::LbvhSeg> segs;
    DevBuf<int> chunk_seg, perm;
    DevBuf<unsigned long long> keys;
    HC_CUDA(keys.reserve(std::max<size_t>(1, std::max(n_tet, n_tri))));
    HC_CUDA(perm.reserve(std::max<size_t>(1, std::max(n_tet, n_tri))));
    if (!sseg.empty()) {
      HC_CUDA(raw.upload(tets, s));
      HC_CUDA(segs.upload(sseg, s));
      HC_CUDA(chunk_seg.upload(s_chunk_seg, s));
      hc::launch_lbvh_order(raw.p, 4, segs.p, (int)sseg.size(), chunk_seg.p, (int)s_chunk_seg.size(), keys.p, perm.p,
                            c->tets.p, c->tet_orig.p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, s);
      HC_CUDA(cudaGetLastError());
    }
    if (!rseg.empty()) {
      HC_CUDA(raw.upload(tris, s));
      HC_CUDA(segs.upload(rseg, s));
      HC_CUDA(chunk_seg.upload(r_chunk_seg, s));
      HC_CUDA(plane_raw.upload(split(tri_plane), s));
      HC_CUDA(edge_raw.upload(split(tri_edges), s));
      HC_CUDA(meta_raw.upload(tri_meta, s));
      hc::launch_lbvh_order(raw.p, 3, segs.p, (int)rseg.size(), chunk_seg.p, (int)r_chunk_seg.size(), keys.p, perm.p,
                            c->tris.p, c->tri_orig.p, plane_raw.p, c->tri_plane.p, edge_raw.p, c->tri_edges.p,
                            meta_raw.p, c->tri_meta.p, s);
      HC_CUDA(cudaGetLastError());
    }
    // the scratch is freed when the order is done
    HC_CUDA(cudaStreamSynchronize(s));
  }
  HC_CUDA(c->tet_props.reserve(std::max<size_t>(2, tets.size() / 2)));
  hc::launch_tet_props(c->tets.p, c->tet_props.p, (int)n_tet, s);
  HC_CUDA(cudaGetLastError());
  // two float4 (lo, hi) per node
  HC_CUDA(c->nodes.reserve(2 * (size_t)std::max(1, node_total)));
  // LBVH node boxes on the device
  auto refit = [&](const std::vector<int>& eoff, const std::vector<int>& ne, const std::vector<int>& noff,
                   const std::vector<int>& L, const float4* elems, int vpe) -> hc_status {
    if (eoff.empty()) return HC_OK;
    DevBuf<int> a, b, d, e;
    std::vector<int> all;
    if (a.upload(eoff, s) || b.upload(ne, s) || d.upload(noff, s) || e.upload(L, s)) return fail(HC_ERR_CUDA, "refit upload");
    hc::launch_refit(elems, vpe, c->nodes.p, a.p, b.p, d.p, e.p, (int)eoff.size(), s);
    cudaError_t err = cudaStreamSynchronize(s);
    a.release(); b.release(); d.release(); e.release();
    if (err != cudaSuccess) return fail(HC_ERR_CUDA, std::string("refit: ") + cudaGetErrorString(err));
    return HC_OK;
  };
  hc_status st = refit(s_eoff, s_ne, s_noff, s_L, c->tets.p, 4);
  if (st) return st;
  st = refit(r_eoff, r_ne, r_noff, r_L, c->tris.p, 3);
  if (st) return st;
  HC_CUDA(cudaGetLastError());
  c->pools_dirty = false;
  invalidate_graph(c);
  return HC_OK;
}

bool finite_all(const double* p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

hc_status ensure_rec_offsets(hc_context* c);

hc_status ensure_items(hc_context* c, int cap) {
  if (cap <= c->item_cap) return HC_OK;
  HC_CUDA(c->items.reserve(cap));
  HC_CUDA(c->item_out.reserve(cap));
  c->item_cap = cap;
  invalidate_graph(c);
  return ensure_rec_offsets(c);
}

// Capacity of the polygon records (kept by steps with sensors or in adjoint
// mode).
// Polygons are kept as records (rays cast and sensors sampled from them, the
// adjoint reads them) in adjoint mode and whenever sensors are attached.
bool keeps_polygons(const hc_context* c) {
  return c->adjoint_mode || c->n_cells > 0 || !c->tsens_h.empty() || !c->csens_h.empty();
}

int initial_rec_cap(const hc_context* c) {
  return c->cfg.face_capacity > 0 ? (int)std::min<int64_t>(c->cfg.face_capacity, (1 << 30) - 1)
                                  : std::max(1 << 15, 4 * c->item_cap);
}

// Per-item record offsets: item_cap + 1 ints and one scan tile state per kBpBlock items.
hc_status ensure_rec_offsets(hc_context* c) {
  if (c->rec_cap == 0) return HC_OK;
  const size_t blocks = (size_t)std::max(1, (c->item_cap + hc::kBpBlock - 1) / hc::kBpBlock);
  if ((size_t)c->item_cap + 1 <= c->item_poly_off.n && blocks <= c->poly_tiles.n) return HC_OK;
  HC_CUDA(c->item_poly_off.reserve((size_t)c->item_cap + 1));
  HC_CUDA(c->poly_tiles.reserve(blocks));
  invalidate_graph(c);
  return HC_OK;
}

hc_status ensure_recs(hc_context* c, int cap) {
  // record slots are 30-bit fields of the sample keys; the all-ones field is
  // the empty sample's, so the largest slot is 2^30 - 2
  cap = std::min(cap, (1 << 30) - 1);
  if (cap > c->rec_cap) {
    HC_CUDA(c->recs.reserve(cap));
    HC_CUDA(c->rec_key.reserve(cap));
    HC_CUDA(c->rec_out.reserve(cap));
    HC_CUDA(c->slot_press.reserve(6 * (size_t)cap));
    HC_CUDA(c->rec_perm.reserve(cap));
    HC_CUDA(c->rec_dst.reserve(cap));
    HC_CUDA(c->rec_grad.reserve(16 * (size_t)cap));
    c->rec_cap = cap;
    invalidate_graph(c);
  }
  if (!c->tsens_h.empty() && c->tsort.n < (size_t)c->rec_cap) {
    HC_CUDA(c->tsort.reserve(c->rec_cap));
    HC_CUDA(c->tidx.reserve(c->rec_cap));
    HC_CUDA(c->tkey.reserve(c->rec_cap));
    invalidate_graph(c);
  }
  bool ai = false;
  for (const TaxelHost& h : c->tsens_h) ai = ai || h.sample_method == HC_SAMPLE_AREA_IMPORTANCE;
  if (ai && c->tat.n < (size_t)c->rec_cap * hc::kMaxPolyV) {
    HC_CUDA(c->tat.reserve((size_t)c->rec_cap * hc::kMaxPolyV));
    invalidate_graph(c);
  }
  return ensure_rec_offsets(c);
}

hc_status build_sensors(hc_context* c) {
  if (!c->sensors_dirty) return HC_OK;
  std::vector<hc::SensorDev> sd;
  std::vector<float> w, coord;
  std::vector<int> cell_sensor, cell_first;
  int64_t smp = 0;
  int cells = 0;
  for (size_t k = 0; k < c->sensors.size(); ++k) {
    SensorHost& S = c->sensors[k];
    const GeomHost& g = c->geoms[S.geom];
    hc::SensorDev d;
    d.geom = S.geom;
    d.cx = S.cx; d.cy = S.cy; d.sr = S.sr;
    d.nx = S.cx * S.sr; d.ny = S.cy * S.sr;
    d.sample_off = smp;
    smp += (int64_t)d.nx * d.ny;
    d.taxel_off = cells;
    cell_first.push_back(cells);
    for (int i = 0; i < S.cx * S.cy; ++i) cell_sensor.push_back((int)k);
    cells += S.cx * S.cy;
    // constants of FlatTactileSensor::load (flat_tactile_sensor.cpp:179-185)
    const double resolution = S.resolution;
    const int sr = S.sr;
    float xs = (float)g.size[0], ys = (float)g.size[1], zs = (float)g.size[2];
    float rSampling_resolution = (float)(resolution / sr);
    d.rmean = (float)(1. / (sr * sr));
    d.zs15 = (float)(1.5 * zs);
    // sample coordinates in the sensor frame (FS:324-327)
    d.samp_off_x = (int)coord.size();
    for (int x = 0; x < S.cx; ++x)
      for (int i = 0; i < sr; ++i)
        coord.push_back((float)((double)(-xs) + x * resolution + (double)(float)(i * rSampling_resolution) +
                                0.5 * rSampling_resolution));
    d.samp_off_y = (int)coord.size();
    for (int y = 0; y < S.cy; ++y)
      for (int j = 0; j < sr; ++j)
        coord.push_back((float)((double)(-ys) + y * resolution + (double)(float)(j * rSampling_resolution) +
                                0.5 * rSampling_resolution));
    // window weights (FS:305-388)
    d.weight_off = (int)w.size();
    float di_factor = (float)(resolution / sr);
    float sub_halfwidth = (float)(di_factor / 2.0f - resolution / 2.0f);
    const float SQRT_2 = 1.41421356237f;
    float max_dist = (float)(SQRT_2 * resolution / 2.0f);
    float sigma = (float)S.sigma;
    float rsigma_squared = S.window == HC_WINDOW_GAUSS ? 0.5f / (sigma * sigma) : 0.f;
    float rtukey = S.window == HC_WINDOW_TUKEY ? 1.f / sigma * sr * sr : 0.f;
    for (int i = 0; i < sr; ++i)
      for (int j = 0; j < sr; ++j) {
        float weight = 1.0f;
        if (S.window == HC_WINDOW_GAUSS) {
          float dist = std::hypot(di_factor * i + sub_halfwidth, di_factor * j + sub_halfwidth) / max_dist;
          weight = std::exp(-(dist * dist) * rsigma_squared);
        } else if (S.window == HC_WINDOW_TUKEY) {
          if (sr / 2 - std::abs(sr / 2 - i) <= sigma * sr / 2)
            weight *= 0.5f * (1.f - cosf((float)(2.f * M_PI * (sr / 2 - std::abs(sr / 2 - i)) * rtukey)));
          if (sr / 2 - std::abs(sr / 2 - j) <= sigma * sr / 2)
            weight *= 0.5f * (1.f - cosf((float)(2.f * M_PI * (sr / 2 - std::abs(sr / 2 - j)) * rtukey)));
        } else if (S.window == HC_WINDOW_SQUARE) {
          float inv_dist = 1 - std::hypot(di_factor * i + sub_halfwidth, di_factor * j + sub_halfwidth) / max_dist;
          weight = inv_dist * inv_dist;
        }
        w.push_back(weight);
      }
    S.dev = d;
    sd.push_back(d);
  }
  cudaStream_t s = c->stream;
  HC_CUDA(c->sensors_d.upload(sd, s));
  HC_CUDA(c->weights.upload(w, s));
  HC_CUDA(c->samp_coord.upload(coord, s));
  HC_CUDA(c->cell_sensor.upload(cell_sensor, s));
  HC_CUDA(c->cell_first.upload(cell_first, s));
  HC_CUDA(c->taxels.reserve(std::max(1, cells)));
  HC_CUDA(c->samples.reserve(std::max<int64_t>(1, smp)));
  if (smp > 0) HC_CUDA(cudaMemsetAsync(c->samples.p, 0xFF, smp * sizeof(unsigned long long), s));
  {
    // every sensor's touched box starts empty (X0 > X1)
    std::vector<int4> empty(std::max<size_t>(1, c->sensors.size()), make_int4(0x7fffffff, -1, 0x7fffffff, -1));
    HC_CUDA(c->sens_box.reserve(empty.size()));
    HC_CUDA(cudaMemcpyAsync(c->sens_box.p, empty.data(), empty.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  }
  if (cells > 0) HC_CUDA(cudaMemsetAsync(c->taxels.p, 0, cells * sizeof(float), s));
  c->n_cells = cells;
  c->sensors_dirty = false;
  invalidate_graph(c);
  return HC_OK;
}

hc::StepArgs make_args(hc_context* c, int want_polys, int want_pair) {
  hc::StepArgs a;
  memset(&a, 0, sizeof(a));
  a.xpos = c->xpos.p;
  a.xmat = c->xmat.p;
  a.vel = c->have_vel ? c->vel.p : nullptr;
  a.pairs = c->pairs.p;
  a.n_pair = (int)c->pairs_h.size();
  a.frames = c->frames.p;
  a.tets = c->tets.p;
  a.tet_props = c->tet_props.p;
  a.tet_orig = c->tet_orig.p;
  a.tris = c->tris.p;
  a.tri_orig = c->tri_orig.p;
  a.nodes = c->nodes.p;
  a.unit_pair = c->unit_pair.p;
  a.unit_cl = c->unit_cl.p;
  a.n_units = c->n_units;
  a.unit_off = c->unit_off.p;
  a.bp_tiles = c->bp_tiles.p;
  a.n_bp_blocks = c->n_bp_blocks;
  a.items = c->items.p;
  a.item_cap = c->item_cap;
  a.reset_words = c->counters.p;   // kResetWords (12) words: total .. the scans' tile counters
  a.tile_ctr = c->counters.p + kCntTile;
  a.item_total = c->counters.p + kCntTotal;
  a.status = c->counters.p + kCntStatus;
  a.cand_count = c->counters.p + kCntCand;
  a.poly_count = c->counters.p + kCntPoly;
  a.item_next = c->counters.p + kCntNext;
  for (int q = 0; q < 3; ++q) {
    a.type_unit_begin[q] = c->type_units[q][0];
    a.type_unit_end[q] = c->type_units[q][1];
  }
  a.tri_plane = c->tri_plane.p;
  a.tri_edges = c->tri_edges.p;
  a.tri_meta = c->tri_meta.p;
  a.item_out = c->item_out.p;
  a.pair_out = c->pair_out.p;
  a.sensors = c->sensors_d.p;
  a.n_sensor = (int)c->sensors.size();
  a.samples = c->samples.p;
  a.sens_box = c->sens_box.p;
  a.taxels = c->taxels.p;
  a.weights = c->weights.p;
  a.samp_coord = c->samp_coord.p;
  a.n_cells_total = c->n_cells;
  a.cell_sensor = c->cell_sensor.p;
  a.cell_first = c->cell_first.p;
  a.repr = c->cfg.representation;
  a.apply_forces = c->cfg.apply_forces;
  a.debug = c->debug;
  a.cand = c->cand.p;
  a.cand_cap = c->cand_cap;
  a.polys = c->polys.p;
  a.poly_cap = c->poly_cap;
  a.want_polys = want_polys;
  a.want_pair = want_pair;
  a.narrow_block = c->narrow_block;
  a.narrow_grid = std::max(1, c->n_sm * c->narrow_ctas_per_sm);
  a.rec_fwd_grid = std::max(1, c->n_sm * c->rec_fwd_ctas);
  a.rec_adj_grid = std::max(1, c->n_sm * c->rec_adj_ctas);
  a.chunk = std::max(1, c->narrow_chunk);
  a.keep_samples = c->adjoint_mode ? 1 : 0;
  a.rec_count = c->counters.p + kCntRec;
  a.adj_skip = (c->debug & HC_DEBUG_CANDIDATES) ? c->counters.p + kCntAdjSkip : nullptr;
  // polygons are kept as records (rays cast and taxels sampled from them,
  // the adjoint reads them) in adjoint mode and whenever sensors are attached
  if (keeps_polygons(c) && c->rec_cap > 0) {
    a.recs = c->recs.p;
    a.rec_key = c->rec_key.p;
    a.rec_cap = c->rec_cap;
    a.rec_out = c->rec_out.p;
    a.slot_press = c->slot_press.p;
    a.rec_perm = c->rec_perm.p;
    a.rec_dst = c->rec_dst.p;
    a.item_poly_off = c->item_poly_off.p;
    a.poly_tiles = c->poly_tiles.p;
    a.n_item_blocks = std::max(1, (c->item_cap + hc::kBpBlock - 1) / hc::kBpBlock);
    a.tsens = c->tsens.p;
    a.n_tsens = (int)c->tsens_h.size();
    a.tsens_pairs = c->tsens_pairs.p;
    a.tsens_enabled = c->tsens_enabled.p;
    a.taxel_pos = c->taxel_pos.p;
    a.taxel_val = c->taxel_val.p;
    a.tpairs = c->tpairs.p;
    a.tpair_ai = c->tpair_ai.p;
    a.n_tpairs = c->n_tpairs;
    a.tat = c->tat.p;
    a.csens = c->csens.p;
    a.n_csens = (int)c->csens_h.size();
    a.csens_pairs = c->csens_pairs.p;
    a.csens_enabled = c->csens_enabled.p;
    a.cpoints = c->cpoints.p;
    a.cnormals = c->cnormals.p;
    a.clist_off = c->clist_off.p;
    a.clist_pt = c->clist_pt.p;
    a.clist_w = c->clist_w.p;
    a.chit = c->chit.p;
    a.cvalues = c->cvalues.p;
    a.tsort = c->tsort.p;
    a.tkey = c->tkey.p;
    a.tidx = c->tidx.p;
  }
  return a;
}

// Launch one step on the context stream (graph when possible).
hc_status run_step(hc_context* c, int want_polys, int want_pair) {
  if (c->pairs_h.empty() && c->sensors.empty()) {
    c->stepped = true;
    return HC_OK;
  }
  hc::StepArgs a = make_args(c, want_polys, want_pair);
  c->recs_step = a.recs != nullptr;
  c->step_checked = false;
  c->last_fused = false;
  // (the step's first kernel zeroes the counters: StepArgs::reset_words)
  // samples an earlier step kept lie inside that step's touched boxes: the
  // step's first kernel clears those boxes (launch_step)
  c->samples_dirty = c->adjoint_mode && c->n_cells > 0;
  c->samples_used = false;
  // With timing on, event records between the stages are part of the
  // launch sequence (and of the captured graph).
  cudaEvent_t* ev = c->timing && !want_polys ? c->ev : nullptr;
  bool use_graph = c->cfg.use_graph && !want_polys;
  if (!use_graph) {
    c->launches_per_step = hc::launch_step(a, c->stream, ev);
    HC_CUDA(cudaGetLastError());
    c->stepped = true;
    return HC_OK;
  }
  if (!c->graph_valid) {
    invalidate_graph(c);
    HC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->launches_per_step = hc::launch_step(a, c->stream, ev);
    cudaError_t e = cudaStreamEndCapture(c->stream, &c->graph);
    if (e != cudaSuccess) return fail(HC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    HC_CUDA(cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
    c->graph_valid = true;
  }
  HC_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
  c->stepped = true;
  return HC_OK;
}

// Check the status word; on item overflow grow the capacity and re-run.
// Once a step has checked clean, later calls return at once.
hc_status finish_step(hc_context* c) {
  if (c->step_checked) return HC_OK;
  HostRange range_("wait for the step");
  for (int attempt = 0; attempt < 4; ++attempt) {
    int cnt[8];
    HC_CUDA(cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    if (cnt[kCntStatus] & kStatusScanWaitBit)
      return fail(HC_ERR_CUDA, "a single-pass scan waited past its bound for an earlier tile");
    if (!(cnt[kCntStatus] & 9)) {
      c->step_checked = true;
      return HC_OK;
    }
    if (cnt[kCntStatus] & 8) {
      // too many polygons for the records (rays and adjoint): grow, re-run
      const int want = std::max(2 * c->rec_cap, cnt[kCntRec] + cnt[kCntRec] / 4 + 1024);
      if (hc_status st = ensure_recs(c, want)) return st;
    }
    if (cnt[kCntStatus] & 1) {
      // item overflow: the scan wrote the full total into unit_off[n_units]
      int total = 0;
      HC_CUDA(cudaMemcpy(&total, c->unit_off.p + c->n_units, sizeof(int), cudaMemcpyDeviceToHost));
      if (hc_status st = ensure_items(c, std::max(2 * c->item_cap, total + total / 4 + 1024))) return st;
    }
    if (hc_status st = run_step(c, 0, -1)) return st;
  }
  return fail(HC_ERR_OVERFLOW, "work-item or polygon-record capacity overflow persisted");
}

hc_status need(hc_context* c) {
  if (!c) return fail(HC_ERR_INVALID_ARG, "null context");
  return HC_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

void hc_config_default(hc_config* cfg) {
  if (!cfg) return;
  memset(cfg, 0, sizeof(*cfg));
  cfg->device = 0;
  cfg->representation = HC_REPR_TRIANGLE;
  cfg->apply_forces = 1;
  cfg->use_graph = 1;
  cfg->item_capacity = 0;
  cfg->face_capacity = 0;
}

const char* hc_last_error(void) { return g_last_error.c_str(); }

const char* hc_version(void) { return "hydroelastic-gb300 0.1 (sm_103a)"; }

hc_status hc_context_create(const hc_config* cfg, hc_context** out) {
  if (!out) return fail(HC_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  hc_config c0;
  hc_config_default(&c0);
  if (cfg) c0 = *cfg;
  if (c0.representation != HC_REPR_TRIANGLE && c0.representation != HC_REPR_POLYGON)
    return fail(HC_ERR_INVALID_ARG, "representation must be HC_REPR_TRIANGLE or HC_REPR_POLYGON");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(HC_ERR_NO_DEVICE, "no CUDA device visible");
  if (c0.device < 0 || c0.device >= ndev) return fail(HC_ERR_INVALID_ARG, "device ordinal out of range");
  HC_CUDA(cudaSetDevice(c0.device));
  HC_CUDA(hc::init_kernel_attributes());
  hc_context* c = new hc_context();
  c->cfg = c0;
  c->device = c0.device;
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, c0.device);
  c->n_sm = prop.multiProcessorCount;
  hc::record_ctas_per_sm(&c->rec_fwd_ctas, &c->rec_adj_ctas);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return fail(HC_ERR_CUDA, "stream create failed");
  }
  for (auto& ev : c->ev) cudaEventCreate(&ev);
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return fail(HC_ERR_CUDA, "stream create failed");
  }
  for (auto& ev : c->xev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (c->counters.reserve(kCntWords) != cudaSuccess) {
    delete c;
    return fail(HC_ERR_CUDA, "counter alloc failed");
  }
  cudaMemset(c->counters.p, 0, kCntWords * sizeof(int));
  *out = c;
  return HC_OK;
}

hc_status hc_context_destroy(hc_context* c) {
  if (!c) return HC_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  invalidate_graph(c);
  cudaStreamSynchronize(c->copy_stream);
  for (auto& ev : c->ev) cudaEventDestroy(ev);
  for (auto& ev : c->xev) cudaEventDestroy(ev);
  cudaStreamDestroy(c->stream);
  cudaStreamDestroy(c->copy_stream);
  delete c;   // every device array is freed by its destructor
  return HC_OK;
}

hc_status hc_reset(hc_context* c) {
  if (hc_status st = need(c)) return st;
  c->stepped = false;
  return HC_OK;
}

hc_status hc_generate_mesh(int type, const double size[3], const double cs5[5], const double* mesh_vert, int nvert,
                           const int* mesh_face, int nface, int* out_kind, int* out_nvert, int* out_nelem,
                           double* vert, double* pressure, int* elems) {
  if (!size || !cs5) return fail(HC_ERR_INVALID_ARG, "size and cs5 are required");
  double E = cs5[0], hint = cs5[2];
  if (out_kind) *out_kind = -1;
  if (E > 0) {
    hc::SoftMesh m;
    std::string err = hc::make_soft_mesh(type, size, E, hint, mesh_vert, nvert, mesh_face, nface, &m);
    if (!err.empty()) {
      bool unsup = type == HC_GEOM_PLANE || type == HC_GEOM_HFIELD || type == HC_GEOM_CAPSULE;
      return fail(unsup ? HC_ERR_UNSUPPORTED : hc::is_degenerate(err) ? HC_ERR_DEGENERATE : HC_ERR_INVALID_ARG, err);
    }
    hc::round_to_float(&m);
    if (std::string d = hc::degenerate_soft(m); !d.empty()) return fail(HC_ERR_DEGENERATE, d);
    if (out_kind) *out_kind = HC_SOFT;
    if (out_nvert) *out_nvert = (int)(m.v.size() / 3);
    if (out_nelem) *out_nelem = (int)(m.t.size() / 4);
    if (vert) memcpy(vert, m.v.data(), m.v.size() * sizeof(double));
    if (pressure) memcpy(pressure, m.p.data(), m.p.size() * sizeof(double));
    if (elems) memcpy(elems, m.t.data(), m.t.size() * sizeof(int));
    return HC_OK;
  }
  hc::RigidMesh m;
  std::string err = hc::make_rigid_mesh(type, size, hint, mesh_vert, nvert, mesh_face, nface, &m);
  if (!err.empty()) {
    bool unsup = type == HC_GEOM_HFIELD || type == HC_GEOM_CAPSULE;
    return fail(unsup ? HC_ERR_UNSUPPORTED : hc::is_degenerate(err) ? HC_ERR_DEGENERATE : HC_ERR_INVALID_ARG, err);
  }
  hc::round_to_float(&m);
  if (std::string d = hc::degenerate_rigid(m, type == HC_GEOM_PLANE); !d.empty()) return fail(HC_ERR_DEGENERATE, d);
  if (out_kind) *out_kind = HC_RIGID;
  if (out_nvert) *out_nvert = (int)(m.v.size() / 3);
  if (out_nelem) *out_nelem = (int)(m.f.size() / 3);
  if (vert) memcpy(vert, m.v.data(), m.v.size() * sizeof(double));
  if (elems) memcpy(elems, m.f.data(), m.f.size() * sizeof(int));
  return HC_OK;
}

static hc_status make_geom_mesh(GeomHost* g) {
  double E = g->cs5[0], hint = g->cs5[2];
  const double* mv = g->mesh_v.empty() ? nullptr : g->mesh_v.data();
  const int* mf = g->mesh_f.empty() ? nullptr : g->mesh_f.data();
  int nv = (int)(g->mesh_v.size() / 3), nf = (int)(g->mesh_f.size() / 3);
  if (E > 0) {
    std::string err = hc::make_soft_mesh(g->type, g->size, E, hint, mv, nv, mf, nf, &g->soft);
    if (!err.empty()) return fail(hc::is_degenerate(err) ? HC_ERR_DEGENERATE : HC_ERR_INVALID_ARG, err);
    hc::round_to_float(&g->soft);
    if (std::string d = hc::degenerate_soft(g->soft); !d.empty()) return fail(HC_ERR_DEGENERATE, d);
    g->kind = HC_SOFT;
  } else {
    std::string err = hc::make_rigid_mesh(g->type, g->size, hint, mv, nv, mf, nf, &g->rigid);
    if (!err.empty()) return fail(hc::is_degenerate(err) ? HC_ERR_DEGENERATE : HC_ERR_INVALID_ARG, err);
    hc::round_to_float(&g->rigid);
    if (std::string d = hc::degenerate_rigid(g->rigid, g->type == HC_GEOM_PLANE); !d.empty())
      return fail(HC_ERR_DEGENERATE, d);
    g->kind = HC_RIGID;
    g->is_plane = g->type == HC_GEOM_PLANE;
  }
  return HC_OK;
}

hc_status hc_add_geom(hc_context* c, int geom_id, int type, const double size[3], const double cs5[5],
                      const double* mesh_vert, int nvert, const int* mesh_face, int nface, int* out_kind) {
  HostRange range_("hc_add_geom");
  if (hc_status st = need(c)) return st;
  if (out_kind) *out_kind = -1;
  if (geom_id < 0) return fail(HC_ERR_INVALID_ARG, "negative geom id");
  if (!size || !cs5) return fail(HC_ERR_INVALID_ARG, "size and cs5 are required");
  if (c->geoms.count(geom_id)) return fail(HC_ERR_INVALID_ARG, "geom id already registered");
  if (!finite_all(size, 3) || !finite_all(cs5, 5)) return fail(HC_ERR_INVALID_ARG, "non-finite size or cs:: values");
  // soft plane, hfield and capsule have no contact surface.
  if (type == HC_GEOM_HFIELD || type == HC_GEOM_CAPSULE || (type == HC_GEOM_PLANE && cs5[0] > 0))
    return fail(HC_ERR_UNSUPPORTED, "geom type has no hydroelastic representation");
  if (type < 0 || type > HC_GEOM_MESH) return fail(HC_ERR_INVALID_ARG, "unknown geom type");
  GeomHost g;
  g.id = geom_id;
  g.type = type;
  memcpy(g.size, size, sizeof(g.size));
  memcpy(g.cs5, cs5, sizeof(g.cs5));
  if (type == HC_GEOM_MESH) {
    if (!mesh_vert || !mesh_face || nvert <= 0 || nface <= 0) return fail(HC_ERR_INVALID_ARG, "mesh geom needs data");
    g.mesh_v.assign(mesh_vert, mesh_vert + 3 * (size_t)nvert);
    g.mesh_f.assign(mesh_face, mesh_face + 3 * (size_t)nface);
  }
  if (hc_status st = make_geom_mesh(&g)) return st;
  g.order = c->n_registered++;
  if (out_kind) *out_kind = g.kind;
  c->max_geom_id = std::max(c->max_geom_id, geom_id);
  c->geoms[geom_id] = std::move(g);
  c->pools_dirty = true;
  c->pairs_h.clear();  // pair tables refer to pool offsets
  return HC_OK;
}

hc_status hc_update_geom_size(hc_context* c, int geom_id, const double size[3]) {
  HostRange range_("hc_update_geom_size");
  if (hc_status st = need(c)) return st;
  auto it = c->geoms.find(geom_id);
  if (it == c->geoms.end()) return fail(HC_ERR_INVALID_ARG, "unknown geom id");
  if (!size || !finite_all(size, 3)) return fail(HC_ERR_INVALID_ARG, "bad size");
  GeomHost& g = it->second;
  double old[3];
  memcpy(old, g.size, sizeof(old));
  memcpy(g.size, size, sizeof(g.size));
  if (hc_status st = make_geom_mesh(&g)) {
    memcpy(g.size, old, sizeof(old));
    make_geom_mesh(&g);
    return st;
  }
  c->pools_dirty = true;
  // Pair tables hold pool offsets: rebuild them for the current pairs.
  if (!c->pairs_h.empty()) {
    std::vector<int> g1 = c->g1_h, g2 = c->g2_h;
    return hc_set_pairs(c, (int)g1.size(), g1.data(), g2.data(), nullptr, nullptr);
  }
  return HC_OK;
}

hc_status hc_get_geom_info(hc_context* c, int geom_id, hc_geom_info* out) {
  if (hc_status st = need(c)) return st;
  auto it = c->geoms.find(geom_id);
  if (it == c->geoms.end() || !out) return fail(HC_ERR_INVALID_ARG, "unknown geom id");
  const GeomHost& g = it->second;
  out->kind = g.kind;
  out->type = g.type;
  out->order = g.order;
  out->n_elements = g.kind == HC_SOFT ? (int)(g.soft.t.size() / 4) : (int)(g.rigid.f.size() / 3);
  out->n_vertices = g.kind == HC_SOFT ? (int)(g.soft.v.size() / 3) : (int)(g.rigid.v.size() / 3);
  out->E = g.cs5[0]; out->dissipation = g.cs5[1]; out->resolution_hint = g.cs5[2];
  out->mu_static = g.cs5[3]; out->mu_dynamic = g.cs5[4];
  return HC_OK;
}

hc_status hc_get_element_order(hc_context* c, int geom_id, int* order) {
  if (hc_status st = need(c)) return st;
  auto it = c->geoms.find(geom_id);
  if (it == c->geoms.end()) return fail(HC_ERR_INVALID_ARG, "unknown geom id");
  if (!order) return fail(HC_ERR_INVALID_ARG, "null output");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = build_pools(c)) return st;
  const GeomHost& g = it->second;
  if (g.n_elem == 0) return HC_OK;
  const int* src = g.kind == HC_SOFT ? c->tet_orig.p : c->tri_orig.p;
  HC_CUDA(cudaStreamSynchronize(c->stream));
  HC_CUDA(cudaMemcpy(order, src + g.elem_off, (size_t)g.n_elem * sizeof(int), cudaMemcpyDeviceToHost));
  return HC_OK;
}

hc_status hc_get_geom_mesh(hc_context* c, int geom_id, double* vert, double* pressure, int* elems) {
  if (hc_status st = need(c)) return st;
  auto it = c->geoms.find(geom_id);
  if (it == c->geoms.end()) return fail(HC_ERR_INVALID_ARG, "unknown geom id");
  const GeomHost& g = it->second;
  if (g.kind == HC_SOFT) {
    if (vert) memcpy(vert, g.soft.v.data(), g.soft.v.size() * sizeof(double));
    if (pressure) memcpy(pressure, g.soft.p.data(), g.soft.p.size() * sizeof(double));
    if (elems) memcpy(elems, g.soft.t.data(), g.soft.t.size() * sizeof(int));
  } else {
    if (vert) memcpy(vert, g.rigid.v.data(), g.rigid.v.size() * sizeof(double));
    if (elems) memcpy(elems, g.rigid.f.data(), g.rigid.f.size() * sizeof(int));
  }
  return HC_OK;
}

hc_status hc_set_poses(hc_context* c, int n_geom, const double* xpos, const double* xmat, const double* vel) {
  if (hc_status st = need(c)) return st;
  if (n_geom <= c->max_geom_id) return fail(HC_ERR_INVALID_ARG, "n_geom must cover every registered geom id");
  if (!xpos || !xmat) return fail(HC_ERR_INVALID_ARG, "xpos and xmat are required");
  HC_CUDA(cudaSetDevice(c->device));
  if ((size_t)n_geom * 3 > c->xpos.n || (size_t)n_geom * 9 > c->xmat.n || (size_t)n_geom * 6 > c->vel.n) {
    HC_CUDA(c->xpos.reserve((size_t)n_geom * 3));
    HC_CUDA(c->xmat.reserve((size_t)n_geom * 9));
    HC_CUDA(c->vel.reserve((size_t)n_geom * 6));
    invalidate_graph(c);
  }
  HC_CUDA(cudaMemcpyAsync(c->xpos.p, xpos, (size_t)n_geom * 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  HC_CUDA(cudaMemcpyAsync(c->xmat.p, xmat, (size_t)n_geom * 9 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  bool hv = vel != nullptr;
  if (hv) HC_CUDA(cudaMemcpyAsync(c->vel.p, vel, (size_t)n_geom * 6 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (hv != c->have_vel) invalidate_graph(c);
  c->have_vel = hv;
  c->n_pose = n_geom;
  c->poses_set = true;
  return HC_OK;
}

hc_status hc_set_poses_device(hc_context* c, int n_geom, const double* d_xpos, const double* d_xmat,
                              const double* d_vel) {
  if (hc_status st = need(c)) return st;
  if (n_geom <= c->max_geom_id) return fail(HC_ERR_INVALID_ARG, "n_geom must cover every registered geom id");
  if (!d_xpos || !d_xmat) return fail(HC_ERR_INVALID_ARG, "xpos and xmat are required");
  HC_CUDA(cudaSetDevice(c->device));
  if ((size_t)n_geom * 3 > c->xpos.n || (size_t)n_geom * 9 > c->xmat.n || (size_t)n_geom * 6 > c->vel.n) {
    HC_CUDA(c->xpos.reserve((size_t)n_geom * 3));
    HC_CUDA(c->xmat.reserve((size_t)n_geom * 9));
    HC_CUDA(c->vel.reserve((size_t)n_geom * 6));
    invalidate_graph(c);
  }
  HC_CUDA(cudaMemcpyAsync(c->xpos.p, d_xpos, (size_t)n_geom * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  HC_CUDA(cudaMemcpyAsync(c->xmat.p, d_xmat, (size_t)n_geom * 9 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  bool hv = d_vel != nullptr;
  if (hv) HC_CUDA(cudaMemcpyAsync(c->vel.p, d_vel, (size_t)n_geom * 6 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  if (hv != c->have_vel) invalidate_graph(c);
  c->have_vel = hv;
  c->n_pose = n_geom;
  c->poses_set = true;
  return HC_OK;
}

hc_status hc_set_pairs(hc_context* c, int n_pair, const int* g1, const int* g2, int* per_pair_status,
                       int* per_pair_query) {
  HostRange range_("hc_set_pairs");
  if (hc_status st = need(c)) return st;
  if (n_pair < 0 || (n_pair > 0 && (!g1 || !g2))) return fail(HC_ERR_INVALID_ARG, "bad pair arrays");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = build_pools(c)) return st;
  if (hc_status st = build_sensors(c)) return st;
  std::vector<hc::PairDev> P(n_pair);
  std::vector<int> upair, ucl;
  hc_status worst = HC_OK;
  for (int i = 0; i < n_pair; ++i) {
    hc::PairDev& p = P[i];
    memset(&p, 0, sizeof(p));
    p.sensor0 = p.sensor1 = -1;
    auto i1 = c->geoms.find(g1[i]), i2 = c->geoms.find(g2[i]);
    int st = HC_OK;
    p.gs = p.gm = std::max(0, g1[i]);
    p.go = p.gn = std::max(0, g2[i]);
    if (g1[i] < 0 || g2[i] < 0 || g1[i] == g2[i]) {
      st = HC_ERR_INVALID_ARG;
    } else if (i1 == c->geoms.end() || i2 == c->geoms.end() ||
               (i1->second.kind == HC_RIGID && i2->second.kind == HC_RIGID)) {
      st = HC_ERR_UNSUPPORTED;
    }
    p.unit_begin = p.unit_end = (int)upair.size();
    if (st == HC_OK) {
      const GeomHost& G1 = i1->second;
      const GeomHost& G2 = i2->second;
      const GeomHost& M = G1.order <= G2.order ? G1 : G2;
      const GeomHost& N = &M == &G1 ? G2 : G1;
      const GeomHost* S;
      const GeomHost* O;
      if (G1.kind == HC_SOFT && G2.kind == HC_SOFT) {
        p.query = HC_QUERY_SOFT_SOFT;
        S = &M; O = &N;
      } else {
        S = G1.kind == HC_SOFT ? &G1 : &G2;
        O = S == &G1 ? &G2 : &G1;
        p.query = O->is_plane ? HC_QUERY_SOFT_HALFSPACE : HC_QUERY_SOFT_RIGID;
      }
      p.gs = S->id; p.go = O->id; p.gm = M.id; p.gn = N.id;
      p.s_is_m = S == &M;
      p.s_elem_off = S->elem_off; p.s_n_elem = S->n_elem; p.s_node_off = S->node_off; p.s_leaves = S->leaves;
      p.o_elem_off = O->elem_off; p.o_n_elem = O->n_elem; p.o_node_off = O->node_off; p.o_leaves = O->leaves;
      p.o_n_clusters = (O->n_elem + hc::kCluster - 1) / hc::kCluster;
      // material combination
      double EM = M.kind == HC_SOFT ? M.cs5[0] : INFINITY, EN = N.kind == HC_SOFT ? N.cs5[0] : INFINITY;
      double dM = M.kind == HC_SOFT ? M.cs5[1] : 1.0, dN = N.kind == HC_SOFT ? N.cs5[1] : 1.0;
      double Es = combined_E(EM, EN), d = 0;
      if (std::isinf(Es)) d = 0.5 * (dM + dN);
      else {
        if (!std::isinf(EM)) d += Es / EM * dM;
        if (!std::isinf(EN)) d += Es / EN * dN;
      }
      double ma = M.cs5[4], mb = N.cs5[4];
      p.damping = (float)d;
      p.mu = (float)(ma + mb == 0 ? 0.0 : 2 * ma * mb / (ma + mb));
      p.E_s = (float)S->cs5[0];
      p.E_o = O->kind == HC_SOFT ? (float)O->cs5[0] : 0.f;
      if (p.query == HC_QUERY_SOFT_SOFT) {   // S = M, O = N
        const double den = (EM + EN) * (EM + EN);
        p.dd_dEs = (float)(EN * (dN - dM) / den);
        p.dd_dEo = (float)(EM * (dM - dN) / den);
      }
      int ns = 0;
      for (size_t k = 0; k < c->sensors.size() && ns < 2; ++k)
        if (c->sensors[k].geom == g1[i] || c->sensors[k].geom == g2[i]) {
          if (ns == 0) p.sensor0 = (int)k; else p.sensor1 = (int)k;
          ++ns;
        }
    } else {
      p.query = HC_QUERY_NONE;
      if (worst == HC_OK) worst = (hc_status)st;
    }
    if (per_pair_status) per_pair_status[i] = st;
    if (per_pair_query) per_pair_query[i] = p.query;
  }
  // Broadphase units ordered by query type, then pair: each narrow-phase
  // kernel works one contiguous item range; each pair's units (and items)
  // stay contiguous for the per-pair reduction.
  const int qorder[3] = {HC_QUERY_SOFT_RIGID, HC_QUERY_SOFT_HALFSPACE, HC_QUERY_SOFT_SOFT};
  for (int qi = 0; qi < 3; ++qi) {
    c->type_units[qi][0] = (int)upair.size();
    for (int i = 0; i < n_pair; ++i) {
      hc::PairDev& p = P[i];
      if (p.query != qorder[qi]) continue;
      p.unit_begin = (int)upair.size();
      if (p.query == HC_QUERY_SOFT_HALFSPACE) {
        upair.push_back(i); ucl.push_back(-1);
      } else {
        for (int k = 0; k < p.o_n_clusters; ++k) { upair.push_back(i); ucl.push_back(k); }
      }
      p.unit_end = (int)upair.size();
    }
    c->type_units[qi][1] = (int)upair.size();
  }
  cudaStream_t s = c->stream;
  c->pairs_h = P;
  c->g1_h.assign(g1, g1 + n_pair);
  c->g2_h.assign(g2, g2 + n_pair);
  HC_CUDA(c->pairs.upload(P, s));
  HC_CUDA(c->frames.reserve(std::max(1, n_pair)));
  HC_CUDA(c->pair_out.reserve(std::max(1, n_pair)));
  c->n_units = (int)upair.size();
  // broadphase: a warp per unit, kBpBlock / 32 units per block
  c->n_bp_blocks = std::max(1, (c->n_units + hc::kBpBlock / 32 - 1) / (hc::kBpBlock / 32));
  HC_CUDA(c->unit_pair.upload(upair, s));
  HC_CUDA(c->unit_cl.upload(ucl, s));
  HC_CUDA(c->unit_off.reserve(c->n_units + 1));
  HC_CUDA(c->bp_tiles.reserve(c->n_bp_blocks));
  int want = c->cfg.item_capacity > 0 ? (int)c->cfg.item_capacity : std::max(1 << 16, 64 * n_pair);
  if (hc_status st = ensure_items(c, want)) return st;
  if (keeps_polygons(c))
    if (hc_status st = ensure_recs(c, initial_rec_cap(c))) return st;
  // curved sensors: the soft-rigid and half-space pairs of each sensor geom
  if (!c->csens_h.empty()) {
    std::vector<hc::CurvedSensorDev> cd;
    std::vector<int> cp, loff(1, 0), lpt;
    std::vector<float4> pts, nrm;
    std::vector<float> lw;
    for (const CurvedHost& h : c->csens_h) {
      hc::CurvedSensorDev d;
      d.geom = h.geom;
      d.n_taxels = h.n_taxels;
      d.taxel_off = (int)loff.size() - 1;
      d.n_points = (int)h.points.size();
      d.point_off = (int)pts.size();
      d.margin = (float)h.margin;
      d.pair_off = (int)cp.size();
      for (int i = 0; i < n_pair; ++i)
        if ((P[i].query == HC_QUERY_SOFT_RIGID || P[i].query == HC_QUERY_SOFT_HALFSPACE) &&
            (g1[i] == h.geom || g2[i] == h.geom))
          cp.push_back(i);
      d.n_pairs = (int)cp.size() - d.pair_off;
      const int base = loff.back();
      for (int i = 0; i < h.n_taxels; ++i) loff.push_back(base + h.off[(size_t)i + 1]);
      lpt.insert(lpt.end(), h.pt.begin(), h.pt.end());
      lw.insert(lw.end(), h.w.begin(), h.w.end());
      pts.insert(pts.end(), h.points.begin(), h.points.end());
      nrm.insert(nrm.end(), h.normals.begin(), h.normals.end());
      cd.push_back(d);
    }
    if (cp.empty()) cp.push_back(0);
    if (lpt.empty()) { lpt.push_back(0); lw.push_back(0.f); }
    if (pts.empty()) { pts.push_back(make_float4(0, 0, 0, 0)); nrm.push_back(make_float4(0, 0, 0, 0)); }
    HC_CUDA(c->csens.upload(cd, s));
    HC_CUDA(c->csens_pairs.upload(cp, s));
    HC_CUDA(c->csens_enabled.upload(c->csens_enabled_h, s));
    HC_CUDA(c->clist_off.upload(loff, s));
    HC_CUDA(c->clist_pt.upload(lpt, s));
    HC_CUDA(c->clist_w.upload(lw, s));
    HC_CUDA(c->cpoints.upload(pts, s));
    HC_CUDA(c->cnormals.upload(nrm, s));
    HC_CUDA(c->chit.reserve(pts.size()));
    if (c->cvalues.n < (size_t)loff.size() - 1 || c->cvalues.p == nullptr) {
      HC_CUDA(c->cvalues.reserve(std::max<size_t>(1, loff.size() - 1)));
      HC_CUDA(cudaMemsetAsync(c->cvalues.p, 0, c->cvalues.n * sizeof(float), s));
    }
  }
  // taxel-point sensors: the soft-rigid and half-space pairs of each sensor
  // geom, in pair order
  if (!c->tsens_h.empty()) {
    std::vector<hc::TaxelSensorDev> td;
    std::vector<int> tp;
    std::vector<float4> pos;
    for (const TaxelHost& h : c->tsens_h) {
      hc::TaxelSensorDev d;
      d.geom = h.geom;
      d.n_taxels = (int)h.taxels.size();
      d.taxel_off = (int)pos.size();
      d.method = h.method;
      d.sample_method = h.sample_method;
      d.visualize = h.visualize;
      d.margin = h.margin;
      d.res = h.res;
      d.pair_off = (int)tp.size();
      for (int i = 0; i < n_pair; ++i)
        if ((P[i].query == HC_QUERY_SOFT_RIGID || P[i].query == HC_QUERY_SOFT_HALFSPACE) &&
            (g1[i] == h.geom || g2[i] == h.geom))
          tp.push_back(i);
      d.n_pairs = (int)tp.size() - d.pair_off;
      pos.insert(pos.end(), h.taxels.begin(), h.taxels.end());
      td.push_back(d);
    }
    HC_CUDA(c->tsens.upload(td, s));
    std::vector<int> up(tp);
    std::sort(up.begin(), up.end());
    up.erase(std::unique(up.begin(), up.end()), up.end());
    c->n_tpairs = (int)up.size();
    // pairs read by an area-importance sensor get their running fan areas
    std::vector<int> uai(up.size(), 0);
    for (size_t k = 0; k < td.size(); ++k) {
      if (td[k].sample_method != HC_SAMPLE_AREA_IMPORTANCE) continue;
      for (int j = 0; j < td[k].n_pairs; ++j) {
        const int pr = tp[td[k].pair_off + j];
        uai[std::lower_bound(up.begin(), up.end(), pr) - up.begin()] = 1;
      }
    }
    if (up.empty()) { up.push_back(0); uai.push_back(0); }
    HC_CUDA(c->tpairs.upload(up, s));
    HC_CUDA(c->tpair_ai.upload(uai, s));
    if (tp.empty()) tp.push_back(0);
    HC_CUDA(c->tsens_pairs.upload(tp, s));
    HC_CUDA(c->tsens_enabled.upload(c->tsens_enabled_h, s));
    HC_CUDA(c->taxel_pos.upload(pos, s));
    if ((int)pos.size() != c->n_taxel_total) {
      HC_CUDA(c->taxel_val.reserve(pos.size()));
      HC_CUDA(cudaMemsetAsync(c->taxel_val.p, 0, pos.size() * sizeof(float), s));
      c->n_taxel_total = (int)pos.size();
    }
  }
  HC_CUDA(cudaStreamSynchronize(s));
  invalidate_graph(c);
  c->stepped = false;
  (void)worst;
  return HC_OK;
}

hc_status hc_step(hc_context* c) {
  HostRange range_("hc_step");
  if (hc_status st = need(c)) return st;
  if (!c->poses_set && !c->pairs_h.empty()) return fail(HC_ERR_NOT_READY, "poses not set");
  HC_CUDA(cudaSetDevice(c->device));
  if (c->pools_dirty || c->sensors_dirty) {
    std::vector<int> g1 = c->g1_h, g2 = c->g2_h;
    if (hc_status st = hc_set_pairs(c, (int)g1.size(), g1.data(), g2.data(), nullptr, nullptr)) return st;
  }
  if ((size_t)c->n_pose * 3 > c->xpos.n || c->n_pose <= c->max_geom_id)
    return fail(HC_ERR_NOT_READY, "poses do not cover every registered geom");
  return run_step(c, 0, -1);
}

hc_status hc_collide_pairs(hc_context* c, int n_pair, const int* g1, const int* g2, int* per_pair_status) {
  if (hc_status st = hc_set_pairs(c, n_pair, g1, g2, per_pair_status, nullptr)) return st;
  return hc_step(c);
}

hc_status hc_get_wrenches(hc_context* c, double* wrench) {
  HostRange range_("hc_get_wrenches");
  if (hc_status st = need(c)) return st;
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  size_t n = c->pairs_h.size();
  if (!wrench || !n) return HC_OK;
  // the wrench of each pair record, straight into the caller's rows
  HC_CUDA(cudaMemcpy2DAsync(wrench, 6 * sizeof(double), c->pair_out.p, sizeof(hc::PairOut), 6 * sizeof(double), n,
                            cudaMemcpyDeviceToHost, c->stream));
  HC_CUDA(cudaStreamSynchronize(c->stream));
  return HC_OK;
}

hc_status hc_get_wrenches_device(hc_context* c, const double** d_wrench) {
  if (hc_status st = need(c)) return st;
  if (!d_wrench) return fail(HC_ERR_INVALID_ARG, "null output");
  *d_wrench = reinterpret_cast<const double*>(c->pair_out.p);
  return HC_OK;
}

hc_status hc_get_pair_order(hc_context* c, int* query, int* m_geom, int* n_geom) {
  if (hc_status st = need(c)) return st;
  for (size_t i = 0; i < c->pairs_h.size(); ++i) {
    if (query) query[i] = c->pairs_h[i].query;
    if (m_geom) m_geom[i] = c->pairs_h[i].gm;
    if (n_geom) n_geom[i] = c->pairs_h[i].gn;
  }
  return HC_OK;
}

hc_status hc_get_pair_stats(hc_context* c, hc_pair_stats* out) {
  if (hc_status st = need(c)) return st;
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  size_t n = c->pairs_h.size();
  if (!out || !n) return HC_OK;
  std::vector<hc::PairOut> o(n);
  HC_CUDA(cudaMemcpy(o.data(), c->pair_out.p, n * sizeof(hc::PairOut), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < n; ++i) {
    out[i].n_polygons = o[i].n_poly;
    out[i].n_faces = o[i].n_faces;
    out[i].n_near_degenerate = o[i].n_near;
    out[i].n_items = o[i].n_items;
    out[i].area = o[i].area;
    out[i].total_fn0 = o[i].total_fn0;
  }
  return HC_OK;
}

hc_status hc_set_debug(hc_context* c, int flags) {
  if (hc_status st = need(c)) return st;
  HC_CUDA(cudaSetDevice(c->device));
  if ((flags & HC_DEBUG_CANDIDATES) && c->cand_cap == 0) {
    c->cand_cap = 1 << 22;
    HC_CUDA(c->cand.reserve(c->cand_cap));
  }
  if (flags != c->debug) invalidate_graph(c);
  c->debug = flags;
  return HC_OK;
}

hc_status hc_get_candidates(hc_context* c, hc_candidate* out, int64_t capacity, int64_t* count) {
  if (hc_status st = need(c)) return st;
  if (!(c->debug & HC_DEBUG_CANDIDATES)) return fail(HC_ERR_NOT_READY, "candidate recording is off");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  int cnt[8];
  HC_CUDA(cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
  if (cnt[kCntStatus] & 2) return fail(HC_ERR_OVERFLOW, "candidate record buffer overflow");
  int64_t n = std::min<int64_t>(cnt[kCntCand], c->cand_cap);
  if (count) *count = n;
  if (out && capacity > 0) {
    int64_t k = std::min(n, capacity);
    std::vector<hc::CandRec> r(k);
    HC_CUDA(cudaMemcpy(r.data(), c->cand.p, k * sizeof(hc::CandRec), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < k; ++i) {
      out[i].pair = r[i].pair; out[i].elem_a = r[i].elem_a; out[i].elem_b = r[i].elem_b;
      out[i].n_vert = r[i].n_vert; out[i].flags = r[i].flags;
    }
  }
  return HC_OK;
}

hc_status hc_get_surface(hc_context* c, int pair, hc_surface_view* view) {
  HostRange range_("hc_get_surface");
  if (hc_status st = need(c)) return st;
  if (!view || pair < 0 || pair >= (int)c->pairs_h.size()) return fail(HC_ERR_INVALID_ARG, "bad pair or view");
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (c->poly_cap == 0) {
    c->poly_cap = 1 << 20;
    HC_CUDA(c->polys.reserve(c->poly_cap));
  }
  // Re-run the (deterministic) step with polygon recording for this pair.
  if (hc_status st = run_step(c, 1, pair)) return st;
  if (hc_status st = finish_step(c)) return st;
  int cnt[8];
  HC_CUDA(cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
  if (cnt[kCntStatus] & 4) return fail(HC_ERR_OVERFLOW, "surface record buffer overflow");
  int n = std::min(cnt[kCntPoly], c->poly_cap);
  std::vector<hc::PolyRec> r(n);
  if (n) HC_CUDA(cudaMemcpy(r.data(), c->polys.p, n * sizeof(hc::PolyRec), cudaMemcpyDeviceToHost));
  std::sort(r.begin(), r.end(), [](const hc::PolyRec& a, const hc::PolyRec& b) {
    return a.elem_a != b.elem_a ? a.elem_a < b.elem_a : a.elem_b < b.elem_b;
  });
  int nv = 0;
  for (auto& p : r) nv += p.nv;
  view->n_poly = n;
  view->n_vert = nv;
  if (!view->poly_offset && !view->vert && !view->vert_pressure && !view->normal && !view->elem_a && !view->elem_b)
    return HC_OK;
  // soft frame -> world
  const hc::PairDev& P = c->pairs_h[pair];
  double R[9], x[3];
  HC_CUDA(cudaMemcpy(R, c->xmat.p + 9 * (size_t)P.gs, sizeof(R), cudaMemcpyDeviceToHost));
  HC_CUDA(cudaMemcpy(x, c->xpos.p + 3 * (size_t)P.gs, sizeof(x), cudaMemcpyDeviceToHost));
  int k = 0;
  for (int i = 0; i < n; ++i) {
    const hc::PolyRec& p = r[i];
    if (view->poly_offset) view->poly_offset[i] = k;
    for (int j = 0; j < p.nv; ++j, ++k) {
      double v[3] = {p.v[j][0], p.v[j][1], p.v[j][2]};
      for (int a = 0; a < 3; ++a)
        if (view->vert) view->vert[3 * k + a] = R[3 * a] * v[0] + R[3 * a + 1] * v[1] + R[3 * a + 2] * v[2] + x[a];
      if (view->vert_pressure) view->vert_pressure[k] = p.v[j][3];
    }
    for (int a = 0; a < 3; ++a)
      if (view->normal) view->normal[3 * i + a] = R[3 * a] * p.n[0] + R[3 * a + 1] * p.n[1] + R[3 * a + 2] * p.n[2];
    if (view->elem_a) view->elem_a[i] = p.elem_a;
    if (view->elem_b) view->elem_b[i] = p.elem_b;
  }
  if (view->poly_offset) view->poly_offset[n] = k;
  return HC_OK;
}

hc_status hc_add_taxel_sensor(hc_context* c, int geom_id, int n_taxels, const double* taxels, int method,
                              double include_margin, double sample_resolution, int sample_method, int visualize,
                              int* out_sensor) {
  HostRange range_("hc_add_taxel_sensor");
  if (hc_status st = need(c)) return st;
  if (!c->geoms.count(geom_id)) return fail(HC_ERR_INVALID_ARG, "sensor geom has no cs:: properties");
  if (n_taxels <= 0 || n_taxels > (1 << 20) || !taxels) return fail(HC_ERR_INVALID_ARG, "1 to 2^20 taxels are needed");
  if (method < HC_TAXEL_CLOSEST || method > HC_TAXEL_SQUARED) return fail(HC_ERR_INVALID_ARG, "bad taxel method");
  if (sample_method != HC_SAMPLE_DEFAULT && sample_method != HC_SAMPLE_AREA_IMPORTANCE)
    return fail(HC_ERR_INVALID_ARG, "bad sample method");
  if (!(include_margin > 0) || !(sample_resolution > 0) || !finite_all(taxels, 3 * (size_t)n_taxels))
    return fail(HC_ERR_INVALID_ARG, "bad margin, resolution or taxel position");
  TaxelHost h;
  h.geom = geom_id;
  h.method = method;
  h.sample_method = sample_method;
  h.visualize = visualize ? 1 : 0;
  h.margin = include_margin;
  h.res = sample_resolution;
  for (int i = 0; i < n_taxels; ++i)
    h.taxels.push_back(make_float4((float)taxels[3 * i], (float)taxels[3 * i + 1], (float)taxels[3 * i + 2], 0.f));
  c->tsens_h.push_back(h);
  c->tsens_enabled_h.push_back(1);
  c->sensors_dirty = true;   // pairs are dispatched again before the next step
  if (out_sensor) *out_sensor = (int)c->tsens_h.size() - 1;
  return HC_OK;
}

hc_status hc_set_taxel_sensor_enabled(hc_context* c, int sensor, int on) {
  if (hc_status st = need(c)) return st;
  if (sensor < 0 || sensor >= (int)c->tsens_h.size()) return fail(HC_ERR_INVALID_ARG, "bad taxel sensor");
  c->tsens_enabled_h[sensor] = on ? 1 : 0;
  if (c->tsens_enabled.n >= c->tsens_enabled_h.size()) {
    HC_CUDA(cudaSetDevice(c->device));
    HC_CUDA(cudaMemcpyAsync(c->tsens_enabled.p + sensor, &c->tsens_enabled_h[sensor], sizeof(int),
                            cudaMemcpyHostToDevice, c->stream));
  }
  return HC_OK;
}

hc_status hc_get_taxel_sensor_values(hc_context* c, int sensor, float* out) {
  if (hc_status st = need(c)) return st;
  if (sensor < 0 || sensor >= (int)c->tsens_h.size() || !out) return fail(HC_ERR_INVALID_ARG, "bad taxel sensor");
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  int cnt[8];
  HC_CUDA(cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
  if (cnt[kCntStatus] & 16)
    return fail(HC_ERR_OVERFLOW, "a taxel sensor exceeded its sample limit in the last step (4096 grid steps per "
                                 "triangle side, 2^20 samples per fan triangle): the sample resolution is too fine");
  int off = 0;
  for (int k = 0; k < sensor; ++k) off += (int)c->tsens_h[k].taxels.size();
  const size_t n = c->tsens_h[sensor].taxels.size();
  if (c->taxel_val.n < (size_t)off + n) return fail(HC_ERR_NOT_READY, "taxel sensor not set up (call hc_set_pairs)");
  HC_CUDA(cudaMemcpy(out, c->taxel_val.p + off, n * sizeof(float), cudaMemcpyDeviceToHost));
  return HC_OK;
}

hc_status hc_get_all_taxel_sensor_values(hc_context* c, float* out, size_t capacity) {
  if (hc_status st = need(c)) return st;
  size_t total = 0;
  for (const TaxelHost& h : c->tsens_h) total += h.taxels.size();
  if (!out || capacity < total) return fail(HC_ERR_INVALID_ARG, "output smaller than the total taxel count");
  if (total == 0) return HC_OK;
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  int cnt[8];
  HC_CUDA(cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
  if (cnt[kCntStatus] & 16)
    return fail(HC_ERR_OVERFLOW, "a taxel sensor exceeded its sample limit in the last step (4096 grid steps per "
                                 "triangle side, 2^20 samples per fan triangle): the sample resolution is too fine");
  if (c->taxel_val.n < total) return fail(HC_ERR_NOT_READY, "taxel sensors not set up (call hc_set_pairs)");
  HC_CUDA(cudaMemcpy(out, c->taxel_val.p, total * sizeof(float), cudaMemcpyDeviceToHost));
  return HC_OK;
}

hc_status hc_sample_surface(int n_vert, const double* vert, int n_face, const int* face, int n_samples,
                            uint64_t seed, int capacity, double* out_points, double* out_normals, int* out_n) {
  if (n_vert <= 0 || n_face <= 0 || !vert || !face || n_samples < 0 || !out_n)
    return fail(HC_ERR_INVALID_ARG, "a mesh with vertices and faces and an output count are needed");
  if (!finite_all(vert, 3 * (size_t)n_vert)) return fail(HC_ERR_INVALID_ARG, "non-finite mesh vertex");
  for (int i = 0; i < 3 * n_face; ++i)
    if (face[i] < 0 || face[i] >= n_vert) return fail(HC_ERR_INVALID_ARG, "face index out of range");
  std::vector<double> p, n;
  const int got = hc::sample_surface(vert, n_vert, face, n_face, std::min(n_samples, 1 << 22), seed, &p, &n, nullptr);
  *out_n = got;
  if (got > capacity || (got > 0 && (!out_points || !out_normals)))
    return fail(HC_ERR_INVALID_ARG, "output capacity smaller than the sample count (see out_n)");
  if (got > 0) {
    std::copy(p.begin(), p.end(), out_points);
    std::copy(n.begin(), n.end(), out_normals);
  }
  return HC_OK;
}

hc_status hc_add_curved_sensor(hc_context* c, int geom_id, int n_taxels, const double* taxels,
                               const double* taxel_normals, double include_margin, int n_points,
                               const double* points, const double* point_normals, int* out_sensor) {
  HostRange range_("hc_add_curved_sensor");
  if (hc_status st = need(c)) return st;
  if (!c->geoms.count(geom_id)) return fail(HC_ERR_INVALID_ARG, "sensor geom has no cs:: properties");
  if (n_taxels <= 0 || n_taxels > (1 << 20) || !taxels) return fail(HC_ERR_INVALID_ARG, "1 to 2^20 taxels are needed");
  if (n_points < 0 || n_points > (1 << 24) || (n_points > 0 && (!points || !point_normals)))
    return fail(HC_ERR_INVALID_ARG, "0 to 2^24 surface points with normals are needed");
  if (!(include_margin > 0) || !std::isfinite(include_margin) || !finite_all(taxels, 3 * (size_t)n_taxels) ||
      (taxel_normals && !finite_all(taxel_normals, 3 * (size_t)n_taxels)) ||
      (n_points > 0 && (!finite_all(points, 3 * (size_t)n_points) || !finite_all(point_normals, 3 * (size_t)n_points))))
    return fail(HC_ERR_INVALID_ARG, "bad margin, taxel, normal or surface point");
  // the taxels' normals, normalised (curved_sensor.cpp:174-189); none = zero
  std::vector<double> tn(3 * (size_t)n_taxels, 0.0);
  if (taxel_normals)
    for (int i = 0; i < n_taxels; ++i) {
      const double* v = taxel_normals + 3 * (size_t)i;
      const double z = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      for (int k = 0; k < 3; ++k) tn[3 * (size_t)i + k] = z > 0 ? v[k] / std::sqrt(z) : 0.0;
    }
  // points near each taxel (curved_sensor.cpp:318-347): the distance-matrix
  // expression, the margin, the 45-degree normal test; weights
  // max(0, margin - d)^2; points kept in order of first use
  const double m2 = include_margin * include_margin, lim = 45 * 3.141592653589793 / 180.;
  std::vector<std::vector<std::pair<int, float>>> lists((size_t)n_taxels);
  std::vector<int> used;
  for (int j = 0; j < n_points; ++j) {
    const double* s = points + 3 * (size_t)j;
    const double* sn = point_normals + 3 * (size_t)j;
    const double ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    bool added = false;
    for (int i = 0; i < n_taxels; ++i) {
      const double* t = taxels + 3 * (size_t)i;
      const double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      const double d = (-2 * (t[0] * s[0] + t[1] * s[1] + t[2] * s[2]) + tt) + ss;
      if (!(d < m2)) continue;
      const double* nt = &tn[3 * (size_t)i];
      if (nt[0] * nt[0] + nt[1] * nt[1] + nt[2] * nt[2] != 0 &&
          !(std::acos(nt[0] * sn[0] + nt[1] * sn[1] + nt[2] * sn[2]) < lim))
        continue;
      if (!added) {
        used.push_back(j);
        added = true;
      }
      const double r = include_margin - std::sqrt(d);
      lists[(size_t)i].push_back({(int)used.size() - 1, (float)(r > 0 ? r * r : 0.0)});
    }
  }
  CurvedHost h;
  h.geom = geom_id;
  h.margin = include_margin;
  h.n_taxels = n_taxels;
  for (int j : used) {
    const double* s = points + 3 * (size_t)j;
    const double* sn = point_normals + 3 * (size_t)j;
    h.points.push_back(make_float4((float)s[0], (float)s[1], (float)s[2], 0.f));
    h.normals.push_back(make_float4((float)sn[0], (float)sn[1], (float)sn[2], 0.f));
  }
  h.off.push_back(0);
  for (const auto& l : lists) {
    for (const auto& e : l) {
      h.pt.push_back(e.first);
      h.w.push_back(e.second);
    }
    h.off.push_back((int)h.pt.size());
  }
  c->csens_h.push_back(std::move(h));
  c->csens_enabled_h.push_back(1);
  c->sensors_dirty = true;   // pairs are dispatched again before the next step
  if (out_sensor) *out_sensor = (int)c->csens_h.size() - 1;
  return HC_OK;
}

hc_status hc_set_curved_sensor_enabled(hc_context* c, int sensor, int on) {
  if (hc_status st = need(c)) return st;
  if (sensor < 0 || sensor >= (int)c->csens_h.size()) return fail(HC_ERR_INVALID_ARG, "bad curved sensor");
  c->csens_enabled_h[sensor] = on ? 1 : 0;
  if (c->csens_enabled.n >= c->csens_enabled_h.size()) {
    HC_CUDA(cudaSetDevice(c->device));
    HC_CUDA(cudaMemcpyAsync(c->csens_enabled.p + sensor, &c->csens_enabled_h[sensor], sizeof(int),
                            cudaMemcpyHostToDevice, c->stream));
  }
  return HC_OK;
}

hc_status hc_get_curved_sensor_values(hc_context* c, int sensor, float* out) {
  if (hc_status st = need(c)) return st;
  if (sensor < 0 || sensor >= (int)c->csens_h.size() || !out) return fail(HC_ERR_INVALID_ARG, "bad curved sensor");
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = finish_step(c)) return st;
  int off = 0;
  for (int k = 0; k < sensor; ++k) off += c->csens_h[k].n_taxels;
  const size_t n = (size_t)c->csens_h[sensor].n_taxels;
  if (c->cvalues.n < (size_t)off + n) return fail(HC_ERR_NOT_READY, "curved sensor not set up (call hc_set_pairs)");
  HC_CUDA(cudaMemcpy(out, c->cvalues.p + off, n * sizeof(float), cudaMemcpyDeviceToHost));
  return HC_OK;
}

hc_status hc_add_flat_sensor(hc_context* c, int geom_id, double resolution, int sampling_resolution, int window,
                             double sigma, int* out_sensor, int* out_cx, int* out_cy) {
  HostRange range_("hc_add_flat_sensor");
  if (hc_status st = need(c)) return st;
  auto it = c->geoms.find(geom_id);
  if (it == c->geoms.end()) return fail(HC_ERR_INVALID_ARG, "sensor geom has no cs:: properties");
  if (!(resolution > 0) || sampling_resolution <= 0) return fail(HC_ERR_INVALID_ARG, "bad resolution");
  if (window < HC_WINDOW_NONE || window > HC_WINDOW_SQUARE) return fail(HC_ERR_INVALID_ARG, "bad window");
  // FS:148-161 default sigmas
  if (window == HC_WINDOW_GAUSS && sigma == -1.0) sigma = 0.1;
  if (window == HC_WINDOW_TUKEY && sigma == -1.0) sigma = 0.3;
  if ((window == HC_WINDOW_GAUSS || window == HC_WINDOW_TUKEY) && !(sigma > 0))
    return fail(HC_ERR_INVALID_ARG, "window needs sigma > 0");
  SensorHost S;
  S.geom = geom_id;
  S.resolution = resolution;
  S.sr = sampling_resolution;
  S.window = window;
  S.sigma = sigma;
  const GeomHost& g = it->second;
  S.cx = (int)floorl(2 * (long double)g.size[0] / resolution + 0.1L);   // FS:196-197
  S.cy = (int)floorl(2 * (long double)g.size[1] / resolution + 0.1L);
  if (S.cx <= 0 || S.cy <= 0) return fail(HC_ERR_INVALID_ARG, "sensor grid is empty");
  c->sensors.push_back(S);
  c->sensors_dirty = true;
  if (out_sensor) *out_sensor = (int)c->sensors.size() - 1;
  if (out_cx) *out_cx = S.cx;
  if (out_cy) *out_cy = S.cy;
  return HC_OK;
}

hc_status hc_get_taxels(hc_context* c, int sensor, float* out) {
  if (hc_status st = need(c)) return st;
  if (sensor < 0 || sensor >= (int)c->sensors.size() || !out) return fail(HC_ERR_INVALID_ARG, "bad sensor");
  if (c->sensors_dirty) return fail(HC_ERR_NOT_READY, "sensor not built; run a step first");
  HC_CUDA(cudaSetDevice(c->device));
  if (c->stepped) {
    if (hc_status st = finish_step(c)) return st;
  }
  const SensorHost& S = c->sensors[sensor];
  HC_CUDA(cudaMemcpy(out, c->taxels.p + S.dev.taxel_off, S.cx * S.cy * sizeof(float), cudaMemcpyDeviceToHost));
  return HC_OK;
}

hc_status hc_get_taxels_all(hc_context* c, float* out, int64_t n_floats) {
  HostRange range_("hc_get_taxels_all");
  if (hc_status st = need(c)) return st;
  if (!out || n_floats < c->n_cells) return fail(HC_ERR_INVALID_ARG, "output too small");
  if (c->sensors_dirty) return fail(HC_ERR_NOT_READY, "sensors not built; run a step first");
  HC_CUDA(cudaSetDevice(c->device));
  if (c->stepped) {
    if (hc_status st = finish_step(c)) return st;
  }
  if (c->n_cells) {
    HC_CUDA(cudaMemcpyAsync(out, c->taxels.p, (size_t)c->n_cells * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return HC_OK;
}

hc_status hc_get_taxels_device(hc_context* c, const float** d_taxels, int64_t* n_floats) {
  if (hc_status st = need(c)) return st;
  if (d_taxels) *d_taxels = c->taxels.p;
  if (n_floats) *n_floats = c->n_cells;
  return HC_OK;
}

hc_status hc_enable_timing(hc_context* c, int enable) {
  if (hc_status st = need(c)) return st;
  if ((enable != 0) != c->timing) invalidate_graph(c);
  c->timing = enable != 0;
  return HC_OK;
}

hc_status hc_get_timings(hc_context* c, hc_timings* out) {
  if (hc_status st = need(c)) return st;
  if (!out) return fail(HC_ERR_INVALID_ARG, "null output");
  if (!c->timing) return fail(HC_ERR_NOT_READY, "timing is off");
  HC_CUDA(cudaEventSynchronize(c->ev[5]));
  float t[5];
  for (int i = 0; i < 5; ++i) cudaEventElapsedTime(&t[i], c->ev[i], c->ev[i + 1]);
  // the narrow-phase stage splits at ev[6] into the narrow kernels and the
  // pass over the kept polygons (zero when none are kept)
  float t_narrow = t[2], t_kept = 0.f;
  if (cudaEventElapsedTime(&t_narrow, c->ev[2], c->ev[6]) == cudaSuccess)
    cudaEventElapsedTime(&t_kept, c->ev[6], c->ev[3]);
  else
    t_narrow = t[2];
  out->ms_setup = t[0];
  out->ms_broadphase = t[1];
  out->ms_narrowphase = t_narrow;
  out->ms_kept_polygons = t_kept;
  out->ms_reduce = t[3];
  out->ms_taxels = t[4];
  cudaEventElapsedTime(&out->ms_total, c->ev[0], c->ev[5]);
  out->ms_adjoint = 0.f;
  if (c->last_fused) {
    HC_CUDA(cudaEventSynchronize(c->ev[7]));
    cudaEventElapsedTime(&out->ms_adjoint, c->ev[5], c->ev[7]);
  }
  int cnt[8];
  HC_CUDA(cudaMemcpy(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost));
  out->n_items = cnt[kCntTotal];
  out->n_polygons = 0;
  return HC_OK;
}

hc_status hc_get_stream(hc_context* c, void** stream) {
  if (hc_status st = need(c)) return st;
  if (!stream) return fail(HC_ERR_INVALID_ARG, "null output");
  *stream = (void*)c->stream;
  return HC_OK;
}

hc_status hc_get_launch_count(hc_context* c, int* n) {
  if (hc_status st = need(c)) return st;
  if (n) *n = c->launches_per_step;
  return HC_OK;
}

// Sweep of the persistent kernels' grid (CTAs per SM) and the soft-rigid
// work-queue chunk on the current pairs and poses: each shape is warmed up
// (graph captured) and timed over three steps with the stage events; the
// fastest step wins.  Results do not depend on the shape (per-item sums are
// deterministic and reduced in a fixed order).
hc_status hc_autotune(hc_context* c, int* chosen_ctas_per_sm, int* chosen_chunk) {
  HostRange range_("hc_autotune");
  if (hc_status st = need(c)) return st;
  if (!c->poses_set || c->pairs_h.empty()) return fail(HC_ERR_NOT_READY, "set pairs and poses before autotuning");
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = hc_step(c)) return st;
  if (hc_status st = finish_step(c)) return st;
  const bool was_timing = c->timing;
  const int old_ctas = c->narrow_ctas_per_sm, old_chunk = c->narrow_chunk;
  c->timing = true;
  static const int kCtas[] = {2, 3, 4, 6, 8};
  static const int kChunks[] = {1, 2, 4, 8, 16};
  float best = INFINITY;
  int best_ctas = old_ctas, best_chunk = old_chunk;
  for (int ct : kCtas) {
    for (int ch : kChunks) {
      c->narrow_ctas_per_sm = ct;
      c->narrow_chunk = ch;
      invalidate_graph(c);
      hc_status st = run_step(c, 0, -1);
      if (!st) st = finish_step(c);
      float tot = 0.f;
      for (int r = 0; r < 3 && !st; ++r) {
        st = run_step(c, 0, -1);
        if (st) break;
        cudaError_t e = cudaEventSynchronize(c->ev[5]);
        if (e != cudaSuccess) { st = fail(HC_ERR_CUDA, cudaGetErrorString(e)); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[0], c->ev[5]);
        tot += ms;
      }
      if (st) {
        c->narrow_ctas_per_sm = old_ctas;
        c->narrow_chunk = old_chunk;
        c->timing = was_timing;
        invalidate_graph(c);
        return st;
      }
      if (tot < best) {
        best = tot;
        best_ctas = ct;
        best_chunk = ch;
      }
    }
  }
  c->narrow_ctas_per_sm = best_ctas;
  c->narrow_chunk = best_chunk;
  c->timing = was_timing;
  invalidate_graph(c);
  if (chosen_ctas_per_sm) *chosen_ctas_per_sm = best_ctas;
  if (chosen_chunk) *chosen_chunk = best_chunk;
  return HC_OK;
}

hc_status hc_set_launch_shape(hc_context* c, int ctas_per_sm, int chunk) {
  if (hc_status st = need(c)) return st;
  if (ctas_per_sm < 1 || ctas_per_sm > 8 || chunk < 1 || chunk > 16)
    return fail(HC_ERR_INVALID_ARG, "ctas_per_sm must be in 1-8 and chunk in 1-16");
  if (ctas_per_sm != c->narrow_ctas_per_sm || chunk != c->narrow_chunk) invalidate_graph(c);
  c->narrow_ctas_per_sm = ctas_per_sm;
  c->narrow_chunk = chunk;
  return HC_OK;
}

hc_status hc_set_adjoint_mode(hc_context* c, int on) {
  if (hc_status st = need(c)) return st;
  if ((on != 0) != c->adjoint_mode) invalidate_graph(c);
  c->adjoint_mode = on != 0;
  if (on) {
    HC_CUDA(cudaSetDevice(c->device));
    if (hc_status st = ensure_recs(c, initial_rec_cap(c))) return st;
  }
  return HC_OK;
}

// Launch the adjoint on device inputs; leaves n_pair x 14 doubles in adj_out.
static hc_status adjoint_launch(hc_context* c, const double* d_dw, const float* d_dt) {
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  const int n_pair = (int)c->pairs_h.size();
  HC_CUDA(c->adj_pair.reserve(8 * (size_t)std::max(1, n_pair)));
  HC_CUDA(c->adj_out.reserve(14 * (size_t)std::max(1, n_pair)));
  HC_CUDA(c->adj_item.reserve(16 * (size_t)std::max(1, c->item_cap)));
  hc::StepArgs a = make_args(c, 0, -1);
  a.adj_wrench = d_dw;
  a.adj_taxel = d_dt && c->n_cells > 0 ? d_dt : nullptr;
  a.adj_pair = c->adj_pair.p;
  a.adj_item = c->adj_item.p;
  a.adj_out = c->adj_out.p;
  if (c->recs_step) {
    // the polygons the last step kept, in the slots it assigned
    a.n_item_blocks = std::max(1, (c->item_cap + hc::kBpBlock - 1) / hc::kBpBlock);
    a.use_recs = 1;
    a.recs = c->recs.p;
    a.rec_key = c->rec_key.p;
    a.rec_cap = c->rec_cap;
    a.rec_out = c->rec_out.p;
    a.item_poly_off = c->item_poly_off.p;
    a.poly_tiles = c->poly_tiles.p;
    a.rec_grad = c->rec_grad.p;
  } else {
    a.recs = nullptr;
    a.rec_key = nullptr;
    a.rec_cap = 0;
  }
  c->adj_launches = hc::launch_adjoint(a, c->stream);
  HC_CUDA(cudaGetLastError());
  // Kept polygons find their samples by slot key and leave them as the step
  // left them (the next step clears them); recomputed ones (no polygons
  // kept, soft-soft pairs) take each won sample once, so a further taxel
  // adjoint of this step needs the step again.
  if (a.adj_taxel && (!c->recs_step || c->type_units[2][1] > c->type_units[2][0])) c->samples_used = true;
  return HC_OK;
}

// Make sure the last step's won samples are available for a taxel adjoint.
static hc_status ensure_kept_samples(hc_context* c) {
  if (hc_status st = finish_step(c)) return st;
  if ((c->samples_dirty && !c->samples_used) || c->n_cells == 0) return HC_OK;
  bool was = c->adjoint_mode;
  c->adjoint_mode = true;
  invalidate_graph(c);
  hc_status st = run_step(c, 0, -1);
  c->adjoint_mode = was;
  invalidate_graph(c);
  if (st) return st;
  return finish_step(c);
}

// The fused step's per-pair results back to back (one contiguous read each
// for the host instead of strided rows): wrench (6), dL/dpose (12), dL/dE (2).

// The forward step and its adjoint as one graph on the context stream: the
// counters and kept samples cleared, the step's kernels, then the adjoint's
// on the upstream gradients at d_dw / d_dt (device; either may be null).
// Adjoint mode must be on.  The adjoint kernels read the step's status on the
// device (records that overflowed are not read; work items never exceed the
// capacity), so nothing waits between the two; the caller checks the status.
static hc_status run_fused(hc_context* c, const double* d_dw, const float* d_dt) {
  const int n_pair = (int)c->pairs_h.size();
  if (n_pair == 0 && c->sensors.empty()) {
    c->stepped = true;
    return HC_OK;
  }
  HC_CUDA(c->adj_pair.reserve(8 * (size_t)std::max(1, n_pair)));
  HC_CUDA(c->adj_out.reserve(14 * (size_t)std::max(1, n_pair)));
  HC_CUDA(c->adj_item.reserve(16 * (size_t)std::max(1, c->item_cap)));
  HC_CUDA(c->out_stage.reserve(20 * (size_t)std::max(1, n_pair)));
  hc::StepArgs a = make_args(c, 0, -1);
  hc::StepArgs b = a;
  b.adj_wrench = d_dw;
  b.adj_taxel = d_dt && c->n_cells > 0 ? d_dt : nullptr;
  b.adj_pair = c->adj_pair.p;
  b.adj_item = c->adj_item.p;
  b.adj_out = c->adj_out.p;
  if (a.recs) {
    b.n_item_blocks = std::max(1, (c->item_cap + hc::kBpBlock - 1) / hc::kBpBlock);
    b.use_recs = 1;
    b.rec_grad = c->rec_grad.p;
  }
  b.out_stage = c->out_stage.p;
  b.fused = 1;
  c->recs_step = a.recs != nullptr;
  c->step_checked = false;
  const void* key[6] = {d_dw, b.adj_taxel, c->adj_pair.p, c->adj_item.p, c->adj_out.p, c->out_stage.p};
  if (c->fused_valid && memcmp(key, c->fused_key, sizeof(key)) != 0) invalidate_graph(c);
  if (!c->fused_valid) {
    invalidate_graph(c);
    cudaEvent_t* ev = c->timing ? c->ev : nullptr;
    HC_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    c->launches_per_step = hc::launch_step(a, c->stream, ev);
    // the forward's results are final here (the taxel maps may leave on
    // the copy stream); the adjoint needs the upstream gradients in
    cudaEventRecordWithFlags(c->xev[1], c->stream, cudaEventRecordExternal);
    cudaStreamWaitEvent(c->stream, c->xev[0], cudaEventWaitExternal);
    c->adj_launches = hc::launch_adjoint(b, c->stream);
    if (ev) cudaEventRecordWithFlags(ev[7], c->stream, cudaEventRecordExternal);
    cudaError_t e = cudaStreamEndCapture(c->stream, &c->fused_graph);
    if (e != cudaSuccess) return fail(HC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    HC_CUDA(cudaGraphInstantiate(&c->fused_exec, c->fused_graph, 0));
    memcpy(c->fused_key, key, sizeof(key));
    c->fused_valid = true;
  }
  HC_CUDA(cudaGraphLaunch(c->fused_exec, c->stream));
  c->stepped = true;
  c->last_fused = true;
  // the step kept its samples (the next step's first kernel clears them);
  // recomputed polygons took theirs
  c->samples_dirty = a.keep_samples && c->n_cells > 0;
  c->samples_used = b.adj_taxel && (!c->recs_step || c->type_units[2][1] > c->type_units[2][0]);
  return HC_OK;
}

// Preconditions of a fused step; turns adjoint mode on when `enable` is set.
static hc_status fused_ready(hc_context* c, bool enable) {
  if (!c->adjoint_mode) {
    if (!enable) return fail(HC_ERR_NOT_READY, "the fused step needs hc_set_adjoint_mode(ctx, 1)");
    if (hc_status st = hc_set_adjoint_mode(c, 1)) return st;
  }
  if (c->pools_dirty || c->sensors_dirty) {
    std::vector<int> g1 = c->g1_h, g2 = c->g2_h;
    if (hc_status st = hc_set_pairs(c, (int)g1.size(), g1.data(), g2.data(), nullptr, nullptr)) return st;
  }
  if (!c->poses_set && !c->pairs_h.empty()) return fail(HC_ERR_NOT_READY, "poses not set");
  if ((size_t)c->n_pose * 3 > c->xpos.n || c->n_pose <= c->max_geom_id)
    return fail(HC_ERR_NOT_READY, "poses do not cover every registered geom");
  return HC_OK;
}

hc_status hc_step_adjoint(hc_context* c, int n_geom, const double* xpos, const double* xmat, const double* vel,
                          const double* dL_dwrench, const float* dL_dtaxel, double* wrench, float* taxels,
                          double* dL_dpose, double* dL_dE) {
  HostRange range_("hc_step_adjoint");
  if (hc_status st = need(c)) return st;
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = hc_set_poses(c, n_geom, xpos, xmat, vel)) return st;
  if (hc_status st = fused_ready(c, true)) return st;
  const int n_pair = (int)c->pairs_h.size();
  const double* d_dw = nullptr;
  const float* d_dt = nullptr;
  // the upstream gradients go in on the copy stream while the forward runs
  // (the adjoint part of the graph waits for xev[0]); the buffers are free:
  // the previous call waited for its graph
  if (dL_dwrench && n_pair) {
    HC_CUDA(c->adj_wrench.reserve(6 * (size_t)n_pair));
    HC_CUDA(cudaMemcpyAsync(c->adj_wrench.p, dL_dwrench, 6 * (size_t)n_pair * sizeof(double), cudaMemcpyHostToDevice,
                            c->copy_stream));
    d_dw = c->adj_wrench.p;
  }
  if (dL_dtaxel && c->n_cells) {
    HC_CUDA(c->adj_taxel.reserve(c->n_cells));
    HC_CUDA(cudaMemcpyAsync(c->adj_taxel.p, dL_dtaxel, (size_t)c->n_cells * sizeof(float), cudaMemcpyHostToDevice,
                            c->copy_stream));
    d_dt = c->adj_taxel.p;
  }
  HC_CUDA(cudaEventRecord(c->xev[0], c->copy_stream));
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (hc_status st = run_fused(c, d_dw, d_dt)) return st;
    if (n_pair == 0 && c->sensors.empty()) return HC_OK;
    // the taxel maps and wrenches leave on the copy stream once the forward
    // is done, while the adjoint runs; the gradients straight into the
    // caller's arrays (each one contiguous copy from the packed results),
    // then the status word; one wait for all of it
    if ((c->n_cells && taxels) || (n_pair && wrench)) HC_CUDA(cudaStreamWaitEvent(c->copy_stream, c->xev[1], 0));
    if (c->n_cells && taxels)
      HC_CUDA(cudaMemcpyAsync(taxels, c->taxels.p, (size_t)c->n_cells * sizeof(float), cudaMemcpyDeviceToHost,
                              c->copy_stream));
    // the wrenches are final with the forward too: the six leading doubles
    // of each 10-double pair record
    if (n_pair && wrench)
      HC_CUDA(cudaMemcpy2DAsync(wrench, 6 * sizeof(double), c->pair_out.p, sizeof(hc::PairOut), 6 * sizeof(double),
                                (size_t)n_pair, cudaMemcpyDeviceToHost, c->copy_stream));
    HC_CUDA(cudaEventRecord(c->xev[2], c->copy_stream));
    HC_CUDA(cudaStreamWaitEvent(c->stream, c->xev[2], 0));
    const double* st = c->out_stage.p;
    if (n_pair && dL_dpose)
      HC_CUDA(cudaMemcpyAsync(dL_dpose, st + 6 * (size_t)n_pair, 12 * (size_t)n_pair * sizeof(double),
                              cudaMemcpyDeviceToHost, c->stream));
    if (n_pair && dL_dE)
      HC_CUDA(cudaMemcpyAsync(dL_dE, st + 18 * (size_t)n_pair, 2 * (size_t)n_pair * sizeof(double),
                              cudaMemcpyDeviceToHost, c->stream));
    int cnt[8];
    HC_CUDA(cudaMemcpyAsync(cnt, c->counters.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
    HC_CUDA(cudaStreamSynchronize(c->stream));
    if (cnt[kCntStatus] & kStatusScanWaitBit)
      return fail(HC_ERR_CUDA, "a single-pass scan waited past its bound for an earlier tile");
    if (!(cnt[kCntStatus] & 9)) {
      c->step_checked = true;
      return HC_OK;
    }
    // a capacity overflowed: grow it and run the whole step again
    if (cnt[kCntStatus] & 8) {
      const int want = std::max(2 * c->rec_cap, cnt[kCntRec] + cnt[kCntRec] / 4 + 1024);
      if (hc_status st = ensure_recs(c, want)) return st;
    }
    if (cnt[kCntStatus] & 1) {
      int total = 0;
      HC_CUDA(cudaMemcpy(&total, c->unit_off.p + c->n_units, sizeof(int), cudaMemcpyDeviceToHost));
      if (hc_status st = ensure_items(c, std::max(2 * c->item_cap, total + total / 4 + 1024))) return st;
    }
  }
  return fail(HC_ERR_OVERFLOW, "work-item or polygon-record capacity overflow persisted");
}

hc_status hc_step_adjoint_device(hc_context* c, const double* d_dL_dwrench, const float* d_dL_dtaxel,
                                 const double** d_grad) {
  HostRange range_("hc_step_adjoint_device");
  if (hc_status st = need(c)) return st;
  HC_CUDA(cudaSetDevice(c->device));
  if (hc_status st = fused_ready(c, false)) return st;
  // the caller's upstream arrays are ordered on the context's stream: the
  // graph's wait for upstream copies is met at once
  HC_CUDA(cudaEventRecord(c->xev[0], c->stream));
  if (hc_status st = run_fused(c, d_dL_dwrench, d_dL_dtaxel)) return st;
  if (d_grad) *d_grad = c->adj_out.p;
  return HC_OK;
}

hc_status hc_adjoint(hc_context* c, const double* dL_dwrench, const float* dL_dtaxel, double* dL_dpose,
                     double* dL_dE) {
  HostRange range_("hc_adjoint");
  if (hc_status st = need(c)) return st;
  if (!c->stepped) return fail(HC_ERR_NOT_READY, "no step has run");
  HC_CUDA(cudaSetDevice(c->device));
  const int n_pair = (int)c->pairs_h.size();
  if (dL_dtaxel) {
    if (hc_status st = ensure_kept_samples(c)) return st;
  } else if (hc_status st = finish_step(c)) {
    return st;
  }
  const double* d_dw = nullptr;
  const float* d_dt = nullptr;
  if (dL_dwrench && n_pair) {
    HC_CUDA(c->adj_wrench.reserve(6 * (size_t)n_pair));
    HC_CUDA(cudaMemcpyAsync(c->adj_wrench.p, dL_dwrench, 6 * (size_t)n_pair * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
    d_dw = c->adj_wrench.p;
  }
  if (dL_dtaxel && c->n_cells) {
    HC_CUDA(c->adj_taxel.reserve(c->n_cells));
    HC_CUDA(cudaMemcpyAsync(c->adj_taxel.p, dL_dtaxel, (size_t)c->n_cells * sizeof(float), cudaMemcpyHostToDevice,
                            c->stream));
    d_dt = c->adj_taxel.p;
  }
  if (hc_status st = adjoint_launch(c, d_dw, d_dt)) return st;
  // rows of 14 doubles per pair: the 12 twist terms and the 2 moduli terms
  // straight into the caller's arrays
  if (n_pair && dL_dpose)
    HC_CUDA(cudaMemcpy2DAsync(dL_dpose, 12 * sizeof(double), c->adj_out.p, 14 * sizeof(double), 12 * sizeof(double),
                              n_pair, cudaMemcpyDeviceToHost, c->stream));
  if (n_pair && dL_dE)
    HC_CUDA(cudaMemcpy2DAsync(dL_dE, 2 * sizeof(double), c->adj_out.p + 12, 14 * sizeof(double), 2 * sizeof(double),
                              n_pair, cudaMemcpyDeviceToHost, c->stream));
  HC_CUDA(cudaStreamSynchronize(c->stream));
  return HC_OK;
}

hc_status hc_adjoint_device(hc_context* c, const double* d_dL_dwrench, const float* d_dL_dtaxel,
                            const double** d_grad) {
  HostRange range_("hc_adjoint_device");
  if (hc_status st = need(c)) return st;
  if (d_dL_dtaxel && !c->samples_dirty && c->n_cells > 0)
    return fail(HC_ERR_NOT_READY, "taxel adjoint needs hc_set_adjoint_mode(ctx, 1) before the step");
  if (d_dL_dtaxel && c->samples_used && c->n_cells > 0)
    return fail(HC_ERR_NOT_READY, "a taxel adjoint of this step already took the samples of its recomputed polygons; "
                                  "step again (hc_adjoint does so itself)");
  if (hc_status st = adjoint_launch(c, d_dL_dwrench, d_dL_dtaxel)) return st;
  if (d_grad) *d_grad = c->adj_out.p;
  return HC_OK;
}

hc_status hc_get_adjoint_skipped(hc_context* c, int* n, float* min_det) {
  if (hc_status st = need(c)) return st;
  if (!(c->debug & HC_DEBUG_CANDIDATES)) return fail(HC_ERR_NOT_READY, "needs debug recording (hc_set_debug)");
  HC_CUDA(cudaSetDevice(c->device));
  HC_CUDA(cudaStreamSynchronize(c->stream));
  int w[2];
  HC_CUDA(cudaMemcpy(w, c->counters.p + kCntAdjSkip, sizeof(w), cudaMemcpyDeviceToHost));
  if (n) *n = w[0];
  if (min_det) memcpy(min_det, &w[1], sizeof(float));
  return HC_OK;
}

hc_status hc_get_adjoint_launch_count(hc_context* c, int* n) {
  if (hc_status st = need(c)) return st;
  if (n) *n = c->adj_launches;
  return HC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Read-only view of a context for hc_step_noalloc (noalloc.cu).
namespace hc {

hc_status set_last_error(hc_status st, const char* msg) { return fail(st, msg); }

hc_status noalloc_view(hc_context* c, NoallocView* v) {
  if (hc_status st = need(c)) return st;
  if (c->pools_dirty || c->sensors_dirty)
    return fail(HC_ERR_NOT_READY, "geoms or sensors changed since hc_set_pairs: call hc_set_pairs first");
  v->args = make_args(c, 0, -1);
  v->device = c->device;
  v->stream = c->stream;
  v->max_geom_id = c->max_geom_id;
  size_t n = 0;
  for (const SensorHost& S : c->sensors) n += (size_t)S.cx * S.sr * S.cy * S.sr;
  v->n_samples = n;
  return HC_OK;
}

}  // namespace hc
