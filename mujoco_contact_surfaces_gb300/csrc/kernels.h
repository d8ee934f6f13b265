// kernels.h — launch wrappers for the device kernels (host-callable).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hc_internal.h"

namespace hc {

// Pairs per block of the per-pair reductions (a warp each): 8 rather than
// 16 gives the 4096-pair step 512 blocks over 152 SMs and a block waits on
// the slowest of fewer pairs (step 1.360 -> 1.350 ms).
constexpr int kReducePairs = 8;

// Step counters the step's first kernel zeroes (StepArgs::reset_words).
constexpr int kResetWords = 12;

struct StepArgs {
  // per-step inputs (device)
  const double* xpos;
  const double* xmat;
  const double* vel;
  // pairs
  const PairDev* pairs;
  int n_pair;
  FrameDev* frames;
  // geometry pools
  const float4* tets;
  const float4* tet_props;   // per tet: (g.xyz, |g|), (kappa, xmax, pmax, hmin) of its field
  const int* tet_orig;
  const float4* tris;
  const DfPlane* tri_plane;   // body-frame unit normal and offset (FP64 as head and tail)
  const DfPlane* tri_edges;   // 3 per triangle: body-frame edge planes
  const float4* tri_meta;     // (min altitude, max edge, max |vertex|, 0)
  const int* tri_orig;
  const float4* nodes;
  // broadphase units and items
  const int* unit_pair;
  const int* unit_cl;
  int n_units;
  int* unit_off;      // n_units + 1
  unsigned long long* bp_tiles;   // per broadphase block: its decoupled look-back state
  int n_bp_blocks;
  int4* items;
  int item_cap;
  int type_unit_begin[3];    // unit range of each query type
  int type_unit_end[3];      // (soft-rigid, half-space, soft-soft)
  int* item_total;
  int* item_next;     // one work counter per query type
  int* status;        // bit 0: item overflow, bit 1: candidate overflow,
                      // bit 2: polygon overflow, bit 3: adjoint record overflow
  ItemOut* item_out;
  PairOut* pair_out;
  // sensors
  const SensorDev* sensors;
  int n_sensor;
  unsigned long long* samples;
  int4* sens_box;     // per flat sensor: the sample box (X0, X1, Y0, Y1) this
                      // step's rays can touch (X0 > X1: none); null: every
                      // sample may be set (the taxel pass reads them all)
  float* taxels;
  const float* weights;
  const float* samp_coord;
  int n_cells_total;
  const int* cell_sensor;   // sensor index per global cell
  const int* cell_first;    // first global cell of each sensor
  // options
  int repr;
  int apply_forces;
  int debug;
  CandRec* cand;
  int cand_cap;
  int* cand_count;
  PolyRec* polys;
  int poly_cap;
  int* poly_count;
  int want_polys;
  int want_pair;      // -1 = all pairs
  // launch shape of the narrow phase
  int narrow_block;
  int narrow_grid;
  int rec_fwd_grid;   // the kept-polygon kernels: every CTA resident at once
  int rec_adj_grid;
  int chunk;          // consecutive items a soft-rigid warp takes at once
  // adjoint
  int keep_samples;          // taxel pass leaves the won samples for the adjoint
  const double* adj_wrench;  // dL/dwrench, n_pair x 6 (device) or null
  const float* adj_taxel;    // dL/dtaxel, all cells (device) or null
  float* adj_pair;           // per pair: dL/dF_S, dL/dT_S in the soft frame (8 floats)
  double* adj_item;          // per item: 13 gradient sums (stride 16)
  double* adj_out;           // per pair: [dL/dtwist M (6), N (6), dL/dE_M, dL/dE_N]
  // adjoint records: polygons kept by the forward (null: none kept)
  AdjPoly* recs;
  int2* rec_key;             // (item, sequence number within the item)
  int rec_cap;
  int* rec_count;
  int* adj_skip;             // with debug recording: [0] adjoint polygon vertices left out
                             // of the contraction, [1] the smallest normalised |det| (bits), else null
  int use_recs;              // the adjoint reads the kept polygons (when none overflowed)
  int* reset_words;          // kResetWords step counters zeroed by the step's first kernel (null: none)
  double* out_stage;         // fused step: the adjoint's last kernel packs the results here
                             // (wrenches n x 6, twist gradients n x 12, moduli n x 2), else null
  int fused;                 // fused step: an overflow re-runs the whole step, so the
                             // recomputing adjoint fallbacks are left out
  int* item_poly_off;        // per item: first record of the item in pair order (item_cap + 1)
  unsigned long long* poly_tiles; // per kBpBlock items: the polygon-slot scan's look-back state
  int* tile_ctr;             // [0] broadphase, [1] polygon slots: the next tile a block takes
  int n_item_blocks;         // item_cap / kBpBlock rounded up
  float* rec_grad;           // per record in pair order: 13 gradient terms (stride 16)
  RecOut* rec_out;           // per record in pair order: forces (forward)
  float4* slot_press;        // per record slot and sensor side (2), three float4:
                             // the linear pressure model (lx0, ly0, p0, px), then
                             // (py, lz0, zx, zy) of the polygon's plane, then its
                             // sample box (X0, X1, Y0, Y1 as ints; X0 > X1: none)
  int* rec_perm;             // per record slot: the record index
  int* rec_dst;              // per record: its slot (-1: none), written by the forward record pass
  // taxel-point sensors
  const TaxelSensorDev* tsens;
  int n_tsens;
  const int* tsens_pairs;
  const int* tsens_enabled;  // per sensor: update in this step
  const float4* taxel_pos;   // geom frame
  float* taxel_val;          // values (kept between updates)
  const int* tpairs;         // the pairs any taxel sensor reads (each once)
  const int* tpair_ai;       // per such pair: read by an area-importance sensor
  int n_tpairs;
  double* tat;               // per record slot x kMaxPolyV: running surface area (area importance)
  // curved sensors
  const CurvedSensorDev* csens;
  int n_csens;
  const int* csens_pairs;
  const int* csens_enabled;
  const float4* cpoints;     // geom frame
  const float4* cnormals;    // geom frame, unit
  const int* clist_off;      // per taxel (all curved sensors' taxels back to back) + 1
  const int* clist_pt;       // point index within the sensor
  const float* clist_w;      // weight
  float* chit;               // per point: hit pressure of its ray (0: no hit)
  float* cvalues;
  int* tsort;                // per record slot of those pairs: the slot in polygon order
  unsigned long long* tkey;  // sort scratch (pairs of more than 2048 polygons)
  int* tidx;
};

constexpr int kBpBlock = 256;

// LBVH build, element order: one geom's elements in the element pools
// (the same offset in the unsorted input and in the pools).
struct LbvhSeg {
  int off;         // first element
  int n;           // elements
  int chunk_off;   // first sort chunk of the geom
  int pad;
  double lo[3], hi[3];   // bounding box of the geom's vertices
};
// Orders each geom's elements (npe float4 each, unsorted in `raw`) along the
// Morton curve of their centroids and gathers them into `out`; orig gets each
// pool element's index in its geom.  Rigid triangles also carry their planes,
// edge planes and metadata (plane_raw / edge_raw / meta_raw; null for tets).
// chunk_seg: the geom of every sort chunk of lbvh_sort_chunk() keys; keys and
// perm: scratch of one entry per element.
void launch_lbvh_order(const float4* raw, int npe, const LbvhSeg* segs, int n_segs, const int* chunk_seg,
                       int n_chunks, unsigned long long* keys, int* perm, float4* out, int* orig,
                       const DfPlane* plane_raw, DfPlane* plane, const DfPlane* edge_raw, DfPlane* edge,
                       const float4* meta_raw, float4* meta, cudaStream_t s);
int lbvh_sort_chunk();

// LBVH build/refit: node boxes of the implicit trees of `n_geoms` geoms.
void launch_refit(const float4* elems, int verts_per_elem, float4* nodes, const int* geom_elem_off,
                  const int* geom_n_elem, const int* geom_node_off, const int* geom_leaves,
                  int n_geoms, cudaStream_t s);

// Per-tet constants of the soft tets (pressure gradient and its norm,
// conditioning, coordinate and pressure magnitudes, minimum height), all in
// the soft body frame: computed once when the pool is built.
void launch_tet_props(const float4* tets, float4* props, int n_tets, cudaStream_t s);

// Kernel attributes (large dynamic shared memory); once per device.
cudaError_t init_kernel_attributes();

// CTAs of 128 threads that fit on one SM for the forward and adjoint passes
// over the kept polygons (their work is split evenly over the grid, so the
// grid is sized to be resident in one wave).
void record_ctas_per_sm(int* fwd, int* adj);

// One step: frames, broadphase, narrow phase, per-pair reduce, taxels.
// Returns the number of kernels launched.
int launch_step(const StepArgs& a, cudaStream_t s, cudaEvent_t* ev /* 7 or null */);

// Adjoint of the last step (all query types).  Returns the
// number of kernels launched.
int launch_adjoint(const StepArgs& a, cudaStream_t s);

}  // namespace hc
