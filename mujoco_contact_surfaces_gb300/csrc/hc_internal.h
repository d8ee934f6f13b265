// hc_internal.h — device data layout shared by the host API and the kernels.
//
// HBM layout (all pools are one allocation each; per-geom offsets index them):
//   tet pool   : float4[4] per tet, vertices (x, y, z, pressure) in the soft
//                geom's body frame, tets in Morton order of their centroids.
//                64 B per tet, read as four 16 B vector loads.
//   tet props  : float4[2] per tet, (g.xyz, |g|) and (kappa, xmax, pmax, hmin)
//                of its linear pressure field, computed on the device once
//                per pool build (constant in the body frame).
//   tri pool   : float4[3] per triangle, vertices (x, y, z, 0) in the rigid
//                geom's body frame, Morton order.  48 B per triangle.
//   node pool  : float4[2] per node (lo.xyz, hi.xyz) of each geom's implicit
//                complete binary tree over 32-element clusters ("LBVH":
//                Morton-sorted leaves, heap-numbered nodes 1..2L-1, leaves at
//                L..2L-1).  Empty leaves are inverted boxes.
//   orig pools : int per element, Morton position -> original element index.
#pragma once
#include <stdint.h>

namespace hc {

// Four doubles, 32-byte aligned (one 32 B load).
// An FP64 plane (x, y, z, w) as FP32 head and tail per component: head + tail
// is the double to 2^-48 relative.
struct alignas(32) DfPlane {
  float4 hi, lo;
};

struct alignas(32) Dbl4 {
  double x, y, z, w;
};

constexpr int kCluster = 32;       // elements per leaf cluster (one warp)
constexpr int kMaxPolyV = 8;       // max vertices of a clipped polygon

// Static per-pair data (set by hc_set_pairs).
struct PairDev {
  int query;            // HC_QUERY_*
  int gs, go;           // soft geom, other geom (soft-soft: gs = M, go = N)
  int gm, gn;           // M and N
  int s_is_m;
  int sensor0, sensor1; // flat sensors attached to a geom of the pair (-1: none)
  int s_elem_off, s_n_elem, s_node_off, s_leaves;   // soft side: tets, tree
  int o_elem_off, o_n_elem, o_node_off, o_leaves;   // other side: elems, tree
  int o_n_clusters;
  int unit_begin, unit_end;                         // broadphase units
  float damping, mu;
  float E_s, E_o;       // moduli (E_o = 0 for rigid)
  float dd_dEs, dd_dEo; // soft-soft: derivatives of the combined damping by E_s, E_o
};

// Per-step frame data of one pair (computed on the device from the poses).
struct FrameDev {
  double R[9];          // other body -> soft body rotation, row-major
  double t[3];          // other body -> soft body translation
  double RS[9];         // soft body -> world rotation
  double xS[3];         // soft body origin (world)
  double xM[3];         // M origin (world)
  double xN[3];         // N origin (world)
  float lin[3];         // relative velocity field in the soft frame:
  float ang[3];         //   v_M - v_N at p = lin + ang x p
  float Rf[9];          // float copies of R, t (heads)
  float tf[3];
  float Rlo[9];         // tails: R - Rf, t - tf (double-float R, t)
  float tlo[3];
  float Rl[9];          // soft -> sensor0 local frame (rotation, translation)
  float tl[3];
  float Rl1[9];         // soft -> sensor1 local frame
  float tl1[3];
  int valid;            // 0 when a pose was non-finite
  int pad;
};

// Per-item outputs (one item = soft leaf cluster x other cluster).
struct ItemOut {
  float hi[8], lo[8];   // F(3), T(3) about the soft origin in the soft frame,
                        // area, total fn0; each the unevaluated sum hi + lo
                        // of a double-float warp reduction (~48-bit)
  int n_poly, n_faces, n_near, pad;
};

// Per-pair outputs.
struct PairOut {
  double wrench[6];
  double area, total_fn0;
  int n_poly, n_faces, n_near, n_items;
};
static_assert(sizeof(PairOut) == 10 * sizeof(double), "PairOut is the 10-double public pair record");

// Flat sensor (device).
struct SensorDev {
  int geom;
  int cx, cy, sr;       // cells and sampling resolution
  int nx, ny;           // samples per axis: cx*sr, cy*sr
  int64_t sample_off;   // offset into the sample pool (uint64 per sample)
  int taxel_off;        // offset into the taxel pool (float per cell)
  int weight_off;       // offset into the weight pool (sr*sr floats)
  float rmean;
  float zs15;           // 1.5 * zs (ray start height and t bound)
  int samp_off_x, samp_off_y;  // offsets into the sample-coordinate pool
};

// Debug record of a non-empty element pair.
struct CandRec {
  int pair, elem_a, elem_b, n_vert, flags;
};

// Surface record (hc_get_surface): one polygon in the soft body frame.
struct PolyRec {
  int pair, elem_a, elem_b, nv;
  float n[4];                  // contact normal (soft frame), out of N into M
  float v[kMaxPolyV][4];       // vertices (x, y, z, pressure), soft frame
};

// Contact polygon kept by a forward step in adjoint mode, with what its
// reverse pass needs (soft frame).  272 B.
struct alignas(16) AdjPoly {
  float v[kMaxPolyV][4];       // vertices relative to anc: x, y, z, pressure
  float anc[3], gint;          // anchor (a tet vertex); gradient along n
  float n[3];                  // section normal (triangle / plane normal)
  int lab0;                    // constraint labels of vertices 0-3 (8 bits each)
  float g[3];                  // soft pressure gradient
  int lab1;                    // labels of vertices 4-7
  float face[4][3];            // unnormalised tet face normals
  float clip[3][3];            // clip-plane normals (soft-rigid)
  int pair, nv, kind;          // kind: 0 soft-rigid, 1 half-space
  int elem_a, elem_b;          // original soft tet, other element (-1: half-space)
};
static_assert(sizeof(AdjPoly) == 288, "AdjPoly layout");

// Taxel-point sensor (device): taxels at given points of a geom, valued from
// samples of the contact surfaces that involve the geom.
struct TaxelSensorDev {
  int geom;
  int n_taxels, taxel_off;     // taxel positions (geom frame) and values
  int method;                  // 0 closest, 1 weighted, 2 mean, 3 squared
  int sample_method;           // 0 default grid, 1 area importance
  int visualize;
  int pair_off, n_pairs;       // the pairs that involve the geom, in pair order
  double margin, res;          // as given (the sample counts use res in double)
};

// Curved sensor (device): rays from points on the geom's surface into the
// contact surfaces; each taxel sums weight x hit pressure over its points.
struct CurvedSensorDev {
  int geom;
  int n_taxels, taxel_off;     // values; per-taxel lists at list offsets [taxel_off + i]
  int n_points, point_off;     // the points some taxel uses (geom frame) and their hit pressures
  int pair_off, n_pairs;       // the soft-rigid and half-space pairs of the geom, in pair order
  float margin;                // rays count hits with 0 < t < margin
};

// Forces of one kept polygon (soft frame), in the pair-ordered record slot.
struct alignas(16) RecOut {
  float F[3], T[3], area, fn0;
  int n_faces, pad[3];
};

}  // namespace hc
