// taxel_sensor.cuh — the taxel-point sensor (included by contact.cu inside
// namespace hc, after adjoint.cuh).
//
// The reference's TaxelSensor::internal_update (mujoco_contact_surface_
// sensors/src/taxel_sensor.cpp:158-478) samples the triangle mesh of every
// contact surface that involves the sensor geom and values each taxel from
// the samples near it.  Two kernels per step:
//
//   taxel_order_kernel (one CTA per pair that any taxel sensor reads): the
//     pair's kept polygons in (soft element, other element) order, the order
//     of hc_get_surface — a bitonic sort of (key, index) in shared memory per
//     2048 polygons and, for longer pairs, the rank of each polygon across
//     the sorted chunks by binary search (stable, no size limit);
//
//   taxel_sensor_kernel (one CTA per sensor): the sensor's pairs in pair
//     order, each pair's polygons in that order, streamed 128 at a time:
//     1. each polygon fanned about its area-weighted centroid c: triangle
//        k = (v_k, v_{k+1}, c) in the world frame (FP64);
//     2. samples per triangle, as the reference: the default grid
//        (st0 = int(|v1-v0|/res)+1, st1 = st2 = int(|v2-v0|/res)+1,
//        st = max(st0, st1); a and b accumulated in double from 0 by 1/st
//        and 1/st2 while <= 1) or area importance (per surface, one sample
//        per res * total_area of running area; a = 1 - sqrt(u0),
//        b = (1-a) u1 from std::uniform_real_distribution over a
//        default-seeded minstd_rand0, which is Park-Miller 16807 mod 2^31-1
//        with two draws per double, so sample g uses draws 4g+1..4g+4 and is
//        generated independently by jumping the state); bary
//        (a, (1-a)(1-b), (1-a)b);
//     3. per taxel over the samples in order: the closest (first minimum of
//        the squared distance) and the squared-weight sum within the margin
//        — per tile of 256 samples, the taxels within the margin of a
//        32-sample sub-tile's bounding box are candidates; one warp scans a
//        candidate's tile (lane j takes samples j, j+32, ...), keeps the
//        first minimum by (distance, index) and sums the weights in a fixed
//        shuffle order;
//     4. values as the reference leaves them: closest -> inside the margin
//        the pressure only with visualisation on and |p| > 1e-6, else 0 (the
//        reference's else binds to its visualisation test); weighted and
//        mean fall through into squared (sum of max(0, margin - sqrt(d))^2
//        |p|, times res); a taxel with no sample within the margin keeps its
//        value; with no samples at all every value is 0.
//
// Which samples a triangle gets (the grid counts, and the running areas of
// the area-importance walk) is decided in FP64 with explicitly rounded
// intrinsics, as the host restatement decides it; sample positions and
// pressures are then formed in FP32 relative to the sensor origin, where the
// distances are taken.  Only samples within the margin of a taxel can change
// its value (the closest value is written only when the closest sample lies
// inside the margin), so a tile of samples whose bounding box is farther than
// the margin from a taxel is skipped for it: the values are those of a scan
// over every sample.

constexpr int kTaxThreads = 256;
constexpr int kTaxWarps = kTaxThreads / 32;
constexpr int kTaxGroup = 512;                      // taxels per pass over the samples
constexpr int kTaxChunk = 128;                      // polygons per chunk
constexpr int kTaxMaxSt = 4096;                     // grid steps per triangle side
constexpr int kTaxMaxTriSamples = 1 << 20;          // samples per fan triangle
constexpr int kSortChunk = 2048;                    // polygons sorted in shared memory at once

struct TaxelTri {
  int cnt, kb;         // samples; b-steps per a-step (default grid)
  float inc_a, inc_b;  // 1/st, 1/st1
};

struct TaxelSmem {
  float4 vtx[kTaxChunk][kMaxPolyV];   // polygon vertices relative to the sensor origin, pressure in w
  float4 cen[kTaxChunk];              // fan centroid relative to the origin, its pressure
  TaxelTri tri[kTaxChunk][kMaxPolyV];
  double tarea[kTaxChunk][kMaxPolyV]; // running surface area after each fan triangle (area importance)
  int nv[kTaxChunk];
  int poff[kTaxChunk + 1];            // exclusive scan of the polygons' sample counts
  int wsum[kTaxWarps];
  float4 tile[kTaxThreads];           // one tile of samples (position, pressure)
  float wbox[kTaxWarps][6];           // per 32-sample sub-tile: bounding box (min, -max)
  float4 tx[kTaxGroup];               // taxels of this pass (world orientation, relative to the origin)
  float best[kTaxGroup], pbest[kTaxGroup], acc[kTaxGroup];
  int ws[kTaxGroup];
  int cand[kTaxGroup];                // taxels within the margin of the tile
  int ncand;
  float fRS[9], fxo[3];               // the pair's soft frame in float, relative to the sensor origin
  float xs_tol;                       // FP64 world-coordinate error bound of the pair
  double area, ares;                  // area-importance walk of the current surface
};
constexpr size_t kTaxelSmemBytes = sizeof(TaxelSmem);

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// World position of a kept polygon's vertex i: R (anc + v) + x, the anchor
// sum in float as the surface records store it.
__device__ __forceinline__ void world_vertex(const AdjPoly& R, int i, const FrameDev& F, double w[3]) {
  const float4 v = *reinterpret_cast<const float4*>(R.v[i]);
  const double p[3] = {(double)(R.anc[0] + v.x), (double)(R.anc[1] + v.y), (double)(R.anc[2] + v.z)};
#pragma unroll
  for (int a = 0; a < 3; ++a)
    w[a] = dadd(dadd(dadd(dmul(F.RS[3 * a], p[0]), dmul(F.RS[3 * a + 1], p[1])), dmul(F.RS[3 * a + 2], p[2])),
                F.xS[a]);
}

__device__ __forceinline__ double dnorm3(const double* a, const double* b) {
  const double d0 = dsub(a[0], b[0]), d1 = dsub(a[1], b[1]), d2 = dsub(a[2], b[2]);
  return sqrt(dadd(dadd(dmul(d0, d0), dmul(d1, d1)), dmul(d2, d2)));
}

__device__ __forceinline__ void dcross(const double* a, const double* b, double* o) {
  o[0] = dsub(dmul(a[1], b[2]), dmul(a[2], b[1]));
  o[1] = dsub(dmul(a[2], b[0]), dmul(a[0], b[2]));
  o[2] = dsub(dmul(a[0], b[1]), dmul(a[1], b[0]));
}

// Iterations of `for (double x = 0; x <= 1; x += 1. / st)` (st <= kTaxMaxSt).
__device__ __forceinline__ int grid_count(int st) {
  const double inc = __ddiv_rn(1.0, (double)st);
  int n = 0;
  for (double x = 0; x <= 1.0; x = dadd(x, inc)) ++n;
  return n;
}

// grid_count(st) for st = 0..kTaxMaxSt, filled once per device.
__device__ int g_grid_tab[kTaxMaxSt + 1];

__global__ void grid_table_kernel() {
  const int st = blockIdx.x * blockDim.x + threadIdx.x;
  if (st >= 1 && st <= kTaxMaxSt) g_grid_tab[st] = grid_count(st);
  if (st == 0) g_grid_tab[0] = 0;
}

// Park-Miller minstd_rand0 (seed 1): state after `n` draws.
__device__ __forceinline__ unsigned long long mod31(unsigned long long p) {
  const unsigned long long M = 0x7fffffffull;
  p = (p & M) + (p >> 31);
  p = (p & M) + (p >> 31);
  return p >= M ? p - M : p;
}
__device__ __forceinline__ unsigned long long minstd_jump(unsigned long long n) {
  unsigned long long x = 1, b = 16807;
  while (n) {
    if (n & 1) x = mod31(x * b);
    b = mod31(b * b);
    n >>= 1;
  }
  return x;
}
// std::generate_canonical<double, 53> of two draws (range 2^31 - 2).
__device__ __forceinline__ double canonical2(unsigned long long d0, unsigned long long d1) {
  const double R = 2147483646.0;
  double sum = (double)(d0 - 1);
  sum = dadd(sum, dmul((double)(d1 - 1), R));
  double r = __ddiv_rn(sum, dmul(R, R));
  if (r >= 1.0) r = 0x1.fffffffffffffp-1;
  return r;
}

// The kept polygons of pair P: record slots [*b, *e).
__device__ __forceinline__ void pair_slots(const StepArgs& a, const PairDev& P, int total_items, int* b, int* e) {
  *b = a.item_poly_off[min(a.unit_off[P.unit_begin], total_items)];
  *e = a.item_poly_off[min(a.unit_off[P.unit_end], total_items)];
}

// Fan of one kept polygon in FP64, as the host restatement forms it: world
// vertices, the area-weighted centroid and its pressure.  Returns false for a
// polygon of zero signed area (no fan).
struct FanD {
  double w[kMaxPolyV][3];
  double c[3], pc;
  int nv;
};

__device__ bool fan_fp64(const StepArgs& a, const AdjPoly& R, FanD& f) {
  const FrameDev& F = a.frames[R.pair];
  const PairDev& P = a.pairs[R.pair];
  const int nv = R.nv;
  f.nv = nv;
  for (int i = 0; i < nv; ++i) world_vertex(R, i, F, f.w[i]);
  // world normal of the contact (out of N into M), for the signed areas
  const double sg = P.s_is_m ? 1.0 : -1.0;
  const double nl[3] = {R.n[0] * sg, R.n[1] * sg, R.n[2] * sg};
  double nw[3];
  for (int c = 0; c < 3; ++c)
    nw[c] = dadd(dadd(dmul(F.RS[3 * c], (double)(float)nl[0]), dmul(F.RS[3 * c + 1], (double)(float)nl[1])),
                 dmul(F.RS[3 * c + 2], (double)(float)nl[2]));
  double A = 0, Sx[3] = {0, 0, 0}, Pp = 0;
  for (int i = 1; i + 1 < nv; ++i) {
    double e1[3], e2[3], cr[3];
    for (int c = 0; c < 3; ++c) { e1[c] = dsub(f.w[i][c], f.w[0][c]); e2[c] = dsub(f.w[i + 1][c], f.w[0][c]); }
    dcross(e1, e2, cr);
    const double ai = dmul(0.5, dadd(dadd(dmul(cr[0], nw[0]), dmul(cr[1], nw[1])), dmul(cr[2], nw[2])));
    A = dadd(A, ai);
    const double a3 = __ddiv_rn(ai, 3.0);
    for (int c = 0; c < 3; ++c) Sx[c] = dadd(Sx[c], dmul(dadd(dadd(f.w[0][c], f.w[i][c]), f.w[i + 1][c]), a3));
    Pp = dadd(Pp, __ddiv_rn(dmul(ai, dadd(dadd((double)R.v[0][3], (double)R.v[i][3]), (double)R.v[i + 1][3])), 3.0));
  }
  if (A == 0) return false;
  for (int k = 0; k < 3; ++k) f.c[k] = __ddiv_rn(Sx[k], A);
  f.pc = __ddiv_rn(Pp, A);
  return true;
}

// Area of fan triangle k, (v_k, v_{k+1}, c), in FP64.
__device__ __forceinline__ double fan_area_fp64(const FanD& f, int k) {
  const double* w0 = f.w[k];
  const double* w1 = f.w[k + 1 == f.nv ? 0 : k + 1];
  double e1[3], e2[3], cr[3];
  for (int m = 0; m < 3; ++m) { e1[m] = dsub(w1[m], w0[m]); e2[m] = dsub(f.c[m], w0[m]); }
  dcross(e1, e2, cr);
  return dmul(0.5, sqrt(dadd(dadd(dmul(cr[0], cr[0]), dmul(cr[1], cr[1])), dmul(cr[2], cr[2]))));
}

// ---------------------------------------------------------------------------
// Polygon order of the pairs the taxel sensors read.

__device__ __forceinline__ unsigned long long poly_order_key(const AdjPoly& R) {
  return ((unsigned long long)((unsigned)R.elem_a ^ 0x80000000u) << 32) | ((unsigned)R.elem_b ^ 0x80000000u);
}

// Keys key[0..n) (ascending): how many are < k, or <= k when `upper`.
__device__ __forceinline__ int sorted_count(const unsigned long long* key, int n, unsigned long long k, bool upper) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const unsigned long long m = key[mid];
    if (m < k || (upper && m == k)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// For a pair read by an area-importance sensor: the running surface area
// after every fan triangle, in polygon order (FP64, summed in order as the
// reference sums it), into tat[slot * kMaxPolyV + k].  The areas are formed
// by all threads, the running sum by one.
__device__ void fan_prefix(const StepArgs& a, int b, int n) {
  if (!a.tpair_ai[blockIdx.x]) return;
  __syncthreads();   // tsort of the pair is complete
  for (int i = threadIdx.x; i < n; i += kTaxThreads) {
    FanD f;
    const AdjPoly& R = a.recs[a.rec_perm[a.tsort[b + i]]];
    const bool ok = fan_fp64(a, R, f);
    double* dst = a.tat + (size_t)(b + i) * kMaxPolyV;
    for (int k = 0; k < kMaxPolyV; ++k) dst[k] = (ok && k < f.nv) ? fan_area_fp64(f, k) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double run = 0;
    for (int i = 0; i < n; ++i) {
      double* dst = a.tat + (size_t)(b + i) * kMaxPolyV;
      double ar[kMaxPolyV];
#pragma unroll
      for (int k = 0; k < kMaxPolyV; ++k) ar[k] = dst[k];
#pragma unroll
      for (int k = 0; k < kMaxPolyV; ++k) {
        if (__double_as_longlong(ar[k]) != 0) run = dadd(run, ar[k]);
        dst[k] = run;
      }
    }
  }
}

__global__ void __launch_bounds__(kTaxThreads) taxel_order_kernel(StepArgs a) {
  __shared__ unsigned long long skey[kSortChunk];
  __shared__ int sidx[kSortChunk];
  if (!rec_ok(a)) return;
  const int tid = threadIdx.x;
  const PairDev& P = a.pairs[a.tpairs[blockIdx.x]];
  int b, e;
  pair_slots(a, P, *a.item_total, &b, &e);
  const int n = e - b;
  if (n <= 0) return;
  const int nch = (n + kSortChunk - 1) / kSortChunk;
  for (int c = 0; c < nch; ++c) {
    const int c0 = c * kSortChunk, m = min(kSortChunk, n - c0);
    int npow = 1;
    while (npow < m) npow <<= 1;
    for (int i = tid; i < npow; i += kTaxThreads) {
      if (i < m) {
        skey[i] = poly_order_key(a.recs[a.rec_perm[b + c0 + i]]);
        sidx[i] = c0 + i;
      } else {
        skey[i] = ~0ull;
        sidx[i] = 0x7fffffff;
      }
    }
    __syncthreads();
    for (int size = 2; size <= npow; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int i = tid; i < npow; i += kTaxThreads) {
          const int j = i ^ stride;
          if (j > i) {
            const bool up = (i & size) == 0;
            const unsigned long long ki = skey[i], kj = skey[j];
            const int ii = sidx[i], ij = sidx[j];
            const bool gt = ki > kj || (ki == kj && ii > ij);
            if (gt == up) {
              skey[i] = kj; skey[j] = ki;
              sidx[i] = ij; sidx[j] = ii;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int i = tid; i < m; i += kTaxThreads) {
      if (nch == 1) {
        a.tsort[b + i] = b + sidx[i];
      } else {
        a.tkey[b + c0 + i] = skey[i];
        a.tidx[b + c0 + i] = sidx[i];
      }
    }
    __syncthreads();
  }
  if (nch == 1) {
    fan_prefix(a, b, n);
    return;
  }
  // rank across the sorted chunks: equal keys keep the index order (chunks
  // before this one hold smaller indices, chunks after it larger ones)
  for (int i = tid; i < n; i += kTaxThreads) {
    const int c = i / kSortChunk;
    const unsigned long long k = a.tkey[b + i];
    int rank = i - c * kSortChunk;
    for (int c2 = 0; c2 < nch; ++c2) {
      if (c2 == c) continue;
      const int base = c2 * kSortChunk;
      rank += sorted_count(a.tkey + b + base, min(kSortChunk, n - base), k, c2 < c);
    }
    a.tsort[b + rank] = b + a.tidx[b + i];
  }
  fan_prefix(a, b, n);
}

// ---------------------------------------------------------------------------
// The sensor.

// Default-grid sample counts of fan triangle k from the FP64 side lengths.
__device__ __forceinline__ TaxelTri grid_tri_fp64(const StepArgs& a, const FanD& f, int k, double res) {
  const double* w0 = f.w[k];
  const double* w1 = f.w[k + 1 == f.nv ? 0 : k + 1];
  TaxelTri t;
  t.cnt = 0; t.kb = 1; t.inc_a = t.inc_b = 0.f;
  const double x0 = __ddiv_rn(dnorm3(w1, w0), res), x1 = __ddiv_rn(dnorm3(f.c, w0), res);
  if (!(x0 < kTaxMaxSt) || !(x1 < kTaxMaxSt)) {
    atomicOr(a.status, 16);   // resolution too fine for this triangle: no samples
    return t;
  }
  const int st1 = (int)x1 + 1, st = max((int)x0 + 1, st1);
  const int na = g_grid_tab[st], nb = g_grid_tab[st1];
  t.kb = nb;
  t.inc_a = 1.f / (float)st;
  t.inc_b = 1.f / (float)st1;
  t.cnt = min(na * nb, kTaxMaxTriSamples);
  if (na * nb > kTaxMaxTriSamples) atomicOr(a.status, 16);
  return t;
}

// FP64 fan of a polygon into chunk position q (the exact path): vertices and
// centroid relative to the sensor origin o, and with `counts` the grid
// sample counts of its triangles.
__device__ void taxel_polygon_fp64(const StepArgs& a, const TaxelSensorDev& T, const AdjPoly& R, const double* o,
                                   TaxelSmem& S, int q, bool counts) {
  FanD f;
  const bool ok = fan_fp64(a, R, f);
  for (int k = 0; k < kMaxPolyV; ++k) S.tri[q][k].cnt = 0;
  S.nv[q] = f.nv;
  if (!ok) return;
  S.cen[q] = make_float4((float)(f.c[0] - o[0]), (float)(f.c[1] - o[1]), (float)(f.c[2] - o[2]), (float)f.pc);
  for (int k = 0; k < f.nv; ++k)
    S.vtx[q][k] = make_float4((float)(f.w[k][0] - o[0]), (float)(f.w[k][1] - o[1]), (float)(f.w[k][2] - o[2]),
                              R.v[k][3]);
  if (counts)
    for (int k = 0; k < f.nv; ++k) S.tri[q][k] = grid_tri_fp64(a, f, k, T.res);
}

// True when the FP32 value x may lie on the other side of an integer
// boundary than its exact value, given |x_float - x_exact| < tol.
__device__ __forceinline__ bool near_integer(float x, float tol) {
  const float fl = floorf(x), fr = x - fl;
  return fr > 1.f - tol || (fl > 0.f && fr < tol);
}

// FP32 fan of a polygon into chunk position q, in the soft frame relative to
// vertex 0, then placed relative to the sensor origin with the pair's float
// frame (S.fRS, S.fxo).  With `counts`, the grid sample counts of its
// triangles — unless a side length over the resolution lies within the FP32
// error bound of an integer, a count exceeds the limits, or the signed area
// is too small to tell from zero: then it returns false and the FP64 path
// decides.  The bound: the vertices are the same floats the FP64 path starts
// from; a side length taken in FP32 from them is within 3e-7 relative of the
// exact length, the centroid offset within 2e-6 of the largest vertex offset,
// and the FP64 path's own error is below 1e-15 of the world coordinates.
__device__ bool taxel_polygon_f32(const StepArgs& a, const TaxelSensorDev& T, const AdjPoly& R, TaxelSmem& S, int q,
                                  bool counts, float inv_res, float xs_scale) {
  const PairDev& P = a.pairs[R.pair];
  const int nv = R.nv;
  float p[kMaxPolyV][3];
  for (int i = 0; i < nv; ++i) {
    const float4 v = *reinterpret_cast<const float4*>(R.v[i]);
    p[i][0] = R.anc[0] + v.x; p[i][1] = R.anc[1] + v.y; p[i][2] = R.anc[2] + v.z;
  }
  const float sg = P.s_is_m ? 1.f : -1.f;
  const float nl[3] = {R.n[0] * sg, R.n[1] * sg, R.n[2] * sg};
  float A = 0.f, co[3] = {0.f, 0.f, 0.f}, Pp = 0.f, maxd = 0.f;
  for (int i = 1; i + 1 < nv; ++i) {
    const float d1[3] = {p[i][0] - p[0][0], p[i][1] - p[0][1], p[i][2] - p[0][2]};
    const float d2[3] = {p[i + 1][0] - p[0][0], p[i + 1][1] - p[0][1], p[i + 1][2] - p[0][2]};
    const float cr[3] = {d1[1] * d2[2] - d1[2] * d2[1], d1[2] * d2[0] - d1[0] * d2[2], d1[0] * d2[1] - d1[1] * d2[0]};
    const float ai = 0.5f * (cr[0] * nl[0] + cr[1] * nl[1] + cr[2] * nl[2]);
    A += ai;
    for (int c = 0; c < 3; ++c) co[c] += (d1[c] + d2[c]) * ai;
    Pp += ai * (R.v[0][3] + R.v[i][3] + R.v[i + 1][3]);
    maxd = fmaxf(maxd, fmaxf(fabsf(d1[0]) + fabsf(d1[1]) + fabsf(d1[2]), fabsf(d2[0]) + fabsf(d2[1]) + fabsf(d2[2])));
  }
  S.nv[q] = nv;
  if (!(fabsf(A) > 1e-5f * maxd * maxd)) return false;
  const float inv3A = 1.f / (3.f * A);
  for (int c = 0; c < 3; ++c) co[c] *= inv3A;
  const float pc = Pp * inv3A;
  for (int k = 0; k < nv; ++k) {
    float w[3];
    for (int r = 0; r < 3; ++r) w[r] = S.fRS[3 * r] * p[k][0] + S.fRS[3 * r + 1] * p[k][1] + S.fRS[3 * r + 2] * p[k][2] + S.fxo[r];
    S.vtx[q][k] = make_float4(w[0], w[1], w[2], R.v[k][3]);
  }
  {
    const float c[3] = {p[0][0] + co[0], p[0][1] + co[1], p[0][2] + co[2]};
    float w[3];
    for (int r = 0; r < 3; ++r) w[r] = S.fRS[3 * r] * c[0] + S.fRS[3 * r + 1] * c[1] + S.fRS[3 * r + 2] * c[2] + S.fxo[r];
    S.cen[q] = make_float4(w[0], w[1], w[2], pc);
  }
  if (!counts) return true;
  const float abs_tol = (4e-6f * maxd + xs_scale) * inv_res + 1e-6f;
  TaxelTri tt[kMaxPolyV];
  for (int k = 0; k < nv; ++k) {
    const int j = k + 1 == nv ? 0 : k + 1;
    const float e[3] = {p[j][0] - p[k][0], p[j][1] - p[k][1], p[j][2] - p[k][2]};
    const float dk[3] = {p[k][0] - p[0][0], p[k][1] - p[0][1], p[k][2] - p[0][2]};
    const float ce[3] = {co[0] - dk[0], co[1] - dk[1], co[2] - dk[2]};
    const float x0 = sqrtf(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * inv_res;
    const float x1 = sqrtf(ce[0] * ce[0] + ce[1] * ce[1] + ce[2] * ce[2]) * inv_res;
    if (!(x0 < kTaxMaxSt - 2) || !(x1 < kTaxMaxSt - 2)) return false;
    if (near_integer(x0, 1e-6f * x0 + abs_tol) || near_integer(x1, 1e-6f * x1 + abs_tol)) return false;
    const int st1 = (int)x1 + 1, st = max((int)x0 + 1, st1);
    const int na = g_grid_tab[st], nb = g_grid_tab[st1];
    if (na * nb > kTaxMaxTriSamples) return false;
    tt[k].cnt = na * nb;
    tt[k].kb = nb;
    tt[k].inc_a = 1.f / (float)st;
    tt[k].inc_b = 1.f / (float)st1;
  }
  for (int k = 0; k < kMaxPolyV; ++k) {
    if (k < nv) S.tri[q][k] = tt[k];
    else S.tri[q][k].cnt = 0;
  }
  return true;
}

// Squared distance from taxel t to a box stored as (min, -max).
__device__ __forceinline__ float box_gap2(const float* box, float4 t) {
  const float gx = fmaxf(fmaxf(box[0] - t.x, t.x + box[3]), 0.f);
  const float gy = fmaxf(fmaxf(box[1] - t.y, t.y + box[4]), 0.f);
  const float gz = fmaxf(fmaxf(box[2] - t.z, t.z + box[5]), 0.f);
  return gx * gx + gy * gy + gz * gz;
}

// Exclusive scan of the chunk's per-polygon sample counts into S.poff
// (thread q < nq holds polygon q).  All threads of the CTA call it.
__device__ __forceinline__ void chunk_scan(TaxelSmem& S, int tid, int nq) {
  int tot = 0;
  if (tid < nq)
    for (int k = 0; k < kMaxPolyV; ++k) tot += S.tri[tid][k].cnt;
  const int lane = tid & 31, warp = tid >> 5;
  int x = tot;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) S.wsum[warp] = x;
  __syncthreads();
  int base = 0;
  for (int w = 0; w < warp; ++w) base += S.wsum[w];
  if (tid < nq) S.poff[tid] = base + x - tot;
  if (tid == nq - 1) S.poff[nq] = base + x;
  __syncthreads();
}

__global__ void __launch_bounds__(kTaxThreads, 3) taxel_sensor_kernel(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TaxelSmem& S = *reinterpret_cast<TaxelSmem*>(smem_raw);
  const int sid = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (!rec_ok(a) || !a.tsens_enabled[sid]) return;
  const TaxelSensorDev T = a.tsens[sid];
  const int total_items = *a.item_total;
  const bool area_imp = T.sample_method == 1;
  // sensor origin and rotation (the geom pose)
  double o[3], Rg[9];
  for (int c = 0; c < 3; ++c) o[c] = a.xpos[3 * (size_t)T.geom + c];
  for (int c = 0; c < 9; ++c) Rg[c] = a.xmat[9 * (size_t)T.geom + c];
  const float margin = (float)T.margin;
  const float r2 = margin * margin;
  const float r2_cull = r2 * 1.0001f;
  const float inv_res = (float)(1.0 / T.res);

  for (int tbase = 0; tbase < T.n_taxels; tbase += kTaxGroup) {
    const int ng = min(kTaxGroup, T.n_taxels - tbase);
    for (int i = tid; i < ng; i += kTaxThreads) {
      const float4 p = a.taxel_pos[T.taxel_off + tbase + i];
      float t[3];
      for (int c = 0; c < 3; ++c) t[c] = (float)(Rg[3 * c] * p.x + Rg[3 * c + 1] * p.y + Rg[3 * c + 2] * p.z);
      S.tx[i] = make_float4(t[0], t[1], t[2], 0.f);
      S.best[i] = INFINITY;
      S.pbest[i] = 0.f;
      S.acc[i] = 0.f;
      S.ws[i] = 0;
    }
    long long g_base = 0;   // samples so far (the area-importance draws follow it)
    for (int k = 0; k < T.n_pairs; ++k) {
      const int pair = a.tsens_pairs[T.pair_off + k];
      int b, e;
      pair_slots(a, a.pairs[pair], total_items, &b, &e);
      if (e <= b) continue;
      if (tid == 0) {
        const FrameDev& F = a.frames[pair];
        for (int i = 0; i < 9; ++i) S.fRS[i] = (float)F.RS[i];
        double xm = 0;
        for (int r = 0; r < 3; ++r) {
          S.fxo[r] = (float)(F.xS[r] - o[r]);
          xm = fmax(xm, fabs(F.xS[r]));
        }
        S.xs_tol = 1e-14f * ((float)xm + 1.f);
        if (area_imp) {
          // one sample per res * (the surface's total area) of running area
          S.ares = dmul(T.res, a.tat[(size_t)(e - 1) * kMaxPolyV + kMaxPolyV - 1]);
          S.area = 0;
        }
      }
      __syncthreads();
      const float xs_tol = S.xs_tol;
      for (int c0 = b; c0 < e; c0 += kTaxChunk) {
        const int nq = min(kTaxChunk, e - c0);
        if (tid < nq) {
          const AdjPoly& R = a.recs[a.rec_perm[a.tsort[c0 + tid]]];
          if (!taxel_polygon_f32(a, T, R, S, tid, !area_imp, inv_res, xs_tol))
            taxel_polygon_fp64(a, T, R, o, S, tid, !area_imp);
          if (area_imp)
            for (int t = 0; t < kMaxPolyV; ++t) S.tarea[tid][t] = a.tat[(size_t)(c0 + tid) * kMaxPolyV + t];
        }
        __syncthreads();
        if (area_imp && tid == 0) {
          // the walk: fan triangle t takes a sample while the running sample
          // area is below the running surface area after t
          double area = S.area;
          const double ares = S.ares;
          for (int q = 0; q < nq; ++q) {
            const int nv = S.nv[q];
            for (int t = 0; t < kMaxPolyV; ++t) {
              int cnt = 0;
              if (t < nv) {
                const double at = S.tarea[q][t];
                while (area < at && cnt < kTaxMaxTriSamples) {
                  area = dadd(area, ares);
                  ++cnt;
                }
                if (area < at) atomicOr(a.status, 16);
              }
              S.tri[q][t].cnt = cnt;
            }
          }
          S.area = area;
        }
        __syncthreads();
        chunk_scan(S, tid, nq);
        const int M = S.poff[nq];
        // 3. the chunk's samples in tiles, in order
        for (int s0 = 0; s0 < M; s0 += kTaxThreads) {
          const int s = s0 + tid;
          float4 smp = make_float4(0.f, 0.f, 0.f, 0.f);
          const bool valid = s < M;
          if (valid) {
            int lo = 0, hi = nq;   // last q with poff[q] <= s
            while (hi - lo > 1) {
              const int mid = (lo + hi) >> 1;
              if (S.poff[mid] <= s) lo = mid; else hi = mid;
            }
            const int q = lo;
            int loc = s - S.poff[q], t = 0;
            while (loc >= S.tri[q][t].cnt) { loc -= S.tri[q][t].cnt; ++t; }
            const int nv = S.nv[q];
            const float4 v0 = S.vtx[q][t], v1 = S.vtx[q][t + 1 == nv ? 0 : t + 1], v2 = S.cen[q];
            float fa, fb;
            if (!area_imp) {
              const TaxelTri tr = S.tri[q][t];
              fa = (float)(loc / tr.kb) * tr.inc_a;
              fb = (float)(loc % tr.kb) * tr.inc_b;
            } else {
              const unsigned long long x = minstd_jump(4ull * (unsigned long long)(g_base + s));
              const unsigned long long d0 = mod31(x * 16807u);
              const unsigned long long d1 = mod31(d0 * 16807u);
              const unsigned long long d2 = mod31(d1 * 16807u);
              const unsigned long long d3 = mod31(d2 * 16807u);
              const double u0 = canonical2(d0, d1), u1 = canonical2(d2, d3);
              const double da = dsub(1.0, sqrt(u0));
              fa = (float)da;
              fb = (float)dmul(dsub(1.0, da), u1);
            }
            const float w0 = fa, w1 = (1.f - fa) * (1.f - fb), w2 = (1.f - fa) * fb;
            smp = make_float4(w0 * v0.x + w1 * v1.x + w2 * v2.x, w0 * v0.y + w1 * v1.y + w2 * v2.y,
                              w0 * v0.z + w1 * v1.z + w2 * v2.z, w0 * v0.w + w1 * v1.w + w2 * v2.w);
          }
          S.tile[tid] = smp;
          // the tile's bounding box (min of the coordinates and of their negatives)
          float bx[6] = {valid ? smp.x : INFINITY,  valid ? smp.y : INFINITY,  valid ? smp.z : INFINITY,
                         valid ? -smp.x : INFINITY, valid ? -smp.y : INFINITY, valid ? -smp.z : INFINITY};
#pragma unroll
          for (int d = 16; d > 0; d >>= 1)
#pragma unroll
            for (int m = 0; m < 6; ++m) bx[m] = fminf(bx[m], __shfl_xor_sync(0xffffffffu, bx[m], d));
          if (lane == 0)
            for (int m = 0; m < 6; ++m) S.wbox[warp][m] = bx[m];
          if (tid == 0) S.ncand = 0;
          __syncthreads();
          const int nt = min(kTaxThreads, M - s0);
          const int nsub = (nt + 31) >> 5;
          // candidates: taxels within the margin of a sub-tile's box
          for (int i = tid; i < ng; i += kTaxThreads) {
            const float4 t = S.tx[i];
            bool near = false;
            for (int w = 0; w < nsub && !near; ++w) near = box_gap2(S.wbox[w], t) <= r2_cull;
            if (near) S.cand[atomicAdd(&S.ncand, 1)] = i;
          }
          __syncthreads();
          const int ncand = S.ncand;
          for (int ci = warp; ci < ncand; ci += kTaxWarps) {
            const int i = S.cand[ci];
            const float4 t = S.tx[i];
            float bd = INFINITY, bp = 0.f, sacc = 0.f;
            int bj = 0x7fffffff, sws = 0;
            for (int w = 0; w < nsub; ++w) {
              if (box_gap2(S.wbox[w], t) > r2_cull) continue;   // warp-uniform
              const int j = (w << 5) + lane;
              if (j < nt) {
                const float4 sp = S.tile[j];
                const float dx = t.x - sp.x, dy = t.y - sp.y, dz = t.z - sp.z;
                const float d = dx * dx + dy * dy + dz * dz;
                if (d < bd) { bd = d; bj = j; bp = sp.w; }
                if (d < r2) {
                  const float wt = fmaxf(0.f, margin - sqrtf(d));
                  sacc += wt * wt * fabsf(sp.w);
                  ++sws;
                }
              }
            }
            // first minimum of the tile by (distance, index); fixed-order sums
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
              const float od = __shfl_xor_sync(0xffffffffu, bd, d);
              const int oj = __shfl_xor_sync(0xffffffffu, bj, d);
              const float op = __shfl_xor_sync(0xffffffffu, bp, d);
              if (od < bd || (od == bd && oj < bj)) { bd = od; bj = oj; bp = op; }
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
              sacc += __shfl_down_sync(0xffffffffu, sacc, d);
              sws += __shfl_down_sync(0xffffffffu, sws, d);
            }
            if (lane == 0) {
              if (bd < S.best[i]) { S.best[i] = bd; S.pbest[i] = bp; }
              S.acc[i] += sacc;
              S.ws[i] += sws;
            }
          }
          __syncthreads();
        }
        g_base += M;
      }
    }
    // 4. values
    for (int i = tid; i < ng; i += kTaxThreads) {
      float* val = a.taxel_val + T.taxel_off + tbase + i;
      if (g_base == 0) {
        *val = 0.f;
      } else if (T.method == 0) {
        if (S.best[i] < r2) *val = (T.visualize && fabsf(S.pbest[i]) > 1e-6f) ? S.pbest[i] : 0.f;
      } else if (S.ws[i] > 0) {
        *val = (float)(S.acc[i] * T.res);
      }
    }
    __syncthreads();
  }
}
