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
  double tarea[kTaxChunk][kMaxPolyV]; // fan triangle areas (area importance)
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
  double area, at, ares;              // area-importance walk of the current surface
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
  if (nch == 1) return;
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
}

// ---------------------------------------------------------------------------
// The sensor.

// Fan of one kept polygon (FP64) into chunk position q: vertices and
// centroid relative to the sensor origin o, and per fan triangle either the
// default-grid sample counts (`counts`) or the area.  A polygon of zero area
// has no fan (all counts and areas 0).
__device__ void taxel_polygon(const StepArgs& a, const TaxelSensorDev& T, const AdjPoly& R, const double* o,
                              TaxelSmem& S, int q, bool counts) {
  const FrameDev& F = a.frames[R.pair];
  const PairDev& P = a.pairs[R.pair];
  const int nv = R.nv;
  double w[kMaxPolyV][3];
  for (int i = 0; i < nv; ++i) world_vertex(R, i, F, w[i]);
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
    for (int c = 0; c < 3; ++c) { e1[c] = dsub(w[i][c], w[0][c]); e2[c] = dsub(w[i + 1][c], w[0][c]); }
    dcross(e1, e2, cr);
    const double ai = dmul(0.5, dadd(dadd(dmul(cr[0], nw[0]), dmul(cr[1], nw[1])), dmul(cr[2], nw[2])));
    A = dadd(A, ai);
    const double a3 = __ddiv_rn(ai, 3.0);
    for (int c = 0; c < 3; ++c) Sx[c] = dadd(Sx[c], dmul(dadd(dadd(w[0][c], w[i][c]), w[i + 1][c]), a3));
    Pp = dadd(Pp, __ddiv_rn(dmul(ai, dadd(dadd((double)R.v[0][3], (double)R.v[i][3]), (double)R.v[i + 1][3])), 3.0));
  }
  for (int k = 0; k < kMaxPolyV; ++k) {
    S.tri[q][k].cnt = 0;
    S.tarea[q][k] = 0;
  }
  S.nv[q] = nv;
  if (A == 0) return;
  double c[3];
  for (int k = 0; k < 3; ++k) c[k] = __ddiv_rn(Sx[k], A);
  const double pc = __ddiv_rn(Pp, A);
  S.cen[q] = make_float4((float)(c[0] - o[0]), (float)(c[1] - o[1]), (float)(c[2] - o[2]), (float)pc);
  for (int k = 0; k < nv; ++k)
    S.vtx[q][k] = make_float4((float)(w[k][0] - o[0]), (float)(w[k][1] - o[1]), (float)(w[k][2] - o[2]), R.v[k][3]);
  for (int k = 0; k < nv; ++k) {
    const double* w0 = w[k];
    const double* w1 = w[k + 1 == nv ? 0 : k + 1];
    if (counts) {
      const double x0 = __ddiv_rn(dnorm3(w1, w0), T.res), x1 = __ddiv_rn(dnorm3(c, w0), T.res);
      if (!(x0 < kTaxMaxSt) || !(x1 < kTaxMaxSt)) {
        atomicOr(a.status, 16);   // resolution too fine for this triangle: no samples
        continue;
      }
      const int st1 = (int)x1 + 1, st = max((int)x0 + 1, st1);
      const int na = grid_count(st), nb = grid_count(st1);
      TaxelTri t;
      t.kb = nb;
      t.inc_a = (float)__ddiv_rn(1.0, (double)st);
      t.inc_b = (float)__ddiv_rn(1.0, (double)st1);
      t.cnt = min(na * nb, kTaxMaxTriSamples);
      if (na * nb > kTaxMaxTriSamples) atomicOr(a.status, 16);
      S.tri[q][k] = t;
    } else {
      double e1[3], e2[3], cr[3];
      for (int m = 0; m < 3; ++m) { e1[m] = dsub(w1[m], w0[m]); e2[m] = dsub(c[m], w0[m]); }
      dcross(e1, e2, cr);
      S.tarea[q][k] = dmul(0.5, sqrt(dadd(dadd(dmul(cr[0], cr[0]), dmul(cr[1], cr[1])), dmul(cr[2], cr[2]))));
    }
  }
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
      const PairDev& P = a.pairs[a.tsens_pairs[T.pair_off + k]];
      int b, e;
      pair_slots(a, P, total_items, &b, &e);
      if (e <= b) continue;
      if (area_imp) {
        // the surface's total area, summed in order
        double total = 0;
        for (int c0 = b; c0 < e; c0 += kTaxChunk) {
          const int nq = min(kTaxChunk, e - c0);
          if (tid < nq) taxel_polygon(a, T, a.recs[a.rec_perm[a.tsort[c0 + tid]]], o, S, tid, false);
          __syncthreads();
          if (tid == 0)
            for (int q = 0; q < nq; ++q)
              for (int t = 0; t < kMaxPolyV; ++t) total = dadd(total, S.tarea[q][t]);
          __syncthreads();
        }
        if (tid == 0) {
          S.ares = dmul(T.res, total);
          S.area = 0;
          S.at = 0;
        }
        __syncthreads();
      }
      for (int c0 = b; c0 < e; c0 += kTaxChunk) {
        const int nq = min(kTaxChunk, e - c0);
        if (tid < nq) taxel_polygon(a, T, a.recs[a.rec_perm[a.tsort[c0 + tid]]], o, S, tid, !area_imp);
        __syncthreads();
        if (area_imp && tid == 0) {
          // one sample per area step of running area (missing and zero-area
          // triangles add no area and take no sample)
          double area = S.area, at = S.at;
          const double ares = S.ares;
          for (int q = 0; q < nq; ++q) {
            for (int t = 0; t < kMaxPolyV; ++t) {
              at = dadd(at, S.tarea[q][t]);
              int cnt = 0;
              while (area < at && cnt < kTaxMaxTriSamples) {
                area = dadd(area, ares);
                ++cnt;
              }
              if (area < at) atomicOr(a.status, 16);
              S.tri[q][t].cnt = cnt;
            }
          }
          S.area = area;
          S.at = at;
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
