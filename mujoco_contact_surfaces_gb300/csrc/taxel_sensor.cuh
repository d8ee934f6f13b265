// taxel_sensor.cuh — the taxel-point sensor (included by contact.cu inside
// namespace hc, after adjoint.cuh).
//
// The reference's TaxelSensor::internal_update (mujoco_contact_surface_
// sensors/src/taxel_sensor.cpp:158-478) samples the triangle mesh of every
// contact surface that involves the sensor geom and values each taxel from
// the samples near it.  Here one CTA serves one sensor per step:
//   1. the kept polygons of the sensor's pairs, in collision order and, per
//      pair, in (soft element, other element) order (the order of
//      hc_get_surface), each fanned about its area-weighted centroid c:
//      triangle k = (v_k, v_{k+1}, c) in the world frame (FP64);
//   2. samples per triangle, as the reference: the default grid
//      (st0 = int(|v1-v0|/res)+1, st1 = st2 = int(|v2-v0|/res)+1,
//      st = max(st0, st1); a and b accumulated in double from 0 by 1/st and
//      1/st2 while <= 1) or area importance (per surface, one sample per
//      res * total_area of running area; a = 1 - sqrt(u0), b = (1-a) u1 from
//      std::uniform_real_distribution over a default-seeded minstd_rand0,
//      which is Park-Miller 16807 mod 2^31-1 with two draws per double, so
//      sample g uses draws 4g+1..4g+4 and is generated independently by
//      jumping the state); bary (a, (1-a)(1-b), (1-a)b);
//   3. per taxel over the samples in order: the closest (first minimum of
//      the squared distance) and the squared-weight sum within the margin;
//   4. values as the reference leaves them: closest -> inside the margin the
//      pressure only with visualisation on and |p| > 1e-6, else 0 (the
//      reference's else binds to its visualisation test); weighted and mean
//      fall through into squared (sum of max(0, margin - sqrt(d))^2 |p|,
//      times res); a taxel with no sample within the margin keeps its
//      value; with no samples at all every value is 0.
// All FP64 arithmetic of steps 1-2 uses explicitly rounded intrinsics
// (no contraction), as the host's restatement of the same steps does.

constexpr int kTaxPolys = 1024;   // kept polygons per sensor per step
constexpr int kTaxPer = 4;        // taxels per thread (n_taxels <= 4 * 256)
constexpr int kTaxThreads = 256;

struct TaxelSmem {
  unsigned long long key[kTaxPolys];
  int slot[kTaxPolys];
  int poff[kTaxPolys + 1];
  unsigned short tcnt[kTaxPolys][kMaxPolyV];
  double tarea[kTaxPolys][kMaxPolyV];
  double cen[kTaxPolys][4];       // fan centroid (world) and its pressure
  float4 tile[kTaxThreads];
  int n_poly, overflow;
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

// Iterations of `for (double x = 0; x <= 1; x += 1. / st)`.
__device__ __forceinline__ int grid_count(int st) {
  const double inc = __ddiv_rn(1.0, (double)st);
  int n = 0;
  for (double x = 0; x <= 1.0; x = dadd(x, inc)) ++n;
  return n;
}

// The k-th value of that loop.
__device__ __forceinline__ double grid_value(int st, int k) {
  const double inc = __ddiv_rn(1.0, (double)st);
  double x = 0;
  for (int i = 0; i < k; ++i) x = dadd(x, inc);
  return x;
}

// Park-Miller minstd_rand0 (seed 1): state after `n` draws, and one draw.
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

// Triangle k of kept polygon q (sorted position): vertices relative to the
// sensor origin o (double) and their pressures.
__device__ __forceinline__ void fan_triangle(const StepArgs& a, const TaxelSmem& S, int q, int k, const double* o,
                                             double v[3][3], double pv[3]) {
  const int r = a.rec_perm[S.slot[q]];
  const AdjPoly& R = a.recs[r];
  const FrameDev& F = a.frames[R.pair];
  const int nv = R.nv;
  const int j = k + 1 == nv ? 0 : k + 1;
  double w[3];
  world_vertex(R, k, F, w);
  for (int c = 0; c < 3; ++c) v[0][c] = w[c];
  world_vertex(R, j, F, w);
  for (int c = 0; c < 3; ++c) v[1][c] = w[c];
  v[2][0] = S.cen[q][0];
  v[2][1] = S.cen[q][1];
  v[2][2] = S.cen[q][2];
  pv[0] = R.v[k][3];
  pv[1] = R.v[j][3];
  pv[2] = S.cen[q][3];
}

__global__ void __launch_bounds__(kTaxThreads) taxel_sensor_kernel(StepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TaxelSmem& S = *reinterpret_cast<TaxelSmem*>(smem_raw);
  const int sid = blockIdx.x, tid = threadIdx.x;
  if (!rec_ok(a) || !a.tsens_enabled[sid]) return;
  const TaxelSensorDev T = a.tsens[sid];
  const int total_items = *a.item_total;
  // sensor origin and rotation (the geom pose)
  double o[3], Rg[9];
  for (int c = 0; c < 3; ++c) o[c] = a.xpos[3 * (size_t)T.geom + c];
  for (int c = 0; c < 9; ++c) Rg[c] = a.xmat[9 * (size_t)T.geom + c];
  // 1. the sensor's kept polygons
  if (tid == 0) {
    int n = 0;
    for (int k = 0; k < T.n_pairs; ++k) {
      const PairDev& P = a.pairs[a.tsens_pairs[T.pair_off + k]];
      const int b = a.item_poly_off[min(a.unit_off[P.unit_begin], total_items)];
      const int e = a.item_poly_off[min(a.unit_off[P.unit_end], total_items)];
      n += e - b;
    }
    S.n_poly = n;
    S.overflow = n > kTaxPolys;
  }
  __syncthreads();
  if (S.overflow) {
    if (tid == 0) atomicOr(a.status, 16);
    return;   // values unchanged; reported by hc_get_taxel_sensor_values
  }
  const int np = S.n_poly;
  {
    int base = 0;
    for (int k = 0; k < T.n_pairs; ++k) {
      const PairDev& P = a.pairs[a.tsens_pairs[T.pair_off + k]];
      const int b = a.item_poly_off[min(a.unit_off[P.unit_begin], total_items)];
      const int e = a.item_poly_off[min(a.unit_off[P.unit_end], total_items)];
      for (int i = tid; i < e - b; i += kTaxThreads) {
        const AdjPoly& R = a.recs[a.rec_perm[b + i]];
        S.key[base + i] = ((unsigned long long)k << 48) | ((unsigned long long)(R.elem_a & 0xFFFFFF) << 24) |
                          (unsigned long long)((R.elem_b + 1) & 0xFFFFFF);
        S.slot[base + i] = b + i;
      }
      base += e - b;
    }
  }
  int npow = 1;
  while (npow < np) npow <<= 1;
  for (int i = np + tid; i < npow; i += kTaxThreads) {
    S.key[i] = ~0ull;
    S.slot[i] = -1;
  }
  __syncthreads();
  // bitonic sort of (key, slot)
  for (int size = 2; size <= npow; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = tid; i < npow; i += kTaxThreads) {
        const int j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long ki = S.key[i], kj = S.key[j];
          if ((ki > kj) == up) {
            S.key[i] = kj; S.key[j] = ki;
            const int t = S.slot[i]; S.slot[i] = S.slot[j]; S.slot[j] = t;
          }
        }
      }
      __syncthreads();
    }
  }
  // 2. per polygon: centroid, triangle sample counts (or areas)
  for (int q = tid; q < np; q += kTaxThreads) {
    const AdjPoly& R = a.recs[a.rec_perm[S.slot[q]]];
    const FrameDev& F = a.frames[R.pair];
    const PairDev& P = a.pairs[R.pair];
    const int nv = R.nv;
    // world normal of the contact (out of N into M), for the signed areas
    const double sg = P.s_is_m ? 1.0 : -1.0;
    const double nl[3] = {R.n[0] * sg, R.n[1] * sg, R.n[2] * sg};
    double nw[3];
    for (int c = 0; c < 3; ++c)
      nw[c] = dadd(dadd(dmul(F.RS[3 * c], (double)(float)nl[0]), dmul(F.RS[3 * c + 1], (double)(float)nl[1])),
                   dmul(F.RS[3 * c + 2], (double)(float)nl[2]));
    double v0[3];
    world_vertex(R, 0, F, v0);
    double A = 0, Sx[3] = {0, 0, 0}, Pp = 0;
    for (int i = 1; i + 1 < nv; ++i) {
      double v1[3], v2[3], e1[3], e2[3], cr[3];
      world_vertex(R, i, F, v1);
      world_vertex(R, i + 1, F, v2);
      for (int c = 0; c < 3; ++c) { e1[c] = dsub(v1[c], v0[c]); e2[c] = dsub(v2[c], v0[c]); }
      dcross(e1, e2, cr);
      const double ai = dmul(0.5, dadd(dadd(dmul(cr[0], nw[0]), dmul(cr[1], nw[1])), dmul(cr[2], nw[2])));
      A = dadd(A, ai);
      const double a3 = __ddiv_rn(ai, 3.0);
      for (int c = 0; c < 3; ++c) Sx[c] = dadd(Sx[c], dmul(dadd(dadd(v0[c], v1[c]), v2[c]), a3));
      Pp = dadd(Pp, __ddiv_rn(dmul(ai, dadd(dadd((double)R.v[0][3], (double)R.v[i][3]), (double)R.v[i + 1][3])), 3.0));
    }
    for (int k = 0; k < kMaxPolyV; ++k) {
      S.tcnt[q][k] = 0;
      S.tarea[q][k] = 0;
    }
    if (A == 0) {
      S.cen[q][0] = S.cen[q][1] = S.cen[q][2] = S.cen[q][3] = 0;
      continue;   // zero-area polygon: no fan
    }
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = __ddiv_rn(Sx[k], A);
    const double pc = __ddiv_rn(Pp, A);
    S.cen[q][0] = c[0]; S.cen[q][1] = c[1]; S.cen[q][2] = c[2]; S.cen[q][3] = pc;
    for (int k = 0; k < nv; ++k) {
      double w0[3], w1[3];
      world_vertex(R, k, F, w0);
      world_vertex(R, k + 1 == nv ? 0 : k + 1, F, w1);
      if (T.sample_method == 0) {
        const int st0 = (int)(__ddiv_rn(dnorm3(w1, w0), T.res)) + 1;
        const int st1 = (int)(__ddiv_rn(dnorm3(c, w0), T.res)) + 1;
        const int st = max(st0, st1);
        const int cnt = grid_count(st) * grid_count(st1);
        S.tcnt[q][k] = (unsigned short)min(cnt, 65535);
      } else {
        double e1[3], e2[3], cr[3];
        for (int m = 0; m < 3; ++m) { e1[m] = dsub(w1[m], w0[m]); e2[m] = dsub(c[m], w0[m]); }
        dcross(e1, e2, cr);
        S.tarea[q][k] = dmul(0.5, sqrt(dadd(dadd(dmul(cr[0], cr[0]), dmul(cr[1], cr[1])), dmul(cr[2], cr[2]))));
      }
    }
  }
  __syncthreads();
  // area importance: the running area per surface decides the counts
  if (T.sample_method == 1 && tid == 0) {
    int q0 = 0;
    while (q0 < np) {
      const unsigned long long pk = S.key[q0] >> 48;
      int q1 = q0;
      while (q1 < np && (S.key[q1] >> 48) == pk) ++q1;
      double total = 0;
      for (int q = q0; q < q1; ++q)
        for (int k = 0; k < kMaxPolyV; ++k) total = dadd(total, S.tarea[q][k]);
      const double ares = dmul(T.res, total);
      double area = 0, at = 0;
      for (int q = q0; q < q1; ++q) {
        for (int k = 0; k < kMaxPolyV; ++k) {
          // (missing and zero-area triangles add no area and take no sample)
          at = dadd(at, S.tarea[q][k]);
          int cnt = 0;
          while (area < at && cnt < 65535) {
            area = dadd(area, ares);
            ++cnt;
          }
          S.tcnt[q][k] = (unsigned short)cnt;
        }
      }
      q0 = q1;
    }
  }
  __syncthreads();
  // exclusive scan of the polygons' sample counts (serial; np <= 1024)
  if (tid == 0) {
    int run = 0;
    for (int q = 0; q < np; ++q) {
      S.poff[q] = run;
      for (int k = 0; k < kMaxPolyV; ++k) run += S.tcnt[q][k];
    }
    S.poff[np] = run;
  }
  __syncthreads();
  const int M = np > 0 ? S.poff[np] : 0;
  // this thread's taxels, relative to the sensor origin
  float tx[kTaxPer][3], best[kTaxPer], pbest[kTaxPer], acc[kTaxPer];
  int ws[kTaxPer];
#pragma unroll
  for (int u = 0; u < kTaxPer; ++u) {
    const int i = tid + u * kTaxThreads;
    best[u] = INFINITY; pbest[u] = 0.f; acc[u] = 0.f; ws[u] = 0;
    tx[u][0] = tx[u][1] = tx[u][2] = 0.f;
    if (i < T.n_taxels) {
      const float4 p = a.taxel_pos[T.taxel_off + i];
      for (int c = 0; c < 3; ++c) tx[u][c] = (float)(Rg[3 * c] * p.x + Rg[3 * c + 1] * p.y + Rg[3 * c + 2] * p.z);
    }
  }
  const float margin = (float)T.margin;
  const float r2 = margin * margin;
  // 3. samples in tiles, in order
  for (int s0 = 0; s0 < M; s0 += kTaxThreads) {
    const int s = s0 + tid;
    if (s < M) {
      int lo = 0, hi = np;   // last q with poff[q] <= s
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (S.poff[mid] <= s) lo = mid; else hi = mid;
      }
      const int q = lo;
      int loc = s - S.poff[q], k = 0;
      while (loc >= S.tcnt[q][k]) { loc -= S.tcnt[q][k]; ++k; }
      double v[3][3], pv[3];
      fan_triangle(a, S, q, k, o, v, pv);
      double aa, bb;
      if (T.sample_method == 0) {
        const int st0 = (int)(__ddiv_rn(dnorm3(v[1], v[0]), T.res)) + 1;
        const int st1 = (int)(__ddiv_rn(dnorm3(v[2], v[0]), T.res)) + 1;
        const int st = max(st0, st1);
        const int kb = grid_count(st1);
        aa = grid_value(st, loc / kb);
        bb = grid_value(st1, loc % kb);
      } else {
        unsigned long long x = minstd_jump(4ull * (unsigned long long)s);
        const unsigned long long d0 = mod31(x * 16807u);
        const unsigned long long d1 = mod31(d0 * 16807u);
        const unsigned long long d2 = mod31(d1 * 16807u);
        const unsigned long long d3 = mod31(d2 * 16807u);
        const double u0 = canonical2(d0, d1), u1 = canonical2(d2, d3);
        aa = dsub(1.0, sqrt(u0));
        bb = dmul(dsub(1.0, aa), u1);
      }
      const double w0 = aa, w1 = dmul(dsub(1.0, aa), dsub(1.0, bb)), w2 = dmul(dsub(1.0, aa), bb);
      float p3[3];
      for (int c = 0; c < 3; ++c)
        p3[c] = (float)dsub(dadd(dadd(dmul(w0, v[0][c]), dmul(w1, v[1][c])), dmul(w2, v[2][c])), o[c]);
      const float pr = (float)dadd(dadd(dmul(w0, pv[0]), dmul(w1, pv[1])), dmul(w2, pv[2]));
      S.tile[tid] = make_float4(p3[0], p3[1], p3[2], pr);
    }
    __syncthreads();
    const int nt = min(kTaxThreads, M - s0);
#pragma unroll
    for (int u = 0; u < kTaxPer; ++u) {
      if (tid + u * kTaxThreads >= T.n_taxels) continue;
      for (int j = 0; j < nt; ++j) {
        const float4 sp = S.tile[j];
        const float dx = tx[u][0] - sp.x, dy = tx[u][1] - sp.y, dz = tx[u][2] - sp.z;
        const float d = dx * dx + dy * dy + dz * dz;
        if (d < best[u]) {
          best[u] = d;
          pbest[u] = sp.w;
        }
        if (d < r2) {
          const float w = fmaxf(0.f, margin - sqrtf(d));
          acc[u] += w * w * fabsf(sp.w);
          ++ws[u];
        }
      }
    }
    __syncthreads();
  }
  // 4. values
#pragma unroll
  for (int u = 0; u < kTaxPer; ++u) {
    const int i = tid + u * kTaxThreads;
    if (i >= T.n_taxels) continue;
    float* val = a.taxel_val + T.taxel_off + i;
    if (M == 0) {
      *val = 0.f;
    } else if (T.method == 0) {
      if (best[u] < r2) *val = (T.visualize && fabsf(pbest[u]) > 1e-6f) ? pbest[u] : 0.f;
    } else if (ws[u] > 0) {
      *val = (float)(acc[u] * T.res);
    }
  }
}
