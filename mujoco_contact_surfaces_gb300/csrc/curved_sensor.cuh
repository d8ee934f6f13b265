// curved_sensor.cuh — the curved sensor (included by contact.cu inside
// namespace hc, after taxel_sensor.cuh).
//
// The reference's CurvedSensor (mujoco_contact_surface_sensors/src/
// curved_sensor.cpp) keeps, from load, the points of the geom's surface that
// lie within the margin of some taxel (with their normals, and per taxel its
// points with weights max(0, margin - d)^2), and in internal_update
// (:367-466) casts from every such point p a ray from p + 1e-8 n along -n
// into the contact surfaces of the geom's collisions: the nearest hit with
// 0 < t < margin gives the pressure there, and each taxel's value is the sum
// of weight x pressure over its points (0 without any collision).
//
// One CTA per sensor: up to 1024 points per pass, four per thread, each with
// its ray relative to the sensor origin in FP32; the kept polygons of the
// sensor's pairs are staged 64 at a time in shared memory (vertices, unit
// plane normal, the linear pressure field, a bounding box); every ray keeps
// its nearest hit (ties: the lower record slot).  A polygon is hit when the
// ray meets its plane at 0 < t < the best t so far and the hit lies inside or
// on every edge.  The pressure is the polygon's linear field at the hit, as
// barycentric interpolation on its fan triangle gives it.  Then one thread
// per taxel sums its points' pressures in list order.

constexpr int kCurvThreads = 256;
constexpr int kCurvPer = 4;
constexpr int kCurvGroup = kCurvThreads * kCurvPer;
constexpr int kCurvTile = 64;

struct CurvPoly {
  float q[kMaxPolyV][3];   // vertices relative to the sensor origin
  float m[3], g[3];        // unit plane normal; pressure gradient
  float lo[3], hi[3];      // bounding box
  float p0;                // pressure at q[0]
  float sgn;               // orientation of the vertex order about m (0: degenerate)
  int nv, slot;
};

__global__ void __launch_bounds__(kCurvThreads) curved_sensor_kernel(StepArgs a) {
  __shared__ CurvPoly P[kCurvTile];
  __shared__ float fRS[9], fxo[3];
  const int sid = blockIdx.x, tid = threadIdx.x;
  if (!rec_ok(a) || !a.csens_enabled[sid]) return;
  const CurvedSensorDev C = a.csens[sid];
  const int total_items = *a.item_total;
  double o[3];
  float Rf[9];
  for (int c = 0; c < 3; ++c) o[c] = a.xpos[3 * (size_t)C.geom + c];
  for (int c = 0; c < 9; ++c) Rf[c] = (float)a.xmat[9 * (size_t)C.geom + c];
  const float margin = C.margin;
  constexpr float kBoxEps = 1e-6f;   // 1 um: far above the FP32 rounding of the coordinates

  for (int pbase = 0; pbase < C.n_points; pbase += kCurvGroup) {
    float O[kCurvPer][3], D[kCurvPer][3], best[kCurvPer], bp[kCurvPer];
    int bs[kCurvPer];
#pragma unroll
    for (int u = 0; u < kCurvPer; ++u) {
      const int j = pbase + tid + u * kCurvThreads;
      best[u] = margin;
      bp[u] = 0.f;
      bs[u] = 0x7fffffff;
      O[u][0] = O[u][1] = O[u][2] = 0.f;
      D[u][0] = D[u][1] = D[u][2] = 0.f;
      if (j < C.n_points) {
        const float4 p = a.cpoints[C.point_off + j], n = a.cnormals[C.point_off + j];
        for (int r = 0; r < 3; ++r) {
          const float pw = Rf[3 * r] * p.x + Rf[3 * r + 1] * p.y + Rf[3 * r + 2] * p.z;
          const float nw = Rf[3 * r] * n.x + Rf[3 * r + 1] * n.y + Rf[3 * r + 2] * n.z;
          O[u][r] = pw + nw * 1e-8f;
          D[u][r] = -nw;
        }
      } else {
        best[u] = -1.f;   // no ray
      }
    }
    for (int k = 0; k < C.n_pairs; ++k) {
      const int pair = a.csens_pairs[C.pair_off + k];
      int b, e;
      pair_slots(a, a.pairs[pair], total_items, &b, &e);
      if (e <= b) continue;
      __syncthreads();   // the previous pair's tiles are no longer read
      if (tid == 0) {
        const FrameDev& F = a.frames[pair];
        for (int i = 0; i < 9; ++i) fRS[i] = (float)F.RS[i];
        for (int r = 0; r < 3; ++r) fxo[r] = (float)(F.xS[r] - o[r]);
      }
      __syncthreads();
      for (int c0 = b; c0 < e; c0 += kCurvTile) {
        const int nq = min(kCurvTile, e - c0);
        if (tid < nq) {
          const AdjPoly& R = a.recs[a.rec_perm[c0 + tid]];
          CurvPoly& Q = P[tid];
          const int nv = R.nv;
          float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
          for (int i = 0; i < nv; ++i) {
            const float4 v = *reinterpret_cast<const float4*>(R.v[i]);
            const float x = R.anc[0] + v.x, y = R.anc[1] + v.y, z = R.anc[2] + v.z;
            for (int r = 0; r < 3; ++r) {
              const float w = fRS[3 * r] * x + fRS[3 * r + 1] * y + fRS[3 * r + 2] * z + fxo[r];
              Q.q[i][r] = w;
              lo[r] = fminf(lo[r], w);
              hi[r] = fmaxf(hi[r], w);
            }
          }
          float m[3], g[3];
          for (int r = 0; r < 3; ++r) {
            m[r] = fRS[3 * r] * R.n[0] + fRS[3 * r + 1] * R.n[1] + fRS[3 * r + 2] * R.n[2];
            g[r] = fRS[3 * r] * R.g[0] + fRS[3 * r + 1] * R.g[1] + fRS[3 * r + 2] * R.g[2];
          }
          const float mn = sqrtf(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
          float A2 = 0.f;
          for (int i = 1; i + 1 < nv; ++i) {
            const float e1[3] = {Q.q[i][0] - Q.q[0][0], Q.q[i][1] - Q.q[0][1], Q.q[i][2] - Q.q[0][2]};
            const float e2[3] = {Q.q[i + 1][0] - Q.q[0][0], Q.q[i + 1][1] - Q.q[0][1], Q.q[i + 1][2] - Q.q[0][2]};
            A2 += (e1[1] * e2[2] - e1[2] * e2[1]) * m[0] + (e1[2] * e2[0] - e1[0] * e2[2]) * m[1] +
                  (e1[0] * e2[1] - e1[1] * e2[0]) * m[2];
          }
          for (int r = 0; r < 3; ++r) {
            Q.m[r] = mn > 0.f ? m[r] / mn : 0.f;
            Q.g[r] = g[r];
            Q.lo[r] = lo[r] - kBoxEps;
            Q.hi[r] = hi[r] + kBoxEps;
          }
          Q.p0 = R.v[0][3];
          Q.sgn = (mn > 0.f && A2 != 0.f) ? (A2 > 0.f ? 1.f : -1.f) : 0.f;
          Q.nv = nv;
          Q.slot = c0 + tid;
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kCurvPer; ++u) {
          if (!(best[u] > 0.f)) continue;
          // the ray segment up to the best hit so far
          float slo[3], shi[3];
          for (int r = 0; r < 3; ++r) {
            const float end = O[u][r] + best[u] * D[u][r];
            slo[r] = fminf(O[u][r], end);
            shi[r] = fmaxf(O[u][r], end);
          }
          for (int qi = 0; qi < nq; ++qi) {
            const CurvPoly& Q = P[qi];
            if (Q.sgn == 0.f) continue;
            if (Q.hi[0] < slo[0] || Q.lo[0] > shi[0] || Q.hi[1] < slo[1] || Q.lo[1] > shi[1] || Q.hi[2] < slo[2] ||
                Q.lo[2] > shi[2])
              continue;
            const float dn = Q.m[0] * D[u][0] + Q.m[1] * D[u][1] + Q.m[2] * D[u][2];
            if (!(fabsf(dn) > 1e-20f)) continue;   // parallel to the polygon's plane
            const float t = (Q.m[0] * (Q.q[0][0] - O[u][0]) + Q.m[1] * (Q.q[0][1] - O[u][1]) +
                             Q.m[2] * (Q.q[0][2] - O[u][2])) / dn;
            if (!(t > 0.f) || t > best[u] || (t == best[u] && Q.slot >= bs[u])) continue;
            const float h[3] = {O[u][0] + t * D[u][0], O[u][1] + t * D[u][1], O[u][2] + t * D[u][2]};
            bool in = true;
            for (int i = 0; i < Q.nv && in; ++i) {
              const int i1 = i + 1 == Q.nv ? 0 : i + 1;
              const float ex = Q.q[i1][0] - Q.q[i][0], ey = Q.q[i1][1] - Q.q[i][1], ez = Q.q[i1][2] - Q.q[i][2];
              const float wx = h[0] - Q.q[i][0], wy = h[1] - Q.q[i][1], wz = h[2] - Q.q[i][2];
              const float s = (ey * wz - ez * wy) * Q.m[0] + (ez * wx - ex * wz) * Q.m[1] + (ex * wy - ey * wx) * Q.m[2];
              in = s * Q.sgn >= 0.f;
            }
            if (!in) continue;
            best[u] = t;
            bs[u] = Q.slot;
            bp[u] = Q.p0 + Q.g[0] * (h[0] - Q.q[0][0]) + Q.g[1] * (h[1] - Q.q[0][1]) + Q.g[2] * (h[2] - Q.q[0][2]);
          }
        }
        __syncthreads();
      }
    }
#pragma unroll
    for (int u = 0; u < kCurvPer; ++u) {
      const int j = pbase + tid + u * kCurvThreads;
      if (j < C.n_points) a.chit[C.point_off + j] = best[u] < margin ? bp[u] : 0.f;
    }
  }
  __syncthreads();   // every point's hit pressure is written
  for (int i = tid; i < C.n_taxels; i += kCurvThreads) {
    const int l0 = a.clist_off[C.taxel_off + i], l1 = a.clist_off[C.taxel_off + i + 1];
    float s = 0.f;
    for (int l = l0; l < l1; ++l) s += a.clist_w[l] * a.chit[C.point_off + a.clist_pt[l]];
    a.cvalues[C.taxel_off + i] = s;
  }
}
