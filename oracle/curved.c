/*
 * curved.c — FP64 restatement of the reference's curved sensor
 * (CurvedSensor, mujoco_contact_surface_sensors/src/curved_sensor.cpp):
 * the choice, at load, of the surface points near each taxel (:251-355) and
 * the per-update rays from those points into the contact surfaces (:367-461).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Parity status: unpinned (the
 * reference draws its surface points with vcglib's Poisson-disk sampler,
 * which is not available here, and intersects Drake's triangle mesh of the
 * contact surface; here the points are given and each polygon is fanned
 * about its area-weighted centroid, as the engine fans it).
 *
 * Selection (:328-347): d(i, j) = (-2 t_i.s_j + |t_i|^2) + |s_j|^2 (the
 * distance-matrix expression); point j belongs to taxel i when
 * d < margin^2 and (the taxel has no normal, or acos(n_i . s_n_j) < 45
 * degrees); its weight is max(0, margin - sqrt(d))^2.  Each taxel's list is
 * in point order.
 *
 * Update (:447-466): the ray of point j starts at p_j + 1e-8 n_j and runs
 * along -n_j; the nearest hit of any fan triangle (Moeller-Trumbore as
 * bvh.cpp:49-74 applies it: |a| < 1e-10 is parallel, u in [0, 1], v >= 0,
 * u + v <= 1, 0 < t < best) counts when t < margin, with the pressure
 * (1-u-v) p0 + u p1 + v p2; taxel i's value is the sum of weight x pressure
 * over its list.  With no surfaces every value is 0.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

int or_curved_select(int n_taxels, const double* taxels, const double* taxel_normals, double margin, int n_points,
                     const double* points, const double* point_normals, int* off, int* pt, double* w) {
  const double m2 = margin * margin;
  const double lim = 45 * M_PI / 180.;
  int n = 0;
  /* the reference appends in point order (outer loop over points) */
  int* cnt = (int*)calloc((size_t)n_taxels + 1, sizeof(int));
  for (int j = 0; j < n_points; ++j) {
    const double* s = points + 3 * (size_t)j;
    const double ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    for (int i = 0; i < n_taxels; ++i) {
      const double* t = taxels + 3 * (size_t)i;
      const double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      const double d = (-2 * (t[0] * s[0] + t[1] * s[1] + t[2] * s[2]) + tt) + ss;
      int ok = d < m2;
      if (ok && taxel_normals) {
        const double* nt = taxel_normals + 3 * (size_t)i;
        const double nn = nt[0] * nt[0] + nt[1] * nt[1] + nt[2] * nt[2];
        if (nn != 0) {
          const double* sn = point_normals + 3 * (size_t)j;
          ok = acos(nt[0] * sn[0] + nt[1] * sn[1] + nt[2] * sn[2]) < lim;
        }
      }
      if (ok) ++cnt[i];
    }
  }
  off[0] = 0;
  for (int i = 0; i < n_taxels; ++i) off[i + 1] = off[i] + cnt[i];
  memset(cnt, 0, (size_t)n_taxels * sizeof(int));
  for (int j = 0; j < n_points; ++j) {
    const double* s = points + 3 * (size_t)j;
    const double ss = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    for (int i = 0; i < n_taxels; ++i) {
      const double* t = taxels + 3 * (size_t)i;
      const double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      const double d = (-2 * (t[0] * s[0] + t[1] * s[1] + t[2] * s[2]) + tt) + ss;
      int ok = d < m2;
      if (ok && taxel_normals) {
        const double* nt = taxel_normals + 3 * (size_t)i;
        const double nn = nt[0] * nt[0] + nt[1] * nt[1] + nt[2] * nt[2];
        if (nn != 0) {
          const double* sn = point_normals + 3 * (size_t)j;
          ok = acos(nt[0] * sn[0] + nt[1] * sn[1] + nt[2] * sn[2]) < lim;
        }
      }
      if (ok) {
        const int k = off[i] + cnt[i]++;
        const double r = margin - sqrt(d);
        pt[k] = j;
        w[k] = r > 0 ? r * r : 0.0;
        ++n;
      }
    }
  }
  free(cnt);
  return n;
}

static void sub3(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Area-weighted centroid of a polygon and its pressure; 0 for zero area. */
static int centroid(const double* vx, const double* vp, int nv, const double* nrm, double c[3], double* pc) {
  double A = 0, S[3] = {0, 0, 0}, P = 0;
  for (int i = 1; i + 1 < nv; ++i) {
    double e1[3], e2[3], cr[3];
    sub3(vx + 3 * i, vx, e1);
    sub3(vx + 3 * (i + 1), vx, e2);
    cross3(e1, e2, cr);
    const double ai = 0.5 * dot3(cr, nrm);
    A += ai;
    for (int k = 0; k < 3; ++k) S[k] += (vx[k] + vx[3 * i + k] + vx[3 * (i + 1) + k]) * (ai / 3.0);
    P += ai * (vp[0] + vp[i] + vp[i + 1]) / 3.0;
  }
  if (A == 0) return 0;
  for (int k = 0; k < 3; ++k) c[k] = S[k] / A;
  *pc = P / A;
  return 1;
}

void or_curved_update(int n_taxels, const int* off, const int* pt, const double* w, int n_points,
                      const double* points, const double* normals, double margin, int n_surf,
                      const int* surf_poly_off, const int* poly_vert_off, const double* vert, const double* vert_p,
                      const double* normal, double* values) {
  if (n_surf == 0) {
    for (int i = 0; i < n_taxels; ++i) values[i] = 0;
    return;
  }
  /* the hit pressure of every point's ray (a point may serve several taxels) */
  double* raw = (double*)malloc((size_t)(n_points > 0 ? n_points : 1) * sizeof(double));
  int* hit = (int*)calloc((size_t)(n_points > 0 ? n_points : 1), sizeof(int));
  const int n_poly = surf_poly_off[n_surf];
  for (int j = 0; j < n_points; ++j) {
    const double* p = points + 3 * (size_t)j;
    const double* nn = normals + 3 * (size_t)j;
    const double O[3] = {p[0] + nn[0] * 1e-8, p[1] + nn[1] * 1e-8, p[2] + nn[2] * 1e-8};
    const double D[3] = {-nn[0], -nn[1], -nn[2]};
    double best = 1e30, bp = 0;
    for (int q = 0; q < n_poly; ++q) {
      const int o = poly_vert_off[q], nv = poly_vert_off[q + 1] - o;
      double c[3], pc;
      if (!centroid(vert + 3 * (size_t)o, vert_p + o, nv, normal + 3 * (size_t)q, c, &pc)) continue;
      for (int k = 0; k < nv; ++k) {
        const int kk = k + 1 == nv ? 0 : k + 1;
        const double* v0 = vert + 3 * (size_t)(o + k);
        const double* v1 = vert + 3 * (size_t)(o + kk);
        double e1[3], e2[3], h[3], s[3], qv[3];
        sub3(v1, v0, e1);
        sub3(c, v0, e2);
        cross3(D, e2, h);
        const double a = dot3(e1, h);
        if (fabs(a) < 1e-10) continue;
        const double f = 1.0 / a;
        sub3(O, v0, s);
        const double u = f * dot3(s, h);
        if (u < 0.0 || u > 1.0) continue;
        cross3(s, e1, qv);
        const double v = f * dot3(D, qv);
        if (v < 0.0 || u + v > 1.0) continue;
        const double t = f * dot3(e2, qv);
        if (t < best && t > 0.0) {
          best = t;
          bp = (1 - u - v) * vert_p[o + k] + u * vert_p[o + kk] + v * pc;
        }
      }
    }
    hit[j] = best < margin && best > 0.0;
    raw[j] = bp;
  }
  for (int i = 0; i < n_taxels; ++i) {
    double s = 0;
    for (int k = off[i]; k < off[i + 1]; ++k)
      if (hit[pt[k]]) s += w[k] * raw[pt[k]];
    values[i] = s;
  }
  free(raw);
  free(hit);
}
