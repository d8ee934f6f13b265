/*
 * taxel.c — FP64 restatement of the reference's taxel-point sensor update
 * (TaxelSensor::internal_update, mujoco_contact_surface_sensors/src/
 * taxel_sensor.cpp:158-478).
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Parity status: unpinned (the
 * sensor samples Drake's triangle mesh of the contact surface; here the
 * surface is given as polygons and fanned as the engine fans them).
 *
 * Input: the contact surfaces that involve the sensor geom, in collision
 * order, each a list of convex polygons (world frame, vertex pressures).
 * Each polygon is fanned about its area-weighted centroid c (pressure pc
 * there): triangle k is (v_k, v_{k+1}, c).  Then, as the reference:
 *   sampling (:183-249)
 *     default: per triangle st0 = int(|v1-v0|/res)+1, st1 = st2 =
 *       int(|v2-v0|/res)+1, st = max(st0, st1); for (a = 0; a <= 1;
 *       a += 1/st) for (b = 0; b <= 1; b += 1/st2): bary (a, (1-a)(1-b),
 *       (1-a)b) (the loops accumulate in double, as written);
 *     area importance: per surface, area_resolution = res * total area;
 *       the running area passes each triangle's cumulative area in
 *       area_resolution steps, one sample per step at bary (a, (1-a)(1-b),
 *       (1-a)b) with a = 1 - sqrt(u0), b = (1-a) u1; u from one
 *       default-seeded std::default_random_engine (minstd_rand0) per update
 *       through std::uniform_real_distribution<double>(0, 1);
 *   distances (:281-286): d = -2 t.s + |t|^2 + |s|^2;
 *   methods (:287-470): closest (first minimum; inside the margin the value
 *     is the pressure only when visualisation is on and |p| > 1e-6, else
 *     0 — the else binds to the visualisation test), weighted, mean and
 *     squared (weighted and mean fall through into squared, so they end
 *     with squared's values: sum of max(0, margin - sqrt(d))^2 |p| times
 *     res); a taxel with no sample inside the margin keeps its value; with
 *     no samples at all every value is 0.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* minstd_rand0 (Park-Miller): x <- 16807 x mod (2^31 - 1), default seed 1. */
typedef struct {
  uint64_t x;
} minstd;

static uint64_t ms_draw(minstd* g) {
  g->x = (g->x * 16807u) % 2147483647u;
  return g->x;
}

/* std::generate_canonical<double, 53> over minstd_rand0 (range R = 2^31 - 2,
 * so k = 2 draws): ((g0 - 1) + (g1 - 1) R) / R^2, kept below 1. */
static double ms_uniform(minstd* g) {
  const double R = 2147483646.0;
  double sum = (double)(ms_draw(g) - 1u);
  double tmp = R;
  sum += (double)(ms_draw(g) - 1u) * tmp;
  tmp *= R;
  double r = sum / tmp;
  if (r >= 1.0) r = nextafter(1.0, 0.0);
  return r;
}

typedef struct {
  double x[3], p;
} sample;

typedef struct {
  sample* s;
  int n, cap;
} samples;

static void push(samples* S, const double v[3][3], const double pv[3], double a, double b) {
  if (S->n == S->cap) {
    S->cap = S->cap ? 2 * S->cap : 1024;
    S->s = (sample*)realloc(S->s, (size_t)S->cap * sizeof(sample));
  }
  const double w0 = a, w1 = (1 - a) * (1 - b), w2 = (1 - a) * b;
  sample* o = &S->s[S->n++];
  for (int k = 0; k < 3; ++k) o->x[k] = w0 * v[0][k] + w1 * v[1][k] + w2 * v[2][k];
  o->p = w0 * pv[0] + w1 * pv[1] + w2 * pv[2];
}

static double dist3(const double* a, const double* b) {
  const double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
  return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

/* Fan triangle k of polygon (verts vx[nv][3], pressures vp[nv]) with its
 * centroid; returns 0 for a polygon of zero area. */
static int polygon_centroid(const double* vx, const double* vp, int nv, const double* nrm, double c[3], double* pc) {
  double A = 0, S[3] = {0, 0, 0}, P = 0;
  for (int i = 1; i + 1 < nv; ++i) {
    const double* v0 = vx;
    const double* v1 = vx + 3 * i;
    const double* v2 = vx + 3 * (i + 1);
    const double e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
    const double e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
    const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double ai = 0.5 * (cr[0] * nrm[0] + cr[1] * nrm[1] + cr[2] * nrm[2]);
    A += ai;
    for (int k = 0; k < 3; ++k) S[k] += (v0[k] + v1[k] + v2[k]) * (ai / 3.0);
    P += ai * (vp[0] + vp[i] + vp[i + 1]) / 3.0;
  }
  if (A == 0) return 0;
  for (int k = 0; k < 3; ++k) c[k] = S[k] / A;
  *pc = P / A;
  return 1;
}

void or_taxel_sensor(const or_taxel_cfg* cfg, int n_surf, const int* surf_poly_off, const int* poly_vert_off,
                     const double* vert, const double* vert_p, const double* normal, double* values) {
  samples S = {0, 0, 0};
  minstd gen = {1};
  for (int si = 0; si < n_surf; ++si) {
    /* the surface's fan triangles, in order */
    int n_tri = 0;
    for (int pi = surf_poly_off[si]; pi < surf_poly_off[si + 1]; ++pi) n_tri += poly_vert_off[pi + 1] - poly_vert_off[pi];
    double* tv = (double*)malloc((size_t)(n_tri > 0 ? n_tri : 1) * 9 * sizeof(double));
    double* tp = (double*)malloc((size_t)(n_tri > 0 ? n_tri : 1) * 3 * sizeof(double));
    int t = 0;
    for (int pi = surf_poly_off[si]; pi < surf_poly_off[si + 1]; ++pi) {
      const int o = poly_vert_off[pi], nv = poly_vert_off[pi + 1] - o;
      double c[3], pc;
      if (!polygon_centroid(vert + 3 * (size_t)o, vert_p + o, nv, normal + 3 * (size_t)pi, c, &pc)) continue;
      for (int k = 0; k < nv; ++k) {
        const int j = k + 1 == nv ? 0 : k + 1;
        for (int q = 0; q < 3; ++q) {
          tv[9 * t + q] = vert[3 * (size_t)(o + k) + q];
          tv[9 * t + 3 + q] = vert[3 * (size_t)(o + j) + q];
          tv[9 * t + 6 + q] = c[q];
        }
        tp[3 * t] = vert_p[o + k];
        tp[3 * t + 1] = vert_p[o + j];
        tp[3 * t + 2] = pc;
        ++t;
      }
    }
    n_tri = t;
    if (cfg->sample_method == 0) {
      for (t = 0; t < n_tri; ++t) {
        double v[3][3];
        memcpy(v, tv + 9 * t, sizeof(v));
        const int st0 = (int)(dist3(v[1], v[0]) / cfg->sample_resolution) + 1;
        const int st1 = (int)(dist3(v[2], v[0]) / cfg->sample_resolution) + 1;
        const int st2 = (int)(dist3(v[2], v[0]) / cfg->sample_resolution) + 1;
        const int st = st0 > st1 ? st0 : st1;
        for (double a = 0; a <= 1; a += 1. / st)
          for (double b = 0; b <= 1; b += 1. / st2) push(&S, v, tp + 3 * t, a, b);
      }
    } else {
      double total = 0;
      for (t = 0; t < n_tri; ++t) {
        const double* v = tv + 9 * t;
        const double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
        const double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
        const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        total += 0.5 * sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      }
      const double area_res = cfg->sample_resolution * total;
      double area = 0, at = 0;
      for (t = 0; t < n_tri; ++t) {
        double v[3][3];
        memcpy(v, tv + 9 * t, sizeof(v));
        const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
        const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
        const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        at += 0.5 * sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        while (area < at) {
          area += area_res;
          const double u0 = ms_uniform(&gen), u1 = ms_uniform(&gen);
          const double a = 1.0 - sqrt(u0);
          const double b = (1.0 - a) * u1;
          push(&S, v, tp + 3 * t, a, b);
        }
      }
    }
    free(tv);
    free(tp);
  }

  const int n = cfg->n_taxels, m = S.n;
  const double r2 = cfg->include_margin * cfg->include_margin;
  if (m == 0) {
    for (int i = 0; i < n; ++i) values[i] = 0;
    free(S.s);
    return;
  }
  for (int i = 0; i < n; ++i) {
    const double* tx = cfg->taxels + 3 * (size_t)i;
    const double tt = tx[0] * tx[0] + tx[1] * tx[1] + tx[2] * tx[2];
    double best = INFINITY, pbest = 0, pw = 0, pm = 0, psq = 0;
    int ws = 0;
    for (int j = 0; j < m; ++j) {
      const sample* s = &S.s[j];
      const double d = (-2 * (tx[0] * s->x[0] + tx[1] * s->x[1] + tx[2] * s->x[2]) + tt) +
                       (s->x[0] * s->x[0] + s->x[1] * s->x[1] + s->x[2] * s->x[2]);
      if (d < best) {
        best = d;
        pbest = s->p;
      }
      if (d < r2) {
        const double ap = fabs(s->p);
        pw += (r2 - d) * ap;
        pm += ap;
        const double w = fmax(0.0, cfg->include_margin - sqrt(d));
        psq += w * w * ap;
        ++ws;
      }
    }
    if (cfg->method == 0) {
      if (best < r2) values[i] = (cfg->visualize && fabs(pbest) > 1e-6) ? pbest : 0.0;
    } else if (ws > 0) {
      /* weighted and mean write their sums, then fall through to squared */
      if (cfg->method == 1) values[i] = pw;
      if (cfg->method <= 2) values[i] = pm;
      values[i] = psq * cfg->sample_resolution;
    }
  }
  free(S.s);
}

/* The n-th draw of a default-constructed minstd_rand0 and the n-th double of
 * std::uniform_real_distribution<double>(0, 1) over it (known-answer hooks). */
uint64_t or_minstd_nth(int n) {
  minstd g = {1};
  uint64_t x = 0;
  for (int i = 0; i < n; ++i) x = ms_draw(&g);
  return x;
}

double or_uniform_nth(int n) {
  minstd g = {1};
  double u = 0;
  for (int i = 0; i < n; ++i) u = ms_uniform(&g);
  return u;
}
