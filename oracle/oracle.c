/*
 * oracle.c — FP64 CPU restatement of the contact-surface path (checker).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
 * the CPU legs of bench.py as the checker.  Never part of the product.
 * Parity status: UNPINNED (see oracle.h).
 *
 * Reference citations are file:line within ubi-agni/mujoco_contact_surfaces:
 *   P  = mujoco_contact_surfaces/src/mujoco_contact_surfaces_plugin.cpp
 *   PH = mujoco_contact_surfaces/include/mujoco_contact_surfaces/mujoco_contact_surfaces_plugin.h
 *   FS = mujoco_contact_surface_sensors/src/flat_tactile_sensor.cpp
 *   BV = mujoco_contact_surface_sensors/src/bvh.cpp
 *
 * Build with -ffp-contract=off: the flat-sensor arithmetic follows the
 * reference's float expressions operation by operation.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NEAR_TOL 1e-12
#define MAXV 16

/* ------------------------------------------------------------------ */
/* small vector helpers                                                */
/* ------------------------------------------------------------------ */
static inline void v_sub(const double* a, const double* b, double* o) {
  o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
static inline double v_dot(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void v_cross(const double* a, const double* b, double* o) {
  double x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
  o[0] = x; o[1] = y; o[2] = z;
}
static inline double v_norm(const double* a) { return sqrt(v_dot(a, a)); }
/* o = R a (R row-major) */
static inline void m_mul(const double* R, const double* a, double* o) {
  double x = R[0] * a[0] + R[1] * a[1] + R[2] * a[2];
  double y = R[3] * a[0] + R[4] * a[1] + R[5] * a[2];
  double z = R[6] * a[0] + R[7] * a[1] + R[8] * a[2];
  o[0] = x; o[1] = y; o[2] = z;
}
/* o = R^T a */
static inline void m_tmul(const double* R, const double* a, double* o) {
  double x = R[0] * a[0] + R[3] * a[1] + R[6] * a[2];
  double y = R[1] * a[0] + R[4] * a[1] + R[7] * a[2];
  double z = R[2] * a[0] + R[5] * a[1] + R[8] * a[2];
  o[0] = x; o[1] = y; o[2] = z;
}

/* ------------------------------------------------------------------ */
/* AABB tree over mesh elements (median split), used only to find       */
/* candidate element pairs; results do not depend on it.                */
/* ------------------------------------------------------------------ */
typedef struct { double lo[3], hi[3]; int left, right, start, count; } bnode;
typedef struct { bnode* nodes; int n_nodes; int* idx; int n; double* lo; double* hi; } btree;

static int g_axis;
static const double* g_cent;
static int cmp_cent(const void* a, const void* b) {
  double x = g_cent[3 * *(const int*)a + g_axis], y = g_cent[3 * *(const int*)b + g_axis];
  if (x < y) return -1;
  if (x > y) return 1;
  return *(const int*)a - *(const int*)b;
}

static int build_rec(btree* t, const double* cent, int start, int count) {
  int id = t->n_nodes++;
  bnode* nd = &t->nodes[id];
  for (int a = 0; a < 3; ++a) { nd->lo[a] = DBL_MAX; nd->hi[a] = -DBL_MAX; }
  for (int i = start; i < start + count; ++i) {
    int e = t->idx[i];
    for (int a = 0; a < 3; ++a) {
      if (t->lo[3 * e + a] < nd->lo[a]) nd->lo[a] = t->lo[3 * e + a];
      if (t->hi[3 * e + a] > nd->hi[a]) nd->hi[a] = t->hi[3 * e + a];
    }
  }
  nd->start = start; nd->count = count; nd->left = nd->right = -1;
  if (count <= 4) return id;
  int axis = 0;
  double ext = -1;
  for (int a = 0; a < 3; ++a)
    if (nd->hi[a] - nd->lo[a] > ext) { ext = nd->hi[a] - nd->lo[a]; axis = a; }
  g_axis = axis; g_cent = cent;
  qsort(t->idx + start, count, sizeof(int), cmp_cent);
  int half = count / 2;
  int l = build_rec(t, cent, start, half);
  int r = build_rec(t, cent, start + half, count - half);
  t->nodes[id].left = l; t->nodes[id].right = r;
  return id;
}

/* Elements with `npe` vertices each. */
static void build_tree(btree* t, const double* v, const int* e, int ne, int npe) {
  t->n = ne;
  t->idx = (int*)malloc(sizeof(int) * (ne > 0 ? ne : 1));
  t->lo = (double*)malloc(sizeof(double) * 3 * (ne > 0 ? ne : 1));
  t->hi = (double*)malloc(sizeof(double) * 3 * (ne > 0 ? ne : 1));
  double* cent = (double*)malloc(sizeof(double) * 3 * (ne > 0 ? ne : 1));
  for (int i = 0; i < ne; ++i) {
    t->idx[i] = i;
    for (int a = 0; a < 3; ++a) { t->lo[3 * i + a] = DBL_MAX; t->hi[3 * i + a] = -DBL_MAX; cent[3 * i + a] = 0; }
    for (int k = 0; k < npe; ++k) {
      const double* x = v + 3 * e[npe * i + k];
      for (int a = 0; a < 3; ++a) {
        if (x[a] < t->lo[3 * i + a]) t->lo[3 * i + a] = x[a];
        if (x[a] > t->hi[3 * i + a]) t->hi[3 * i + a] = x[a];
        cent[3 * i + a] += x[a] / npe;
      }
    }
  }
  t->nodes = (bnode*)malloc(sizeof(bnode) * (2 * ne + 1));
  t->n_nodes = 0;
  if (ne > 0) build_rec(t, cent, 0, ne);
  free(cent);
}

static void free_tree(btree* t) { free(t->nodes); free(t->idx); free(t->lo); free(t->hi); }

static int cmp_int(const void* a, const void* b) { return *(const int*)a - *(const int*)b; }

/* Elements whose AABB overlaps [lo, hi]; sorted ascending. */
static int query_tree(const btree* t, const double* lo, const double* hi, int* out, int cap) {
  if (t->n_nodes == 0) return 0;
  int stack[128], sp = 0, n = 0;
  stack[sp++] = 0;
  while (sp) {
    const bnode* nd = &t->nodes[stack[--sp]];
    int ov = 1;
    for (int a = 0; a < 3; ++a) ov &= nd->lo[a] <= hi[a] && nd->hi[a] >= lo[a];
    if (!ov) continue;
    if (nd->left < 0) {
      for (int i = nd->start; i < nd->start + nd->count; ++i) {
        int e = t->idx[i];
        int ok = 1;
        for (int a = 0; a < 3; ++a) ok &= t->lo[3 * e + a] <= hi[a] && t->hi[3 * e + a] >= lo[a];
        if (ok && n < cap) out[n++] = e;
      }
    } else {
      stack[sp++] = nd->left;
      stack[sp++] = nd->right;
    }
  }
  qsort(out, n, sizeof(int), cmp_int);
  return n;
}

/* ------------------------------------------------------------------ */
struct or_ctx {
  or_geom* g;
  int n_geom;
  btree* tree;   /* per geom (soft: tets, rigid: triangles) */
};

or_ctx* or_create(const or_geom* geoms, int n_geom) {
  or_ctx* c = (or_ctx*)calloc(1, sizeof(or_ctx));
  c->n_geom = n_geom;
  c->g = (or_geom*)malloc(sizeof(or_geom) * n_geom);
  memcpy(c->g, geoms, sizeof(or_geom) * n_geom);
  c->tree = (btree*)calloc(n_geom, sizeof(btree));
  for (int i = 0; i < n_geom; ++i) {
    const or_geom* g = &c->g[i];
    if (g->kind == 1) build_tree(&c->tree[i], g->v, g->e, g->ne, 4);
    else if (g->kind == 0 && !g->is_plane && g->ne > 0) build_tree(&c->tree[i], g->v, g->e, g->ne, 3);
  }
  return c;
}

void or_destroy(or_ctx* c) {
  if (!c) return;
  for (int i = 0; i < c->n_geom; ++i)
    if (c->tree[i].nodes) free_tree(&c->tree[i]);
  free(c->tree);
  free(c->g);
  free(c);
}

/* ------------------------------------------------------------------ */
/* polygons                                                              */
/* ------------------------------------------------------------------ */
typedef struct {
  int nv;
  double x[MAXV][3];  /* world frame after finish_polygon */
  double pr[MAXV];    /* pressure at the vertices          */
  double n[3];        /* unit normal, out of N into M      */
  double gM, gN;      /* pressure gradients along n */
  double grad[3];     /* soft M-side gradient for the field at the centroid */
  double pc;          /* pressure at the area-weighted centroid */
  double c[3];        /* area-weighted centroid            */
  int elem_a, elem_b, flags;
} poly;

typedef struct { poly* p; int n, cap; } polylist;

static poly* pl_push(polylist* l) {
  if (l->n == l->cap) {
    l->cap = l->cap ? 2 * l->cap : 64;
    l->p = (poly*)realloc(l->p, sizeof(poly) * l->cap);
  }
  return &l->p[l->n++];
}

/* Linear field of a tet: p(x) = g.x + c, from its four vertex values. */
static int tet_field(const double X[4][3], const double P[4], double g[3], double* c) {
  double e1[3], e2[3], e3[3], c23[3], c31[3], c12[3];
  v_sub(X[1], X[0], e1); v_sub(X[2], X[0], e2); v_sub(X[3], X[0], e3);
  v_cross(e2, e3, c23); v_cross(e3, e1, c31); v_cross(e1, e2, c12);
  double det = v_dot(e1, c23);
  if (det == 0) { g[0] = g[1] = g[2] = 0; *c = P[0]; return 0; }
  double d1 = P[1] - P[0], d2 = P[2] - P[0], d3 = P[3] - P[0];
  for (int a = 0; a < 3; ++a) g[a] = (d1 * c23[a] + d2 * c31[a] + d3 * c12[a]) / det;
  *c = P[0] - v_dot(g, X[0]);
  return 1;
}

/* Inward face planes of a positively oriented tet: unit normal n_k and
 * offset so that dist(x) = n_k.x - o_k >= 0 inside; face k is opposite
 * vertex k. */
static void tet_planes(const double X[4][3], double n[4][3], double o[4]) {
  static const int fv[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
  for (int k = 0; k < 4; ++k) {
    double e1[3], e2[3];
    v_sub(X[fv[k][1]], X[fv[k][0]], e1);
    v_sub(X[fv[k][2]], X[fv[k][0]], e2);
    v_cross(e1, e2, n[k]);
    double d[3];
    v_sub(X[k], X[fv[k][0]], d);
    if (v_dot(n[k], d) < 0) { n[k][0] = -n[k][0]; n[k][1] = -n[k][1]; n[k][2] = -n[k][2]; }
    double l = v_norm(n[k]);
    if (l > 0) { n[k][0] /= l; n[k][1] /= l; n[k][2] /= l; }
    o[k] = v_dot(n[k], X[fv[k][0]]);
  }
}

/* Sutherland-Hodgman clip of a polygon (in place) by dist >= 0 of a plane.
 * Sets *flags bit 0 when any vertex lies within NEAR_TOL of the plane. */
static int clip_plane(double (*x)[3], int n, const double* pn, double po, int* flags) {
  double y[MAXV][3], d[MAXV];
  for (int i = 0; i < n; ++i) {
    d[i] = v_dot(pn, x[i]) - po;
    if (fabs(d[i]) < NEAR_TOL) *flags |= 1;
  }
  int m = 0;
  for (int i = 0; i < n; ++i) {
    int j = (i + 1) % n;
    int in_i = d[i] >= 0, in_j = d[j] >= 0;
    if (in_i) { if (m < MAXV) { memcpy(y[m], x[i], sizeof(y[m])); } ++m; }
    if (in_i != in_j) {
      double t = d[i] / (d[i] - d[j]);
      if (m < MAXV)
        for (int a = 0; a < 3; ++a) y[m][a] = x[i][a] + t * (x[j][a] - x[i][a]);
      ++m;
    }
  }
  if (m > MAXV) m = MAXV;
  for (int i = 0; i < m; ++i) memcpy(x[i], y[i], sizeof(y[i]));
  return m;
}

/* Cross-section of a tet with the plane s(x) = 0 given the vertex values
 * s[k]; the crossing points are ordered counter-clockwise about `nrm`. */
static int tet_section(const double X[4][3], const double s[4], const double nrm[3],
                       double out[4][3], int* flags) {
  static const int edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  int n = 0;
  for (int k = 0; k < 4; ++k)
    if (fabs(s[k]) < NEAR_TOL) *flags |= 1;
  for (int e = 0; e < 6; ++e) {
    int a = edges[e][0], b = edges[e][1];
    if ((s[a] >= 0) != (s[b] >= 0)) {
      double t = s[a] / (s[a] - s[b]);
      for (int q = 0; q < 3; ++q) out[n][q] = X[a][q] + t * (X[b][q] - X[a][q]);
      ++n;
    }
  }
  if (n < 3) return n;
  double c[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < 3; ++q) c[q] += out[i][q] / n;
  double u[3], w[3];
  /* in-plane basis u, w = nrm x u */
  double ax[3] = {1, 0, 0};
  if (fabs(nrm[0]) > 0.6) { ax[0] = 0; ax[1] = 1; }
  v_cross(nrm, ax, u);
  double lu = v_norm(u);
  for (int q = 0; q < 3; ++q) u[q] /= lu;
  v_cross(nrm, u, w);
  double ang[4];
  for (int i = 0; i < n; ++i) {
    double d[3];
    v_sub(out[i], c, d);
    ang[i] = atan2(v_dot(d, w), v_dot(d, u));
  }
  for (int i = 1; i < n; ++i)
    for (int j = i; j > 0 && ang[j] < ang[j - 1]; --j) {
      double ta = ang[j]; ang[j] = ang[j - 1]; ang[j - 1] = ta;
      double tx[3];
      memcpy(tx, out[j], sizeof(tx)); memcpy(out[j], out[j - 1], sizeof(tx)); memcpy(out[j - 1], tx, sizeof(tx));
    }
  return n;
}

static double bary_eval(const double X[4][3], const double P[4], const double x[3]) {
  double g[3], c;
  tet_field(X, P, g, &c);
  return v_dot(g, x) + c;
}

/* cos(5*pi/8): faces whose normal makes a larger angle with the pressure
 * gradient are culled (the published method's back-face test). */
static int normal_ok(const double n[3], const double g[3], int* flags) {
  const double kCosAlpha = cos(5.0 * M_PI / 8.0);
  double gl = v_norm(g);
  if (!(gl > 0)) return 0;
  double c = v_dot(n, g) / gl;
  if (fabs(c - kCosAlpha) < NEAR_TOL) *flags |= 1;
  return c > kCosAlpha;
}

static void get_tet(const or_geom* g, int t, double X[4][3], double P[4]) {
  for (int k = 0; k < 4; ++k) {
    int vi = g->e[4 * t + k];
    X[k][0] = g->v[3 * vi]; X[k][1] = g->v[3 * vi + 1]; X[k][2] = g->v[3 * vi + 2];
    P[k] = g->p[vi];
  }
}

/* ---- soft (S) vs rigid surface (R): ComputeContactSurfaceFromSoftVolume-
 * RigidSurface restated (called at P:301-303).  The contact surface is the
 * part of R's triangles inside S's tets; normals are R's outward normals
 * (out of R into S); pressure is S's field.  Computed in S's frame.      */
static void soft_rigid(const or_ctx* c, int gs, int gr, const double* xpos, const double* xmat,
                       int s_is_m, polylist* out) {
  const or_geom* S = &c->g[gs];
  const or_geom* R = &c->g[gr];
  const double *RS = xmat + 9 * gs, *xS = xpos + 3 * gs, *RR = xmat + 9 * gr, *xR = xpos + 3 * gr;
  int* cand = (int*)malloc(sizeof(int) * (S->ne > 0 ? S->ne : 1));
  for (int j = 0; j < R->ne; ++j) {
    double Y[3][3], w[3], d[3];
    for (int k = 0; k < 3; ++k) {
      m_mul(RR, R->v + 3 * R->e[3 * j + k], w);
      for (int a = 0; a < 3; ++a) w[a] += xR[a];
      v_sub(w, xS, d);
      m_tmul(RS, d, Y[k]);
    }
    double e1[3], e2[3], nt[3];
    v_sub(Y[1], Y[0], e1); v_sub(Y[2], Y[0], e2); v_cross(e1, e2, nt);
    double ln = v_norm(nt);
    if (!(ln > 0)) continue;
    for (int a = 0; a < 3; ++a) nt[a] /= ln;
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = fmin(Y[0][a], fmin(Y[1][a], Y[2][a]));
      hi[a] = fmax(Y[0][a], fmax(Y[1][a], Y[2][a]));
    }
    int nc = query_tree(&c->tree[gs], lo, hi, cand, S->ne);
    for (int ci = 0; ci < nc; ++ci) {
      int t = cand[ci];
      double X[4][3], P[4], g[3], cc;
      get_tet(S, t, X, P);
      tet_field(X, P, g, &cc);
      int flags = 0;
      /* tet vertices against the triangle's plane (near-degeneracy only) */
      for (int k = 0; k < 4; ++k) {
        double dd[3];
        v_sub(X[k], Y[0], dd);
        if (fabs(v_dot(nt, dd)) < NEAR_TOL) flags |= 1;
      }
      if (!normal_ok(nt, g, &flags)) continue;
      double pn[4][3], po[4];
      tet_planes(X, pn, po);
      double x[MAXV][3];
      memcpy(x[0], Y[0], sizeof(x[0])); memcpy(x[1], Y[1], sizeof(x[1])); memcpy(x[2], Y[2], sizeof(x[2]));
      int n = 3;
      for (int k = 0; k < 4 && n > 0; ++k) n = clip_plane(x, n, pn[k], po[k], &flags);
      if (n < 3) continue;
      poly* pg = pl_push(out);
      memset(pg, 0, sizeof(*pg));
      pg->nv = n;
      for (int i = 0; i < n; ++i) {
        memcpy(pg->x[i], x[i], sizeof(x[i]));
        pg->pr[i] = v_dot(g, x[i]) + cc;
      }
      double sgn = s_is_m ? 1.0 : -1.0;
      for (int a = 0; a < 3; ++a) { pg->n[a] = sgn * nt[a]; pg->grad[a] = g[a]; }
      pg->elem_a = t; pg->elem_b = j; pg->flags = flags;
    }
  }
  free(cand);
}

/* ---- soft (S) vs rigid half-space: ...SoftVolumeRigidHalfSpace restated
 * (called at P:298-299).  The half-space is z <= 0 of the plane geom's
 * frame; the surface is the plane's section of S's tets; the normal is the
 * plane's +z (out of the half-space into S).                              */
static void soft_halfspace(const or_ctx* c, int gs, int gp, const double* xpos, const double* xmat,
                           int s_is_m, polylist* out) {
  const or_geom* S = &c->g[gs];
  const double *RS = xmat + 9 * gs, *xS = xpos + 3 * gs, *RP = xmat + 9 * gp, *xP = xpos + 3 * gp;
  double nw[3] = {RP[2], RP[5], RP[8]}, np[3], d[3], pp[3];
  m_tmul(RS, nw, np);
  v_sub(xP, xS, d);
  m_tmul(RS, d, pp);
  double off = v_dot(np, pp);
  for (int t = 0; t < S->ne; ++t) {
    double X[4][3], P[4], s[4];
    get_tet(S, t, X, P);
    int pos = 0, neg = 0;
    for (int k = 0; k < 4; ++k) {
      s[k] = v_dot(np, X[k]) - off;
      if (s[k] >= 0) ++pos; else ++neg;
    }
    if (!pos || !neg) continue;
    double g[3], cc;
    tet_field(X, P, g, &cc);
    int flags = 0;
    if (!normal_ok(np, g, &flags)) continue;
    double sec[4][3];
    int n = tet_section(X, s, np, sec, &flags);
    if (n < 3) continue;
    poly* pg = pl_push(out);
    memset(pg, 0, sizeof(*pg));
    pg->nv = n;
    for (int i = 0; i < n; ++i) {
      memcpy(pg->x[i], sec[i], sizeof(sec[i]));
      pg->pr[i] = v_dot(g, sec[i]) + cc;
    }
    double sgn = s_is_m ? 1.0 : -1.0;
    for (int a = 0; a < 3; ++a) { pg->n[a] = sgn * np[a]; pg->grad[a] = g[a]; }
    pg->elem_a = t; pg->elem_b = -1; pg->flags = flags;
  }
}

/* ---- soft (A) vs soft (B): ComputeContactSurfaceFromCompliantVolumes
 * restated (called at P:284-286).  For each overlapping tet pair the
 * equal-pressure plane p_A(x) = p_B(x) (both fields linear) is cut by tet
 * A and clipped by tet B.  The normal points along grad(p_A - p_B), i.e.
 * into A; computed in A's frame.  A is M.                                 */
static void soft_soft(const or_ctx* c, int ga, int gb, const double* xpos, const double* xmat,
                      polylist* out) {
  const or_geom* A = &c->g[ga];
  const or_geom* B = &c->g[gb];
  const double *RA = xmat + 9 * ga, *xA = xpos + 3 * ga, *RB = xmat + 9 * gb, *xB = xpos + 3 * gb;
  /* Rrel = RA^T RB (B frame -> A frame), trel = RA^T (xB - xA) */
  double Rrel[9], trel[3], d[3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      Rrel[3 * i + j] = RA[i] * RB[j] + RA[3 + i] * RB[3 + j] + RA[6 + i] * RB[6 + j];
  v_sub(xB, xA, d);
  m_tmul(RA, d, trel);
  int* cand = (int*)malloc(sizeof(int) * (B->ne > 0 ? B->ne : 1));
  for (int ta = 0; ta < A->ne; ++ta) {
    double XA[4][3], PA[4], ga_[3], ca;
    get_tet(A, ta, XA, PA);
    /* A's tet AABB in B's frame: x_B = Rrel^T (x_A - trel) */
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int k = 0; k < 4; ++k) {
      double q[3], xb[3];
      v_sub(XA[k], trel, q);
      m_tmul(Rrel, q, xb);
      for (int a = 0; a < 3; ++a) { lo[a] = fmin(lo[a], xb[a]); hi[a] = fmax(hi[a], xb[a]); }
    }
    int nc = query_tree(&c->tree[gb], lo, hi, cand, B->ne);
    if (!nc) continue;
    tet_field(XA, PA, ga_, &ca);
    for (int ci = 0; ci < nc; ++ci) {
      int tb = cand[ci];
      double XB0[4][3], PB[4], XB[4][3], gb_[3], cb;
      get_tet(B, tb, XB0, PB);
      for (int k = 0; k < 4; ++k) {
        m_mul(Rrel, XB0[k], XB[k]);
        for (int a = 0; a < 3; ++a) XB[k][a] += trel[a];
      }
      tet_field(XB, PB, gb_, &cb);
      double m[3] = {ga_[0] - gb_[0], ga_[1] - gb_[1], ga_[2] - gb_[2]};
      double lm = v_norm(m);
      if (!(lm > 0)) continue;
      double nrm[3] = {m[0] / lm, m[1] / lm, m[2] / lm};
      int flags = 0;
      double mgb[3] = {-gb_[0], -gb_[1], -gb_[2]};
      if (!normal_ok(nrm, ga_, &flags)) continue;
      if (!normal_ok(nrm, mgb, &flags)) continue;
      double s[4];
      int pos = 0, neg = 0;
      for (int k = 0; k < 4; ++k) {
        s[k] = (PA[k] - (v_dot(gb_, XA[k]) + cb)) / lm;
        if (s[k] >= 0) ++pos; else ++neg;
      }
      if (!pos || !neg) continue;
      double x[MAXV][3], sec[4][3];
      int n = tet_section(XA, s, nrm, sec, &flags);
      for (int i = 0; i < n; ++i) memcpy(x[i], sec[i], sizeof(sec[i]));
      double pn[4][3], po[4];
      tet_planes(XB, pn, po);
      for (int k = 0; k < 4 && n >= 3; ++k) n = clip_plane(x, n, pn[k], po[k], &flags);
      if (n < 3) continue;
      poly* pg = pl_push(out);
      memset(pg, 0, sizeof(*pg));
      pg->nv = n;
      for (int i = 0; i < n; ++i) {
        memcpy(pg->x[i], x[i], sizeof(x[i]));
        pg->pr[i] = v_dot(ga_, x[i]) + ca;
      }
      for (int a = 0; a < 3; ++a) { pg->n[a] = nrm[a]; pg->grad[a] = ga_[a]; }
      /* gM = gradA.n, gN = -gradB.n; kept in A's frame, a
       * rotation leaves the dot products unchanged */
      pg->gM = v_dot(ga_, nrm);
      pg->gN = -v_dot(gb_, nrm);
      if (fabs(pg->gM) < 1e-9 * v_norm(ga_)) pg->gM = 0.0;
      if (fabs(pg->gN) < 1e-9 * v_norm(gb_)) pg->gN = 0.0;
      pg->elem_a = ta; pg->elem_b = tb; pg->flags = flags;
    }
  }
  free(cand);
}

/* Move a polygon from body frame (R, x) to world, compute its area-weighted
 * centroid and the field value there.  gM/gN: soft-rigid and half-space
 * use the soft side's gradient, the rigid side is infinite. */
static void finish_polygon(poly* pg, const double* R, const double* x, int query, int s_is_m) {
  for (int i = 0; i < pg->nv; ++i) {
    double w[3];
    m_mul(R, pg->x[i], w);
    for (int a = 0; a < 3; ++a) pg->x[i][a] = w[a] + x[a];
  }
  double nw[3], gw[3];
  m_mul(R, pg->n, nw);
  m_mul(R, pg->grad, gw);
  memcpy(pg->n, nw, sizeof(nw));
  memcpy(pg->grad, gw, sizeof(gw));
  if (query != 3) {
    /* gradient into the soft body along the normal; a component below
     * 1e-9 of the gradient's magnitude is rounding noise of a gradient
     * perpendicular to the face and counts as zero (face skipped) */
    double gs = v_dot(gw, nw);
    if (fabs(gs) < 1e-9 * v_norm(gw)) gs = 0.0;
    if (s_is_m) { pg->gM = gs; pg->gN = INFINITY; }
    else { pg->gM = INFINITY; pg->gN = gs == 0.0 ? 0.0 : -gs; }
  }
  /* area-weighted centroid by a fan from vertex 0 */
  double A = 0, c[3] = {0, 0, 0}, pc = 0;
  for (int i = 1; i + 1 < pg->nv; ++i) {
    double e1[3], e2[3], cr[3];
    v_sub(pg->x[i], pg->x[0], e1);
    v_sub(pg->x[i + 1], pg->x[0], e2);
    v_cross(e1, e2, cr);
    double ai = 0.5 * v_dot(cr, pg->n);
    A += ai;
    for (int a = 0; a < 3; ++a) c[a] += ai * (pg->x[0][a] + pg->x[i][a] + pg->x[i + 1][a]) / 3.0;
    pc += ai * (pg->pr[0] + pg->pr[i] + pg->pr[i + 1]) / 3.0;
  }
  if (A != 0) {
    for (int a = 0; a < 3; ++a) pg->c[a] = c[a] / A;
    pg->pc = pc / A;
  } else {
    for (int a = 0; a < 3; ++a) {
      pg->c[a] = 0;
      for (int i = 0; i < pg->nv; ++i) pg->c[a] += pg->x[i][a] / pg->nv;
    }
    pg->pc = 0;
    for (int i = 0; i < pg->nv; ++i) pg->pc += pg->pr[i] / pg->nv;
  }
}

static int cmp_poly(const void* a, const void* b) {
  const poly *p = (const poly*)a, *q = (const poly*)b;
  if (p->elem_a != q->elem_a) return p->elem_a < q->elem_a ? -1 : 1;
  if (p->elem_b != q->elem_b) return p->elem_b < q->elem_b ? -1 : 1;
  return 0;
}

/* Dispatch of collision_cb: classify, order soft-first, run
 * the query, then order by registration.  Returns the query
 * kind; polygons end in world frame with normals out of N into M. */
static int run_pair(const or_ctx* c, int g1, int g2, const double* xpos, const double* xmat,
                    int* m_out, int* n_out, polylist* pl) {
  const or_geom *G1 = &c->g[g1], *G2 = &c->g[g2];
  *m_out = g1; *n_out = g2;
  if (G1->kind < 0 || G2->kind < 0 || (G1->kind == 0 && G2->kind == 0)) return 0;
  int m = G1->order <= G2->order ? g1 : g2;
  int n = m == g1 ? g2 : g1;
  *m_out = m; *n_out = n;
  if (G1->kind == 1 && G2->kind == 1) {
    soft_soft(c, m, n, xpos, xmat, pl);
    for (int i = 0; i < pl->n; ++i) finish_polygon(&pl->p[i], xmat + 9 * m, xpos + 3 * m, 3, 1);
    qsort(pl->p, pl->n, sizeof(poly), cmp_poly);
    return 3;
  }
  int gs = G1->kind == 1 ? g1 : g2;
  int gr = gs == g1 ? g2 : g1;
  int s_is_m = gs == m;
  int q;
  if (c->g[gr].is_plane) { soft_halfspace(c, gs, gr, xpos, xmat, s_is_m, pl); q = 2; }
  else { soft_rigid(c, gs, gr, xpos, xmat, s_is_m, pl); q = 1; }
  for (int i = 0; i < pl->n; ++i) finish_polygon(&pl->p[i], xmat + 9 * gs, xpos + 3 * gs, q, s_is_m);
  qsort(pl->p, pl->n, sizeof(poly), cmp_poly);
  return q;
}

/* ------------------------------------------------------------------ */
/* material combination and friction combination */
/* ------------------------------------------------------------------ */
static double E_of(const or_geom* g) { return g->kind == 1 ? g->E : INFINITY; }
static double d_of(const or_geom* g) { return g->kind == 1 ? g->d : 1.0; }  /* rigid: PH:198-199 */

static double combined_E(double ea, double eb) {
  if (isinf(ea)) return eb;
  if (isinf(eb)) return ea;
  return ea * eb / (ea + eb);
}
static double combined_d(const or_geom* a, const or_geom* b) {
  double ea = E_of(a), eb = E_of(b), es = combined_E(ea, eb);
  if (isinf(es)) return 0.5 * (d_of(a) + d_of(b));
  double d = 0;
  if (!isinf(ea)) d += es / ea * d_of(a);
  if (!isinf(eb)) d += es / eb * d_of(b);
  return d;
}
/* Coulomb friction of two surfaces: 2 mu_a mu_b / (mu_a + mu_b); only the
 * dynamic coefficient is used. */
static double combined_mu(double a, double b) {
  if (a + b == 0) return 0;
  return 2 * a * b / (a + b);
}

/* ------------------------------------------------------------------ */
/* one quadrature point: P:345-404 then the force law P:440-482          */
/* ------------------------------------------------------------------ */
typedef struct {
  const double *xM, *xN, *VM, *VN;
  double damping, mu;
  int apply;
  double F[3], T[3];
  double area, total_fn0;
  int n_faces;
} accum;

static void point_force(accum* ac, double A, const double p[3], const double n[3], double gM,
                        double gN, double p0) {
  if (!(A > 1.0e-14)) return;
  const double kGradientEpsilon = 1.0e-14;
  if (gM < kGradientEpsilon || gN < kGradientEpsilon) return;
  double g = 1.0 / (1.0 / gM + 1.0 / gN);
  double fn0 = A * p0;
  double k = A * g;
  ac->area += A;
  ac->total_fn0 += fn0;
  ac->n_faces++;
  /* V_WAq = V_WA.Shift(p - x_A): v + w x r */
  double rA[3], rB[3], vA[3], vB[3], v[3];
  v_sub(p, ac->xM, rA);
  v_sub(p, ac->xN, rB);
  v_cross(ac->VM, rA, vA);
  v_cross(ac->VN, rB, vB);
  for (int a = 0; a < 3; ++a) v[a] = (ac->VM[3 + a] + vA[a]) - (ac->VN[3 + a] + vB[a]);
  double vn = v_dot(v, n);
  double fn = fmax(0.0, 1.0 - ac->damping * vn) * (fn0 - 0.001 * k * vn);
  if (!ac->apply) return;
  const double stiction_tolerance = 1.0e-4, relative_tolerance = 1.0e-2;
  double vt[3];
  for (int a = 0; a < 3; ++a) vt[a] = v[a] - n[a] * vn;
  double eps = stiction_tolerance * relative_tolerance;
  eps = eps * eps;
  double v_slip = sqrt(v_dot(vt, vt) + eps);
  double mu_reg = ac->mu;
  double s = v_slip / stiction_tolerance;
  if (s < 1) mu_reg = ac->mu * s * (2.0 - s);
  double f[3];
  for (int a = 0; a < 3; ++a) f[a] = -mu_reg * (vt[a] / v_slip) * fn + fn * n[a];
  double r[3], tq[3];
  v_sub(p, ac->xM, r);
  v_cross(r, f, tq);
  for (int a = 0; a < 3; ++a) { ac->F[a] += f[a]; ac->T[a] += tq[a]; }
}

/* Quadrature of one polygon.  kPolygon: one point at the
 * area-weighted centroid with p0 = field at the centroid.
 * kTriangle: the polygon is fanned about its centroid; each triangle is one
 * point with p0 at barycentric (1/3,1/3,1/3). */
static void integrate_polygon(accum* ac, const poly* pg, int repr) {
  if (repr == 1) {
    double A = 0;
    for (int i = 1; i + 1 < pg->nv; ++i) {
      double e1[3], e2[3], cr[3];
      v_sub(pg->x[i], pg->x[0], e1);
      v_sub(pg->x[i + 1], pg->x[0], e2);
      v_cross(e1, e2, cr);
      A += 0.5 * v_dot(cr, pg->n);
    }
    point_force(ac, fabs(A), pg->c, pg->n, pg->gM, pg->gN, pg->pc);
    return;
  }
  for (int i = 0; i < pg->nv; ++i) {
    const double *a = pg->x[i], *b = pg->x[(i + 1) % pg->nv];
    double e1[3], e2[3], cr[3], cen[3];
    v_sub(a, pg->c, e1);
    v_sub(b, pg->c, e2);
    v_cross(e1, e2, cr);
    double A = 0.5 * v_norm(cr);
    for (int q = 0; q < 3; ++q) cen[q] = (pg->c[q] + a[q] + b[q]) / 3.0;
    double p0 = pg->pc / 3.0 + pg->pr[i] / 3.0 + pg->pr[(i + 1) % pg->nv] / 3.0;
    point_force(ac, A, cen, pg->n, pg->gM, pg->gN, p0);
  }
}

/* ------------------------------------------------------------------ */
/* flat tactile sensor (FS:262-402), float arithmetic as the reference   */
/* ------------------------------------------------------------------ */
typedef struct { float v0[3], v1[3], v2[3]; double e0, e1, e2; } ftri;
typedef struct { ftri* t; int n, cap; } ftrilist;

static void f_sub(const float* a, const float* b, float* o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }
static void f_cross(const float* a, const float* b, float* o) {
  float x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
  o[0] = x; o[1] = y; o[2] = z;
}
static float f_dot(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* Moeller-Trumbore as BV:49-74. */
static void intersect_tri(const float* O, const float* D, const ftri* tri, int id, float* t_hit,
                          float* u_hit, float* v_hit, int* id_hit) {
  float edge1[3], edge2[3], h[3], s[3], q[3];
  f_sub(tri->v1, tri->v0, edge1);
  f_sub(tri->v2, tri->v0, edge2);
  f_cross(D, edge2, h);
  float a = f_dot(edge1, h);
  if (fabsf(a) < 1e-10f) return;
  float f = 1.0f / a;
  f_sub(O, tri->v0, s);
  float u = f * f_dot(s, h);
  if (u < 0.0f || u > 1.0f) return;
  f_cross(s, edge1, q);
  float v = f * f_dot(D, q);
  if (v < 0.0f || u + v > 1.0f) return;
  float t = f * f_dot(edge2, q);
  if (t < *t_hit && t > 0.0f) { *t_hit = t; *u_hit = u; *v_hit = v; *id_hit = id; }
}

void or_sensor_grid(double xs, double ys, double resolution, int* cx, int* cy) {
  *cx = (int)floorl(2 * (long double)xs / resolution + 0.1L);   /* FS:196-197 */
  *cy = (int)floorl(2 * (long double)ys / resolution + 0.1L);
}

static void sensor_update(or_sensor* sn, const double* xpos, const double* xmat, const ftrilist* tl) {
  int cx = sn->cx, cy = sn->cy;
  float* out = sn->taxels;
  if (!out) return;
  for (int i = 0; i < cx * cy; ++i) out[i] = 0.f;
  if (tl->n == 0) return;                                        /* FS:290-296 */
  const int id = sn->geom;
  float xs = (float)sn->size[0], ys = (float)sn->size[1], zs = (float)sn->size[2];
  double resolution = sn->resolution;
  int sr = sn->sampling_resolution;
  /* FS:179-185 */
  float di_factor = (float)(resolution / sr);
  float sub_halfwidth = (float)(di_factor / 2.0f - resolution / 2.0f);
  float rmean = (float)(1. / (sr * sr));
  float rSampling_resolution = (float)(resolution / sr);
  const float SQRT_2 = 1.41421356237f;
  float max_dist = (float)(SQRT_2 * resolution / 2.0f);
  const double* rot = xmat + 9 * id;
  float sensor_normal[3] = {(float)rot[2], (float)rot[5], (float)rot[8]};
  double sensor_topleft[3] = {-xs, -ys, zs};
  float rsigma_squared = 0.f, rtukey = 0.f;
  float sigma = (float)sn->sigma;
  if (sn->window == 1) rsigma_squared = 0.5f / (sigma * sigma);
  else if (sn->window == 2) rtukey = 1.f / sigma * sr * sr;

  /* bucket triangles by the cells their sensor-frame footprint touches;
   * hits are still decided by the exact per-triangle test below */
  int ncell = cx * cy;
  int* cnt = (int*)calloc(ncell + 1, sizeof(int));
  int* lo_hi = (int*)malloc(sizeof(int) * 4 * tl->n);
  for (int k = 0; k < tl->n; ++k) {
    double mn[2] = {DBL_MAX, DBL_MAX}, mx[2] = {-DBL_MAX, -DBL_MAX};
    const float* vs[3] = {tl->t[k].v0, tl->t[k].v1, tl->t[k].v2};
    for (int q = 0; q < 3; ++q) {
      double w[3] = {vs[q][0] - xpos[3 * id], vs[q][1] - xpos[3 * id + 1], vs[q][2] - xpos[3 * id + 2]}, l[3];
      m_tmul(rot, w, l);
      for (int a = 0; a < 2; ++a) { mn[a] = fmin(mn[a], l[a]); mx[a] = fmax(mx[a], l[a]); }
    }
    int x0 = (int)floor((mn[0] - 1e-6 + xs) / resolution), x1 = (int)floor((mx[0] + 1e-6 + xs) / resolution);
    int y0 = (int)floor((mn[1] - 1e-6 + ys) / resolution), y1 = (int)floor((mx[1] + 1e-6 + ys) / resolution);
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (x1 > cx - 1) x1 = cx - 1;
    if (y1 > cy - 1) y1 = cy - 1;
    lo_hi[4 * k] = x0; lo_hi[4 * k + 1] = x1; lo_hi[4 * k + 2] = y0; lo_hi[4 * k + 3] = y1;
    for (int x = x0; x <= x1; ++x)
      for (int y = y0; y <= y1; ++y) cnt[x * cy + y + 1]++;
  }
  for (int i = 0; i < ncell; ++i) cnt[i + 1] += cnt[i];
  int* fill = (int*)malloc(sizeof(int) * (ncell + 1));
  memcpy(fill, cnt, sizeof(int) * (ncell + 1));
  int* items = (int*)malloc(sizeof(int) * (cnt[ncell] > 0 ? cnt[ncell] : 1));
  for (int k = 0; k < tl->n; ++k)
    for (int x = lo_hi[4 * k]; x <= lo_hi[4 * k + 1]; ++x)
      for (int y = lo_hi[4 * k + 2]; y <= lo_hi[4 * k + 3]; ++y) items[fill[x * cy + y]++] = k;

  for (int x = 0; x < cx; x++) {
    for (int y = 0; y < cy; y++) {
      float avg_pressure = 0;
      for (int i = 0; i < sr; i++) {
        for (int j = 0; j < sr; j++) {
          /* FS:324-331 */
          double pos[3] = {sensor_topleft[0] + x * resolution + (double)(float)(i * rSampling_resolution) +
                               0.5 * rSampling_resolution,
                           sensor_topleft[1] + y * resolution + (double)(float)(j * rSampling_resolution) +
                               0.5 * rSampling_resolution,
                           1.5 * zs};
          double rp[3];
          m_mul(rot, pos, rp);
          for (int a = 0; a < 3; ++a) rp[a] += xpos[3 * id + a];
          float sp[3] = {(float)rp[0], (float)rp[1], (float)rp[2]};
          /* FS:336-339 */
          float O[3], D[3];
          for (int a = 0; a < 3; ++a) {
            O[a] = sp[a] + sensor_normal[a] * 1e-8f;
            D[a] = -sensor_normal[a];
          }
          float t_hit = 1e30f, u_hit = 0, v_hit = 0;
          int hid = -1;
          for (int it = cnt[x * cy + y]; it < cnt[x * cy + y + 1]; ++it) {
            int k = items[it];
            intersect_tri(O, D, &tl->t[k], k, &t_hit, &u_hit, &v_hit, &hid);
          }
          if (hid >= 0 && t_hit < 1.5 * zs && t_hit > 0.0f) {    /* FS:346 */
            float b0 = 1 - u_hit - v_hit;
            double bary[3] = {b0, u_hit, v_hit};
            const ftri* tr = &tl->t[hid];
            double ev = bary[0] * tr->e0 + bary[1] * tr->e1 + bary[2] * tr->e2;
            float raw = (float)(ev * rmean);
            float weight = 1.0f;
            if (sn->window == 1) {                                 /* FS:355-361 */
              float dist = hypotf(di_factor * i + sub_halfwidth, di_factor * j + sub_halfwidth) / max_dist;
              weight = expf(-(dist * dist) * rsigma_squared);
            } else if (sn->window == 2) {                          /* FS:367-380 */
              if (sr / 2 - abs(sr / 2 - i) <= sigma * sr / 2)
                weight *= 0.5f * (1.f - cosf((float)(2.f * M_PI * (sr / 2 - abs(sr / 2 - i)) * rtukey)));
              if (sr / 2 - abs(sr / 2 - j) <= sigma * sr / 2)
                weight *= 0.5f * (1.f - cosf((float)(2.f * M_PI * (sr / 2 - abs(sr / 2 - j)) * rtukey)));
            } else if (sn->window == 3) {                          /* FS:383-388 */
              float inv_dist = 1 - hypotf(di_factor * i + sub_halfwidth, di_factor * j + sub_halfwidth) / max_dist;
              weight = inv_dist * inv_dist;
            }
            avg_pressure += weight * raw;
          }
        }
      }
      out[x + cy * y] = avg_pressure;                            /* FS:396 */
    }
  }
  free(cnt); free(fill); free(items); free(lo_hi);
}

/* The same ray sampling evaluated in FP64 throughout (sample origins, ray
 * test, pressure and sums), for central-difference gradient checks; the
 * fan triangles come from the FP64 polygons. */
typedef struct { double v0[3], v1[3], v2[3]; double e0, e1, e2; } dtri;

static void sensor_update64(or_sensor* sn, const double* xpos, const double* xmat, const dtri* tr, int nt) {
  int cx = sn->cx, cy = sn->cy, sr = sn->sampling_resolution;
  double* out = sn->taxels64;
  for (int i = 0; i < cx * cy; ++i) out[i] = 0.0;
  const int id = sn->geom;
  const double xs = sn->size[0], ys = sn->size[1], zs = sn->size[2], res = sn->resolution;
  const double rsr = res / sr, rmean = 1.0 / (sr * sr);
  const double* rot = xmat + 9 * id;
  const double D[3] = {-rot[2], -rot[5], -rot[8]};
  const double di = res / sr, sub = di / 2.0 - res / 2.0, max_dist = sqrt(2.0) * res / 2.0;
  for (int x = 0; x < cx; ++x)
    for (int y = 0; y < cy; ++y) {
      double acc = 0;
      for (int i = 0; i < sr; ++i)
        for (int j = 0; j < sr; ++j) {
          double pos[3] = {-xs + x * res + (i + 0.5) * rsr, -ys + y * res + (j + 0.5) * rsr, 1.5 * zs}, O[3];
          m_mul(rot, pos, O);
          for (int a = 0; a < 3; ++a) O[a] += xpos[3 * id + a];
          double tb = 1e300, ub = 0, vb = 0;
          int hb = -1;
          for (int k = 0; k < nt; ++k) {
            double e1[3], e2[3], h[3], s[3], q[3];
            v_sub(tr[k].v1, tr[k].v0, e1);
            v_sub(tr[k].v2, tr[k].v0, e2);
            v_cross(D, e2, h);
            double a = v_dot(e1, h);
            if (fabs(a) < 1e-10) continue;
            double f = 1.0 / a;
            v_sub(O, tr[k].v0, s);
            double u = f * v_dot(s, h);
            if (u < 0 || u > 1) continue;
            v_cross(s, e1, q);
            double v = f * v_dot(D, q);
            if (v < 0 || u + v > 1) continue;
            double t = f * v_dot(e2, q);
            if (t < tb && t > 0) { tb = t; ub = u; vb = v; hb = k; }
          }
          if (hb < 0 || !(tb < 1.5 * zs && tb > 0)) continue;
          double p = (1 - ub - vb) * tr[hb].e0 + ub * tr[hb].e1 + vb * tr[hb].e2;
          double w = 1.0;
          double dist = hypot(di * i + sub, di * j + sub) / max_dist;
          if (sn->window == 1) w = exp(-(dist * dist) * 0.5 / (sn->sigma * sn->sigma));
          else if (sn->window == 3) w = (1 - dist) * (1 - dist);
          else if (sn->window == 2) {
            double rt = 1.0 / sn->sigma * sr * sr;
            if (sr / 2 - abs(sr / 2 - i) <= sn->sigma * sr / 2) w *= 0.5 * (1 - cos(2 * M_PI * (sr / 2 - abs(sr / 2 - i)) * rt));
            if (sr / 2 - abs(sr / 2 - j) <= sn->sigma * sr / 2) w *= 0.5 * (1 - cos(2 * M_PI * (sr / 2 - abs(sr / 2 - j)) * rt));
          }
          acc += w * p * rmean;
        }
      out[x + cy * y] = acc;
    }
}

static void push_fan64(dtri** t, int* n, int* cap, const poly* pg) {
  for (int i = 0; i < pg->nv; ++i) {
    if (*n == *cap) {
      *cap = *cap ? 2 * *cap : 256;
      *t = (dtri*)realloc(*t, sizeof(dtri) * *cap);
    }
    dtri* d = &(*t)[(*n)++];
    int j = (i + 1) % pg->nv;
    memcpy(d->v0, pg->x[i], sizeof(d->v0));
    memcpy(d->v1, pg->x[j], sizeof(d->v1));
    memcpy(d->v2, pg->c, sizeof(d->v2));
    d->e0 = pg->pr[i]; d->e1 = pg->pr[j]; d->e2 = pg->pc;
  }
}

/* kTriangle fan of a polygon as float world triangles with the field
 * values at their vertices (the tri_e_MN the sensor evaluates). */
static void push_fan(ftrilist* tl, const poly* pg) {
  for (int i = 0; i < pg->nv; ++i) {
    if (tl->n == tl->cap) {
      tl->cap = tl->cap ? 2 * tl->cap : 256;
      tl->t = (ftri*)realloc(tl->t, sizeof(ftri) * tl->cap);
    }
    ftri* t = &tl->t[tl->n++];
    int j = (i + 1) % pg->nv;
    for (int a = 0; a < 3; ++a) {
      t->v0[a] = (float)pg->x[i][a];
      t->v1[a] = (float)pg->x[j][a];
      t->v2[a] = (float)pg->c[a];
    }
    t->e0 = pg->pr[i]; t->e1 = pg->pr[j]; t->e2 = pg->pc;
  }
}

/* ------------------------------------------------------------------ */
int or_collide(or_ctx* c, const double* xpos, const double* xmat, const double* vel, int n_pair,
               const int* g1, const int* g2, const or_options* opt, or_pair_result* out,
               or_sensor* sensors, int n_sensor, or_candidate* cand, int64_t cand_cap,
               int64_t* n_cand) {
  static const double zero6[6] = {0, 0, 0, 0, 0, 0};
  polylist* lists = (polylist*)calloc(n_pair > 0 ? n_pair : 1, sizeof(polylist));
  int nth = opt->n_threads;
#ifdef _OPENMP
  if (nth <= 0) nth = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
#endif
  for (int i = 0; i < n_pair; ++i) {
    int m, n;
    int q = run_pair(c, g1[i], g2[i], xpos, xmat, &m, &n, &lists[i]);
    or_pair_result* r = &out[i];
    memset(r, 0, sizeof(*r));
    r->query = q; r->m = m; r->n = n;
    if (!q) continue;
    const or_geom *GM = &c->g[m], *GN = &c->g[n];
    accum ac;
    memset(&ac, 0, sizeof(ac));
    ac.xM = xpos + 3 * m; ac.xN = xpos + 3 * n;
    ac.VM = vel ? vel + 6 * m : zero6;
    ac.VN = vel ? vel + 6 * n : zero6;
    ac.damping = combined_d(GM, GN);
    ac.mu = combined_mu(GM->mu_d, GN->mu_d);
    ac.apply = opt->apply_forces;
    double sa = 0.0, sc[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < lists[i].n; ++k) {
      const poly* pg = &lists[i].p[k];
      integrate_polygon(&ac, pg, opt->representation);
      if (pg->flags & 1) r->n_near_degenerate++;
      double A = 0.0;
      for (int q = 1; q + 1 < pg->nv; ++q) {
        double e1[3], e2[3], cr[3];
        v_sub(pg->x[q], pg->x[0], e1);
        v_sub(pg->x[q + 1], pg->x[0], e2);
        v_cross(e1, e2, cr);
        A += 0.5 * v_dot(cr, pg->n);
      }
      A = fabs(A);
      sa += A;
      for (int a = 0; a < 3; ++a) sc[a] += A * pg->c[a];
    }
    for (int a = 0; a < 3; ++a) r->centroid[a] = sa > 0.0 ? sc[a] / sa : 0.0;
    r->n_polygons = lists[i].n;
    r->n_faces = ac.n_faces;
    r->area = ac.area;
    r->total_fn0 = ac.total_fn0;
    for (int a = 0; a < 3; ++a) { r->wrench[a] = ac.F[a]; r->wrench[3 + a] = ac.T[a]; }
  }
  if (n_cand) {
    int64_t k = 0;
    for (int i = 0; i < n_pair; ++i)
      for (int j = 0; j < lists[i].n; ++j) {
        if (cand && k < cand_cap) {
          cand[k].pair = i;
          cand[k].elem_a = lists[i].p[j].elem_a;
          cand[k].elem_b = lists[i].p[j].elem_b;
          cand[k].n_vert = lists[i].p[j].nv;
          cand[k].flags = lists[i].p[j].flags;
        }
        ++k;
      }
    *n_cand = k;
  }
  for (int s = 0; s < n_sensor; ++s) {
    or_sensor* sn = &sensors[s];
    or_sensor_grid(sn->size[0], sn->size[1], sn->resolution, &sn->cx, &sn->cy);
    ftrilist tl = {0, 0, 0};
    for (int i = 0; i < n_pair; ++i) {
      if (!out[i].query || (g1[i] != sn->geom && g2[i] != sn->geom)) continue;
      for (int k = 0; k < lists[i].n; ++k) push_fan(&tl, &lists[i].p[k]);
    }
    sensor_update(sn, xpos, xmat, &tl);
    free(tl.t);
    if (sn->taxels64) {
      dtri* dt = NULL;
      int nd = 0, cap = 0;
      for (int i = 0; i < n_pair; ++i) {
        if (!out[i].query || (g1[i] != sn->geom && g2[i] != sn->geom)) continue;
        for (int k = 0; k < lists[i].n; ++k) push_fan64(&dt, &nd, &cap, &lists[i].p[k]);
      }
      sensor_update64(sn, xpos, xmat, dt, nd);
      free(dt);
    }
  }
  for (int i = 0; i < n_pair; ++i) free(lists[i].p);
  free(lists);
  return 0;
}

int or_surface(or_ctx* c, const double* xpos, const double* xmat, int g1, int g2, int* n_poly,
               int* n_vert, int* poly_offset, double* vert, double* vert_pressure, double* normal,
               int* elem_a, int* elem_b) {
  polylist pl = {0, 0, 0};
  int m, n;
  run_pair(c, g1, g2, xpos, xmat, &m, &n, &pl);
  int nv = 0;
  for (int k = 0; k < pl.n; ++k) {
    if (poly_offset) poly_offset[k] = nv;
    for (int i = 0; i < pl.p[k].nv; ++i) {
      if (vert) for (int a = 0; a < 3; ++a) vert[3 * (nv + i) + a] = pl.p[k].x[i][a];
      if (vert_pressure) vert_pressure[nv + i] = pl.p[k].pr[i];
    }
    if (normal) for (int a = 0; a < 3; ++a) normal[3 * k + a] = pl.p[k].n[a];
    if (elem_a) elem_a[k] = pl.p[k].elem_a;
    if (elem_b) elem_b[k] = pl.p[k].elem_b;
    nv += pl.p[k].nv;
  }
  if (poly_offset) poly_offset[pl.n] = nv;
  *n_poly = pl.n;
  *n_vert = nv;
  free(pl.p);
  return 0;
}
