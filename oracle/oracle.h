/*
 * oracle.h — FP64 CPU restatement of the reference's contact-surface path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline / reference legs of bench.py may load this library, and only
 * as the checker.  The product (libhc) never links or calls it.
 *
 * Parity status: UNPINNED.  The reference has no tests, golden vectors or
 * fixtures, and its contact-surface arithmetic lives in Drake v1.8.0
 * (drake-20220919-focal), which is not vendored and cannot be built here
 * (no Drake, MuJoCo, ROS or Eigen).  The in-repo parts are restated line by
 * line (quadrature, material combination, force law, flat-sensor sampling);
 * the Drake queries are restated from the published hydroelastic method
 * (Elandt et al. 2019, arXiv 1904.11433; Masterjohn et al. 2021, arXiv
 * 2110.04157).  Analytic known-answer tests anchor what they can.
 */
#ifndef HC_ORACLE_H_
#define HC_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int kind;          /* 1 soft, 0 rigid, -1 no cs:: properties            */
  int is_plane;      /* rigid half-space z <= 0 of the geom frame          */
  int order;         /* registration order (M is the smaller)              */
  double E, d, mu_s, mu_d;
  int nv;
  const double* v;   /* 3 per vertex, body frame                           */
  const double* p;   /* pressure per vertex (soft)                          */
  int ne;
  const int* e;      /* 4 per tet (soft) / 3 per triangle (rigid)           */
} or_geom;

typedef struct {
  int representation;  /* 0 triangle fan, 1 polygon                         */
  int apply_forces;
  int n_threads;       /* OpenMP threads over pairs (<=0: all)              */
} or_options;

typedef struct {
  int query;              /* 0 none, 1 soft-rigid, 2 soft-halfspace, 3 soft-soft */
  int m, n;               /* geom ids after ordering                          */
  double wrench[6];       /* force on M, torque about x_M, world              */
  int n_polygons, n_faces, n_near_degenerate;
  double area, total_fn0;
} or_pair_result;

typedef struct {
  int32_t pair, elem_a, elem_b, n_vert, flags;
} or_candidate;

typedef struct {
  int geom;
  double resolution;
  int sampling_resolution;
  int window;             /* 0 none, 1 gauss, 2 tukey, 3 square              */
  double sigma;
  double size[3];         /* geom half sizes                                  */
  int cx, cy;             /* filled by or_collide                             */
  float* taxels;          /* cx*cy output, caller-owned (may be NULL)         */
  double* taxels64;       /* cx*cy output of the same sampling evaluated in
                             FP64 (gradient checks), may be NULL             */
} or_sensor;

typedef struct or_ctx or_ctx;

or_ctx* or_create(const or_geom* geoms, int n_geom);
void or_destroy(or_ctx* c);

/* One step: every pair, then every sensor.  cand may be NULL. */
int or_collide(or_ctx* c, const double* xpos, const double* xmat, const double* vel, int n_pair,
               const int* g1, const int* g2, const or_options* opt, or_pair_result* out,
               or_sensor* sensors, int n_sensor, or_candidate* cand, int64_t cand_cap,
               int64_t* n_cand);

/* The contact surface of one pair (world frame, canonical order).  Call with
 * NULL arrays for sizes.                                                    */
int or_surface(or_ctx* c, const double* xpos, const double* xmat, int g1, int g2, int* n_poly,
               int* n_vert, int* poly_offset, double* vert, double* vert_pressure, double* normal,
               int* elem_a, int* elem_b);

/* Flat-sensor grid size as FlatTactileSensor::load computes it. */
void or_sensor_grid(double xs, double ys, double resolution, int* cx, int* cy);

#ifdef __cplusplus
}
#endif
#endif
