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
  double centroid[3];     /* area-weighted centroid of the surface, world (the
                             point a reference-free torque error is taken at) */
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

/* Taxel-point sensor update (taxel.c; TaxelSensor::internal_update,
 * mujoco_contact_surface_sensors/src/taxel_sensor.cpp:158-478). */
typedef struct {
  int n_taxels;
  const double* taxels;     /* world positions, 3 per taxel                  */
  int method;               /* 0 closest, 1 weighted, 2 mean, 3 squared      */
  double include_margin;
  double sample_resolution;
  int sample_method;        /* 0 default grid, 1 area importance             */
  int visualize;            /* changes the closest method's values (:311-327) */
} or_taxel_cfg;
/* Surfaces in collision order: surf_poly_off[n_surf+1] into polygons,
 * poly_vert_off[n_poly+1] into vert (3 doubles, world) / vert_p; normal: 3
 * per polygon.  values: n_taxels, in/out (kept where nothing is sampled
 * within the margin).                                                      */
void or_taxel_sensor(const or_taxel_cfg* cfg, int n_surf, const int* surf_poly_off, const int* poly_vert_off,
                     const double* vert, const double* vert_p, const double* normal, double* values);
/* Known-answer hooks of the sensor's random stream. */
uint64_t or_minstd_nth(int n);
double or_uniform_nth(int n);

/* Curved sensor (curved.c; CurvedSensor, mujoco_contact_surface_sensors/
 * src/curved_sensor.cpp).  Selection at load: taxels and surface points in
 * the geom frame (3 doubles each), taxel_normals NULL or unit vectors (zero =
 * none), point_normals unit; per taxel i its points pt[off[i]..off[i+1]) in
 * point order with weights w (off: n_taxels+1; pt, w: n_taxels * n_points
 * at most).  Returns the number of (taxel, point) entries.                 */
int or_curved_select(int n_taxels, const double* taxels, const double* taxel_normals, double margin, int n_points,
                     const double* points, const double* point_normals, int* off, int* pt, double* w);
/* Update: points and normals in the world frame; surfaces as for
 * or_taxel_sensor; values: n_taxels (every value is written).               */
void or_curved_update(int n_taxels, const int* off, const int* pt, const double* w, int n_points,
                      const double* points, const double* normals, double margin, int n_surf,
                      const int* surf_poly_off, const int* poly_vert_off, const double* vert, const double* vert_p,
                      const double* normal, double* values);

#ifdef __cplusplus
}
#endif
#endif
