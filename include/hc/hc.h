/*
 * hc.h — C ABI of the GB300 hydroelastic contact engine.
 *
 * This is the drop-in boundary for the contact-surface path of the MuJoCo
 * contact-surfaces plugin (ubi-agni/mujoco_contact_surfaces).  Every entry
 * point takes plain pointers and sizes; no C++ or torch types cross it.
 * Each entry point names the reference interface it replaces, as
 * `file:line` within the reference project:
 *
 *   P  = mujoco_contact_surfaces/src/mujoco_contact_surfaces_plugin.cpp
 *   PH = mujoco_contact_surfaces/include/mujoco_contact_surfaces/mujoco_contact_surfaces_plugin.h
 *   CT = mujoco_contact_surfaces/include/mujoco_contact_surfaces/common_types.h
 *   UH = mujoco_contact_surfaces/include/mujoco_contact_surfaces/plugin_utils.h
 *   FS = mujoco_contact_surface_sensors/src/flat_tactile_sensor.cpp
 *
 * Conventions
 *   - Geoms are addressed by the caller's geom id (MuJoCo geom index).
 *     Geom types use MuJoCo's mjtGeom numbering.
 *   - Poses are MuJoCo's geom_xpos (3 doubles) and geom_xmat (9 doubles,
 *     row-major) per geom id; velocities are mj_objectVelocity(...,
 *     flg_local=0) 6-vectors [omega; v] at the geom origin, world aligned.
 *   - The contact pair (g1, g2) is re-ordered so that M is the geom that was
 *     registered first (the reference orders by Drake geometry id, which it
 *     assigns in parse order).  Wrenches are reported on M:
 *     force on M and torque on M about M's origin (geom_xpos of M).  The
 *     wrench on N is the negative force and
 *     -(torque + (x_M - x_N) x force) about N's origin.
 *   - Every function returns hc_status; HC_OK is 0.  hc_last_error() gives
 *     a message for the calling thread's last failure.
 *   - A context owns one CUDA stream and all device buffers.  Calls on one
 *     context are not thread safe; different contexts are independent.
 *   - Allocation happens only in create / add_geom / set_pairs /
 *     add_flat_sensor and when a capacity grows; hc_step allocates nothing.
 */
#ifndef HC_HC_H_
#define HC_HC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HC_API __attribute__((visibility("default")))

typedef enum {
  HC_OK = 0,
  HC_ERR_INVALID_ARG = 1,  /* bad id, size, NaN/Inf pose, bad mesh          */
  HC_ERR_UNSUPPORTED = 2,  /* pair or geom type without a contact surface:
                              the caller falls back to its default narrow
                              phase exactly as P:270-271 does              */
  HC_ERR_OVERFLOW = 3,     /* a fixed-capacity device buffer overflowed;
                              results are incomplete, grow and re-run      */
  HC_ERR_TIMEOUT = 4,      /* a bounded device-side wait gave up            */
  HC_ERR_CUDA = 5,         /* CUDA runtime error (message in hc_last_error) */
  HC_ERR_DEGENERATE = 6,   /* degenerate input geometry (zero-volume mesh)  */
  HC_ERR_NOT_READY = 7,    /* step not run yet / no such output             */
  HC_ERR_NO_DEVICE = 8     /* no CUDA device visible                        */
} hc_status;

/* MuJoCo mjtGeom numbering. */
enum {
  HC_GEOM_PLANE = 0,
  HC_GEOM_HFIELD = 1,
  HC_GEOM_SPHERE = 2,
  HC_GEOM_CAPSULE = 3,
  HC_GEOM_ELLIPSOID = 4,
  HC_GEOM_CYLINDER = 5,
  HC_GEOM_BOX = 6,
  HC_GEOM_MESH = 7
};

/* cs::HydroelasticContactRepresentation (PH:251, P:574-591). */
enum { HC_REPR_TRIANGLE = 0, HC_REPR_POLYGON = 1 };

/* Contact kinds (PH:134-138). */
enum { HC_RIGID = 0, HC_SOFT = 1 };

/* Query kinds chosen by the pair dispatch. */
enum {
  HC_QUERY_NONE = 0,        /* default narrow phase            */
  HC_QUERY_SOFT_RIGID = 1,  /* ComputeContactSurfaceFromSoftVolumeRigidSurface */
  HC_QUERY_SOFT_HALFSPACE = 2, /* ...SoftVolumeRigidHalfSpace              */
  HC_QUERY_SOFT_SOFT = 3    /* ComputeContactSurfaceFromCompliantVolumes    */
};

/* Flat sensor windows (FS:140-168). */
enum { HC_WINDOW_NONE = 0, HC_WINDOW_GAUSS = 1, HC_WINDOW_TUKEY = 2, HC_WINDOW_SQUARE = 3 };

/* Debug flags for hc_set_debug. */
enum {
  HC_DEBUG_CANDIDATES = 1  /* record every non-empty element pair (for the
                              canonical-sort parity check)                 */
};

typedef struct hc_context hc_context;

typedef struct {
  int device;               /* CUDA device ordinal                          */
  int representation;       /* HC_REPR_TRIANGLE (default) or HC_REPR_POLYGON */
  int apply_forces;         /* cs::ApplyContactSurfaceForces (default 1)     */
  int use_graph;            /* capture hc_step in a CUDA graph (default 1)   */
  int64_t item_capacity;    /* cluster-pair work items (0 = automatic)       */
  int64_t face_capacity;    /* initial capacity of the contact polygons a
                               step keeps when sensors are attached or in
                               adjoint mode (0 = automatic; on overflow the
                               next synchronising call grows it and re-runs
                               the step)                                    */
} hc_config;

/* Fill a config with defaults. */
HC_API void hc_config_default(hc_config* cfg);

/* Message of the calling thread's last failing call ("" when none). */
HC_API const char* hc_last_error(void);

/* Library version string. */
HC_API const char* hc_version(void);

/* ---- context ------------------------------------------------------------
 * Replaces the plugin object's construction and load(m, d).    */
HC_API hc_status hc_context_create(const hc_config* cfg, hc_context** out);
/* Replaces the plugin destructor. */
HC_API hc_status hc_context_destroy(hc_context* ctx);
/* Replaces reset(): forgets the last step's outputs. */
HC_API hc_status hc_reset(hc_context* ctx);

/* ---- geoms --------------------------------------------------------------
 * Replaces the per-geom branch of parseMujocoCustomFields:
 * `cs5` is the cs::<geom> numeric [E, dissipation, resolutionHint,
 * mu_static, mu_dynamic].  E > 0 makes a soft geom (tet mesh +
 * linear pressure field E*extent), E <= 0 a rigid one (triangle mesh; a
 * plane is a rigid half-space).  `size` is MuJoCo's geom_size (half sizes).
 * `mesh_vert`/`mesh_face` are used for HC_GEOM_MESH only (nvert x 3
 * doubles, nface x 3 ints, outward counter-clockwise faces).
 * `out_kind` receives HC_SOFT / HC_RIGID, or -1 when the geom type has no
 * contact surface (capsule, hfield, soft plane: P:634-647).  Registration
 * order defines the M/N order of every pair.                    */
HC_API hc_status hc_add_geom(hc_context* ctx, int geom_id, int type, const double size[3],
                             const double cs5[5], const double* mesh_vert, int nvert,
                             const int* mesh_face, int nface, int* out_kind);

/* Replaces onGeomChanged: regenerate the geom's mesh and
 * pressure field for a new size and rebuild or refit its LBVH.           */
HC_API hc_status hc_update_geom_size(hc_context* ctx, int geom_id, const double size[3]);

typedef struct {
  int kind;          /* HC_SOFT / HC_RIGID / -1                           */
  int type;          /* mjtGeom                                            */
  int order;         /* registration index (the reference's Drake id order) */
  int n_elements;    /* tets (soft) or triangles (rigid); 0 for a plane      */
  int n_vertices;
  double E, dissipation, resolution_hint, mu_static, mu_dynamic;
} hc_geom_info;
HC_API hc_status hc_get_geom_info(hc_context* ctx, int geom_id, hc_geom_info* out);

/* The geom's elements in the order of its LBVH leaves (built on the device:
 * the Morton curve of their centroids in the geom's bounding box): order[k]
 * is the index, in the geom's mesh, of the k-th element (n_elements ints).
 * A diagnostic of the LBVH build; builds the element pools if needed.  No
 * counterpart in the reference (its BVHs live inside Drake).               */
HC_API hc_status hc_get_element_order(hc_context* ctx, int geom_id, int* order);

/* Copy the geom's mesh as stored (vertices rounded to float, body frame).
 * Soft: elems = 4 ints per tet, pressure = one value per vertex.
 * Rigid: elems = 3 ints per triangle, pressure untouched.  Pass NULL
 * pointers to query sizes only.                                           */
HC_API hc_status hc_get_geom_mesh(hc_context* ctx, int geom_id, double* vert, double* pressure,
                                  int* elems);

/* Stateless mesh generation (host only, no device needed): the same
 * generator hc_add_geom uses.  Two calls: first with NULL outputs to get
 * the sizes.                                                             */
HC_API hc_status hc_generate_mesh(int type, const double size[3], const double cs5[5],
                                  const double* mesh_vert, int nvert, const int* mesh_face,
                                  int nface, int* out_kind, int* out_nvert, int* out_nelem,
                                  double* vert, double* pressure, int* elems);

/* ---- per-step inputs ----------------------------------------------------
 * Poses and velocities for geom ids [0, n_geom).  Replaces getGeomPose
 * and getGeomVelocity.  Host pointers; copied to
 * the device on the context stream.  `vel` may be NULL (zero velocity).  */
HC_API hc_status hc_set_poses(hc_context* ctx, int n_geom, const double* xpos,
                              const double* xmat, const double* vel);
/* Same with device pointers (already in HBM, same layout).               */
HC_API hc_status hc_set_poses_device(hc_context* ctx, int n_geom, const double* d_xpos,
                                     const double* d_xmat, const double* d_vel);

/* ---- pair dispatch ------------------------------------------------------
 * Replaces the classification part of collision_cb: decides
 * per pair which contact-surface query runs (or HC_ERR_UNSUPPORTED when
 * either geom lacks cs:: properties or both are rigid, the P:270-271
 * fallback).  per_pair_status and per_pair_query may be NULL.            */
HC_API hc_status hc_set_pairs(hc_context* ctx, int n_pair, const int* g1, const int* g2,
                              int* per_pair_status, int* per_pair_query);

/* Runs one step over the current pairs and poses: broadphase, clipping,
 * quadrature, the force law and the per-pair
 * wrench, plus taxel binning for every flat sensor (FS:262-402).
 * Asynchronous on the context stream.                                    */
HC_API hc_status hc_step(hc_context* ctx);

/* Convenience: hc_set_pairs + hc_step. */
HC_API hc_status hc_collide_pairs(hc_context* ctx, int n_pair, const int* g1, const int* g2,
                                  int* per_pair_status);

/* Per-pair wrench on M about M's origin, world frame: n_pair x
 * [fx fy fz tx ty tz] doubles.  Synchronises the context stream.        */
HC_API hc_status hc_get_wrenches(hc_context* ctx, double* wrench);
/* Device pointer to the per-pair records of the last step (valid until the
 * next hc_set_pairs): n_pair records of HC_PAIR_RECORD_DOUBLES doubles each,
 * the wrench (as hc_get_wrenches) in the first 6, then area and total fn0
 * (hc_pair_stats), then the four int32 counters of hc_pair_stats.        */
#define HC_PAIR_RECORD_DOUBLES 10
HC_API hc_status hc_get_wrenches_device(hc_context* ctx, const double** d_wrench);
/* The query kind and M/N order chosen for each pair: m_geom/n_geom ids. */
HC_API hc_status hc_get_pair_order(hc_context* ctx, int* query, int* m_geom, int* n_geom);

typedef struct {
  int32_t n_polygons;       /* non-empty clipped element pairs            */
  int32_t n_faces;          /* quadrature points kept (area > 1e-14 and
                               gradient checks)           */
  int32_t n_near_degenerate;/* polygons with a vertex within 1e-12 of a
                               clip plane                                 */
  int32_t n_items;          /* cluster-pair work items visited            */
  double area;              /* total contact area (faces kept)            */
  double total_fn0;         /* sum of A*p0                    */
} hc_pair_stats;
HC_API hc_status hc_get_pair_stats(hc_context* ctx, hc_pair_stats* out);

/* Contact surface of one pair, copied to host memory, world frame, in a
 * canonical order (soft element, other element).  Polygons are stored as
 * vertex lists: poly_offset[n_poly+1] into vert (3 doubles each) and
 * vert_pressure; normal (3 per polygon, out of N into M); elem_a/elem_b
 * (original element indices: soft tet, and rigid triangle / soft tet of
 * the second body / -1 for a half-space).  Call with NULL arrays to get
 * the counts.  Replaces access to ContactSurface (CT:59-66).             */
typedef struct {
  int n_poly;
  int n_vert;
  int* poly_offset;
  double* vert;
  double* vert_pressure;
  double* normal;
  int* elem_a;
  int* elem_b;
} hc_surface_view;
HC_API hc_status hc_get_surface(hc_context* ctx, int pair, hc_surface_view* view);

/* Debug record of every non-empty element pair (HC_DEBUG_CANDIDATES). */
typedef struct {
  int32_t pair;
  int32_t elem_a;
  int32_t elem_b;
  int32_t n_vert;   /* vertices of the clipped polygon                  */
  int32_t flags;    /* bit 0: near-degenerate                           */
} hc_candidate;
HC_API hc_status hc_set_debug(hc_context* ctx, int flags);
HC_API hc_status hc_get_candidates(hc_context* ctx, hc_candidate* out, int64_t capacity,
                                   int64_t* count);

/* ---- flat tactile sensor ------------------------------------------------
 * Replaces FlatTactileSensor::load (FS:127-214) and bvh_update
 * (FS:262-402): a cx x cy taxel grid on the top face of a box geom at
 * `resolution`, sampling_resolution^2 rays per cell, optional window.
 * cx = floor(2*xs/resolution + 0.1) (FS:196-197).                       */
HC_API hc_status hc_add_flat_sensor(hc_context* ctx, int geom_id, double resolution,
                                    int sampling_resolution, int window, double sigma,
                                    int* out_sensor, int* out_cx, int* out_cy);
/* The sensor's taxel map of the last step (cx*cy floats, index x + cy*y as
 * FS:396-397).  Synchronises the context stream.                        */
HC_API hc_status hc_get_taxels(hc_context* ctx, int sensor, float* out);
/* All sensors' taxel maps in one host copy (sensor-major, cx*cy floats
 * each, in hc_add_flat_sensor order).  n_floats: capacity of `out`. */
HC_API hc_status hc_get_taxels_all(hc_context* ctx, float* out, int64_t n_floats);
/* Device pointer to all sensors' taxel maps (sensor-major). */
HC_API hc_status hc_get_taxels_device(hc_context* ctx, const float** d_taxels,
                                      int64_t* n_floats);

/* ---- taxel-point sensor -------------------------------------------------
 * Replaces TaxelSensor::load / internal_update (mujoco_contact_surface_
 * sensors/src/taxel_sensor.cpp:46-156, 158-478): n_taxels points fixed in the
 * geom's frame (n x 3 doubles), each valued from samples of the contact
 * surfaces that involve the geom (in collision order, each polygon fanned
 * about its area-weighted centroid): `method` HC_TAXEL_CLOSEST, _WEIGHTED,
 * _MEAN, _SQUARED; `sample_method` HC_SAMPLE_DEFAULT (barycentric grid at
 * `sample_resolution`) or HC_SAMPLE_AREA_IMPORTANCE (`sample_resolution` of
 * each surface's area per sample, the reference's default-seeded
 * minstd_rand0 stream); `include_margin` in metres.  The reference's
 * quirks are kept: weighted and mean fall through into squared; closest
 * reports 0 inside the margin unless `visualize` is set (its else binds to
 * the visualisation test); taxels with no sample inside the margin keep
 * their value.  Soft-rigid and half-space contacts; 1 to 2^20 taxels; any
 * number of contact polygons.  A triangle side of more than 4096 grid
 * steps, or more than 2^20 samples in one fan triangle, makes the next read
 * return HC_ERR_OVERFLOW (the resolution is too fine for the contact).      */
enum { HC_TAXEL_CLOSEST = 0, HC_TAXEL_WEIGHTED = 1, HC_TAXEL_MEAN = 2, HC_TAXEL_SQUARED = 3 };
enum { HC_SAMPLE_DEFAULT = 0, HC_SAMPLE_AREA_IMPORTANCE = 1 };
HC_API hc_status hc_add_taxel_sensor(hc_context* ctx, int geom_id, int n_taxels, const double* taxels, int method,
                                     double include_margin, double sample_resolution, int sample_method,
                                     int visualize, int* out_sensor);
/* Whether the next steps update the sensor (the update-rate gate of
 * TactileSensorBase::update, tactile_sensor_base.cpp:89-120): a disabled
 * sensor keeps its values.                                                */
HC_API hc_status hc_set_taxel_sensor_enabled(hc_context* ctx, int sensor, int on);
/* The sensor's values after the last step (n_taxels floats, taxel order).
 * Synchronises the context stream.                                        */
HC_API hc_status hc_get_taxel_sensor_values(hc_context* ctx, int sensor, float* out);
/* Every taxel sensor's values after the last step, sensor after sensor in
 * the order they were added, in one copy (`capacity` floats at `out`; it
 * must hold the total taxel count).  Synchronises the context stream.      */
HC_API hc_status hc_get_all_taxel_sensor_values(hc_context* ctx, float* out, size_t capacity);

/* ---- curved sensor ------------------------------------------------------
 * Replaces CurvedSensor::load / internal_update (mujoco_contact_surface_
 * sensors/src/curved_sensor.cpp:111-365, 367-466).
 *
 * hc_sample_surface: blue-noise points on a triangle mesh (n_vert x 3
 * doubles, n_face x 3 indices, counter-clockwise outward), with the unit
 * normal of each point's triangle — the load-time surface sampling, which
 * the reference does with vcglib's Poisson-disk sampler (:260-268; not
 * reproduced: the points differ, their spacing is alike).  At most
 * `n_samples` points (the reference asks for (int)sample_resolution *
 * area); deterministic for a `seed`.  *out_n receives the count; the
 * outputs (capacity x 3 doubles each) must hold it.  Needs no context.      */
HC_API hc_status hc_sample_surface(int n_vert, const double* vert, int n_face, const int* face, int n_samples,
                                   uint64_t seed, int capacity, double* out_points, double* out_normals,
                                   int* out_n);
/* A curved sensor on geom_id: n_taxels points fixed in the geom's frame
 * (n x 3 doubles) with optional normals (NULL, or n x 3; normalised; a zero
 * normal means none), and n_points surface points with unit normals (geom
 * frame; e.g. from hc_sample_surface).  As the reference: surface point j
 * serves taxel i when their squared distance is below include_margin^2 and
 * (the taxel has no normal or the normals are less than 45 degrees apart),
 * with weight max(0, include_margin - distance)^2; each step, the ray of
 * point j from p_j + 1e-8 n_j along -n_j takes the pressure of the nearest
 * contact surface it meets at 0 < t < include_margin, and taxel i's value is
 * the sum of weight x pressure over its points (0 without contact).
 * Soft-rigid and half-space contacts.                                       */
HC_API hc_status hc_add_curved_sensor(hc_context* ctx, int geom_id, int n_taxels, const double* taxels,
                                      const double* taxel_normals, double include_margin, int n_points,
                                      const double* points, const double* point_normals, int* out_sensor);
/* Whether the next steps update the sensor (the update-rate gate); a
 * disabled sensor keeps its values.                                          */
HC_API hc_status hc_set_curved_sensor_enabled(hc_context* ctx, int sensor, int on);
/* The sensor's values after the last step (n_taxels floats, taxel order).
 * Synchronises the context stream.                                          */
HC_API hc_status hc_get_curved_sensor_values(hc_context* ctx, int sensor, float* out);

/* ---- adjoint -------------------------------------------------------------
 * Gradient of L with respect to both geoms' 6-DoF poses (twist
 * [dtheta; dx], world frame, applied as X <- exp(dtheta) X, x <- x + dx)
 * and the soft moduli, given dL/dwrench (n_pair x 6 doubles, may be NULL)
 * and dL/dtaxel (all sensors' maps, may be NULL).  Reads the polygons the
 * step kept (adjoint mode, or sensors attached) and otherwise recomputes
 * them.  Outputs: dL_dpose n_pair x 2 x 6 (M then N), dL_dE n_pair x 2 (M
 * then N; 0 for a rigid geom).                                            */
HC_API hc_status hc_adjoint(hc_context* ctx, const double* dL_dwrench, const float* dL_dtaxel,
                            double* dL_dpose, double* dL_dE);
/* Keep each step's ray-sample hits for a following taxel adjoint (without
 * this, hc_adjoint with dL_dtaxel re-runs the step once to recover them).  */
HC_API hc_status hc_set_adjoint_mode(hc_context* ctx, int on);
/* hc_adjoint on device buffers, asynchronous on the context stream.  The
 * result is n_pair x 14 doubles: [dL/dtwist M (6), N (6), dL/dE_M, dL/dE_N],
 * valid until the next adjoint.  A taxel adjoint needs adjoint mode on
 * before the step, and where polygons are recomputed (none kept, or
 * soft-soft pairs) it takes the step's ray samples: one taxel adjoint per
 * step (hc_adjoint re-runs the step for a second one).                   */
HC_API hc_status hc_adjoint_device(hc_context* ctx, const double* d_dL_dwrench, const float* d_dL_dtaxel,
                                   const double** d_grad);
/* Kernels the last adjoint launched. */
HC_API hc_status hc_get_adjoint_launch_count(hc_context* ctx, int* n);
/* Diagnostic (needs HC_DEBUG_CANDIDATES): polygon vertices the last adjoint
 * left out of its contraction because their three constraint rows were
 * linearly dependent (normalised determinant below 1e-4; soft-soft vertices
 * on the line where both surfaces meet are carried by their two face rows
 * instead and are not counted), and the smallest normalised determinant it
 * met (+infinity when none).  Either output may be NULL.  No counterpart in
 * the reference.                                                          */
HC_API hc_status hc_get_adjoint_skipped(hc_context* ctx, int* n, float* min_det);
/* Forward step and adjoint as one graph launch with one wait: the
 * training-style step of a caller that knows dL/dwrench and dL/dtaxel before
 * the step (a fixed linear loss, identification against target maps).  The
 * reference has no gradient; this replaces the sequence hc_set_poses,
 * hc_step, hc_get_wrenches, hc_get_taxels_all, hc_adjoint with identical
 * results.  Inputs as hc_set_poses and hc_adjoint (host arrays; page-locked
 * memory makes the copies direct); outputs (each may be NULL): wrench
 * n_pair x 6, taxels (all flat sensors' maps), dL_dpose n_pair x 2 x 6,
 * dL_dE n_pair x 2.  Turns adjoint mode on if it is off.  A step whose
 * work items or kept polygons overflow grows the capacity and runs again
 * before the call returns.                                                 */
HC_API hc_status hc_step_adjoint(hc_context* ctx, int n_geom, const double* xpos, const double* xmat,
                                 const double* vel, const double* dL_dwrench, const float* dL_dtaxel,
                                 double* wrench, float* taxels, double* dL_dpose, double* dL_dE);
/* The same on device buffers, asynchronous on the context stream: poses as
 * last set (hc_set_poses / hc_set_poses_device), upstream gradients as
 * hc_adjoint_device (either may be NULL), *d_grad as hc_adjoint_device.
 * Needs adjoint mode on.  The graph is kept while the upstream pointers stay
 * the same.  An overflowing step is found by the next synchronising call
 * (hc_get_wrenches, ...), which grows the capacity and re-runs the forward
 * step alone: call this again for its gradient.                             */
HC_API hc_status hc_step_adjoint_device(hc_context* ctx, const double* d_dL_dwrench, const float* d_dL_dtaxel,
                                        const double** d_grad);

/* ---- measurement --------------------------------------------------------*/
typedef struct {
  float ms_setup, ms_broadphase, ms_narrowphase, ms_reduce, ms_taxels, ms_total;
  float ms_kept_polygons;   /* forces and rays of the kept polygons (part of
                               the narrow-phase stage, not of ms_narrowphase) */
  int64_t n_items;
  int64_t n_polygons;
  float ms_adjoint;         /* the adjoint of a fused step (hc_step_adjoint*),
                               else 0                                        */
} hc_timings;
/* Enable CUDA-event timing of the stages of hc_step (the event records
 * become part of the captured graph).                                    */
HC_API hc_status hc_enable_timing(hc_context* ctx, int enable);
HC_API hc_status hc_get_timings(hc_context* ctx, hc_timings* out);
/* The context's CUDA stream (cudaStream_t), for callers that order their
 * own work against hc_step.                                             */
HC_API hc_status hc_get_stream(hc_context* ctx, void** stream);
/* Number of kernels one hc_step launches for the current pairs/sensors. */
HC_API hc_status hc_get_launch_count(hc_context* ctx, int* n);
/* Autotune the launch shape on the current pairs and poses: the grid of the
 * persistent kernels (CTAs per SM, 2-8) and the soft-rigid work-queue chunk
 * (consecutive work items a warp takes, 1-16), timed over three steps each;
 * the fastest is kept for later steps.  Outputs may be NULL.              */
HC_API hc_status hc_autotune(hc_context* ctx, int* chosen_ctas_per_sm, int* chosen_chunk);
/* Set the launch shape directly (CTAs per SM 1-8, work-queue chunk 1-16),
 * e.g. to a shape an earlier hc_autotune chose.                           */
HC_API hc_status hc_set_launch_shape(hc_context* ctx, int ctas_per_sm, int chunk);

/* ---- step without device allocation -------------------------------------
 * No counterpart in the reference: the plugin has no such call.
 *
 * hc_step keeps its working buffers (per-pair frames and sums, broadphase
 * counts and offsets, the cluster-pair work items and their partial sums,
 * the ray-sample keys of the sensors) in device memory that the context
 * allocates, and grows the work-item buffers when a step needs more.  Some
 * callers cannot have device memory allocated while they run: a real-time
 * control loop that fixes its memory at start-up and must not stall in the
 * allocator, a process whose device memory is owned by another framework's
 * pool allocator, or code running where the CUDA allocator may not be
 * called.  hc_step_noalloc runs the same forward step with all of that
 * working memory inside one static device array of HC_NOALLOC_SCRATCH_BYTES
 * (32 MiB) compiled into the library, and calls no allocating routine.
 *
 *   n_geom, d_xpos, d_xmat, d_vel: device poses and velocities for geom ids
 *       [0, n_geom), in the layout of hc_set_poses (d_vel may be NULL);
 *   d_wrench: device output, n_pair x 6 doubles, as hc_get_wrenches;
 *   d_taxels: device output, all flat sensors' taxel maps, as
 *       hc_get_taxels_device (NULL allowed when the context has no sensor);
 *       a context with taxel-point (hc_add_taxel_sensor) or curved
 *       (hc_add_curved_sensor) sensors is refused with HC_ERR_UNSUPPORTED:
 *       those sensors read kept polygons, which this step does not keep;
 *   stream: the cudaStream_t to run on, or NULL for the context's stream.
 *
 * The context must be ready: hc_set_pairs called after the last change of
 * geoms or sensors (that call allocates; this one then does not).  The step
 * reads the context's geometry but writes nothing in it, so hc_get_*,
 * hc_get_surface and hc_adjoint keep referring to the last hc_step.  The
 * call is synchronous: it waits for the stream to read back the step's
 * status word.  A step whose working set does not fit in the array fails
 * with HC_ERR_OVERFLOW and a message giving the pair, sample or work-item
 * count that did not fit; its outputs are then incomplete.
 * The first call on each device looks up the array's device address with
 * that device current (cudaGetSymbolAddress, once per device); make that
 * first call before any stream capture.  All calls, from every context and
 * thread, share the one array, and each call leaves its contents behind: the
 * call clears what must start cleared, but two calls whose work overlaps on
 * the GPU race on the array and give wrong results, so serialise them (one
 * stream, or events between streams).                                       */
#define HC_NOALLOC_SCRATCH_BYTES (32u << 20)
HC_API hc_status hc_step_noalloc(hc_context* ctx, int n_geom, const double* d_xpos,
                                 const double* d_xmat, const double* d_vel, double* d_wrench,
                                 float* d_taxels, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HC_HC_H_ */
