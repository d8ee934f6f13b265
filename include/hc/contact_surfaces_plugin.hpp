// contact_surfaces_plugin.hpp — header-only C++ host class with the method
// names and semantics of the reference's MuJoCo plugin, backed by the C ABI
// of hc.h.
//
// Reference interface mirrored (paths within ubi-agni/mujoco_contact_surfaces):
//   MujocoContactSurfacesPlugin        mujoco_contact_surfaces/include/mujoco_contact_surfaces/
//                                      mujoco_contact_surfaces_plugin.h:215-266
//     load / reset                     mujoco_contact_surfaces/src/mujoco_contact_surfaces_plugin.cpp:208-253
//     collision_cb                     ...plugin.cpp:255-318
//     passiveCallback (force law)      ...plugin.cpp:411-523
//     parseMujocoCustomFields          ...plugin.cpp:571-813
//     onGeomChanged                    ...plugin.cpp:828-975
//   SurfacePlugin::update              mujoco_contact_surfaces/include/mujoco_contact_surfaces/plugin_utils.h:94
//   TactileSensorBase::update          mujoco_contact_surface_sensors/src/tactile_sensor_base.cpp:89-120
//   FlatTactileSensor::load            mujoco_contact_surface_sensors/src/flat_tactile_sensor.cpp:127-214
//   TaxelSensor::load                  mujoco_contact_surface_sensors/src/taxel_sensor.cpp:46-156
//   CurvedSensor::load                 mujoco_contact_surface_sensors/src/curved_sensor.cpp:111-365
//
// The class is a template over an `Api` traits type that names the MuJoCo
// types and the four MuJoCo calls the plugin needs, so it compiles against
// the real mujoco.h (see the integration notes for the ten-line traits type)
// and against the small model/data fakes the tests use.  Fields read from the
// model and data follow MuJoCo's names: ngeom, geom_type, geom_size,
// geom_bodyid, geom_dataid, nnumeric, numeric_adr, numeric_size,
// numeric_data, ntext, text_adr, text_size, text_data, mesh_vertadr,
// mesh_vertnum, mesh_vert, mesh_faceadr, mesh_facenum, mesh_face;
// geom_xpos, geom_xmat, qfrc_passive, time.
//
// Differences from the reference, by design:
//   - collision_cb only records the pair; the whole batch of pairs is
//     computed on the GPU in passiveCallback (one hc_step), where the
//     reference computes each surface inside collision_cb.  Poses are the
//     same in both places (MuJoCo does not move geoms between the two).
//   - The wrench of each pair is applied with two mj_applyFT calls (on M and,
//     negated, on N, both at M's origin) instead of two per quadrature point;
//     the generalised force is the same up to rounding.
//   - Rendering (VisualizeSurfaces) and ROS plumbing are not part of it.
//   - `cs::ApplyContactSurfaceForces` and `cs::VisualizeSurfaces` sizes are
//     read by numeric id (the reference indexes numeric_size by the data
//     address, plugin.cpp:596,606).
#ifndef HC_CONTACT_SURFACES_PLUGIN_HPP_
#define HC_CONTACT_SURFACES_PLUGIN_HPP_

#include <algorithm>
#include <array>
#include <cmath>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "hc.h"

namespace hc_plugin {

const std::string kPrefix = "cs::";

// One cs::<geom> numeric custom field (plugin.cpp:613-626).
struct GeomProperties {
  int geom_id = -1;
  std::string geom_name;
  double cs5[5] = {0, 0, 0, 0, 0};  // E, dissipation, resolutionHint, mu_static, mu_dynamic
};

// What parseMujocoCustomFields reads from a model.
struct ParsedFields {
  int representation = HC_REPR_TRIANGLE;  // default kTriangle (mujoco_contact_surfaces_plugin.h:251)
  bool visualize = false;
  bool apply_forces = true;
  std::vector<GeomProperties> geoms;  // in numeric-field order = registration order
};

template <class Api>
ParsedFields parse_custom_fields(const typename Api::Model* m) {
  ParsedFields out;
  const int text_id = Api::name2id(m, Api::kObjText, (kPrefix + "HydroelasticContactRepresentation").c_str());
  if (text_id >= 0 && m->text_adr[text_id] >= 0) {
    const std::string s(&m->text_data[m->text_adr[text_id]], (size_t)m->text_size[text_id]);
    if (s.find("kTriangle") != std::string::npos) out.representation = HC_REPR_TRIANGLE;
    else if (s.find("kPolygon") != std::string::npos) out.representation = HC_REPR_POLYGON;
  }
  auto flag = [&](const char* name, bool& value) {
    const int id = Api::name2id(m, Api::kObjNumeric, (kPrefix + name).c_str());
    if (id >= 0 && m->numeric_size[id] == 1) value = m->numeric_data[m->numeric_adr[id]] != 0;
  };
  flag("VisualizeSurfaces", out.visualize);
  flag("ApplyContactSurfaceForces", out.apply_forces);
  for (int i = 0; i < m->nnumeric; ++i) {
    const char* full = Api::id2name(m, Api::kObjNumeric, i);
    if (!full) continue;
    const std::string name(full);
    if (name.rfind(kPrefix, 0) != 0) continue;
    const std::string geom = name.substr(kPrefix.size());
    const int id = Api::name2id(m, Api::kObjGeom, geom.c_str());
    if (id < 0 || m->numeric_adr[i] < 0 || m->numeric_size[i] != 5) continue;
    GeomProperties g;
    g.geom_id = id;
    g.geom_name = geom;
    for (int k = 0; k < 5; ++k) g.cs5[k] = m->numeric_data[m->numeric_adr[i] + k];
    out.geoms.push_back(g);
  }
  return out;
}

// What a surface plugin sees of one step: the pairs with their M/N order,
// wrenches and statistics, and the engine context for surfaces and taxels.
struct StepView {
  hc_context* ctx = nullptr;
  const std::vector<int>* m_geom = nullptr;
  const std::vector<int>* n_geom = nullptr;
  const std::vector<double>* wrench = nullptr;  // n_pair x 6, on M about M's origin
  int n_pair = 0;
};

// SurfacePlugin-shaped base (plugin_utils.h:53-119): load once, update each
// step with the step's contact surfaces, reset.
template <class Api>
class SurfacePlugin {
 public:
  virtual ~SurfacePlugin() = default;
  virtual bool load(const typename Api::Model* m, typename Api::Data* d, hc_context* ctx) = 0;
  virtual void reset() {}
  // Called before the step that update() will report (d->time is the
  // step's time): a plugin whose device work is gated can switch it here.
  virtual void before_step(const typename Api::Model*, typename Api::Data*) {}
  virtual void update(const typename Api::Model* m, typename Api::Data* d, const StepView& step) = 0;
};

// Flat tactile sensor (flat_tactile_sensor.cpp:127-214) with the update-rate
// gate of TactileSensorBase::update (tactile_sensor_base.cpp:89-120).
struct FlatSensorConfig {
  std::string sensor_name;
  std::string geom_name;
  double update_rate = 100.0;
  double resolution = 0.005;
  int sampling_resolution = 5;
  std::string windowing;  // "", "gauss", "tukey" or "square"
  double sigma = -1.0;
};

template <class Api>
class FlatTactileSensor : public SurfacePlugin<Api> {
 public:
  explicit FlatTactileSensor(FlatSensorConfig cfg) : cfg_(std::move(cfg)) {}

  bool load(const typename Api::Model* m, typename Api::Data*, hc_context* ctx) override {
    ctx_ = ctx;
    geom_id_ = Api::name2id(m, Api::kObjGeom, cfg_.geom_name.c_str());
    if (geom_id_ < 0 || cfg_.update_rate <= 0 || cfg_.resolution <= 0) return false;
    int window = HC_WINDOW_NONE;
    double sigma = cfg_.sigma;
    if (cfg_.windowing == "gauss") {
      window = HC_WINDOW_GAUSS;
      if (sigma == -1.0) sigma = 0.1;
    } else if (cfg_.windowing == "tukey") {
      window = HC_WINDOW_TUKEY;
      if (sigma == -1.0) sigma = 0.3;
    } else if (cfg_.windowing == "square") {
      window = HC_WINDOW_SQUARE;
    }
    if (hc_add_flat_sensor(ctx, geom_id_, cfg_.resolution, cfg_.sampling_resolution, window, sigma, &sensor_,
                           &cx_, &cy_) != HC_OK)
      return false;
    values_.assign((size_t)cx_ * cy_, 0.f);
    period_ = 1.0 / cfg_.update_rate;
    last_update_ = -1e300;
    return true;
  }

  void reset() override { last_update_ = -1e300; }

  void update(const typename Api::Model*, typename Api::Data* d, const StepView&) override {
    const double now = d->time;
    if (now < last_update_) last_update_ = -1e300;  // time jumped back
    if (now - last_update_ >= period_) {
      last_update_ = now;
      if (hc_get_taxels(ctx_, sensor_, values_.data()) == HC_OK) ++n_updates_;
    }
  }

  // The sensor channel (tactile_msgs ChannelFloat32 values, index x + cy*y).
  const std::vector<float>& values() const { return values_; }
  const std::string& name() const { return cfg_.sensor_name; }
  int cx() const { return cx_; }
  int cy() const { return cy_; }
  int n_updates() const { return n_updates_; }

 private:
  FlatSensorConfig cfg_;
  hc_context* ctx_ = nullptr;
  int geom_id_ = -1, sensor_ = -1, cx_ = 0, cy_ = 0, n_updates_ = 0;
  double period_ = 0.0, last_update_ = -1e300;
  std::vector<float> values_;
};

// Maps points (x, y, z triples) by the inverse of the pose (p, unit
// quaternion q = w, x, y, z): t <- R(q)^T (t - p), the mju_negPose /
// mju_quat2Mat product of taxel_sensor.cpp:130-140.  The identity pose leaves
// the points as they are.
inline void apply_inverse_pose(const double p[3], const double q[4], std::vector<double>& t) {
  if (p[0] == 0 && p[1] == 0 && p[2] == 0 && q[0] == 1 && q[1] == 0 && q[2] == 0 && q[3] == 0) return;
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double Rq[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
  double R[9], o[3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) R[3 * r + c] = Rq[3 * c + r];
  for (int r = 0; r < 3; ++r) o[r] = -(R[3 * r] * p[0] + R[3 * r + 1] * p[1] + R[3 * r + 2] * p[2]);
  for (size_t i = 0; i + 2 < t.size(); i += 3) {
    const double a0 = t[i], a1 = t[i + 1], a2 = t[i + 2];
    for (int r = 0; r < 3; ++r) t[i + r] = R[3 * r] * a0 + R[3 * r + 1] * a1 + R[3 * r + 2] * a2 + o[r];
  }
}

// Taxel-point sensor (taxel_sensor.cpp:46-156 load, 158-478 update): taxels
// at points of the geom's frame, valued on the device from samples of the
// contact surfaces; the update-rate gate switches the device update on for
// the steps it reports.  For a mesh geom with a local pose (Api::kGeomLocalPose
// and a non-identity geom_pos / geom_quat) the taxels are moved by the
// inverse of that pose, as the reference does (taxel_sensor.cpp:121-147).
struct TaxelSensorConfig {
  std::string sensor_name;
  std::string geom_name;
  double update_rate = 100.0;
  std::vector<std::array<double, 3>> taxels;
  std::string method = "closest";          // closest, weighted, mean, squared
  double include_margin = 0.0;
  double sample_resolution = 0.0;
  std::string sample_method = "default";   // default, area_importance
  bool visualize = false;
};

template <class Api>
class TaxelSensor : public SurfacePlugin<Api> {
 public:
  explicit TaxelSensor(TaxelSensorConfig cfg) : cfg_(std::move(cfg)) {}

  bool load(const typename Api::Model* m, typename Api::Data*, hc_context* ctx) override {
    ctx_ = ctx;
    const int g = Api::name2id(m, Api::kObjGeom, cfg_.geom_name.c_str());
    if (g < 0 || cfg_.taxels.empty() || cfg_.update_rate <= 0) return false;
    int method = -1, sample = -1;
    if (cfg_.method == "closest") method = HC_TAXEL_CLOSEST;
    else if (cfg_.method == "weighted") method = HC_TAXEL_WEIGHTED;
    else if (cfg_.method == "mean") method = HC_TAXEL_MEAN;
    else if (cfg_.method == "squared") method = HC_TAXEL_SQUARED;
    if (cfg_.sample_method == "default") sample = HC_SAMPLE_DEFAULT;
    else if (cfg_.sample_method == "area_importance") sample = HC_SAMPLE_AREA_IMPORTANCE;
    if (method < 0 || sample < 0) return false;
    std::vector<double> t;
    for (const auto& p : cfg_.taxels) t.insert(t.end(), p.begin(), p.end());
    move_to_geom_frame(m, g, t);
    if (hc_add_taxel_sensor(ctx, g, (int)cfg_.taxels.size(), t.data(), method, cfg_.include_margin,
                            cfg_.sample_resolution, sample, cfg_.visualize ? 1 : 0, &sensor_) != HC_OK)
      return false;
    values_.assign(cfg_.taxels.size(), 0.f);
    period_ = 1.0 / cfg_.update_rate;
    last_update_ = -1e300;
    return true;
  }

  void reset() override { last_update_ = -1e300; }

  void before_step(const typename Api::Model*, typename Api::Data* d) override {
    due_ = d->time < last_update_ || d->time - last_update_ >= period_;
    hc_set_taxel_sensor_enabled(ctx_, sensor_, due_ ? 1 : 0);
  }

  void update(const typename Api::Model*, typename Api::Data* d, const StepView&) override {
    if (!due_) return;
    last_update_ = d->time;
    if (hc_get_taxel_sensor_values(ctx_, sensor_, values_.data()) == HC_OK) ++n_updates_;
  }

  const std::vector<float>& values() const { return values_; }
  const std::string& name() const { return cfg_.sensor_name; }
  int n_updates() const { return n_updates_; }

 private:
  template <class A = Api>
  static auto local_pose(const typename A::Model* m, int g, double p[3], double q[4])
      -> decltype(A::kGeomLocalPose, void()) {
    for (int k = 0; k < 3; ++k) p[k] = m->geom_pos[3 * g + k];
    for (int k = 0; k < 4; ++k) q[k] = m->geom_quat[4 * g + k];
  }
  static void local_pose(...) {}

  void move_to_geom_frame(const typename Api::Model* m, int g, std::vector<double>& t) const {
    double p[3] = {0, 0, 0}, q[4] = {1, 0, 0, 0};
    local_pose(m, g, p, q);
    if (m->geom_type[g] == HC_GEOM_MESH) apply_inverse_pose(p, q, t);
  }

  TaxelSensorConfig cfg_;
  hc_context* ctx_ = nullptr;
  int sensor_ = -1, n_updates_ = 0;
  bool due_ = false;
  double period_ = 0.0, last_update_ = -1e300;
  std::vector<float> values_;
};

// Curved sensor (curved_sensor.cpp:111-365 load, 367-466 update): taxels
// (with optional normals) on a mesh geom, valued from rays cast from points
// sampled on the mesh surface at load (hc_sample_surface replaces vcglib's
// Poisson-disk sampler; the reference asks it for (int)sample_resolution *
// area points, the integer cast binding to sample_resolution, and so does
// this class).  Mesh geoms only, as the reference.  `method` and
// `sample_method` are checked as the reference checks them; the values do
// not depend on them.  The update-rate gate switches the device update on
// for the steps it reports.
struct CurvedSensorConfig {
  std::string sensor_name;
  std::string geom_name;
  double update_rate = 100.0;
  std::vector<std::array<double, 3>> taxels;
  std::vector<std::array<double, 3>> normals;   // empty, or up to one per taxel (missing: none)
  std::string method = "closest";
  double include_margin = 0.0;
  double sample_resolution = 0.0;               // surface points per square metre
  std::string sample_method = "default";
  uint64_t seed = 42;
};

template <class Api>
class CurvedSensor : public SurfacePlugin<Api> {
 public:
  explicit CurvedSensor(CurvedSensorConfig cfg) : cfg_(std::move(cfg)) {}

  bool load(const typename Api::Model* m, typename Api::Data*, hc_context* ctx) override {
    ctx_ = ctx;
    const int g = Api::name2id(m, Api::kObjGeom, cfg_.geom_name.c_str());
    if (g < 0 || cfg_.taxels.empty() || cfg_.update_rate <= 0 || cfg_.normals.size() > cfg_.taxels.size())
      return false;
    if (cfg_.method != "closest" && cfg_.method != "weighted" && cfg_.method != "mean" && cfg_.method != "squared")
      return false;
    if (cfg_.sample_method != "default" && cfg_.sample_method != "area_importance") return false;
    if (m->geom_type[g] != HC_GEOM_MESH || m->geom_dataid[g] < 0) return false;
    const int mesh = m->geom_dataid[g];
    const int va = m->mesh_vertadr[mesh], vn = m->mesh_vertnum[mesh];
    const int fa = m->mesh_faceadr[mesh], fn = m->mesh_facenum[mesh];
    if (vn <= 0 || fn <= 0 || va < 0 || fa < 0) return false;
    std::vector<double> mv(m->mesh_vert + 3 * (size_t)va, m->mesh_vert + 3 * (size_t)(va + vn));
    std::vector<int> mf(m->mesh_face + 3 * (size_t)fa, m->mesh_face + 3 * (size_t)(fa + fn));
    double area = 0;
    for (int f = 0; f < fn; ++f) {
      const double* a = &mv[3 * (size_t)mf[3 * (size_t)f]];
      const double* b = &mv[3 * (size_t)mf[3 * (size_t)f + 1]];
      const double* c = &mv[3 * (size_t)mf[3 * (size_t)f + 2]];
      const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
      const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      area += 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    }
    const int n_samples = (int)((double)(int)cfg_.sample_resolution * area);
    std::vector<double> pts(3 * (size_t)std::max(n_samples, 1)), nrm(pts.size());
    int got = 0;
    if (n_samples > 0 &&
        hc_sample_surface(vn, mv.data(), fn, mf.data(), n_samples, cfg_.seed, n_samples, pts.data(), nrm.data(),
                          &got) != HC_OK)
      return false;
    std::vector<double> t, tn(3 * cfg_.taxels.size(), 0.0);
    for (const auto& p : cfg_.taxels) t.insert(t.end(), p.begin(), p.end());
    for (size_t i = 0; i < cfg_.normals.size(); ++i)
      for (int k = 0; k < 3; ++k) tn[3 * i + k] = cfg_.normals[i][k];
    move_to_geom_frame(m, g, t, tn);
    if (hc_add_curved_sensor(ctx, g, (int)cfg_.taxels.size(), t.data(), tn.data(), cfg_.include_margin, got,
                             pts.data(), nrm.data(), &sensor_) != HC_OK)
      return false;
    n_points_ = got;
    values_.assign(cfg_.taxels.size(), 0.f);
    period_ = 1.0 / cfg_.update_rate;
    last_update_ = -1e300;
    return true;
  }

  void reset() override { last_update_ = -1e300; }

  void before_step(const typename Api::Model*, typename Api::Data* d) override {
    due_ = d->time < last_update_ || d->time - last_update_ >= period_;
    hc_set_curved_sensor_enabled(ctx_, sensor_, due_ ? 1 : 0);
  }

  void update(const typename Api::Model*, typename Api::Data* d, const StepView&) override {
    if (!due_) return;
    last_update_ = d->time;
    if (hc_get_curved_sensor_values(ctx_, sensor_, values_.data()) == HC_OK) ++n_updates_;
  }

  const std::vector<float>& values() const { return values_; }
  const std::string& name() const { return cfg_.sensor_name; }
  int n_updates() const { return n_updates_; }
  int n_surface_points() const { return n_points_; }

 private:
  template <class A = Api>
  static auto local_pose(const typename A::Model* m, int g, double p[3], double q[4])
      -> decltype(A::kGeomLocalPose, void()) {
    for (int k = 0; k < 3; ++k) p[k] = m->geom_pos[3 * g + k];
    for (int k = 0; k < 4; ++k) q[k] = m->geom_quat[4 * g + k];
  }
  static void local_pose(...) {}

  // Taxels by the inverse local pose, normals by its rotation
  // (curved_sensor.cpp:193-226).
  void move_to_geom_frame(const typename Api::Model* m, int g, std::vector<double>& t, std::vector<double>& tn) const {
    double p[3] = {0, 0, 0}, q[4] = {1, 0, 0, 0};
    local_pose(m, g, p, q);
    apply_inverse_pose(p, q, t);
    const double zero[3] = {0, 0, 0};
    if (p[0] != 0 || p[1] != 0 || p[2] != 0 || q[0] != 1 || q[1] != 0 || q[2] != 0 || q[3] != 0)
      apply_inverse_pose(zero, q, tn);
  }

  CurvedSensorConfig cfg_;
  hc_context* ctx_ = nullptr;
  int sensor_ = -1, n_updates_ = 0, n_points_ = 0;
  bool due_ = false;
  double period_ = 0.0, last_update_ = -1e300;
  std::vector<float> values_;
};

template <class Api>
class MujocoContactSurfacesPlugin {
 public:
  using Model = typename Api::Model;
  using Data = typename Api::Data;
  using Contact = typename Api::Contact;
  using Real = typename Api::Real;
  // MuJoCo's default narrow phase for a pair (mjCOLLISIONFUNC entry).
  using CollisionFn = int (*)(const Model*, const Data*, Contact*, int, int, Real);

  explicit MujocoContactSurfacesPlugin(int device = 0) : device_(device) {}
  ~MujocoContactSurfacesPlugin() {
    if (ctx_) hc_context_destroy(ctx_);
  }
  MujocoContactSurfacesPlugin(const MujocoContactSurfacesPlugin&) = delete;
  MujocoContactSurfacesPlugin& operator=(const MujocoContactSurfacesPlugin&) = delete;

  void add_plugin(std::unique_ptr<SurfacePlugin<Api>> p) { plugins_.push_back(std::move(p)); }

  // plugin.cpp:208-245: parse the cs:: fields, register the geoms, load the
  // surface plugins.  Returns false on failure (message in last_error()).
  bool load(const Model* m, Data* d) {
    fields_ = parse_custom_fields<Api>(m);
    hc_config cfg;
    hc_config_default(&cfg);
    cfg.device = device_;
    cfg.representation = fields_.representation;
    cfg.apply_forces = fields_.apply_forces ? 1 : 0;
    if (ctx_) hc_context_destroy(ctx_);
    ctx_ = nullptr;
    if (hc_context_create(&cfg, &ctx_) != HC_OK) return fail();
    kind_.assign((size_t)m->ngeom, -1);
    for (const GeomProperties& g : fields_.geoms) {
      const int id = g.geom_id;
      const double size[3] = {m->geom_size[3 * id], m->geom_size[3 * id + 1], m->geom_size[3 * id + 2]};
      std::vector<double> mv;
      std::vector<int> mf;
      if (m->geom_type[id] == HC_GEOM_MESH && m->geom_dataid[id] >= 0) {
        const int mesh = m->geom_dataid[id];
        const int va = m->mesh_vertadr[mesh], vn = m->mesh_vertnum[mesh];
        const int fa = m->mesh_faceadr[mesh], fn = m->mesh_facenum[mesh];
        mv.assign(m->mesh_vert + 3 * (size_t)va, m->mesh_vert + 3 * (size_t)(va + vn));
        mf.assign(m->mesh_face + 3 * (size_t)fa, m->mesh_face + 3 * (size_t)(fa + fn));
      }
      int kind = -1;
      const hc_status st = hc_add_geom(ctx_, id, m->geom_type[id], size, g.cs5, mv.empty() ? nullptr : mv.data(),
                                       (int)(mv.size() / 3), mf.empty() ? nullptr : mf.data(), (int)(mf.size() / 3),
                                       &kind);
      if (st != HC_OK && st != HC_ERR_UNSUPPORTED) return fail();
      kind_[(size_t)id] = kind;  // -1: no contact surface (plugin.cpp:634-647)
    }
    ready_.clear();
    for (auto& p : plugins_)
      if (p->load(m, d, ctx_)) ready_.push_back(p.get());
    m_ = m;
    d_ = d;
    return true;
  }

  // plugin.cpp:247-253
  void reset() {
    g1_.clear();
    g2_.clear();
    if (ctx_) hc_reset(ctx_);
    for (auto& p : plugins_) p->reset();
  }

  // plugin.cpp:255-318.  Pairs without two cs:: geoms, or with two rigid
  // ones, go to MuJoCo's default function; in force mode a surface pair
  // writes no mjContact, in point-contact mode
  // (cs::ApplyContactSurfaceForces = 0) it also gets MuJoCo's contacts.
  int collision_cb(const Model* m, const Data* d, Contact* con, int g1, int g2, Real margin, CollisionFn fallback) {
    const int k1 = g1 >= 0 && g1 < (int)kind_.size() ? kind_[(size_t)g1] : -1;
    const int k2 = g2 >= 0 && g2 < (int)kind_.size() ? kind_[(size_t)g2] : -1;
    if (k1 < 0 || k2 < 0 || (k1 == HC_RIGID && k2 == HC_RIGID))
      return fallback ? fallback(m, d, con, g1, g2, margin) : 0;
    g1_.push_back(g1);
    g2_.push_back(g2);
    if (fields_.apply_forces) return 0;
    return fallback ? fallback(m, d, con, g1, g2, margin) : 0;
  }

  // plugin.cpp:411-523: the force law over all recorded surface pairs (one
  // device step), the wrenches applied to qfrc_passive, then the surface
  // plugins' updates; the recorded pairs are cleared.
  void passiveCallback(const Model* m, Data* d) {
    const int n = (int)g1_.size();
    step_ok_ = true;
    if (n > 0 || !ready_.empty()) {
      vel_.assign(6 * (size_t)m->ngeom, 0.0);
      for (int i = 0; i < n; ++i)
        for (int g : {g1_[(size_t)i], g2_[(size_t)i]}) Api::object_velocity(m, d, g, &vel_[6 * (size_t)g]);
      if (g1_ != last_g1_ || g2_ != last_g2_) {
        if (hc_set_pairs(ctx_, n, g1_.data(), g2_.data(), nullptr, nullptr) != HC_OK) step_ok_ = false;
        last_g1_ = g1_;
        last_g2_ = g2_;
        m_geom_.assign((size_t)n, 0);
        n_geom_.assign((size_t)n, 0);
        if (step_ok_ && hc_get_pair_order(ctx_, nullptr, m_geom_.data(), n_geom_.data()) != HC_OK) step_ok_ = false;
      }
      if (step_ok_ && hc_set_poses(ctx_, m->ngeom, d->geom_xpos, d->geom_xmat, vel_.data()) != HC_OK) step_ok_ = false;
      for (SurfacePlugin<Api>* p : ready_) p->before_step(m, d);
      if (step_ok_ && hc_step(ctx_) != HC_OK) step_ok_ = false;
      wrench_.assign(6 * (size_t)n, 0.0);
      if (step_ok_ && n > 0 && hc_get_wrenches(ctx_, wrench_.data()) != HC_OK) step_ok_ = false;
      if (step_ok_ && fields_.apply_forces) {
        for (int i = 0; i < n; ++i) {
          const int gm = m_geom_[(size_t)i], gn = n_geom_[(size_t)i];
          const Real* xm = d->geom_xpos + 3 * (size_t)gm;
          const double* w = &wrench_[6 * (size_t)i];
          const Real fa[3] = {w[0], w[1], w[2]}, ta[3] = {w[3], w[4], w[5]};
          const Real fb[3] = {-w[0], -w[1], -w[2]}, tb[3] = {-w[3], -w[4], -w[5]};
          Api::apply_ft(m, d, fa, ta, xm, m->geom_bodyid[gm], d->qfrc_passive);
          Api::apply_ft(m, d, fb, tb, xm, m->geom_bodyid[gn], d->qfrc_passive);
        }
      }
      if (step_ok_) {
        StepView v;
        v.ctx = ctx_;
        v.m_geom = &m_geom_;
        v.n_geom = &n_geom_;
        v.wrench = &wrench_;
        v.n_pair = n;
        for (SurfacePlugin<Api>* p : ready_) p->update(m, d, v);
      }
    }
    g1_.clear();
    g2_.clear();
  }

  // plugin.cpp:828-975: regenerate the geom's mesh and field for its new size.
  void onGeomChanged(const Model* m, Data*, int geom_id) {
    if (!ctx_ || geom_id < 0 || geom_id >= (int)kind_.size() || kind_[(size_t)geom_id] < 0) return;
    if (hc_update_geom_size(ctx_, geom_id, m->geom_size + 3 * (size_t)geom_id) != HC_OK) step_ok_ = false;
    last_g1_.clear();  // the pairs are dispatched again at the next step
    last_g2_.clear();
  }

  hc_context* context() const { return ctx_; }
  const ParsedFields& fields() const { return fields_; }
  const std::vector<double>& last_wrenches() const { return wrench_; }
  bool last_step_ok() const { return step_ok_; }
  static std::string last_error() { return hc_last_error(); }

 private:
  bool fail() { return false; }

  int device_ = 0;
  hc_context* ctx_ = nullptr;
  const Model* m_ = nullptr;
  Data* d_ = nullptr;
  ParsedFields fields_;
  std::vector<int> kind_;
  std::vector<int> g1_, g2_, last_g1_, last_g2_, m_geom_, n_geom_;
  std::vector<double> vel_, wrench_;
  bool step_ok_ = true;
  std::vector<std::unique_ptr<SurfacePlugin<Api>>> plugins_;
  std::vector<SurfacePlugin<Api>*> ready_;
};

}  // namespace hc_plugin

#endif  // HC_CONTACT_SURFACES_PLUGIN_HPP_
