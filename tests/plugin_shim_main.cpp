// Test driver for include/hc/contact_surfaces_plugin.hpp over a small fake of
// MuJoCo's model and data (the fields and calls the plugin uses).
//
//   plugin_shim_main parse   : parse the cs:: custom fields (no device)
//   plugin_shim_main step    : load, record pairs, passive step, sensors
//
// Output: "key value..." lines read by tests/test_plugin_shim.py.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hc/contact_surfaces_plugin.hpp"

struct FakeContact {};

struct FakeModel {
  int ngeom = 0;
  int* geom_type = nullptr;
  double* geom_size = nullptr;
  int* geom_bodyid = nullptr;
  int* geom_dataid = nullptr;
  int nnumeric = 0;
  int* numeric_adr = nullptr;
  int* numeric_size = nullptr;
  double* numeric_data = nullptr;
  int ntext = 0;
  int* text_adr = nullptr;
  int* text_size = nullptr;
  char* text_data = nullptr;
  int* mesh_vertadr = nullptr;
  int* mesh_vertnum = nullptr;
  float* mesh_vert = nullptr;
  int* mesh_faceadr = nullptr;
  int* mesh_facenum = nullptr;
  int* mesh_face = nullptr;
  double* geom_pos = nullptr;
  double* geom_quat = nullptr;
  // storage
  std::vector<std::string> geom_names, numeric_names, text_names;
  std::vector<int> v_type, v_body, v_dataid, v_nadr, v_nsize, v_tadr, v_tsize;
  std::vector<double> v_size, v_ndata, v_pos, v_quat;
  std::vector<int> v_mvadr, v_mvnum, v_mfadr, v_mfnum, v_mface;
  std::vector<float> v_mvert;
  std::vector<char> v_tdata;

  int add_geom(const std::string& name, int type, double sx, double sy, double sz, int body) {
    geom_names.push_back(name);
    v_type.push_back(type);
    v_size.insert(v_size.end(), {sx, sy, sz});
    v_body.push_back(body);
    v_dataid.push_back(-1);
    v_pos.insert(v_pos.end(), {0, 0, 0});
    v_quat.insert(v_quat.end(), {1, 0, 0, 0});
    return (int)geom_names.size() - 1;
  }
  // A mesh geom: vertices (3 floats each) and faces (3 indices each).
  int add_mesh_geom(const std::string& name, const std::vector<float>& vert, const std::vector<int>& face, int body) {
    const int g = add_geom(name, 7, 0, 0, 0, body);
    v_dataid[(size_t)g] = (int)v_mvadr.size();
    v_mvadr.push_back((int)v_mvert.size() / 3);
    v_mvnum.push_back((int)vert.size() / 3);
    v_mfadr.push_back((int)v_mface.size() / 3);
    v_mfnum.push_back((int)face.size() / 3);
    v_mvert.insert(v_mvert.end(), vert.begin(), vert.end());
    v_mface.insert(v_mface.end(), face.begin(), face.end());
    return g;
  }
  void add_numeric(const std::string& name, std::vector<double> vals) {
    numeric_names.push_back(name);
    v_nadr.push_back((int)v_ndata.size());
    v_nsize.push_back((int)vals.size());
    v_ndata.insert(v_ndata.end(), vals.begin(), vals.end());
  }
  void add_text(const std::string& name, const std::string& s) {
    text_names.push_back(name);
    v_tadr.push_back((int)v_tdata.size());
    v_tsize.push_back((int)s.size() + 1);
    v_tdata.insert(v_tdata.end(), s.begin(), s.end());
    v_tdata.push_back('\0');
  }
  void finalize() {
    ngeom = (int)geom_names.size();
    geom_type = v_type.data();
    geom_size = v_size.data();
    geom_bodyid = v_body.data();
    geom_dataid = v_dataid.data();
    geom_pos = v_pos.data();
    geom_quat = v_quat.data();
    mesh_vertadr = v_mvadr.data();
    mesh_vertnum = v_mvnum.data();
    mesh_vert = v_mvert.data();
    mesh_faceadr = v_mfadr.data();
    mesh_facenum = v_mfnum.data();
    mesh_face = v_mface.data();
    nnumeric = (int)numeric_names.size();
    numeric_adr = v_nadr.data();
    numeric_size = v_nsize.data();
    numeric_data = v_ndata.data();
    ntext = (int)text_names.size();
    text_adr = v_tadr.data();
    text_size = v_tsize.data();
    text_data = v_tdata.data();
  }
};

struct FakeData {
  double time = 0.0;
  std::vector<double> xpos, xmat, qfrc, vel;
  double* geom_xpos = nullptr;
  double* geom_xmat = nullptr;
  double* qfrc_passive = nullptr;
  // applied wrenches per body: force, torque about the world origin
  std::vector<double> body_wrench;
  int n_apply = 0;
};

struct FakeApi {
  using Model = FakeModel;
  using Data = FakeData;
  using Contact = FakeContact;
  using Real = double;
  static constexpr int kObjGeom = 5, kObjNumeric = 18, kObjText = 19;
  static constexpr bool kGeomLocalPose = true;  // the model has geom_pos / geom_quat
  static int name2id(const Model* m, int type, const char* name) {
    const std::vector<std::string>* v = type == kObjGeom ? &m->geom_names
                                        : type == kObjNumeric ? &m->numeric_names
                                        : type == kObjText ? &m->text_names : nullptr;
    if (!v) return -1;
    for (size_t i = 0; i < v->size(); ++i)
      if ((*v)[i] == name) return (int)i;
    return -1;
  }
  static const char* id2name(const Model* m, int type, int id) {
    if (type == kObjNumeric && id >= 0 && id < (int)m->numeric_names.size()) return m->numeric_names[id].c_str();
    if (type == kObjGeom && id >= 0 && id < (int)m->geom_names.size()) return m->geom_names[id].c_str();
    return nullptr;
  }
  static void object_velocity(const Model*, const Data* d, int geom, Real res[6]) {
    for (int k = 0; k < 6; ++k) res[k] = d->vel[6 * (size_t)geom + k];
  }
  // Records force and the torque about the world origin on `body`.
  static void apply_ft(const Model*, Data* d, const Real f[3], const Real t[3], const Real p[3], int body, Real*) {
    double* w = &d->body_wrench[6 * (size_t)body];
    for (int k = 0; k < 3; ++k) w[k] += f[k];
    w[3] += t[0] + p[1] * f[2] - p[2] * f[1];
    w[4] += t[1] + p[2] * f[0] - p[0] * f[2];
    w[5] += t[2] + p[0] * f[1] - p[1] * f[0];
    ++d->n_apply;
  }
};

static int default_calls = 0;
static int default_collision(const FakeModel*, const FakeData*, FakeContact*, int, int, double) {
  ++default_calls;
  return 1;
}

using Plugin = hc_plugin::MujocoContactSurfacesPlugin<FakeApi>;

static void build_model(FakeModel& m, bool force_mode) {
  // geoms: 0 soft sphere (body 1), 1 rigid box plate (body 2), 2 rigid plane
  // (world), 3 capsule without cs:: fields (body 3), 4 soft box (body 4)
  m.add_geom("ball", 2, 0.03, 0, 0, 1);
  m.add_geom("plate", 6, 0.04, 0.04, 0.005, 2);
  m.add_geom("floor", 0, 0, 0, 1, 0);
  m.add_geom("stick", 3, 0.01, 0.05, 0, 3);
  m.add_geom("cube", 6, 0.02, 0.02, 0.02, 4);
  m.add_text("cs::HydroelasticContactRepresentation", "kTriangle");
  m.add_numeric("cs::ApplyContactSurfaceForces", {force_mode ? 1.0 : 0.0});
  m.add_numeric("cs::ball", {2e5, 1.0, 0.006, 0.5, 0.5});
  m.add_numeric("cs::plate", {0, 1.0, 0, 0.4, 0.4});
  m.add_numeric("cs::floor", {0, 1.0, 0, 0.6, 0.6});
  m.add_numeric("cs::nosuchgeom", {1, 2, 3, 4, 5});
  m.add_numeric("cs::cube", {1e5, 0.5, 0.01, 0.3, 0.3});
  m.add_numeric("unrelated", {1, 2, 3, 4, 5});
  m.finalize();
}

static void set_pose(FakeData& d, int g, double x, double y, double z) {
  d.xpos[3 * g] = x;
  d.xpos[3 * g + 1] = y;
  d.xpos[3 * g + 2] = z;
  for (int k = 0; k < 9; ++k) d.xmat[9 * g + k] = (k % 4 == 0) ? 1.0 : 0.0;
}

// A soft box mesh pressed into the floor, read by a curved sensor on its
// bottom face (50 Hz, three steps at 100 Hz).
static int run_curved() {
  FakeModel m;
  m.add_geom("floor", 0, 0, 0, 1, 0);
  const float hx = 0.02f, hy = 0.02f, hz = 0.01f;
  std::vector<float> vert;
  for (int sx = -1; sx <= 1; sx += 2)
    for (int sy = -1; sy <= 1; sy += 2)
      for (int sz = -1; sz <= 1; sz += 2) vert.insert(vert.end(), {sx * hx, sy * hy, sz * hz});
  const std::vector<int> face = {0, 1, 3, 0, 3, 2, 4, 6, 7, 4, 7, 5, 0, 4, 5, 0, 5, 1,
                                 2, 3, 7, 2, 7, 6, 0, 2, 6, 0, 6, 4, 1, 5, 7, 1, 7, 3};
  const int tip = m.add_mesh_geom("tip", vert, face, 1);
  m.add_text("cs::HydroelasticContactRepresentation", "kTriangle");
  m.add_numeric("cs::floor", {0, 1.0, 0, 0.5, 0.5});
  m.add_numeric("cs::tip", {1e5, 1.0, 0.004, 0.5, 0.5});
  m.finalize();
  FakeData d;
  d.xpos.assign(3 * (size_t)m.ngeom, 0.0);
  d.xmat.assign(9 * (size_t)m.ngeom, 0.0);
  d.vel.assign(6 * (size_t)m.ngeom, 0.0);
  d.qfrc.assign(8, 0.0);
  d.body_wrench.assign(6 * 2, 0.0);
  set_pose(d, 0, 0, 0, 0);
  set_pose(d, tip, 0.001, -0.002, hz - 0.002);
  d.geom_xpos = d.xpos.data();
  d.geom_xmat = d.xmat.data();
  d.qfrc_passive = d.qfrc.data();
  Plugin plugin(0);
  hc_plugin::CurvedSensorConfig cc;
  cc.sensor_name = "tip_skin";
  cc.geom_name = "tip";
  cc.update_rate = 50.0;
  for (int i = -1; i <= 1; ++i)
    for (int j = -1; j <= 1; ++j) cc.taxels.push_back({0.006 * i, 0.006 * j, -hz});
  cc.normals = {{0, 0, -1}, {0, 0, 0}, {0, 0, -3}};
  cc.include_margin = 0.004;
  cc.sample_resolution = 200000.7;   // the integer part counts
  auto cs = std::make_unique<hc_plugin::CurvedSensor<FakeApi>>(cc);
  hc_plugin::CurvedSensor<FakeApi>* cp = cs.get();
  plugin.add_plugin(std::move(cs));
  if (!plugin.load(&m, &d)) {
    printf("load_failed %s\n", Plugin::last_error().c_str());
    return 1;
  }
  FakeContact con[1];
  for (int step = 0; step < 3; ++step) {
    d.time = 0.01 * step;
    plugin.collision_cb(&m, &d, con, tip, 0, 0.0, default_collision);
    plugin.passiveCallback(&m, &d);
    printf("cstep %d ok %d updates %d\n", step, plugin.last_step_ok() ? 1 : 0, cp->n_updates());
  }
  printf("points %d\n", cp->n_surface_points());
  printf("curved_values");
  for (float v : cp->values()) printf(" %.9g", v);
  printf("\n");
  // a primitive geom is rejected, as the reference rejects it
  hc_plugin::CurvedSensorConfig bad = cc;
  bad.geom_name = "floor";
  hc_plugin::CurvedSensor<FakeApi> reject(bad);
  printf("reject_primitive %d\n", reject.load(&m, &d, nullptr) ? 0 : 1);
  return 0;
}

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "parse";
  if (mode == "curved") return run_curved();
  if (mode == "parse") {
    for (int force = 0; force < 2; ++force) {
      FakeModel m;
      build_model(m, force != 0);
      hc_plugin::ParsedFields f = hc_plugin::parse_custom_fields<FakeApi>(&m);
      printf("repr %d apply %d visualize %d ngeoms %zu\n", f.representation, f.apply_forces ? 1 : 0,
             f.visualize ? 1 : 0, f.geoms.size());
      for (const auto& g : f.geoms)
        printf("geom %d %s %g %g %g %g %g\n", g.geom_id, g.geom_name.c_str(), g.cs5[0], g.cs5[1], g.cs5[2],
               g.cs5[3], g.cs5[4]);
    }
    FakeModel m;
    m.add_text("cs::HydroelasticContactRepresentation", "kPolygon please");
    m.finalize();
    printf("repr2 %d\n", hc_plugin::parse_custom_fields<FakeApi>(&m).representation);
    // taxels of a mesh geom with a local pose move by the inverse pose
    const double p0[3] = {0.1, -0.2, 0.3};
    const double h = std::sqrt(0.5), q0[4] = {h, 0, 0, h};  // 90 degrees about z
    std::vector<double> t = {1.0, 2.0, 3.0, 0.1, -0.2, 0.3};
    hc_plugin::apply_inverse_pose(p0, q0, t);
    printf("invpose %.17g %.17g %.17g %.17g %.17g %.17g\n", t[0], t[1], t[2], t[3], t[4], t[5]);
    const double pi[3] = {0, 0, 0}, qi[4] = {1, 0, 0, 0};
    std::vector<double> u = {1.0, 2.0, 3.0};
    hc_plugin::apply_inverse_pose(pi, qi, u);
    printf("identity %.17g %.17g %.17g\n", u[0], u[1], u[2]);
    return 0;
  }
  // step: ball pressed into the plate, cube resting on the floor, stick
  // touching the ball (default collision path)
  FakeModel m;
  build_model(m, true);
  FakeData d;
  d.xpos.assign(3 * (size_t)m.ngeom, 0.0);
  d.xmat.assign(9 * (size_t)m.ngeom, 0.0);
  d.vel.assign(6 * (size_t)m.ngeom, 0.0);
  d.qfrc.assign(8, 0.0);
  d.body_wrench.assign(6 * 5, 0.0);
  set_pose(d, 0, 0.004, -0.003, 0.005 + 0.03 - 0.002);
  set_pose(d, 1, 0, 0, 0);
  set_pose(d, 2, 0, 0, -0.2);
  set_pose(d, 3, 0.5, 0.5, 0.5);
  set_pose(d, 4, 0.3, 0.0, -0.2 + 0.02 - 0.001);
  d.vel[6 * 0 + 5] = -0.01;  // ball moving down
  d.vel[6 * 4 + 3] = 0.02;   // cube sliding along x
  d.geom_xpos = d.xpos.data();
  d.geom_xmat = d.xmat.data();
  d.qfrc_passive = d.qfrc.data();

  Plugin plugin(0);
  hc_plugin::FlatSensorConfig sc;
  sc.sensor_name = "plate_sensor";
  sc.geom_name = "plate";
  sc.update_rate = 50.0;  // every 0.02 s of simulated time
  auto sensor = std::make_unique<hc_plugin::FlatTactileSensor<FakeApi>>(sc);
  hc_plugin::FlatTactileSensor<FakeApi>* sp = sensor.get();
  plugin.add_plugin(std::move(sensor));
  // taxel sensors on the plate's top face: a 5 x 5 grid, squared-distance
  // ("mean" falls through to it) and closest with visualisation
  hc_plugin::TaxelSensorConfig tc;
  tc.sensor_name = "plate_taxels";
  tc.geom_name = "plate";
  tc.update_rate = 50.0;
  for (int i = 0; i < 5; ++i)
    for (int j = 0; j < 5; ++j) tc.taxels.push_back({-0.01 + 0.005 * i, -0.01 + 0.005 * j, 0.005});
  tc.method = "mean";
  tc.include_margin = 0.004;
  tc.sample_resolution = 0.002;
  auto taxel = std::make_unique<hc_plugin::TaxelSensor<FakeApi>>(tc);
  hc_plugin::TaxelSensor<FakeApi>* tp = taxel.get();
  plugin.add_plugin(std::move(taxel));
  tc.sensor_name = "plate_closest";
  tc.method = "closest";
  tc.visualize = true;
  tc.sample_method = "area_importance";
  tc.sample_resolution = 0.01;
  auto closest = std::make_unique<hc_plugin::TaxelSensor<FakeApi>>(tc);
  hc_plugin::TaxelSensor<FakeApi>* cp = closest.get();
  plugin.add_plugin(std::move(closest));
  if (!plugin.load(&m, &d)) {
    printf("load_failed %s\n", Plugin::last_error().c_str());
    return 1;
  }
  FakeContact con[4];
  int n_default = 0, n_surface = 0;
  const int pairs[4][2] = {{1, 0}, {3, 0}, {4, 2}, {1, 2}};  // plate-ball, stick-ball, cube-floor, plate-floor
  for (int step = 0; step < 3; ++step) {
    d.time = 0.01 * step;
    std::fill(d.body_wrench.begin(), d.body_wrench.end(), 0.0);
    d.n_apply = 0;
    for (const auto& p : pairs) {
      const int before = default_calls;
      int r = plugin.collision_cb(&m, &d, con, p[0], p[1], 0.0, default_collision);
      if (default_calls > before) n_default += 1;
      else n_surface += 1;
      (void)r;
    }
    plugin.passiveCallback(&m, &d);
    printf("step %d ok %d applies %d sensor_updates %d taxel_updates %d %d\n", step, plugin.last_step_ok() ? 1 : 0,
           d.n_apply, sp->n_updates(), tp->n_updates(), cp->n_updates());
  }
  printf("counts default %d surface %d\n", n_default, n_surface);
  const std::vector<double>& w = plugin.last_wrenches();
  for (size_t i = 0; i < w.size() / 6; ++i)
    printf("wrench %zu %.17g %.17g %.17g %.17g %.17g %.17g\n", i, w[6 * i], w[6 * i + 1], w[6 * i + 2], w[6 * i + 3],
           w[6 * i + 4], w[6 * i + 5]);
  for (int b = 0; b < 5; ++b) {
    const double* bw = &d.body_wrench[6 * (size_t)b];
    printf("body %d %.17g %.17g %.17g %.17g %.17g %.17g\n", b, bw[0], bw[1], bw[2], bw[3], bw[4], bw[5]);
  }
  double tsum = 0, tmax = 0;
  for (float v : sp->values()) {
    tsum += v;
    tmax = std::max(tmax, (double)v);
  }
  printf("taxels %d %d %.9g %.9g\n", sp->cx(), sp->cy(), tsum, tmax);
  printf("taxel_values");
  for (float v : tp->values()) printf(" %.9g", v);
  printf("\nclosest_values");
  for (float v : cp->values()) printf(" %.9g", v);
  printf("\n");
  // geom resize: the ball grows, next step sees a deeper contact
  m.v_size[0] = 0.031;
  m.finalize();
  plugin.onGeomChanged(&m, &d, 0);
  for (const auto& p : pairs) plugin.collision_cb(&m, &d, con, p[0], p[1], 0.0, default_collision);
  plugin.passiveCallback(&m, &d);
  const std::vector<double>& w2 = plugin.last_wrenches();
  printf("resized ok %d fz %.17g\n", plugin.last_step_ok() ? 1 : 0, w2.size() ? w2[2] : 0.0);
  return 0;
}
