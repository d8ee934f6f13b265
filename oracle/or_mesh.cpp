// or_mesh.cpp — the scene meshes for the oracle, generated on the host.
//
// TEST INFRASTRUCTURE ONLY.  The inputs of every workload are synthetic
// meshes made by the package's own generator (mujoco_contact_surfaces_gb300/
// csrc/meshgen.cpp, the stand-in for the Drake generators the reference
// calls at mujoco_contact_surfaces_plugin.cpp:648-807).  The oracle library
// compiles that source itself, so a process that runs only the oracle (the
// CPU baseline) never loads the engine's library.  The result is the one
// hc_generate_mesh returns: the same generator, rounded to float the same
// way, with floating-point contraction off in both builds.
#include <cstring>
#include <string>

#include "../mujoco_contact_surfaces_gb300/csrc/meshgen.h"

extern "C" {

// Returns 0 on success, 1 on a generator error (message in err, may be
// NULL).  kind: 1 soft (cs5[0] = E > 0), 0 rigid.  Call with NULL arrays
// for the sizes, then again with arrays of those sizes.
int or_generate_mesh(int type, const double size[3], const double cs5[5], const double* mesh_vert, int nvert,
                     const int* mesh_face, int nface, int* out_kind, int* out_nvert, int* out_nelem, double* vert,
                     double* pressure, int* elems, char* err, int err_len) {
  std::string e;
  const double E = cs5[0], hint = cs5[2];
  if (E > 0) {
    hc::SoftMesh m;
    e = hc::make_soft_mesh(type, size, E, hint, mesh_vert, nvert, mesh_face, nface, &m);
    if (e.empty()) {
      hc::round_to_float(&m);
      e = hc::degenerate_soft(m);
    }
    if (e.empty()) {
      *out_kind = 1;
      *out_nvert = (int)(m.v.size() / 3);
      *out_nelem = (int)(m.t.size() / 4);
      if (vert) std::memcpy(vert, m.v.data(), m.v.size() * sizeof(double));
      if (pressure) std::memcpy(pressure, m.p.data(), m.p.size() * sizeof(double));
      if (elems) std::memcpy(elems, m.t.data(), m.t.size() * sizeof(int));
      return 0;
    }
  } else {
    hc::RigidMesh m;
    e = hc::make_rigid_mesh(type, size, hint, mesh_vert, nvert, mesh_face, nface, &m);
    if (e.empty()) {
      hc::round_to_float(&m);
      e = hc::degenerate_rigid(m, type == 0);
    }
    if (e.empty()) {
      *out_kind = 0;
      *out_nvert = (int)(m.v.size() / 3);
      *out_nelem = (int)(m.f.size() / 3);
      if (vert) std::memcpy(vert, m.v.data(), m.v.size() * sizeof(double));
      if (elems) std::memcpy(elems, m.f.data(), m.f.size() * sizeof(int));
      return 0;
    }
  }
  if (err && err_len > 0) {
    std::strncpy(err, e.c_str(), (size_t)err_len - 1);
    err[err_len - 1] = 0;
  }
  return 1;
}

}  // extern "C"
