// meshgen.h — builder-owned tetrahedral / triangle mesh and pressure-field
// generators for the primitive geoms.
//
// Replaces the Drake generators the reference calls while parsing cs::
// properties (mujoco_contact_surfaces_plugin.cpp:648-807): soft sphere and
// ellipsoid (single interior vertex tessellation), soft box
// (P:723-727), soft cylinder, soft convex mesh (centroid fan,
// P:766-789, CalcCentroidOfEnclosedVolume P:161-187) and the rigid surface
// meshes.  The tessellations are
// our own; the pressure field is E * extent with extent 0 on the surface and 1
// on the deepest interior points, linear inside each tetrahedron.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace hc {

struct SoftMesh {
  std::vector<double> v;   // 3 per vertex, body frame
  std::vector<double> p;   // pressure per vertex (Pa)
  std::vector<int> t;      // 4 per tet, positive orientation
};

struct RigidMesh {
  std::vector<double> v;   // 3 per vertex
  std::vector<int> f;      // 3 per triangle, outward counter-clockwise
};

// Returns "" on success, else an error message.  `hint` is the resolution
// hint (m); hint <= 0 picks the coarse default the reference's "WithMa"
// variants stand for.
std::string make_soft_mesh(int type, const double size[3], double E, double hint,
                           const double* mesh_v, int nv, const int* mesh_f, int nf,
                           SoftMesh* out);
std::string make_rigid_mesh(int type, const double size[3], double hint, const double* mesh_v,
                            int nv, const int* mesh_f, int nf, RigidMesh* out);

// Round every coordinate and pressure to the nearest float, the precision
// the device stores; the oracle reads the rounded values.
void round_to_float(SoftMesh* m);
void round_to_float(RigidMesh* m);

// Messages that start with kDegenerate report degenerate input geometry
// (the API's HC_ERR_DEGENERATE), all others invalid arguments.
constexpr const char* kDegenerate = "degenerate: ";
inline bool is_degenerate(const std::string& err) { return err.rfind(kDegenerate, 0) == 0; }

// Degenerate generated meshes, checked after rounding to float: no elements,
// a tetrahedron of volume at most 1e-12 L^3 or a triangle of area at most
// 1e-12 L^2 (L: the mesh's largest extent).  "" when none.
std::string degenerate_soft(const SoftMesh& m);
std::string degenerate_rigid(const RigidMesh& m, bool plane);

// Signed volume of tet (a, b, c, d): (b-a).((c-a)x(d-a)) / 6.
double tet_volume(const double* a, const double* b, const double* c, const double* d);

// Blue-noise points on a triangle mesh surface, for the curved sensor (the
// reference draws them with vcglib's Poisson-disk sampler at load,
// curved_sensor.cpp:260-268, which is not reproduced): `n` candidates
// spread uniformly by area are thinned greedily so that no two kept points
// are closer than a radius, and the radius is shrunk until at least n points
// survive; the first n are kept.  Each point carries the unit normal of its
// triangle (outward for counter-clockwise faces).  Deterministic for a seed
// on every host.  Returns the number of points (<= n).
int sample_surface(const double* v, int nv, const int* f, int nf, int n, uint64_t seed, std::vector<double>* pts,
                   std::vector<double>* nrm, double* radius);

}  // namespace hc
