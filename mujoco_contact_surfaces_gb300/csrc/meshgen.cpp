// meshgen.cpp — primitive tessellations and pressure fields (load time only).
#include "meshgen.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <unordered_map>
#include <utility>

#include "../../include/hc/hc.h"

namespace hc {
namespace {

const double kPi = 3.14159265358979323846;

// Refinement level of the octahedral sphere: the smallest L whose great-arc
// edge length pi*R/(2*2^L) is at most the hint.  Capped so a mesh stays
// below ~2M elements.
int sphere_level(double R, double hint) {
  if (!(hint > 0)) return 2;
  int L = 0;
  while (L < 9 && kPi * R / (2.0 * std::ldexp(1.0, L)) > hint) ++L;
  return L;
}

// Unit sphere surface: octahedron refined `level` times, every new vertex
// projected back to the sphere.  Faces are outward counter-clockwise.
void unit_sphere(int level, std::vector<double>* v, std::vector<int>* f) {
  const double oct_v[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  const int oct_f[8][3] = {{0, 2, 4}, {2, 1, 4}, {1, 3, 4}, {3, 0, 4},
                           {2, 0, 5}, {1, 2, 5}, {3, 1, 5}, {0, 3, 5}};
  v->assign(&oct_v[0][0], &oct_v[0][0] + 18);
  f->assign(&oct_f[0][0], &oct_f[0][0] + 24);
  for (int l = 0; l < level; ++l) {
    std::map<std::pair<int, int>, int> mid;
    std::vector<int> nf;
    nf.reserve(f->size() * 4);
    auto midpoint = [&](int a, int b) {
      std::pair<int, int> key(std::min(a, b), std::max(a, b));
      auto it = mid.find(key);
      if (it != mid.end()) return it->second;
      double x = (*v)[3 * a] + (*v)[3 * b], y = (*v)[3 * a + 1] + (*v)[3 * b + 1],
             z = (*v)[3 * a + 2] + (*v)[3 * b + 2];
      double n = std::sqrt(x * x + y * y + z * z);
      int id = (int)(v->size() / 3);
      v->push_back(x / n);
      v->push_back(y / n);
      v->push_back(z / n);
      mid.emplace(key, id);
      return id;
    };
    for (size_t i = 0; i < f->size(); i += 3) {
      int a = (*f)[i], b = (*f)[i + 1], c = (*f)[i + 2];
      int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
      int tri[4][3] = {{a, ab, ca}, {ab, b, bc}, {ca, bc, c}, {ab, bc, ca}};
      for (auto& t : tri) nf.insert(nf.end(), t, t + 3);
    }
    f->swap(nf);
  }
}

void orient_tets(SoftMesh* m) {
  for (size_t i = 0; i < m->t.size(); i += 4) {
    int* t = &m->t[i];
    if (tet_volume(&m->v[3 * t[0]], &m->v[3 * t[1]], &m->v[3 * t[2]], &m->v[3 * t[3]]) < 0)
      std::swap(t[2], t[3]);
  }
}

// Soft body made of one interior vertex fanned to every surface triangle
// (the single-interior-vertex strategy of P:652-653 and the convex-mesh
// fan of P:766-789).  The interior vertex carries pressure E, the surface
// vertices 0.
void fan_soft(const std::vector<double>& sv, const std::vector<int>& sf, const double c[3],
              double E, SoftMesh* out) {
  out->v = sv;
  out->v.insert(out->v.end(), c, c + 3);
  int ci = (int)(sv.size() / 3);
  out->p.assign(sv.size() / 3, 0.0);
  out->p.push_back(E);
  out->t.clear();
  out->t.reserve(sf.size() / 3 * 4);
  for (size_t i = 0; i < sf.size(); i += 3) {
    int tet[4] = {ci, sf[i], sf[i + 1], sf[i + 2]};
    out->t.insert(out->t.end(), tet, tet + 4);
  }
  orient_tets(out);
}

// Kuhn (Freudenthal) split of the logical hex [i,i+1]x[j,j+1]x[k,k+1] into
// six tets sharing the diagonal corner0 -> corner7; every hex face is cut on
// its min->max diagonal, so neighbouring cells agree.  `vid(di,dj,dk)` maps a
// logical corner to a vertex id; tets with a repeated vertex (collapsed
// corners) are dropped.
template <class F>
void kuhn_cell(F vid, std::vector<int>* tets) {
  const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  for (auto& p : perm) {
    int c[3] = {0, 0, 0};
    int ids[4];
    ids[0] = vid(0, 0, 0);
    for (int s = 0; s < 3; ++s) {
      c[p[s]] = 1;
      ids[s + 1] = vid(c[0], c[1], c[2]);
    }
    bool dup = false;
    for (int a = 0; a < 4; ++a)
      for (int b = a + 1; b < 4; ++b) dup |= ids[a] == ids[b];
    if (!dup) tets->insert(tets->end(), ids, ids + 4);
  }
}

int even_count(double extent, double hint, int min_n) {
  int n = min_n;
  if (hint > 0) n = std::max(min_n, 2 * (int)std::ceil(extent / (2.0 * hint) - 1e-9));
  if (n % 2) ++n;
  return n;
}

void soft_box(const double h[3], double E, double hint, SoftMesh* out) {
  // Even cell counts put a vertex layer on every mid-plane, so the extent
  // field min_i(h_i - |x_i|) / min_i(h_i) is captured exactly in the
  // thinnest direction.  Each cell's Kuhn diagonal starts at the cell corner
  // nearest the centre (the cell is mirrored in every axis where it lies in
  // the lower half), which is strictly inside the box: every tet then has a
  // vertex of positive pressure, also along the box's edges and corners
  // (with one diagonal direction for all cells, some tets there have all
  // four vertices on the surface and carry no pressure).  Cells on either
  // side of a mid-plane are mirror images, so their shared faces are cut
  // alike.
  int n[3];
  for (int a = 0; a < 3; ++a) n[a] = even_count(2 * h[a], hint, 2);
  auto id = [&](int i, int j, int k) { return (k * (n[1] + 1) + j) * (n[0] + 1) + i; };
  double hmin = std::min(h[0], std::min(h[1], h[2]));
  out->v.clear();
  out->p.clear();
  for (int k = 0; k <= n[2]; ++k)
    for (int j = 0; j <= n[1]; ++j)
      for (int i = 0; i <= n[0]; ++i) {
        double x = -h[0] + 2 * h[0] * i / n[0], y = -h[1] + 2 * h[1] * j / n[1],
               z = -h[2] + 2 * h[2] * k / n[2];
        out->v.insert(out->v.end(), {x, y, z});
        double d = std::min(h[0] - std::fabs(x), std::min(h[1] - std::fabs(y), h[2] - std::fabs(z)));
        out->p.push_back(E * std::max(0.0, d) / hmin);
      }
  out->t.clear();
  for (int k = 0; k < n[2]; ++k)
    for (int j = 0; j < n[1]; ++j)
      for (int i = 0; i < n[0]; ++i) {
        const bool fi = 2 * i < n[0], fj = 2 * j < n[1], fk = 2 * k < n[2];
        kuhn_cell([&](int a, int b, int c) { return id(i + (fi ? 1 - a : a), j + (fj ? 1 - b : b), k + (fk ? 1 - c : c)); },
                  &out->t);
      }
  orient_tets(out);
}

void soft_cylinder(double R, double hl, double E, double hint, SoftMesh* out) {
  int nr = std::max(1, hint > 0 ? (int)std::ceil(R / hint - 1e-9) : 1);
  int ns = std::max(12, 4 * (int)std::ceil(2 * kPi * R / (4 * (hint > 0 ? hint : R)) - 1e-9));
  int nz = even_count(2 * hl, hint, 2);
  // Vertex ids: per layer k, the axis vertex then rings 1..nr with ns each.
  int per_layer = 1 + nr * ns;
  auto id = [&](int i, int j, int k) {
    if (i == 0) return k * per_layer;
    return k * per_layer + 1 + (i - 1) * ns + ((j % ns) + ns) % ns;
  };
  double dmax = std::min(R, hl);
  out->v.clear();
  out->p.clear();
  for (int k = 0; k <= nz; ++k) {
    double z = -hl + 2 * hl * k / nz;
    for (int i = 0; i <= nr; ++i) {
      int jn = i == 0 ? 1 : ns;
      for (int j = 0; j < jn; ++j) {
        double r = R * i / nr, th = 2 * kPi * j / ns;
        out->v.insert(out->v.end(), {r * std::cos(th), r * std::sin(th), z});
        double d = std::min(R - r, hl - std::fabs(z));
        out->p.push_back(E * std::max(0.0, d) / dmax);
      }
    }
  }
  // Each cell's Kuhn diagonal starts at its inner ring and at the layer
  // nearer the mid-plane (cells of the lower half mirrored in z): that
  // corner is inside the cylinder, so every tet carries pressure, also where
  // the mantle meets the caps.
  out->t.clear();
  for (int k = 0; k < nz; ++k) {
    const bool fk = 2 * k < nz;
    for (int j = 0; j < ns; ++j)
      for (int i = 0; i < nr; ++i)
        kuhn_cell([&](int a, int b, int c) { return id(i + a, j + b, k + (fk ? 1 - c : c)); }, &out->t);
  }
  orient_tets(out);
}

void rigid_box(const double h[3], double hint, RigidMesh* out) {
  out->v.clear();
  out->f.clear();
  // Each face: axis a normal, sign s; in-plane axes u, v chosen so that
  // u x v = s * e_a (outward counter-clockwise).
  for (int a = 0; a < 3; ++a)
    for (int s = -1; s <= 1; s += 2) {
      int u = (a + 1) % 3, w = (a + 2) % 3;
      if (s < 0) std::swap(u, w);
      int nu = hint > 0 ? std::max(1, (int)std::ceil(2 * h[u] / hint - 1e-9)) : 1;
      int nw = hint > 0 ? std::max(1, (int)std::ceil(2 * h[w] / hint - 1e-9)) : 1;
      int base = (int)(out->v.size() / 3);
      for (int jw = 0; jw <= nw; ++jw)
        for (int iu = 0; iu <= nu; ++iu) {
          double p[3];
          p[a] = s * h[a];
          p[u] = -h[u] + 2 * h[u] * iu / nu;
          p[w] = -h[w] + 2 * h[w] * jw / nw;
          out->v.insert(out->v.end(), p, p + 3);
        }
      for (int jw = 0; jw < nw; ++jw)
        for (int iu = 0; iu < nu; ++iu) {
          int v00 = base + jw * (nu + 1) + iu, v10 = v00 + 1, v01 = v00 + nu + 1, v11 = v01 + 1;
          out->f.insert(out->f.end(), {v00, v10, v11, v00, v11, v01});
        }
    }
}

void rigid_cylinder(double R, double hl, double hint, RigidMesh* out) {
  int ns = std::max(12, 4 * (int)std::ceil(2 * kPi * R / (4 * (hint > 0 ? hint : R)) - 1e-9));
  int nz = hint > 0 ? std::max(1, (int)std::ceil(2 * hl / hint - 1e-9)) : 1;
  out->v.clear();
  out->f.clear();
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j < ns; ++j) {
      double th = 2 * kPi * j / ns;
      out->v.insert(out->v.end(), {R * std::cos(th), R * std::sin(th), -hl + 2 * hl * k / nz});
    }
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ns; ++j) {
      int a = k * ns + j, b = k * ns + (j + 1) % ns, c = a + ns, d = b + ns;
      out->f.insert(out->f.end(), {a, b, d, a, d, c});
    }
  int cb = (int)(out->v.size() / 3);
  out->v.insert(out->v.end(), {0, 0, -hl});
  out->v.insert(out->v.end(), {0, 0, hl});
  for (int j = 0; j < ns; ++j) {
    int a = j, b = (j + 1) % ns;
    out->f.insert(out->f.end(), {cb, b, a});                      // bottom, -z
    out->f.insert(out->f.end(), {cb + 1, nz * ns + a, nz * ns + b});  // top, +z
  }
}

// Centroid of the volume enclosed by a closed, outward oriented triangle
// mesh: signed-volume weighted centroids of the tets (origin, p, q, r).
// Same quantity as CalcCentroidOfEnclosedVolume.
bool enclosed_centroid(const double* v, const int* f, int nf, double c[3]) {
  double six_total = 0, acc[3] = {0, 0, 0};
  for (int i = 0; i < nf; ++i) {
    const double *p = v + 3 * f[3 * i], *q = v + 3 * f[3 * i + 1], *r = v + 3 * f[3 * i + 2];
    double cx = q[1] * r[2] - q[2] * r[1], cy = q[2] * r[0] - q[0] * r[2], cz = q[0] * r[1] - q[1] * r[0];
    double six = p[0] * cx + p[1] * cy + p[2] * cz;
    six_total += six;
    for (int a = 0; a < 3; ++a) acc[a] += six * (p[a] + q[a] + r[a]);
  }
  if (!(std::fabs(six_total) > 0)) return false;
  for (int a = 0; a < 3; ++a) c[a] = acc[a] / (4 * six_total);
  return true;
}

bool finite3(const double* s) {
  return std::isfinite(s[0]) && std::isfinite(s[1]) && std::isfinite(s[2]);
}

}  // namespace

double tet_volume(const double* a, const double* b, const double* c, const double* d) {
  double e1[3], e2[3], e3[3];
  for (int i = 0; i < 3; ++i) e1[i] = b[i] - a[i], e2[i] = c[i] - a[i], e3[i] = d[i] - a[i];
  double cx = e2[1] * e3[2] - e2[2] * e3[1], cy = e2[2] * e3[0] - e2[0] * e3[2],
         cz = e2[0] * e3[1] - e2[1] * e3[0];
  return (e1[0] * cx + e1[1] * cy + e1[2] * cz) / 6.0;
}

std::string make_soft_mesh(int type, const double size[3], double E, double hint,
                           const double* mesh_v, int nv, const int* mesh_f, int nf, SoftMesh* out) {
  if (!(E > 0) || !std::isfinite(E)) return "soft geom needs a finite modulus E > 0";
  if (!finite3(size)) return "non-finite geom size";
  switch (type) {
    case HC_GEOM_SPHERE:
    case HC_GEOM_ELLIPSOID: {
      double ax[3];
      if (type == HC_GEOM_SPHERE) ax[0] = ax[1] = ax[2] = size[0];
      else for (int a = 0; a < 3; ++a) ax[a] = size[a];
      if (!(ax[0] > 0 && ax[1] > 0 && ax[2] > 0)) return "sphere/ellipsoid needs positive radii";
      std::vector<double> sv;
      std::vector<int> sf;
      unit_sphere(sphere_level(std::max(ax[0], std::max(ax[1], ax[2])), hint), &sv, &sf);
      for (size_t i = 0; i < sv.size(); ++i) sv[i] *= ax[i % 3];
      const double c[3] = {0, 0, 0};
      fan_soft(sv, sf, c, E, out);
      return "";
    }
    case HC_GEOM_BOX: {
      if (!(size[0] > 0 && size[1] > 0 && size[2] > 0)) return "box needs positive half sizes";
      soft_box(size, E, hint, out);
      return "";
    }
    case HC_GEOM_CYLINDER: {
      // A soft cylinder with hint <= 0 reads an uninitialised mesh in the
      // reference; here it is rejected.
      if (!(hint > 0)) return "soft cylinder needs a positive resolution hint";
      if (!(size[0] > 0 && size[1] > 0)) return "cylinder needs positive radius and half length";
      soft_cylinder(size[0], size[1], E, hint, out);
      return "";
    }
    case HC_GEOM_MESH: {
      if (!mesh_v || !mesh_f) return "mesh geom needs vertices and faces";
      if (nv < 4 || nf < 4) return std::string(kDegenerate) + "a soft mesh needs at least 4 vertices and 4 faces";
      for (int i = 0; i < 3 * nf; ++i)
        if (mesh_f[i] < 0 || mesh_f[i] >= nv) return "mesh face index out of range";
      double c[3];
      if (!enclosed_centroid(mesh_v, mesh_f, nf, c)) return std::string(kDegenerate) + "mesh encloses zero volume";
      std::vector<double> sv(mesh_v, mesh_v + 3 * nv);
      std::vector<int> sf(mesh_f, mesh_f + 3 * nf);
      fan_soft(sv, sf, c, E, out);
      return "";
    }
    case HC_GEOM_PLANE: return "soft plane collision not implemented";
    case HC_GEOM_HFIELD: return "hfield collision not implemented";
    case HC_GEOM_CAPSULE: return "capsule collision not implemented";
    default: return "unknown geom type";
  }
}

std::string make_rigid_mesh(int type, const double size[3], double hint, const double* mesh_v,
                            int nv, const int* mesh_f, int nf, RigidMesh* out) {
  if (!finite3(size)) return "non-finite geom size";
  switch (type) {
    case HC_GEOM_PLANE: out->v.clear(); out->f.clear(); return "";
    case HC_GEOM_SPHERE:
    case HC_GEOM_ELLIPSOID: {
      double ax[3];
      if (type == HC_GEOM_SPHERE) ax[0] = ax[1] = ax[2] = size[0];
      else for (int a = 0; a < 3; ++a) ax[a] = size[a];
      if (!(ax[0] > 0 && ax[1] > 0 && ax[2] > 0)) return "sphere/ellipsoid needs positive radii";
      unit_sphere(sphere_level(std::max(ax[0], std::max(ax[1], ax[2])), hint), &out->v, &out->f);
      for (size_t i = 0; i < out->v.size(); ++i) out->v[i] *= ax[i % 3];
      return "";
    }
    case HC_GEOM_BOX:
      if (!(size[0] > 0 && size[1] > 0 && size[2] > 0)) return "box needs positive half sizes";
      rigid_box(size, hint, out);
      return "";
    case HC_GEOM_CYLINDER:
      if (!(size[0] > 0 && size[1] > 0)) return "cylinder needs positive radius and half length";
      rigid_cylinder(size[0], size[1], hint, out);
      return "";
    case HC_GEOM_MESH:
      if (!mesh_v || !mesh_f) return "mesh geom needs vertices and faces";
      if (nv < 3 || nf < 1) return std::string(kDegenerate) + "empty rigid mesh";
      for (int i = 0; i < 3 * nf; ++i)
        if (mesh_f[i] < 0 || mesh_f[i] >= nv) return "mesh face index out of range";
      out->v.assign(mesh_v, mesh_v + 3 * nv);
      out->f.assign(mesh_f, mesh_f + 3 * nf);
      return "";
    case HC_GEOM_HFIELD: return "hfield collision not implemented";
    case HC_GEOM_CAPSULE: return "capsule collision not implemented";
    default: return "unknown geom type";
  }
}

void round_to_float(SoftMesh* m) {
  for (double& x : m->v) x = (double)(float)x;
  for (double& x : m->p) x = (double)(float)x;
  // Rounding can flip a sliver's orientation; re-orient.
  orient_tets(m);
}

void round_to_float(RigidMesh* m) {
  for (double& x : m->v) x = (double)(float)x;
}

namespace {

// splitmix64: a seedable 64-bit generator (Steele, Lea and Flood 2014).
struct Split64 {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }   // [0, 1)
};

struct Candidate {
  double x[3];
  int face;
};

// Greedy thinning in candidate order with a hash grid of cell size r.
int thin(const std::vector<Candidate>& c, double r, int want, std::vector<int>* kept) {
  kept->clear();
  std::unordered_map<int64_t, std::vector<int>> grid;
  const double r2 = r * r;
  auto key = [](int64_t i, int64_t j, int64_t k) { return (i * 73856093) ^ (j * 19349663) ^ (k * 83492791); };
  for (int idx = 0; idx < (int)c.size(); ++idx) {
    const double* p = c[idx].x;
    const int64_t ci = (int64_t)std::floor(p[0] / r), cj = (int64_t)std::floor(p[1] / r),
                  ck = (int64_t)std::floor(p[2] / r);
    bool ok = true;
    for (int64_t di = -1; di <= 1 && ok; ++di)
      for (int64_t dj = -1; dj <= 1 && ok; ++dj)
        for (int64_t dk = -1; dk <= 1 && ok; ++dk) {
          auto it = grid.find(key(ci + di, cj + dj, ck + dk));
          if (it == grid.end()) continue;
          for (int o : it->second) {
            const double* q = c[o].x;
            const double d0 = p[0] - q[0], d1 = p[1] - q[1], d2 = p[2] - q[2];
            if (d0 * d0 + d1 * d1 + d2 * d2 < r2) { ok = false; break; }
          }
        }
    if (!ok) continue;
    grid[key(ci, cj, ck)].push_back(idx);
    kept->push_back(idx);
    if (want > 0 && (int)kept->size() >= want) break;
  }
  return (int)kept->size();
}

}  // namespace

int sample_surface(const double* v, int nv, const int* f, int nf, int n, uint64_t seed, std::vector<double>* pts,
                   std::vector<double>* nrm, double* radius) {
  pts->clear();
  nrm->clear();
  if (radius) *radius = 0;
  if (n <= 0 || nf <= 0 || nv <= 0) return 0;
  std::vector<double> cdf((size_t)nf + 1, 0.0), fn(3 * (size_t)nf, 0.0);
  for (int t = 0; t < nf; ++t) {
    double a = 0;
    const int i0 = f[3 * t], i1 = f[3 * t + 1], i2 = f[3 * t + 2];
    if (i0 >= 0 && i1 >= 0 && i2 >= 0 && i0 < nv && i1 < nv && i2 < nv) {
      const double* p0 = v + 3 * i0;
      const double* p1 = v + 3 * i1;
      const double* p2 = v + 3 * i2;
      const double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
      const double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
      const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                            e1[0] * e2[1] - e1[1] * e2[0]};
      const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      a = 0.5 * len;
      if (len > 0)
        for (int k = 0; k < 3; ++k) fn[3 * (size_t)t + k] = cr[k] / len;
    }
    cdf[(size_t)t + 1] = cdf[t] + a;
  }
  const double A = cdf[nf];
  if (!(A > 0) || !std::isfinite(A)) return 0;
  // candidates, uniform by area: face by the area CDF, point by the
  // square-root warp of two uniforms
  const int64_t n_cand = std::min<int64_t>(std::max<int64_t>(32 * (int64_t)n, 1024), 1 << 23);
  std::vector<Candidate> cand((size_t)n_cand);
  Split64 rng{seed};
  for (int64_t k = 0; k < n_cand; ++k) {
    const double u = rng.uniform() * A;
    int t = (int)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) - 1;
    t = std::max(0, std::min(nf - 1, t));
    while (t > 0 && !(cdf[(size_t)t + 1] > cdf[t])) --t;
    const double r1 = std::sqrt(rng.uniform()), r2 = rng.uniform();
    const double w0 = 1 - r1, w1 = r1 * (1 - r2), w2 = r1 * r2;
    const double* p0 = v + 3 * f[3 * t];
    const double* p1 = v + 3 * f[3 * t + 1];
    const double* p2 = v + 3 * f[3 * t + 2];
    for (int c = 0; c < 3; ++c) cand[(size_t)k].x[c] = w0 * p0[c] + w1 * p1[c] + w2 * p2[c];
    cand[(size_t)k].face = t;
  }
  // radius: start at the spacing of a hexagonal packing of n points (an
  // upper bound) and shrink until n points survive the thinning
  double r = std::sqrt(2.0 * A / (std::sqrt(3.0) * n));
  std::vector<int> kept;
  for (int it = 0; it < 40; ++it) {
    const int got = thin(cand, r, n, &kept);
    if (got >= n) break;
    r *= std::max(0.5, std::sqrt((double)std::max(got, 1) / n) * 0.98);
  }
  if (radius) *radius = r;
  for (int idx : kept) {
    for (int c = 0; c < 3; ++c) pts->push_back(cand[(size_t)idx].x[c]);
    for (int c = 0; c < 3; ++c) nrm->push_back(fn[3 * (size_t)cand[(size_t)idx].face + c]);
  }
  return (int)kept.size();
}

}  // namespace hc

namespace hc {

namespace {
double extent(const std::vector<double>& v) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (size_t i = 0; i < v.size(); ++i) {
    lo[i % 3] = std::min(lo[i % 3], v[i]);
    hi[i % 3] = std::max(hi[i % 3], v[i]);
  }
  return std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
}
}  // namespace

std::string degenerate_soft(const SoftMesh& m) {
  const size_t n = m.t.size() / 4;
  if (n == 0) return std::string(kDegenerate) + "soft mesh without tetrahedra";
  const double L = extent(m.v), tol = 1e-12 * L * L * L;
  for (size_t k = 0; k < n; ++k) {
    const int* t = &m.t[4 * k];
    const double vol = tet_volume(&m.v[3 * t[0]], &m.v[3 * t[1]], &m.v[3 * t[2]], &m.v[3 * t[3]]);
    if (!(std::fabs(vol) > tol)) return std::string(kDegenerate) + "zero-volume tetrahedron " + std::to_string(k);
  }
  return "";
}

std::string degenerate_rigid(const RigidMesh& m, bool plane) {
  const size_t n = m.f.size() / 3;
  if (plane) return "";
  if (n == 0) return std::string(kDegenerate) + "rigid mesh without triangles";
  const double L = extent(m.v), tol = 1e-12 * L * L;
  for (size_t k = 0; k < n; ++k) {
    const double* a = &m.v[3 * m.f[3 * k]];
    const double* b = &m.v[3 * m.f[3 * k + 1]];
    const double* c = &m.v[3 * m.f[3 * k + 2]];
    const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const double x = e1[1] * e2[2] - e1[2] * e2[1], y = e1[2] * e2[0] - e1[0] * e2[2], z = e1[0] * e2[1] - e1[1] * e2[0];
    if (!(std::sqrt(x * x + y * y + z * z) > tol)) return std::string(kDegenerate) + "zero-area triangle " + std::to_string(k);
  }
  return "";
}

}  // namespace hc
