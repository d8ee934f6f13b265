// adjoint.cuh — reverse pass of the soft-rigid and half-space contact path
// (included by contact.cu inside namespace hc, after narrow.cuh).
//
// The adjoint recomputes each item's contact polygons instead of storing
// them.  Per polygon the geometry is differentiated forward-mode with six
// tangents: the twist xi = (w, v) of the other body's points in the soft
// frame (dY = w x Y + v).  The force law and the velocity field are
// differentiated reverse-mode by hand.  Per lane the contributions to
// dL/dxi, dL/dlin, dL/dang (the relative velocity field v = lin + ang x p of
// the soft frame) and the taxel part of dL/dE are accumulated and reduced
// per item in FP64, then per pair, where the chain rule maps them to the
// world twists of both bodies.

// Reverse of the force law at one quadrature point: the
// velocity-field adjoints are added to G; the adjoints of the point's inputs
// (area, position, normal, pressure, gM, gN) are returned in `b`.  Returns
// false (and no contribution) where the forward skips the point (P:345,
// P:361-368).  upstream: fbar = gF + gT x p (force and torque about the soft
// origin).
struct PointBar {
  float A, p0, gM, gN, d;   // d: dL/d(damping)
  V3<float> p, n;
};

__device__ __forceinline__ bool point_reverse(AdjAcc& G, const FrameDev& F, float damping, float mu, V3<float> gFv,
                                              V3<float> gTv, float A, V3<float> pv, V3<float> nv, float gMv,
                                              float gNv, float p0, PointBar& b) {
  if (!(A > 1.0e-14f)) return false;
  if (gMv < 1.0e-14f || gNv < 1.0e-14f) return false;
  // forward values
  const float g = 1.0f / (1.0f / gMv + 1.0f / gNv);
  const float fn0 = A * p0, k = A * g;
  const V3<float> lin = mk(F.lin[0], F.lin[1], F.lin[2]), ang = mk(F.ang[0], F.ang[1], F.ang[2]);
  const V3<float> v = lin + cross(ang, pv);
  const float vn = dot(v, nv);
  const float h = 1.f - damping * vn, hp = fmaxf(0.f, h);
  const float fnb = fn0 - 0.001f * k * vn;
  const float fn = hp * fnb;
  const V3<float> vt = v - nv * vn;
  const float eps = (1.0e-4f * 1.0e-2f) * (1.0e-4f * 1.0e-2f);
  const float vs = sqrtf(dot(vt, vt) + eps);
  const float s = vs / 1.0e-4f;
  const float mur = s < 1.f ? mu * s * (2.f - s) : mu;
  const V3<float> u = vt * (1.f / vs);
  const V3<float> q = nv - u * mur;
  const V3<float> f = q * fn;
  const V3<float> fbar = gFv + cross(gTv, pv);
  // reverse
  const float Lfn = dot(fbar, q);
  const V3<float> qbar = fbar * fn;
  V3<float> nbar = qbar;
  const float murbar = -dot(qbar, u);
  const V3<float> ubar = qbar * (-mur);
  V3<float> vtbar = ubar * (1.f / vs);
  float vsbar = -dot(ubar, vt) / (vs * vs);
  vsbar += murbar * (s < 1.f ? mu * (2.f - 2.f * s) / 1.0e-4f : 0.f);
  vtbar = vtbar + vt * (vsbar / vs);
  // vt = v - n vn
  V3<float> vbar = vtbar;
  float vnbar = -dot(vtbar, nv);
  nbar = nbar - vtbar * vn;
  // fn = hp (fn0 - 0.001 k vn)
  const float hbar = h > 0.f ? Lfn * fnb : 0.f;
  b.d = -hbar * vn;
  const float fn0bar = Lfn * hp;
  const float kbar = -Lfn * hp * 0.001f * vn;
  vnbar += -Lfn * hp * 0.001f * k - damping * hbar;
  // vn = v . n
  vbar = vbar + nv * vnbar;
  nbar = nbar + v * vnbar;
  // k = A g, fn0 = A p0, g = 1 / (1/gM + 1/gN)
  b.A = kbar * g + fn0bar * p0;
  const float gbar = kbar * A;
  b.p0 = fn0bar * A;
  b.gM = gbar * (g / gMv) * (g / gMv);
  b.gN = gbar * (g / gNv) * (g / gNv);
  // v = lin + ang x p
  G.glin[0] += vbar.x; G.glin[1] += vbar.y; G.glin[2] += vbar.z;
  const V3<float> angbar = cross(pv, vbar);
  G.gang[0] += angbar.x; G.gang[1] += angbar.y; G.gang[2] += angbar.z;
  b.p = cross(vbar, ang) + cross(f, gTv);
  b.n = nbar;
  return true;
}

// A polygon vertex whose three constraint rows are linearly dependent
// (normalised |det| below kDetTol) is not fixed by them.  Soft-soft polygons
// have such vertices wherever an edge on one body's surface meets the other
// body's surface: both pressures vanish there, so the section plane
// p_M = p_N contains the line where the two surface faces meet, and a
// vertex recorded on those two faces lies on that line.  Its motion is the
// line's, carried by the two face rows alone (wrench_adjoint_ss); in the
// soft-rigid and half-space contractions such a triple is accidental and
// the vertex is left out.  In FP32 the determinant of a dependent triple is
// rounding noise (~1e-7 relative), not zero, so the tolerance sits far above
// that and far below the vertices of well-formed polygons (0.008 and up on
// the soft-soft test scenes).
constexpr float kDetTol = 1e-4f;

// Debug statistics of the contraction (StepArgs::adj_skip: [0] vertices left
// out, [1] the smallest normalised |det| seen, as the bits of a non-negative
// float, so an integer minimum orders them).
__device__ __forceinline__ void det_stat(const StepArgs& a, float det, float sc) {
  if (!a.adj_skip) return;
  const float r = sc > 0.f ? fabsf(det) / sc : 0.f;
  atomicMin(a.adj_skip + 1, __float_as_int(r));
}

__device__ __forceinline__ void adj_zero(AdjAcc& g) {
#pragma unroll
  for (int i = 0; i < 6; ++i) g.gx[i] = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) g.glin[i] = g.gang[i] = 0.f;
  g.gE = 0.f;
}

// Wrench adjoint of one contact polygon.  The quadrature and the
// force law are reversed by hand to per-vertex adjoints xbar_v, pbar_v, the
// normal's nbar and the gradient term's gbar; those are then contracted with
// the geometric tangents under the twist xi = (w, v) of the other body in the
// soft frame:
//   vertex x_v: on the section plane (moving) and its two labelled
//     constraints (tet faces fixed, clip planes moving); with the rows r_k and
//     the 3x3 inverse by cross products a_k / det, b_k = xbar.a_k / det and
//     B = sum over moving rows of b_k r_k give dL/dv += B, dL/dw += x_v x B;
//   pressure p_v = g . x_v + c: pbar_v adds pbar_v g to xbar_v;
//   normal ns (rotates with the other body): dL/dw += ns x nbar;
//   gint = g . n (n rotates): dL/dw += gbar (n x g).
// poly: the forward polygon relative to anc; n: the section normal (soft
// frame); sgn: +1 when the soft geom is M (normal out of N into M);
// face: unnormalised tet face normals; clipn: clip-plane normals.
template <int ND>
__device__ __noinline__ void wrench_adjoint(AdjAcc& G, const StepArgs& a, const PairDev& P, const FrameDev& F,
                                            const float* gF, const float* gT, const PV<float, ND>* poly, int nv,
                                            V3<float> anc, V3<float> n, float sgn, const V3<float>* face,
                                            const V3<float>* clipn, V3<float> g, float gint) {
  V3<float> x[kMaxPolyV], xb[kMaxPolyV];
  float pv[kMaxPolyV], pb[kMaxPolyV];
  for (int i = 0; i < nv; ++i) {
    x[i] = pv_pos(poly[i]);
    pv[i] = poly[i].p;
    xb[i] = mk(0.f, 0.f, 0.f);
    pb[i] = 0.f;
  }
  const V3<float> ns = n * sgn;
  const V3<float> gFv = mk(gF[0], gF[1], gF[2]), gTv = mk(gT[0], gT[1], gT[2]);
  // forward fan sums
  float A = 0.f, Sp = 0.f;
  V3<float> Sc = mk(0.f, 0.f, 0.f);
  for (int i = 1; i + 1 < nv; ++i) {
    const float ai = 0.5f * dot(cross(x[i] - x[0], x[i + 1] - x[0]), ns);
    A += ai;
    Sc = Sc + (x[0] + x[i] + x[i + 1]) * (ai * (1.f / 3.f));
    Sp += ai * (pv[0] + pv[i] + pv[i + 1]) * (1.f / 3.f);
  }
  if (A == 0.f) return;
  const float iA = 1.f / A;
  const V3<float> c = Sc * iA;
  const float pc = Sp * iA;
  const float inf = INFINITY;
  const float gMv = P.s_is_m ? gint : inf, gNv = P.s_is_m ? inf : gint;
  V3<float> nbar = mk(0.f, 0.f, 0.f), cbar = mk(0.f, 0.f, 0.f);
  float gbar = 0.f, pcbar = 0.f, Abar = 0.f;
  PointBar b;
  if (a.repr == 1) {
    if (point_reverse(G, F, P.damping, P.mu, gFv, gTv, fabsf(A), anc + c, ns, gMv, gNv, pc, b)) {
      Abar += A < 0.f ? -b.A : b.A;
      cbar = cbar + b.p;
      pcbar += b.p0;
      nbar = nbar + b.n;
      gbar += P.s_is_m ? b.gM : b.gN;
    }
  } else {
    for (int i = 0; i < nv; ++i) {
      const int j = i + 1 == nv ? 0 : i + 1;
      const V3<float> u = x[i] - c, w = x[j] - c;
      const V3<float> cr = cross(u, w);
      const float len = norm(cr);
      const V3<float> cen = anc + (c + x[i] + x[j]) * (1.f / 3.f);
      const float p0 = pc / 3.f + pv[i] / 3.f + pv[j] / 3.f;
      if (!point_reverse(G, F, P.damping, P.mu, gFv, gTv, 0.5f * len, cen, ns, gMv, gNv, p0, b)) continue;
      nbar = nbar + b.n;
      gbar += P.s_is_m ? b.gM : b.gN;
      if (len > 0.f) {   // A_e = |u x w| / 2
        const V3<float> crb = cr * (0.5f * b.A / len);
        const V3<float> ub = cross(w, crb), wb = cross(crb, u);
        xb[i] = xb[i] + ub;
        xb[j] = xb[j] + wb;
        cbar = cbar - ub - wb;
      }
      const V3<float> c3 = b.p * (1.f / 3.f);
      cbar = cbar + c3;
      xb[i] = xb[i] + c3;
      xb[j] = xb[j] + c3;
      const float p3 = b.p0 * (1.f / 3.f);
      pcbar += p3;
      pb[i] += p3;
      pb[j] += p3;
    }
  }
  // c = Sc / A, pc = Sp / A
  const V3<float> Scb = cbar * iA;
  const float Spb = pcbar * iA;
  Abar -= (dot(cbar, c) + pcbar * pc) * iA;
  for (int i = 1; i + 1 < nv; ++i) {
    const V3<float> e1 = x[i] - x[0], e2 = x[i + 1] - x[0];
    const V3<float> cr = cross(e1, e2);
    const float ai = 0.5f * dot(cr, ns);
    const float aib = Abar + dot(Scb, x[0] + x[i] + x[i + 1]) * (1.f / 3.f) +
                      Spb * (pv[0] + pv[i] + pv[i + 1]) * (1.f / 3.f);
    const V3<float> sx = Scb * (ai * (1.f / 3.f));
    const float sp = Spb * ai * (1.f / 3.f);
    xb[0] = xb[0] + sx; xb[i] = xb[i] + sx; xb[i + 1] = xb[i + 1] + sx;
    pb[0] += sp; pb[i] += sp; pb[i + 1] += sp;
    // a_i = n . (e1 x e2) / 2
    nbar = nbar + cr * (0.5f * aib);
    const V3<float> e1b = cross(e2, ns) * (0.5f * aib), e2b = cross(ns, e1) * (0.5f * aib);
    xb[i] = xb[i] + e1b;
    xb[i + 1] = xb[i + 1] + e2b;
    xb[0] = xb[0] - e1b - e2b;
  }
  // contraction with the tangents
  V3<float> rot = cross(ns, nbar), tr = mk(0.f, 0.f, 0.f);
  if (gint != 0.f) rot = rot + cross(n, g) * gbar;
  for (int v = 0; v < nv; ++v) {
    const V3<float> xe = xb[v] + g * pb[v];
    const V3<float> X = anc + x[v];
    const int l0 = poly[v].lab & 15, l1 = poly[v].lab >> 4;
    const V3<float> r0 = n;
    const V3<float> r1 = l0 < 4 ? face[l0] : clipn[l0 - 4];
    const V3<float> r2 = l1 < 4 ? face[l1] : clipn[l1 - 4];
    const V3<float> a0 = cross(r1, r2), a1 = cross(r2, r0), a2 = cross(r0, r1);
    const float det = dot(r0, a0);
    const float sc = norm(r0) * norm(r1) * norm(r2);
    det_stat(a, det, sc);
    if (!(fabsf(det) > kDetTol * sc)) {
      if (a.adj_skip) atomicAdd(a.adj_skip, 1);
      continue;
    }
    const float id = 1.f / det;
    V3<float> B = r0 * (dot(xe, a0) * id);
    if (l0 >= 4) B = B + r1 * (dot(xe, a1) * id);
    if (l1 >= 4) B = B + r2 * (dot(xe, a2) * id);
    tr = tr + B;
    rot = rot + cross(X, B);
  }
  G.gx[0] += rot.x; G.gx[1] += rot.y; G.gx[2] += rot.z;
  G.gx[3] += tr.x; G.gx[4] += tr.y; G.gx[5] += tr.z;
}

// Wrench adjoint of one soft-soft polygon (soft frame = M's; the twist moves
// N).  The quadrature and force law reverse as in wrench_adjoint; the
// contraction differs where the section is not a rigid plane:
//   section row p_M(x) - p_N(x) = 0, m = g_M - g_N, n = m / |m|: under the
//     twist N's field moves, p_N(y) <- p_N(y - (w x y + v)), so the vertex
//     obeys n . dx = -g_N . (w x x + v) / |m| and the row adds
//     -b_0 g_N / |m| to B (b_0 = xbar . a_0 / det as for the other rows);
//     the moduli enter as n . dx = (-p / E_M dE_M + p / E_N dE_N) / |m|;
//   faces of tet M fixed, faces of tet N (clip planes) moving rigidly;
//   normal: dm = -(w x g_N) + g_M dE_M / E_M - g_N dE_N / E_N, and
//     dn = (I - n n^T) dm / |m|;
//   gM = g_M . n, gN = -g_N . n (g_N turns with N, both scale with E);
//   vertex pressure p_M(x): dp = g_M . dx + p dE_M / E_M;
//   damping d(E_M, E_N) of the combined dissipation: dL/dd summed in ss.gD.
__device__ __noinline__ void wrench_adjoint_ss(AdjAcc& G, SsAdj& ss, const StepArgs& a, const PairDev& P,
                                               const FrameDev& F, const float* gF, const float* gT,
                                               const PV<float, 4>* poly, int nv, V3<float> anc, V3<float> n,
                                               const V3<float>* face, const V3<float>* clipn, float gMv, float gNv) {
  V3<float> x[kMaxPolyV], xb[kMaxPolyV];
  float pv[kMaxPolyV], pb[kMaxPolyV];
  for (int i = 0; i < nv; ++i) {
    x[i] = pv_pos(poly[i]);
    pv[i] = poly[i].p;
    xb[i] = mk(0.f, 0.f, 0.f);
    pb[i] = 0.f;
  }
  const V3<float> gFv = mk(gF[0], gF[1], gF[2]), gTv = mk(gT[0], gT[1], gT[2]);
  float A = 0.f, Sp = 0.f;
  V3<float> Sc = mk(0.f, 0.f, 0.f);
  for (int i = 1; i + 1 < nv; ++i) {
    const float ai = 0.5f * dot(cross(x[i] - x[0], x[i + 1] - x[0]), n);
    A += ai;
    Sc = Sc + (x[0] + x[i] + x[i + 1]) * (ai * (1.f / 3.f));
    Sp += ai * (pv[0] + pv[i] + pv[i + 1]) * (1.f / 3.f);
  }
  if (A == 0.f) return;
  const float iA = 1.f / A;
  const V3<float> c = Sc * iA;
  const float pc = Sp * iA;
  V3<float> nbar = mk(0.f, 0.f, 0.f), cbar = mk(0.f, 0.f, 0.f);
  float gMbar = 0.f, gNbar = 0.f, pcbar = 0.f, Abar = 0.f;
  PointBar b;
  if (a.repr == 1) {
    if (point_reverse(G, F, P.damping, P.mu, gFv, gTv, fabsf(A), anc + c, n, gMv, gNv, pc, b)) {
      Abar += A < 0.f ? -b.A : b.A;
      cbar = cbar + b.p;
      pcbar += b.p0;
      nbar = nbar + b.n;
      gMbar += b.gM;
      gNbar += b.gN;
      ss.gD += b.d;
    }
  } else {
    for (int i = 0; i < nv; ++i) {
      const int j = i + 1 == nv ? 0 : i + 1;
      const V3<float> u = x[i] - c, w = x[j] - c;
      const V3<float> cr = cross(u, w);
      const float len = norm(cr);
      const V3<float> cen = anc + (c + x[i] + x[j]) * (1.f / 3.f);
      const float p0 = pc / 3.f + pv[i] / 3.f + pv[j] / 3.f;
      if (!point_reverse(G, F, P.damping, P.mu, gFv, gTv, 0.5f * len, cen, n, gMv, gNv, p0, b)) continue;
      nbar = nbar + b.n;
      gMbar += b.gM;
      gNbar += b.gN;
      ss.gD += b.d;
      if (len > 0.f) {
        const V3<float> crb = cr * (0.5f * b.A / len);
        const V3<float> ub = cross(w, crb), wb = cross(crb, u);
        xb[i] = xb[i] + ub;
        xb[j] = xb[j] + wb;
        cbar = cbar - ub - wb;
      }
      const V3<float> c3 = b.p * (1.f / 3.f);
      cbar = cbar + c3;
      xb[i] = xb[i] + c3;
      xb[j] = xb[j] + c3;
      const float p3 = b.p0 * (1.f / 3.f);
      pcbar += p3;
      pb[i] += p3;
      pb[j] += p3;
    }
  }
  const V3<float> Scb = cbar * iA;
  const float Spb = pcbar * iA;
  Abar -= (dot(cbar, c) + pcbar * pc) * iA;
  for (int i = 1; i + 1 < nv; ++i) {
    const V3<float> e1 = x[i] - x[0], e2 = x[i + 1] - x[0];
    const V3<float> cr = cross(e1, e2);
    const float ai = 0.5f * dot(cr, n);
    const float aib = Abar + dot(Scb, x[0] + x[i] + x[i + 1]) * (1.f / 3.f) +
                      Spb * (pv[0] + pv[i] + pv[i + 1]) * (1.f / 3.f);
    const V3<float> sx = Scb * (ai * (1.f / 3.f));
    const float sp = Spb * ai * (1.f / 3.f);
    xb[0] = xb[0] + sx; xb[i] = xb[i] + sx; xb[i + 1] = xb[i + 1] + sx;
    pb[0] += sp; pb[i] += sp; pb[i + 1] += sp;
    nbar = nbar + cr * (0.5f * aib);
    const V3<float> e1b = cross(e2, n) * (0.5f * aib), e2b = cross(n, e1) * (0.5f * aib);
    xb[i] = xb[i] + e1b;
    xb[i + 1] = xb[i + 1] + e2b;
    xb[0] = xb[0] - e1b - e2b;
  }
  // normal and gradient terms
  nbar = nbar + ss.ga * gMbar - ss.gb * gNbar;
  const V3<float> np = nbar - n * dot(nbar, n);
  const float il = 1.f / ss.lm;
  V3<float> rot = cross(np, ss.gb) * il + cross(n, ss.gb) * gNbar, tr = mk(0.f, 0.f, 0.f);
  float gEa = (dot(np, ss.ga) * il + gMbar * gMv) * ss.iEa;
  float gEb = (gNbar * gNv - dot(np, ss.gb) * il) * ss.iEb;
  for (int v = 0; v < nv; ++v) {
    const V3<float> xe = xb[v] + ss.ga * pb[v];
    gEa += pb[v] * pv[v] * ss.iEa;
    const V3<float> X = anc + x[v];
    const int l0 = poly[v].lab & 15, l1 = poly[v].lab >> 4;
    const V3<float> r0 = n;
    const V3<float> r1 = l0 < 4 ? face[l0] : clipn[l0 - 4];
    const V3<float> r2 = l1 < 4 ? face[l1] : clipn[l1 - 4];
    const V3<float> a0 = cross(r1, r2), a1 = cross(r2, r0), a2 = cross(r0, r1);
    const float det = dot(r0, a0);
    const float sc = norm(r0) * norm(r1) * norm(r2);
    if (!(fabsf(det) > kDetTol * sc)) {
      // dependent rows (an edge on both bodies' surfaces): the vertex lies on
      // the line where the two faces meet, which the section contains; the
      // two face rows alone carry its motion (minimum norm: no slide along
      // the line, where its position is set by rounding in the clip)
      const float g11 = dot(r1, r1), g12 = dot(r1, r2), g22 = dot(r2, r2);
      const float gd = g11 * g22 - g12 * g12;
      if (!(gd > kDetTol * g11 * g22)) {
        if (a.adj_skip) atomicAdd(a.adj_skip, 1);
        continue;
      }
      const float q1 = dot(r1, xe), q2 = dot(r2, xe), igd = 1.f / gd;
      V3<float> B = mk(0.f, 0.f, 0.f);
      if (l0 >= 4) B = B + r1 * ((g22 * q1 - g12 * q2) * igd);
      if (l1 >= 4) B = B + r2 * ((g11 * q2 - g12 * q1) * igd);
      tr = tr + B;
      rot = rot + cross(X, B);
      continue;
    }
    const float id = 1.f / det;
    const float b0 = dot(xe, a0) * id;
    V3<float> B = ss.gb * (-b0 * il);
    if (l0 >= 4) B = B + r1 * (dot(xe, a1) * id);
    if (l1 >= 4) B = B + r2 * (dot(xe, a2) * id);
    tr = tr + B;
    rot = rot + cross(X, B);
    gEa -= b0 * pv[v] * il * ss.iEa;
    gEb += b0 * pv[v] * il * ss.iEb;
  }
  G.gx[0] += rot.x; G.gx[1] += rot.y; G.gx[2] += rot.z;
  G.gx[3] += tr.x; G.gx[4] += tr.y; G.gx[5] += tr.z;
  G.gE += gEa;
  ss.gEb += gEb;
}

__device__ __forceinline__ void adj_reduce_store(const StepArgs& a, const AdjAcc& G, int item, int lane) {
  double v[13];
#pragma unroll
  for (int i = 0; i < 6; ++i) v[i] = G.gx[i];
#pragma unroll
  for (int i = 0; i < 3; ++i) v[6 + i] = G.glin[i], v[9 + i] = G.gang[i];
  v[12] = G.gE;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int i = 0; i < 13; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < 13; ++i) a.adj_item[(size_t)item * 16 + i] = v[i];
}

// True when the step keeps its polygons as records and none overflowed.
__device__ __forceinline__ bool rec_ok(const StepArgs& a) { return a.recs != nullptr && !(*a.status & 8); }
// True when the adjoint can read the polygons the forward kept.
__device__ __forceinline__ bool recs_valid(const StepArgs& a) { return a.use_recs && rec_ok(a); }

// Recompute path (no records kept, or the record buffer overflowed): one warp
// per item repeats the forward's staging and clipping.
__global__ void __launch_bounds__(128, 4) adjoint_sr_kernel(StepArgs a) {
  if (recs_valid(a)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  SrWarpSmem& W = reinterpret_cast<SrWarpSmem*>(smem_raw)[wid];
  while (true) {
    int ie;
    const int item = next_item(a, 0, lane, ie);
    if (item >= ie) break;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    const float* gF = a.adj_pair + 8 * (size_t)it.x;
    const float* gT = gF + 3;
    AdjAcc G;
    adj_zero(G);
    const int sl = it.y, oc = it.z;
    if (F.valid) {
      stage_tri(a, P, F, oc * kCluster + lane, W.tri[lane]);
      stage_tet(a, P, sl * kCluster + lane, W.tet[lane]);
    } else {
      W.tri[lane].valid = 0;
      W.tet[lane].valid = 0;
    }
    __syncwarp();
    unsigned mask = 0;
    const TetStage& me = W.tet[lane];
    if (me.valid) {
      float mlo[3], mhi[3];
      tet_box(me, mlo, mhi);
      const int n_o = min(kCluster, P.o_n_elem - oc * kCluster);
      for (int j = 0; j < n_o; ++j) {
        const TriStage& T = W.tri[j];
        if (!T.valid || !aabb_overlap(mlo, mhi, T.lo, T.hi)) continue;
        const float margin = 4e-6f * (me.xmax + fabsf(T.o) + T.Lt);
        if (one_sided32(me.X, T.n, T.o, margin) || edge_outside32(me.X, T, me.xmax)) continue;
        mask |= 1u << j;
      }
    }
    const int total = build_queue(mask, W.q, lane);
    __syncwarp();
    const float sgn = P.s_is_m ? 1.f : -1.f;
    for (int base = 0; base < total; base += 32) {
      queue_window(mask, W.q, lane, base);
      const int k = base + lane;
      if (k >= total) continue;
      const int e = W.q[k % kQCap];
      const int i = e & 31, j = e >> 5;
      const TetStage& TS = W.tet[i];
      const TriStage& T = W.tri[j];
      float s[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q] = plane_df(T.n, T.nl, T.o, T.ol, TS.X[q][0], TS.X[q][1], TS.X[q][2]);
      constexpr float tol = (float)kNearTol;
      const bool allp = s[0] > tol && s[1] > tol && s[2] > tol && s[3] > tol;
      const bool alln = s[0] < -tol && s[1] < -tol && s[2] < -tol && s[3] < -tol;
      if (allp || alln) continue;
      TetIn<float> t;
      unstage_tet(TS, t);
      const V3<float> n = mk(T.n[0], T.n[1], T.n[2]);
      // forward polygon (the taxel keys must equal the forward's)
      PV<float, 0> poly[kMaxPolyV];
      Decide dc;
      int anc = 0;
      int nv = sr_poly_f(t, s, T, n, fmaxf(T.M, t.xmax), dc, anc, poly);
      const int tet_idx = P.s_elem_off + sl * kCluster + i;
      float gint = 0.f;
      if (dc.unc) {
        bool near;
        nv = sr_fp64(a, T, tet_idx, anc, poly, near, gint);
        orient_ccw(poly, nv, n);
      } else if (nv >= 3) {
        gint = dot(t.g, n);
        if (fabsf(gint) <= 1e-5f * t.gl) {
          double n64[3], o64;
          tri_plane64(T, n64, o64);
          gint = grad_along64(a, tet_idx, n64[0], n64[1], n64[2]);
        }
      }
      if (nv < 3) continue;
      // taxel adjoint on the forward polygon
      if (a.adj_taxel) {
        if (P.sensor0 >= 0)
          raster_keys<0>(a, P.sensor0, F.Rl, F.tl, poly, nv, t.X[anc], t.g, n, a.sensors[P.sensor0].geom == P.gs,
                         &G);
        if (P.sensor1 >= 0)
          raster_keys<0>(a, P.sensor1, F.Rl1, F.tl1, poly, nv, t.X[anc], t.g, n, a.sensors[P.sensor1].geom == P.gs,
                         &G);
      }
      if (!a.adj_wrench || !a.apply_forces) continue;
      V3<float> face[4];
      tet_face_normals(t.X, face);
      const V3<float> clipn[3] = {mk(T.en[0][0], T.en[0][1], T.en[0][2]), mk(T.en[1][0], T.en[1][1], T.en[1][2]),
                                  mk(T.en[2][0], T.en[2][1], T.en[2][2])};
      wrench_adjoint<0>(G, a, P, F, gF, gT, poly, nv, t.X[anc], n, sgn, face, clipn, t.g, gint);
    }
    __syncwarp();
    adj_reduce_store(a, G, item, lane);
  }
}

__global__ void __launch_bounds__(128, 4) adjoint_hs_kernel(StepArgs a) {
  if (recs_valid(a)) return;
  __shared__ TetStage s_tet[kNarrowWarps][kCluster];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  while (true) {
    int ie;
    const int item = next_item(a, 1, lane, ie);
    if (item >= ie) break;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    const float* gF = a.adj_pair + 8 * (size_t)it.x;
    const float* gT = gF + 3;
    AdjAcc G;
    adj_zero(G);
    const int sl = it.y;
    if (F.valid) stage_tet(a, P, sl * kCluster + lane, s_tet[wid][lane]);
    else s_tet[wid][lane].valid = 0;
    const double n64[3] = {F.R[2], F.R[5], F.R[8]};
    const double o64 = F.R[2] * F.t[0] + F.R[5] * F.t[1] + F.R[8] * F.t[2];
    const float nf[3] = {F.Rf[2], F.Rf[5], F.Rf[8]};
    const float of = (float)o64;
    bool cand;
    {
      const TetStage& me = s_tet[wid][lane];
      cand = me.valid && !one_sided32(me.X, nf, of, 4e-6f * (me.xmax + fabsf(of)));
    }
    const unsigned ballot = __ballot_sync(0xffffffffu, cand);
    const int total = __popc(ballot);
    const float sgn = P.s_is_m ? 1.f : -1.f;
    if (lane < total) {
      unsigned msk = ballot;
      for (int r = 0; r < lane; ++r) msk &= msk - 1;
      const int i = __ffs(msk) - 1;
      const TetStage& TS = s_tet[wid][i];
      double s[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q] = plane64(n64, o64, TS.X[q][0], TS.X[q][1], TS.X[q][2]);
      TetIn<float> t;
      unstage_tet(TS, t);
      const V3<float> n = mk(nf[0], nf[1], nf[2]);
      PV<float, 1> poly[kMaxPolyV];
      Decide dc;
      int anc = 0;
      int nv = hs_poly_f(t, s, n, dc, anc, poly);
      const int tet_idx = P.s_elem_off + sl * kCluster + i;
      float gint = 0.f;
      if (dc.unc) {
        bool near;
        nv = hs_fp64(a, F, tet_idx, s, anc, poly, near, gint);
        orient_ccw(poly, nv, n);
      } else if (nv >= 3) {
        gint = dot(t.g, n);
        if (fabsf(gint) <= 1e-5f * t.gl) gint = grad_along64(a, tet_idx, n64[0], n64[1], n64[2]);
      }
      if (nv >= 3) {
        if (a.adj_taxel) {
          if (P.sensor0 >= 0)
            raster_keys<1>(a, P.sensor0, F.Rl, F.tl, poly, nv, t.X[anc], t.g, n,
                           a.sensors[P.sensor0].geom == P.gs, &G);
          if (P.sensor1 >= 0)
            raster_keys<1>(a, P.sensor1, F.Rl1, F.tl1, poly, nv, t.X[anc], t.g, n,
                           a.sensors[P.sensor1].geom == P.gs, &G);
        }
        if (a.adj_wrench && a.apply_forces) {
          V3<float> face[4];
          tet_face_normals(t.X, face);
          wrench_adjoint<1>(G, a, P, F, gF, gT, poly, nv, t.X[anc], n, sgn, face, face, t.g, gint);
        }
      }
    }
    __syncwarp();
    adj_reduce_store(a, G, item, lane);
  }
}

// Soft-soft pairs (no records are kept for them): one warp per item repeats
// the forward's staging and clipping and reverses each polygon.  The item's
// sums go to adj_item: the 13 of adj_reduce_store, then dL/dE_N and
// dL/d(damping); here entry 12 is dL/dE_M itself.
__global__ void __launch_bounds__(128, 2) adjoint_ss_kernel(StepArgs a) {
  __shared__ TetBStage s_tb[kNarrowWarps][kCluster];
  __shared__ TetStage s_tet[kNarrowWarps][kCluster];
  __shared__ unsigned short s_q[kNarrowWarps][kQCap];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  while (true) {
    int ie;
    const int item = next_item(a, 2, lane, ie);
    if (item >= ie) break;
    const int4 it = a.items[item];
    const PairDev& P = a.pairs[it.x];
    const FrameDev& F = a.frames[it.x];
    const float* gF = a.adj_pair + 8 * (size_t)it.x;
    const float* gT = gF + 3;
    AdjAcc G;
    adj_zero(G);
    SsAdj ss;
    ss.gEb = ss.gD = 0.f;
    ss.iEa = 1.f / P.E_s;
    ss.iEb = 1.f / P.E_o;
    const int sl = it.y, oc = it.z;
    unsigned mask;
    const int total = ss_stage_item(a, P, F, sl, oc, s_tb[wid], s_tet[wid], s_q[wid], lane, mask);
    for (int base = 0; base < total; base += 32) {
      queue_window(mask, s_q[wid], lane, base);
      const int k = base + lane;
      if (k >= total) continue;
      const int e = s_q[wid][k % kQCap];
      const int i = e & 31, j = e >> 5;
      const TetStage& TS = s_tet[wid][i];
      const TetBStage& B = s_tb[wid][j];
      TetIn<float> t;
      unstage_tet(TS, t);
      PV<float, 4> poly[kMaxPolyV];
      int anc = 0, flags = 0;
      V3<float> nrm;
      float gM, gN;
      const int ta_idx = P.s_elem_off + sl * kCluster + i, tb_idx = P.o_elem_off + oc * kCluster + j;
      const int nv = ss_element_pair(a, F, t, B, ta_idx, tb_idx, poly, anc, nrm, gM, gN, flags);
      if (nv < 3) continue;
      ss.ga = t.g;
      ss.gb = mk(B.g[0], B.g[1], B.g[2]);
      ss.lm = norm(ss.ga - ss.gb);
      // taxel adjoint on the forward polygon (same keys as the forward's)
      if (a.adj_taxel) {
        if (P.sensor0 >= 0)
          raster_keys<4, true>(a, P.sensor0, F.Rl, F.tl, poly, nv, t.X[anc], t.g, nrm,
                               a.sensors[P.sensor0].geom == P.gs, &G, &ss);
        if (P.sensor1 >= 0)
          raster_keys<4, true>(a, P.sensor1, F.Rl1, F.tl1, poly, nv, t.X[anc], t.g, nrm,
                               a.sensors[P.sensor1].geom == P.gs, &G, &ss);
      }
      if (!a.adj_wrench || !a.apply_forces) continue;
      V3<float> face[4];
      tet_face_normals(t.X, face);
      const V3<float> clipn[4] = {mk(B.pn[0][0], B.pn[0][1], B.pn[0][2]), mk(B.pn[1][0], B.pn[1][1], B.pn[1][2]),
                                  mk(B.pn[2][0], B.pn[2][1], B.pn[2][2]), mk(B.pn[3][0], B.pn[3][1], B.pn[3][2])};
      wrench_adjoint_ss(G, ss, a, P, F, gF, gT, poly, nv, t.X[anc], nrm, face, clipn, gM, gN);
    }
    __syncwarp();
    adj_reduce_store(a, G, item, lane);
    float v[2] = {ss.gEb, ss.gD};
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
      for (int q = 0; q < 2; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if (lane == 0) {
      a.adj_item[(size_t)item * 16 + 13] = v[0];
      a.adj_item[(size_t)item * 16 + 14] = v[1];
    }
  }
}

// ---- record path ------------------------------------------------------------
// Records are kept in the order warps reached the counter; their gradients
// are stored in pair order (items are ordered by pair): slot = first record
// of the item (exclusive scan of the items' polygon counts) + sequence number.
// Soft-soft items keep no records and are left out of the scan.
__device__ __forceinline__ int rec_items_end(const StepArgs& a) {
  const int total = *a.item_total;
  return min(a.unit_off[a.type_unit_begin[2]], total);
}

// Items per thread of the slot scan (a tile is kBpBlock x kSlotItems items).
constexpr int kSlotItems = 4;

// Each item's first slot in one pass: a block per tile of kBpBlock x
// kSlotItems items (tiles taken in order from a counter) scans its items'
// polygon counts and adds the tiles before it (decoupled look-back,
// tile_lookback).  Tiles past the last record-keeping item return at once
// (no tile that is needed waits on them); the tile holding that item gives
// the items from rec_items_end on (soft-soft, no records) and the end
// sentinel the grand total.
__global__ void poly_slots_kernel(StepArgs a) {
  if (!rec_ok(a)) return;
  __shared__ int tile_s, excl_s, tot;
  if (threadIdx.x == 0) tile_s = atomicAdd(a.tile_ctr + 1, 1);
  __syncthreads();
  const int tile = tile_s;
  const int end = rec_items_end(a);
  constexpr int kTile = kBpBlock * kSlotItems;
  const int last = end > 0 ? (end - 1) / kTile : 0;
  if (tile > last) return;
  const int i0 = tile * kTile + threadIdx.x * kSlotItems;
  int v[kSlotItems], sum = 0;
#pragma unroll
  for (int j = 0; j < kSlotItems; ++j) {
    v[j] = i0 + j < end ? a.item_out[i0 + j].n_poly : 0;
    sum += v[j];
  }
  int ex = block_excl_scan(sum, &tot);
  if (threadIdx.x == 0) excl_s = tile_lookback(a.poly_tiles, tile, tot, a.status);
  __syncthreads();
  ex += excl_s;
#pragma unroll
  for (int j = 0; j < kSlotItems; ++j) {
    if (i0 + j < end) a.item_poly_off[i0 + j] = ex;
    ex += v[j];
  }
  if (tile == last) {
    const int total = *a.item_total, grand = excl_s + tot;
    for (int k = end + threadIdx.x; k <= total; k += blockDim.x) a.item_poly_off[k] = grand;
  }
}

// ---- record kernels: a group of G lanes per kept polygon ------------------
// The lanes of a group share the polygon's work: its quadrature points
// (kTriangle: one fan triangle per lane), its ray samples (strided over the
// bounding box), and in the adjoint one vertex per lane.  Polygons of up to
// 4 vertices (triangles and quads, about 99 % of them) take groups of 4
// lanes, larger ones groups of 8.  Group sums use a fixed shuffle order, so
// results are deterministic; a polygon's sums are the same in either group
// size (the lanes past its vertices add zeros).
constexpr int kGroup = 8;        // lanes per polygon of more than 4 vertices
constexpr int kGroupSmall = 4;   // lanes per polygon of at most 4 vertices

template <int G>
__device__ __forceinline__ float gsum(float v) {
  if constexpr (G >= 8) v += __shfl_xor_sync(0xffffffffu, v, 4);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}
template <int G>
__device__ __forceinline__ V3<float> gsum3(V3<float> v) { return mk(gsum<G>(v.x), gsum<G>(v.y), gsum<G>(v.z)); }

__device__ __forceinline__ float4 rec_vtx(const AdjPoly& R, int i) { return *reinterpret_cast<const float4*>(R.v[i]); }
__device__ __forceinline__ V3<float> rec_pos(const AdjPoly& R, int i) {
  const float4 v = rec_vtx(R, i);
  return mk(v.x, v.y, v.z);
}

// Polygon sums of the quadrature: signed area A, the
// area-weighted centroid c and the pressure pc there, shared by the group:
// lane t adds fan triangle (0, t, t+1); fixed-order shuffle sums.  Every
// lane of the warp calls it.
template <int G>
__device__ __forceinline__ void rec_fan_group(const AdjPoly& R, int nv, V3<float> n, int sub, float& A, V3<float>& c,
                                              float& pc) {
  float ai = 0.f, pp = 0.f;
  V3<float> cc = mk(0.f, 0.f, 0.f);
  if (sub >= 1 && sub + 1 < nv) {
    const float4 v0 = rec_vtx(R, 0), vi = rec_vtx(R, sub), vj = rec_vtx(R, sub + 1);
    const V3<float> x0 = mk(v0.x, v0.y, v0.z), xi = mk(vi.x, vi.y, vi.z), xj = mk(vj.x, vj.y, vj.z);
    ai = 0.5f * dot(cross(xi - x0, xj - x0), n);
    cc = (x0 + xi + xj) * (ai * (1.f / 3.f));
    pp = ai * (v0.w + vi.w + vj.w) * (1.f / 3.f);
  }
  A = gsum<G>(ai);
  c = gsum3<G>(cc);
  pc = gsum<G>(pp);
}

// The lane's share of a kept polygon's forces (its quadrature point).
// Every lane of the warp calls it (shuffles); `on`: the group holds a polygon.
template <int G, int kRepr>
__device__ __forceinline__ void rec_forces_part(const StepArgs& a, const AdjPoly& R, int sub, bool on, Acc& ac) {
  const PairDev& P = a.pairs[R.pair];
  const FrameDev& F = a.frames[R.pair];
  const int nv = on ? R.nv : 0;
  const V3<float> anc = mk(R.anc[0], R.anc[1], R.anc[2]);
  const V3<float> nc = mk(R.n[0], R.n[1], R.n[2]) * (P.s_is_m ? 1.f : -1.f);
  const float gM = P.s_is_m ? R.gint : INFINITY, gN = P.s_is_m ? INFINITY : R.gint;
  float A, pcen;
  V3<float> c;
  rec_fan_group<G>(R, nv, nc, sub, A, c, pcen);
  if (!on) return;
  if (A != 0.f) {
    c = c * (1.f / A);
    pcen /= A;
  } else {
    c = mk(0.f, 0.f, 0.f);
    pcen = 0.f;
    for (int i = 0; i < nv; ++i) {
      c = c + rec_pos(R, i) * (1.f / nv);
      pcen += rec_vtx(R, i).w / nv;
    }
  }
  if constexpr (kRepr == 1) {
    if (sub == 0) point_force(ac, F, P.damping, P.mu, a.apply_forces, fabsf(A), anc + c, nc, gM, gN, pcen);
  } else if (sub < nv) {
    const int j = sub + 1 == nv ? 0 : sub + 1;
    const float4 vi = rec_vtx(R, sub), vj = rec_vtx(R, j);
    const V3<float> xi = mk(vi.x, vi.y, vi.z), xj = mk(vj.x, vj.y, vj.z);
    const float Ai = 0.5f * norm(cross(xi - c, xj - c));
    const V3<float> cen = anc + (c + xi + xj) * (1.f / 3.f);
    const float p0 = pcen / 3.f + vi.w / 3.f + vj.w / 3.f;
    point_force(ac, F, P.damping, P.mu, a.apply_forces, Ai, cen, nc, gM, gN, p0);
  }
}

// raster_prepare for a kept polygon, shared by its group of G lanes:
// lane k transforms vertex k into the sensor frame and the group exchanges
// them by shuffles (the group's lanes follow one control path, so the
// shuffles name only the group's lanes); divisions are reciprocal products.
// The forward and the adjoint both prepare through it, so they compute the
// same sample keys.
template <int G>
__device__ __forceinline__ bool raster_prepare_group(const StepArgs& a, const SensorDev& S, const float* Rl,
                                                     const float* tl, const AdjPoly& R, V3<float> anc,
                                                     V3<float> g_soft, int sub, RasterPoly& rp) {
  const int nv = R.nv;
  // a group of G lanes holds polygons of at most G vertices: the loops stop
  // there (the vertices past nv add nothing)
  constexpr int MV = G < kMaxPolyV ? G : kMaxPolyV;
  const int base = (threadIdx.x & 31) & ~(G - 1);
  const unsigned gm = ((1u << G) - 1u) << base;
  float mx = 0.f, my = 0.f, mz = 0.f, mp = 0.f;
  if (sub < nv) {
    const float4 v = rec_vtx(R, sub);
    const float X = __fadd_rn(anc.x, v.x), Y = __fadd_rn(anc.y, v.y), Z = __fadd_rn(anc.z, v.z);
    mx = __fadd_rn(dot3_rn(Rl, X, Y, Z), tl[0]);
    my = __fadd_rn(dot3_rn(Rl + 3, X, Y, Z), tl[1]);
    mz = __fadd_rn(dot3_rn(Rl + 6, X, Y, Z), tl[2]);
    mp = v.w;
  }
  float lz[kMaxPolyV];
  float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
#pragma unroll
  for (int i = 0; i < MV; ++i) {
    rp.lx[i] = __shfl_sync(gm, mx, base + i);
    rp.ly[i] = __shfl_sync(gm, my, base + i);
    lz[i] = __shfl_sync(gm, mz, base + i);
    if (i < nv) {
      mnx = fminf(mnx, rp.lx[i]); mxx = fmaxf(mxx, rp.lx[i]);
      mny = fminf(mny, rp.ly[i]); mxy = fmaxf(mxy, rp.ly[i]);
    }
  }
  rp.p0 = __shfl_sync(gm, mp, base);
  float A2 = 0.f;
#pragma unroll
  for (int i = 1; i + 1 < MV; ++i)
    if (i + 1 < nv)
      A2 = __fadd_rn(A2, __fsub_rn(__fmul_rn(__fsub_rn(rp.lx[i], rp.lx[0]), __fsub_rn(rp.ly[i + 1], rp.ly[0])),
                                   __fmul_rn(__fsub_rn(rp.ly[i], rp.ly[0]), __fsub_rn(rp.lx[i + 1], rp.lx[0]))));
  if (!(fabsf(A2) >= 1e-10f)) return false;
  rp.pos = A2 > 0.f;
  // the polygon lies in its triangle's (or the half-space's) plane: the
  // record's unit normal, in the sensor frame
  const float nx = dot3_rn(Rl, R.n[0], R.n[1], R.n[2]);
  const float ny = dot3_rn(Rl + 3, R.n[0], R.n[1], R.n[2]);
  const float nz = dot3_rn(Rl + 6, R.n[0], R.n[1], R.n[2]);
  if (!(fabsf(nz) > 0.f)) return false;
  const float inz = __frcp_rn(nz);
  rp.zx = __fmul_rn(-nx, inz);   // dz/dx, dz/dy on the plane
  rp.zy = __fmul_rn(-ny, inz);
  const float glx = dot3_rn(Rl, g_soft.x, g_soft.y, g_soft.z);
  const float gly = dot3_rn(Rl + 3, g_soft.x, g_soft.y, g_soft.z);
  const float glz = dot3_rn(Rl + 6, g_soft.x, g_soft.y, g_soft.z);
  rp.px = __fadd_rn(glx, __fmul_rn(glz, rp.zx));   // dp/dx, dp/dy on the plane
  rp.py = __fadd_rn(gly, __fmul_rn(glz, rp.zy));
  rp.lz0 = lz[0];
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  const float x0 = sx[0], dx = S.nx > 1 ? __fsub_rn(sx[1], sx[0]) : 1.f;
  const float y0 = sy[0], dy = S.ny > 1 ? __fsub_rn(sy[1], sy[0]) : 1.f;
  const float idx = __frcp_rn(dx), idy = __frcp_rn(dy);
  // the sample box, widened by 1e-3 of a sample step (a conservative bound:
  // inclusion is decided by the probe)
  const float fx0 = ceilf(__fsub_rn(__fmul_rn(__fsub_rn(mnx, x0), idx), 1e-3f));
  const float fx1 = floorf(__fadd_rn(__fmul_rn(__fsub_rn(mxx, x0), idx), 1e-3f));
  const float fy0 = ceilf(__fsub_rn(__fmul_rn(__fsub_rn(mny, y0), idy), 1e-3f));
  const float fy1 = floorf(__fadd_rn(__fmul_rn(__fsub_rn(mxy, y0), idy), 1e-3f));
  if (!(fx1 >= 0.f && fy1 >= 0.f && fx0 <= (float)(S.nx - 1) && fy0 <= (float)(S.ny - 1))) return false;
  rp.X0 = max(0, (int)fx0); rp.X1 = min(S.nx - 1, (int)fx1);
  rp.Y0 = max(0, (int)fy0); rp.Y1 = min(S.ny - 1, (int)fy1);
  rp.nv = nv;
#pragma unroll
  for (int i = 0; i < MV; ++i) {
    const bool last = i + 1 >= nv;
    const float nxv = last ? rp.lx[0] : rp.lx[i + 1 < MV ? i + 1 : 0];
    const float nyv = last ? rp.ly[0] : rp.ly[i + 1 < MV ? i + 1 : 0];
    rp.ex[i] = __fsub_rn(nxv, rp.lx[i]);
    rp.ey[i] = __fsub_rn(nyv, rp.ly[i]);
  }
  return true;
}

// The lane's share of a kept polygon's ray samples on one sensor (side 0:
// the pair's sensor0, 1: sensor1), forward: binning with slot keys; lane 0
// keeps the polygon's plane, pressure model and sample box for the taxel
// pass and the adjoint.
template <int G>
__device__ __forceinline__ void rec_rays_fwd(const StepArgs& a, const AdjPoly& R, int dst, int side, int sid,
                                             const float* Rl, const float* tl, int sub) {
  const SensorDev S = a.sensors[sid];
  RasterPoly rp;
  float4* sp = a.slot_press + 6 * (size_t)dst + 3 * side;
  if (!raster_prepare_group<G>(a, S, Rl, tl, R, mk(R.anc[0], R.anc[1], R.anc[2]), mk(R.g[0], R.g[1], R.g[2]), sub,
                               rp)) {
    if (sub == 0) sp[2] = make_float4(__int_as_float(1), __int_as_float(0), __int_as_float(1), __int_as_float(0));
    return;
  }
  if (sub == 0) {
    sp[0] = make_float4(rp.lx[0], rp.ly[0], rp.p0, rp.px);
    sp[1] = make_float4(rp.py, rp.lz0, rp.zx, rp.zy);
    sp[2] = make_float4(__int_as_float(rp.X0), __int_as_float(rp.X1), __int_as_float(rp.Y0), __int_as_float(rp.Y1));
    if (a.sens_box && rp.X0 <= rp.X1 && rp.Y0 <= rp.Y1) grow_box(a.sens_box + sid, rp.X0, rp.X1, rp.Y0, rp.Y1);
  }
  unsigned long long* smp = a.samples + S.sample_off;
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  const int nY = rp.Y1 - rp.Y0 + 1;
  const int cnt = (rp.X1 - rp.X0 + 1) * nY;
  if (nY <= 0 || cnt <= 0) return;   // the box holds no sample
  // sample idx = sub, sub + G, ... of the box, row-major in (X, Y):
  // one division up front, then stepped
  const int dq = G / nY, dr = G % nY;
  int X = rp.X0 + sub / nY, Y = rp.Y0 + sub % nY;
  for (int idx = sub; idx < cnt; idx += G, X += dq, Y += dr) {
    if (Y > rp.Y1) { Y -= nY; ++X; }
    float t, z, pr;
    if (raster_probe<(G < kMaxPolyV ? G : kMaxPolyV)>(rp, S, sx[X], sy[Y], t, z, pr))
      atomicMin(&smp[(size_t)X * S.ny + Y], key_slot(t, dst, side));
  }
}

// Adjoint of the samples a kept polygon won on one sensor: the forward's
// plane and box; the won samples are known by their keys (the low word names
// the polygon and side), so no inside test is needed.
template <int Gs>
__device__ __forceinline__ void rec_rays_adj(const StepArgs& a, const AdjPoly& R, int dst, int side, int sid,
                                             const float* Rl, const float* tl, int soft_is_sensor, int sub,
                                             AdjAcc& G) {
  const float4* sp = a.slot_press + 6 * (size_t)dst + 3 * side;
  const float4 bx = sp[2];
  const int X0 = __float_as_int(bx.x), X1 = __float_as_int(bx.y), Y0 = __float_as_int(bx.z),
            Y1 = __float_as_int(bx.w);
  const int nY = Y1 - Y0 + 1;
  const int cnt = (X1 - X0 + 1) * nY;
  if (X0 > X1 || nY <= 0 || cnt <= 0) return;
  const SensorDev S = a.sensors[sid];
  const float4 m0 = sp[0], m1 = sp[1];
  const unsigned long long* smp = a.samples + S.sample_off;
  const float* sx = a.samp_coord + S.samp_off_x;
  const float* sy = a.samp_coord + S.samp_off_y;
  const unsigned own = (unsigned)key_slot(0.f, dst, side);
  const V3<float> g = mk(R.g[0], R.g[1], R.g[2]);
  const int dq = Gs / nY, dr = Gs % nY;
  // the lane's samples two at a time: both keys in flight before either is
  // tested (adjoint 0.506 -> 0.492 ms), one copy of the won-sample code
  int X = X0 + sub / nY, Y = Y0 + sub % nY;
  for (int idx = sub; idx < cnt; idx += 2 * Gs) {
    int Xb = X + dq, Yb = Y + dr;
    if (Yb > Y1) { Yb -= nY; ++Xb; }
    const bool hb = idx + Gs < cnt;
    const unsigned ka = (unsigned)smp[(size_t)X * S.ny + Y];
    const unsigned kb = hb ? (unsigned)smp[(size_t)Xb * S.ny + Yb] : 0u;   // own is never 0
#pragma unroll 1
    for (int u = 0; u < 2; ++u) {
      if ((u ? kb : ka) != own) continue;   // won by another polygon, or missed
      const int Xs = u ? Xb : X, Ys = u ? Yb : Y;
      const float qx = sx[Xs], qy = sy[Ys];
      const float z = raster_height(m0.x, m0.y, m1.y, m1.z, m1.w, qx, qy);
      const float pr = raster_pressure(m0.x, m0.y, m0.z, m0.w, m1.x, qx, qy);
      sample_adjoint<false>(a, S, Rl, tl, qx, qy, z, pr, Xs, Ys, g, mk(R.n[0], R.n[1], R.n[2]), soft_is_sensor, G,
                            nullptr);
    }
    X = Xb + dq;
    Y = Yb + dr;
    if (Y > Y1) { Y -= nY; ++X; }
  }
}

// The pair's sensors (one per geom at most), a side at a time (one copy of
// the ray code).
template <int Gs>
__device__ __forceinline__ void rec_rays(const StepArgs& a, const AdjPoly& R, int dst, int sub, AdjAcc* G) {
  const PairDev& P = a.pairs[R.pair];
  const FrameDev& F = a.frames[R.pair];
#pragma unroll 1
  for (int side = 0; side < 2; ++side) {
    const int sid = side ? P.sensor1 : P.sensor0;
    if (sid < 0) continue;
    const float* Rl = side ? F.Rl1 : F.Rl;
    const float* tl = side ? F.tl1 : F.tl;
    if (!G) rec_rays_fwd<Gs>(a, R, dst, side, sid, Rl, tl, sub);
    else rec_rays_adj<Gs>(a, R, dst, side, sid, Rl, tl, a.sensors[sid].geom == P.gs, sub, *G);
  }
}

// Record r's pair-ordered slot (-1: none).
__device__ __forceinline__ int rec_slot(const StepArgs& a, int r, int n) {
  if (r >= n) return -1;
  const int2 key = a.rec_key[r];
  const int dst = a.item_poly_off[key.x] + key.y;
  return dst >= 0 && dst < a.rec_cap ? dst : -1;
}

// The polygons of more than 4 vertices among a warp's 8 records of one
// round (records base .. base + 7, record k held by lanes 4k .. 4k + 3):
// lane 4k flags record k (`flag`) and holds its slot (`dst`); the warp's
// four 8-lane groups take the flagged records four at a time in record
// order.  Calls body(r, dst, on, sub) once per turn on every lane (`on`:
// the lane's group holds a record this turn).  Every lane of the warp calls
// it.
template <class Body>
__device__ __forceinline__ void rec_large_turns(bool flag, int base, int dst, int lane, Body body) {
  unsigned big = __ballot_sync(0xffffffffu, flag);
  while (big) {
    unsigned m = big;
    for (int q = 0; q < (lane >> 3); ++q) m &= m - 1;
    const int pick = m ? __ffs(m) - 1 : 0;
    const bool on = m != 0;
    const int dst8 = __shfl_sync(0xffffffffu, dst, pick);
    body(base + (pick >> 2), dst8, on, lane & (kGroup - 1));
#pragma unroll
    for (int q = 0; q < 32 / kGroup; ++q) big &= big - 1;
  }
}

// The adjoint defers the polygons of more than 4 vertices (about 1 in 100)
// across rounds instead: lane i of the warp holds the i-th deferred
// (record, slot), and whenever four are held the warp's four 8-lane groups
// take them in one turn.  A turn in every round that held one (about 1
// round in 13) left most of the warp idle (adjoint 0.483 -> 0.473 ms; the
// forward record pass measured 0.319 -> 0.325 ms with it, at its 72-register
// bound, and keeps the turns in the round).  Each polygon writes only its
// own slot, so the order does not change any result.
struct LargeQueue {
  int r, dst, n;   // this lane's entry; entries held (the same on every lane)
};

// Appends the records whose lane 4k sets `flag` (record r, slot dst), in
// lane order.  Every lane of the warp calls it.
__device__ __forceinline__ void large_push(LargeQueue& q, bool flag, int r, int dst, int lane) {
  const unsigned big = __ballot_sync(0xffffffffu, flag);
  const int cnt = __popc(big), j = lane - q.n;
  unsigned m = big;
  for (int t = 0; t < j && t < cnt; ++t) m &= m - 1;
  const bool take = j >= 0 && j < cnt;
  const int src = take ? __ffs(m) - 1 : lane;
  const int rr = __shfl_sync(0xffffffffu, r, src), dd = __shfl_sync(0xffffffffu, dst, src);
  if (take) {
    q.r = rr;
    q.dst = dd;
  }
  q.n += cnt;
}

// Turns of four held polygons while four are held (all held ones when
// `all`): body(r, dst, on, sub) on every lane, `on` when the lane's 8-lane
// group holds one this turn.  Every lane of the warp calls it.
template <class Body>
__device__ __forceinline__ void large_turns(LargeQueue& q, bool all, int lane, Body body) {
  while (q.n >= 4 || (all && q.n > 0)) {
    const int g = lane >> 3;
    const int r8 = __shfl_sync(0xffffffffu, q.r, g), d8 = __shfl_sync(0xffffffffu, q.dst, g);
    body(r8, d8, g < q.n, lane & (kGroup - 1));
    q.r = __shfl_down_sync(0xffffffffu, q.r, 4);
    q.dst = __shfl_down_sync(0xffffffffu, q.dst, 4);
    q.n = max(0, q.n - 4);
  }
}

// The forward pass over one kept polygon by a group of G lanes: forces into
// its pair-ordered slot, then the sensors' rays.
template <int G, int kRepr>
__device__ __forceinline__ void rec_fwd_one(const StepArgs& a, int r, int dst, bool on, int sub) {
  const AdjPoly& R = a.recs[on ? r : 0];
  Acc ac;
  acc_zero(ac);
  rec_forces_part<G, kRepr>(a, R, sub, on, ac);
  float v[9] = {ac.F[0], ac.F[1], ac.F[2], ac.T[0], ac.T[1], ac.T[2], ac.area, ac.fn0, (float)ac.n_faces};
#pragma unroll
  for (int k = 0; k < 9; ++k) v[k] = gsum<G>(v[k]);
  if (on && sub == 0) {
    a.rec_perm[dst] = r;
    RecOut o;
    o.F[0] = v[0]; o.F[1] = v[1]; o.F[2] = v[2];
    o.T[0] = v[3]; o.T[1] = v[4]; o.T[2] = v[5];
    o.area = v[6]; o.fn0 = v[7]; o.n_faces = (int)v[8];
    o.pad[0] = o.pad[1] = o.pad[2] = 0;
    a.rec_out[dst] = o;
  }
  __syncwarp();   // the groups enter the shuffled ray preparation together
  if (on) rec_rays<G>(a, R, dst, sub, nullptr);
}

// The next round's eight records (8 x 288 B: 18 lines of 128 B), one line
// per lane, and their keys, requested into L1 before this round's work: the
// record kernels wait on their records' loads more than on arithmetic
// (adjoint 0.57 -> 0.54 ms when it prefetched too; into L2 alone gained a
// little less).
__device__ __forceinline__ void prefetch_records(const StepArgs& a, int base, int n, int lane) {
  if (base >= n) return;
  const int nrec = min(8, n - base);
  const char* p = reinterpret_cast<const char*>(a.recs + base);
  const int lines = (nrec * (int)sizeof(AdjPoly) + 127) / 128;
  if (lane < lines) asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 128 * lane));
  if (lane == 31) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.rec_key + base));
}

// The adjoint's round of eight records staged in shared memory instead,
// double-buffered per warp (the next round's copies in flight while this
// round runs).  The copies bypass L1 and are marked evict-first in L2: the
// pass reads each record once, and what it shares with the other passes
// (sample keys, pressure models, gradients) should stay in L2.  Adjoint
// 0.492 -> 0.483 ms against the L1 prefetch; the forward record pass
// measured 0.320 -> 0.323 ms with it and keeps the prefetch.
struct RecStage {
  AdjPoly r[2][8];
};

__device__ __forceinline__ unsigned long long evict_first_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// Records base .. base + 7 (those below n) into dst, 16 B per copy across
// the lanes, as one commit group (empty past the end); lane 31 requests the
// round's stored slots into L1.
__device__ __forceinline__ void stage_round(const StepArgs& a, AdjPoly* dst, int base, int n, int lane,
                                            unsigned long long pol) {
  if (base < n) {
    const int chunks = min(8, n - base) * (int)(sizeof(AdjPoly) / 16);
    const char* src = reinterpret_cast<const char*>(a.recs + base);
    const unsigned d0 = (unsigned)__cvta_generic_to_shared(dst);
    for (int c = lane; c < chunks; c += 32)
      asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(d0 + 16 * c),
                   "l"(src + 16 * c), "l"(pol)
                   : "memory");
    if (lane == 31) asm volatile("prefetch.global.L1 [%0];" ::"l"(a.rec_dst + base));
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// This round's group complete on every lane (the next one may be in flight).
__device__ __forceinline__ void stage_wait() {
  asm volatile("cp.async.wait_group 1;" ::: "memory");
  __syncwarp();
}

// Forward pass over the kept polygons, eight records per warp and round:
// those of up to 4 vertices in groups of 4 lanes, the rest after them in
// groups of 8.
// kRepr: the quadrature (0 kTriangle, 1 kPolygon), fixed per launch.
// 8 CTAs per SM (64 registers, 28 B spilled) measured faster than 7 (72) and
// 6: 0.319 -> 0.313 ms.
template <int kRepr>
__global__ void __launch_bounds__(128, 8) rec_forward_kernel(StepArgs a) {
  if (!rec_ok(a)) return;   // records incomplete: the step is re-run after growth
  const int n = min(*a.rec_count, a.rec_cap);
  const int lane = threadIdx.x & 31, sub = lane & (kGroupSmall - 1), grp = lane / kGroupSmall;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  constexpr int kPer = 32 / kGroupSmall;
  for (int base = warp * kPer; base < n; base += n_warps * kPer) {
    prefetch_records(a, base + n_warps * kPer, n, lane);
    const int r = base + grp;
    const int dst = rec_slot(a, r, n);
    if (r < n && sub == 0) a.rec_dst[r] = dst;   // the adjoint's lookup
    const int nv = dst >= 0 ? a.recs[r].nv : 0;
    rec_fwd_one<kGroupSmall, kRepr>(a, r, dst, dst >= 0 && nv <= kGroupSmall, sub);
    __syncwarp();
    rec_large_turns(dst >= 0 && nv > kGroupSmall && sub == 0, base, dst, lane,
                    [&](int r8, int dst8, bool on8, int sub8) { rec_fwd_one<kGroup, kRepr>(a, r8, dst8, on8, sub8); });
  }
}

// Wrench adjoint of one kept polygon, distributed over the group (the
// serial form is wrench_adjoint): lane k reverses the quadrature point of
// fan triangle k, lane v owns vertex v for the fan reverse and the
// constraint contraction.  Every lane of the warp calls it (shuffles).
template <int Gs, int kRepr>
__device__ __forceinline__ void rec_wrench_group(const StepArgs& a, const AdjPoly& R, bool on, int lane, int sub,
                                                 AdjAcc& G) {
  const int nv = on ? R.nv : 0;
  const int pair = on ? R.pair : 0;
  const PairDev& P = a.pairs[pair];
  const FrameDev& F = a.frames[pair];
  const float sgn = P.s_is_m ? 1.f : -1.f;
  const V3<float> n = mk(R.n[0], R.n[1], R.n[2]), ns = n * sgn;
  const V3<float> g = mk(R.g[0], R.g[1], R.g[2]);
  const V3<float> anc = mk(R.anc[0], R.anc[1], R.anc[2]);
  const float gint = R.gint;
  const float* gF = a.adj_pair + 8 * (size_t)pair;
  const V3<float> gFv = mk(gF[0], gF[1], gF[2]), gTv = mk(gF[3], gF[4], gF[5]);
  float A = 0.f, pc = 0.f;
  V3<float> c = mk(0.f, 0.f, 0.f);
  rec_fan_group<Gs>(R, nv, ns, sub, A, c, pc);
  const bool live = on && A != 0.f;
  const float iA = live ? 1.f / A : 0.f;
  c = c * iA;
  pc = pc * iA;
  const float gMv = P.s_is_m ? gint : INFINITY, gNv = P.s_is_m ? INFINITY : gint;
  // quadrature points
  V3<float> xbi = mk(0.f, 0.f, 0.f), xbj = xbi, nbar = xbi, cbar = xbi;
  float pbi = 0.f, pbj = 0.f, gbar = 0.f, pcbar = 0.f, Abar = 0.f;
  PointBar b;
  if (live) {
    if constexpr (kRepr == 1) {
      if (sub == 0 && point_reverse(G, F, P.damping, P.mu, gFv, gTv, fabsf(A), anc + c, ns, gMv, gNv, pc, b)) {
        Abar += A < 0.f ? -b.A : b.A;
        cbar = cbar + b.p;
        pcbar += b.p0;
        nbar = nbar + b.n;
        gbar += P.s_is_m ? b.gM : b.gN;
      }
    } else if (sub < nv) {
      const int j = sub + 1 == nv ? 0 : sub + 1;
      const float4 vi = rec_vtx(R, sub), vj = rec_vtx(R, j);
      const V3<float> xi = mk(vi.x, vi.y, vi.z), xj = mk(vj.x, vj.y, vj.z);
      const V3<float> u = xi - c, w = xj - c;
      const V3<float> cr = cross(u, w);
      const float len = norm(cr);
      const V3<float> cen = anc + (c + xi + xj) * (1.f / 3.f);
      const float p0 = pc / 3.f + vi.w / 3.f + vj.w / 3.f;
      if (point_reverse(G, F, P.damping, P.mu, gFv, gTv, 0.5f * len, cen, ns, gMv, gNv, p0, b)) {
        nbar = nbar + b.n;
        gbar += P.s_is_m ? b.gM : b.gN;
        if (len > 0.f) {   // A_e = |u x w| / 2
          const V3<float> crb = cr * (0.5f * b.A / len);
          const V3<float> ub = cross(w, crb), wb = cross(crb, u);
          xbi = xbi + ub;
          xbj = xbj + wb;
          cbar = cbar - ub - wb;
        }
        const V3<float> c3 = b.p * (1.f / 3.f);
        cbar = cbar + c3;
        xbi = xbi + c3;
        xbj = xbj + c3;
        const float p3 = b.p0 * (1.f / 3.f);
        pcbar += p3;
        pbi += p3;
        pbj += p3;
      }
    }
  }
  nbar = gsum3<Gs>(nbar);
  cbar = gsum3<Gs>(cbar);
  gbar = gsum<Gs>(gbar);
  pcbar = gsum<Gs>(pcbar);
  Abar = gsum<Gs>(Abar);
  // vertex v collects its share as "i" (own lane) and as "j" (lane v - 1)
  const int src = (lane & ~(Gs - 1)) | (sub == 0 ? (nv > 0 ? nv - 1 : 0) : sub - 1);
  V3<float> xb = xbi + mk(__shfl_sync(0xffffffffu, xbj.x, src), __shfl_sync(0xffffffffu, xbj.y, src),
                          __shfl_sync(0xffffffffu, xbj.z, src));
  float pb = pbi + __shfl_sync(0xffffffffu, pbj, src);
  // c = Sc / A, pc = Sp / A
  const V3<float> Scb = cbar * iA;
  const float Spb = pcbar * iA;
  Abar -= (dot(cbar, c) + pcbar * pc) * iA;
  {
    // fan triangle t = sub reversed by its lane: its shares go to vertex 0
    // (a group sum), vertex t (this lane) and vertex t+1 (the next lane)
    V3<float> nb = mk(0.f, 0.f, 0.f), to0 = nb, to_next = nb;
    float p_to0 = 0.f, p_next = 0.f;
    if (live && sub >= 1 && sub + 1 < nv) {
      const float4 v0 = rec_vtx(R, 0), vi = rec_vtx(R, sub), vj = rec_vtx(R, sub + 1);
      const V3<float> x0 = mk(v0.x, v0.y, v0.z), xi = mk(vi.x, vi.y, vi.z), xj = mk(vj.x, vj.y, vj.z);
      const V3<float> e1 = xi - x0, e2 = xj - x0;
      const V3<float> cr = cross(e1, e2);
      const float ai = 0.5f * dot(cr, ns);
      const float aib = Abar + dot(Scb, x0 + xi + xj) * (1.f / 3.f) + Spb * (v0.w + vi.w + vj.w) * (1.f / 3.f);
      const V3<float> sx = Scb * (ai * (1.f / 3.f));
      const float sp = Spb * ai * (1.f / 3.f);
      // a_t = n . (e1 x e2) / 2
      nb = cr * (0.5f * aib);
      const V3<float> e1b = cross(e2, ns) * (0.5f * aib), e2b = cross(ns, e1) * (0.5f * aib);
      to0 = sx - e1b - e2b;
      p_to0 = sp;
      xb = xb + sx + e1b;
      pb += sp;
      to_next = sx + e2b;
      p_next = sp;
    }
    const int prev = (lane & ~(Gs - 1)) | (sub == 0 ? 0 : sub - 1);
    const V3<float> in = mk(__shfl_sync(0xffffffffu, to_next.x, prev), __shfl_sync(0xffffffffu, to_next.y, prev),
                            __shfl_sync(0xffffffffu, to_next.z, prev));
    const float pin = __shfl_sync(0xffffffffu, p_next, prev);
    if (sub > 0) { xb = xb + in; pb += pin; }
    const V3<float> s0 = gsum3<Gs>(to0);
    const float ps0 = gsum<Gs>(p_to0);
    if (sub == 0) { xb = xb + s0; pb += ps0; }
    nbar = nbar + gsum3<Gs>(nb);
  }
  // contraction with the tangents of the lane's vertex
  V3<float> rot = mk(0.f, 0.f, 0.f), tr = rot;
  if (live && sub < nv) {
    const V3<float> xe = xb + g * pb;
    const V3<float> X = anc + rec_pos(R, sub);
    const int lab = (sub < 4 ? R.lab0 >> (8 * sub) : R.lab1 >> (8 * (sub - 4))) & 0xFF;
    const int l0 = lab & 15, l1 = lab >> 4;
    const V3<float> r0 = n;
    const V3<float> r1 = l0 < 4 ? mk(R.face[l0][0], R.face[l0][1], R.face[l0][2])
                                : mk(R.clip[l0 - 4][0], R.clip[l0 - 4][1], R.clip[l0 - 4][2]);
    const V3<float> r2 = l1 < 4 ? mk(R.face[l1][0], R.face[l1][1], R.face[l1][2])
                                : mk(R.clip[l1 - 4][0], R.clip[l1 - 4][1], R.clip[l1 - 4][2]);
    const V3<float> a0 = cross(r1, r2), a1 = cross(r2, r0), a2 = cross(r0, r1);
    const float det = dot(r0, a0);
    const float sc = norm(r0) * norm(r1) * norm(r2);
    det_stat(a, det, sc);
    if (fabsf(det) > kDetTol * sc) {
      const float id = 1.f / det;
      V3<float> B = r0 * (dot(xe, a0) * id);
      if (l0 >= 4) B = B + r1 * (dot(xe, a1) * id);
      if (l1 >= 4) B = B + r2 * (dot(xe, a2) * id);
      tr = B;
      rot = cross(X, B);
    } else if (a.adj_skip) {
      atomicAdd(a.adj_skip, 1);
    }
  }
  if (live && sub == 0) {
    rot = rot + cross(ns, nbar);
    if (gint != 0.f) rot = rot + cross(n, g) * gbar;
  }
  G.gx[0] += rot.x; G.gx[1] += rot.y; G.gx[2] += rot.z;
  G.gx[3] += tr.x; G.gx[4] += tr.y; G.gx[5] += tr.z;
}

// The reverse pass over one kept polygon by a group of G lanes: the taxel
// samples it won, then the wrench; its 13 gradient terms into its slot.
// rs: the round's staged records, k: this one's index among them.
template <int G, int kRepr>
__device__ __forceinline__ void rec_adj_one(const StepArgs& a, const AdjPoly* rs, int k, int dst, bool on, int lane,
                                            int sub) {
  const AdjPoly& R = rs[on ? k : 0];
  AdjAcc G_;
  adj_zero(G_);
  __syncwarp();   // the groups enter the shuffled ray preparation together
  if (a.adj_taxel != nullptr && on) rec_rays<G>(a, R, dst, sub, &G_);
  __syncwarp();
  if (a.adj_wrench != nullptr && a.apply_forces) rec_wrench_group<G, kRepr>(a, R, on, lane, sub, G_);
  float v[13] = {G_.gx[0], G_.gx[1], G_.gx[2], G_.gx[3], G_.gx[4], G_.gx[5], G_.glin[0], G_.glin[1], G_.glin[2],
                 G_.gang[0], G_.gang[1], G_.gang[2], G_.gE};
#pragma unroll
  for (int k = 0; k < 13; ++k) v[k] = gsum<G>(v[k]);
  if (on && sub == 0) {
    float4* o = reinterpret_cast<float4*>(a.rec_grad + 16 * (size_t)dst);
    o[0] = make_float4(v[0], v[1], v[2], v[3]);
    o[1] = make_float4(v[4], v[5], v[6], v[7]);
    o[2] = make_float4(v[8], v[9], v[10], v[11]);
    o[3] = make_float4(v[12], 0.f, 0.f, 0.f);
  }
}

// Reverse pass over the kept polygons, eight records per warp and round (as
// rec_forward_kernel: groups of 4 lanes, then groups of 8 for the larger).
// 6 CTAs per SM (80 registers; 396 B spilled, mostly around the wrench
// reverse) measured faster than 5 (96) once the records were staged in
// shared memory: 0.468 -> 0.459 ms.
template <int kRepr>
__global__ void __launch_bounds__(128, 6) adjoint_rec_kernel(StepArgs a) {
  if (!recs_valid(a)) return;
  const int n = min(*a.rec_count, a.rec_cap);
  const int lane = threadIdx.x & 31, sub = lane & (kGroupSmall - 1), grp = lane / kGroupSmall;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  constexpr int kPer = 32 / kGroupSmall;
  __shared__ RecStage stage[4];   // per warp (128 threads)
  RecStage& St = stage[threadIdx.x >> 5];
  const unsigned long long pol = evict_first_policy();
  LargeQueue lq = {0, -1, 0};
  auto large = [&](int r8, int dst8, bool on8, int sub8) { rec_adj_one<kGroup, kRepr>(a, a.recs, r8, dst8, on8, lane, sub8); };
  int buf = 0;
  stage_round(a, St.r[0], warp * kPer, n, lane, pol);
  for (int base = warp * kPer; base < n; base += n_warps * kPer, buf ^= 1) {
    stage_round(a, St.r[buf ^ 1], base + n_warps * kPer, n, lane, pol);
    stage_wait();
    const AdjPoly* rs = St.r[buf];
    const int r = base + grp;
    // the slot the forward record pass stored (one load where the key and
    // the item's offset were two dependent ones: adjoint 0.523 -> 0.516 ms)
    const int dst = r < n ? a.rec_dst[r] : -1;
    const int nv = dst >= 0 ? rs[grp].nv : 0;
    rec_adj_one<kGroupSmall, kRepr>(a, rs, grp, dst, dst >= 0 && nv <= kGroupSmall, lane, sub);
    __syncwarp();   // the round's records read before their buffer is refilled
    // the held larger polygons are read from global memory (their round's
    // buffer is gone by the time four are held)
    large_push(lq, dst >= 0 && nv > kGroupSmall && sub == 0, r, dst, lane);
    large_turns(lq, false, lane, large);
  }
  large_turns(lq, true, lane, large);
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Per pair: upstream adjoints of the soft-frame sums from dL/dwrench
// (wrench = [R_S F_S ; R_S T_S + (x_S - x_M) x R_S F_S]).
__global__ void adjoint_setup_kernel(StepArgs a) {
  // the work counters of the adjoint's kernels reuse the narrow phase's
  if (blockIdx.x == 0) {
    if (threadIdx.x < 3) a.item_next[threadIdx.x] = 0;
    if (threadIdx.x == 3 && a.adj_skip) {
      a.adj_skip[0] = 0;
      a.adj_skip[1] = 0x7f800000;   // +infinity
    }
  }
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.n_pair) return;
  const FrameDev& F = a.frames[p];
  float* o = a.adj_pair + 8 * (size_t)p;
  if (!a.adj_wrench || !F.valid) {
    for (int i = 0; i < 8; ++i) o[i] = 0.f;
    return;
  }
  const double* w = a.adj_wrench + 6 * (size_t)p;
  const V3<double> aF = mk(w[0], w[1], w[2]), aT = mk(w[3], w[4], w[5]);
  const V3<double> r = mk(F.xS[0] - F.xM[0], F.xS[1] - F.xM[1], F.xS[2] - F.xM[2]);
  const V3<double> gF = mat_tmul<double>(F.RS, aF + cross(aT, r));
  const V3<double> gT = mat_tmul<double>(F.RS, aT);
  o[0] = (float)gF.x; o[1] = (float)gF.y; o[2] = (float)gF.z;
  o[3] = (float)gT.x; o[4] = (float)gT.y; o[5] = (float)gT.z;
  o[6] = o[7] = 0.f;
}

// Per pair: sum of the item gradients (fixed order, FP64) and the chain rule
// to the world twists of M and N, plus dL/dE.
// The pair's sums by one warp: double-float on the FP32 pipe, in a fixed
// order (lane-strided, then a fixed butterfly); lane 0 holds them.
__device__ __forceinline__ void adjoint_sums(const StepArgs& a, int p, int lane, float vh[15], float vl[15]) {
  const PairDev& P = a.pairs[p];
  const int total = *a.item_total;
  const int b = min(a.unit_off[P.unit_begin], total), e = min(a.unit_off[P.unit_end], total);
#pragma unroll
  for (int k = 0; k < 15; ++k) vh[k] = vl[k] = 0.f;
  const bool ssp = P.query == 3;   // soft-soft: dL/dE_M, dL/dE_N, dL/d(damping) in entries 12-14
  if (recs_valid(a) && !ssp) {
    // the pair's records, in pair order
    const int rb = a.item_poly_off[b], re = a.item_poly_off[e];
    // four records per lane in flight, then summed in the same order (with
    // the forward's reduction batched likewise: adjoint stage 0.517 ->
    // 0.506 ms, step 1.411 -> 1.394 ms)
    int i = rb + lane;
    for (; i + 96 < re; i += 128) {
      float4 q0[4], q1[4], q2[4];
      float q3[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4* g = reinterpret_cast<const float4*>(a.rec_grad + 16 * (size_t)(i + 32 * u));
        q0[u] = g[0];
        q1[u] = g[1];
        q2[u] = g[2];
        q3[u] = reinterpret_cast<const float*>(g + 3)[0];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float x[13] = {q0[u].x, q0[u].y, q0[u].z, q0[u].w, q1[u].x, q1[u].y, q1[u].z, q1[u].w,
                             q2[u].x, q2[u].y, q2[u].z, q2[u].w, q3[u]};
#pragma unroll
        for (int k = 0; k < 13; ++k) df_add(vh[k], vl[k], x[k], 0.f);
      }
    }
    for (; i < re; i += 32) {
      const float4* g = reinterpret_cast<const float4*>(a.rec_grad + 16 * (size_t)i);
      const float4 g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
      const float x[13] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w, g2.x, g2.y, g2.z, g2.w, g3.x};
#pragma unroll
      for (int k = 0; k < 13; ++k) df_add(vh[k], vl[k], x[k], 0.f);
    }
  } else {
    for (int i = b + lane; i < e; i += 32) {
      const double* x = a.adj_item + (size_t)i * 16;
#pragma unroll
      for (int k = 0; k < 15; ++k) {
        if (k >= 13 && !ssp) break;
        const float h = (float)x[k];
        df_add(vh[k], vl[k], h, (float)(x[k] - (double)h));
      }
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1)
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      const float h2 = __shfl_xor_sync(0xffffffffu, vh[k], o), l2 = __shfl_xor_sync(0xffffffffu, vl[k], o);
      df_add(vh[k], vl[k], h2, l2);
    }
}

// The pair's FP64 chain rule from its sums v to both world twists and dE
// (one thread; FP64 from here on).
__device__ __forceinline__ void adjoint_tail(const StepArgs& a, int p, const double v[15]) {
  const PairDev& P = a.pairs[p];
  const bool ssp = P.query == 3;
  double* out = a.adj_out + 14 * (size_t)p;   // [M twist 6, N twist 6, dE_M, dE_N]
  for (int k = 0; k < 14; ++k) out[k] = 0.0;
  const FrameDev& F = a.frames[p];
  if (!F.valid || P.query == 0) return;
  const V3<double> Gw = mk(v[0], v[1], v[2]), Gv = mk(v[3], v[4], v[5]);
  const V3<double> Glin = mk(v[6], v[7], v[8]), Gang = mk(v[9], v[10], v[11]);
  const V3<double> t = mk(F.t[0], F.t[1], F.t[2]);
  // relative pose (other body in the soft frame)
  V3<double> thO = mat_mul<double>(F.RS, Gw - cross(t, Gv));
  V3<double> xO = mat_mul<double>(F.RS, Gv);
  V3<double> thS = mat_mul<double>(F.RS, Gw) * -1.0;
  V3<double> xS = xO * -1.0;
  // velocity field: lin = R_S^T (c + w x x_S), ang = R_S^T w
  const V3<double> lin = mk((double)F.lin[0], (double)F.lin[1], (double)F.lin[2]);
  const V3<double> ang = mk((double)F.ang[0], (double)F.ang[1], (double)F.ang[2]);
  thS = thS - mat_mul<double>(F.RS, cross(lin, Glin) + cross(ang, Gang));
  const V3<double> RGl = mat_mul<double>(F.RS, Glin);
  V3<double> wM = mk(0.0, 0.0, 0.0), wN = wM;
  if (a.vel) {
    wM = mk(a.vel[6 * (size_t)P.gm], a.vel[6 * (size_t)P.gm + 1], a.vel[6 * (size_t)P.gm + 2]);
    wN = mk(a.vel[6 * (size_t)P.gn], a.vel[6 * (size_t)P.gn + 1], a.vel[6 * (size_t)P.gn + 2]);
  }
  const V3<double> w = wM - wN;
  xS = xS + cross(RGl, w);
  V3<double> xM = cross(wM, RGl);
  V3<double> xN = cross(RGl, wN);
  // world wrench transform
  if (a.adj_wrench) {
    const double* aw = a.adj_wrench + 6 * (size_t)p;
    const V3<double> aF = mk(aw[0], aw[1], aw[2]), aT = mk(aw[3], aw[4], aw[5]);
    const PairOut& po = a.pair_out[p];
    const V3<double> FW = mk(po.wrench[0], po.wrench[1], po.wrench[2]);
    const V3<double> TW = mk(po.wrench[3], po.wrench[4], po.wrench[5]);
    const V3<double> r = mk(F.xS[0] - F.xM[0], F.xS[1] - F.xM[1], F.xS[2] - F.xM[2]);
    const V3<double> TWs = TW - cross(r, FW);
    thS = thS + cross(FW, aF) + cross(TWs, aT) + cross(FW, cross(aT, r));
    xS = xS + cross(FW, aT);
    xM = xM + cross(aT, FW);
  }
  // assemble per body (M first)
  double* gm = out;
  double* gn = out + 6;
  const bool sm = P.s_is_m;
  double* gs = sm ? gm : gn;
  double* go = sm ? gn : gm;
  gs[0] += thS.x; gs[1] += thS.y; gs[2] += thS.z; gs[3] += xS.x; gs[4] += xS.y; gs[5] += xS.z;
  go[0] += thO.x; go[1] += thO.y; go[2] += thO.z; go[3] += xO.x; go[4] += xO.y; go[5] += xO.z;
  gm[3] += xM.x; gm[4] += xM.y; gm[5] += xM.z;
  gn[3] += xN.x; gn[4] += xN.y; gn[5] += xN.z;
  // modulus: soft-soft sums hold dL/dE_M and dL/dE_N themselves, plus the
  // damping term (d = (E_N d_M + E_M d_N) / (E_M + E_N))
  if (ssp) {
    out[12] = v[12] + v[14] * (double)P.dd_dEs;
    out[13] = v[13] + v[14] * (double)P.dd_dEo;
    return;
  }
  // soft-rigid / half-space wrench and taxels are linear in E_s
  if (P.E_s > 0.f) {
    double dE = v[12];
    if (a.adj_wrench) {
      const double* aw = a.adj_wrench + 6 * (size_t)p;
      const PairOut& po = a.pair_out[p];
      for (int k = 0; k < 6; ++k) dE += aw[k] * po.wrench[k];
    }
    dE /= (double)P.E_s;
    out[12 + (sm ? 0 : 1)] = dE;
  }
}

// kReducePairs pairs per block: warp w sums pair w of the block
// (adjoint_sums), then the first kReducePairs threads run the pairs' FP64
// chain rules side by side (an FP64 warp instruction costs the FP64 pipe the
// same with one active lane as with 32: one tail per warp made this kernel
// FP64-bound).  In a fused step each also packs its pair's results for the
// host copy: its wrench, its two twist gradients and its two moduli terms,
// each kind back to back over the pairs.
__global__ void __launch_bounds__(kReducePairs * 32) adjoint_reduce_kernel(StepArgs a) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ float sh[kReducePairs][15], sl[kReducePairs][15];
  const int pw = blockIdx.x * kReducePairs + w;
  if (pw < a.n_pair) {
    float vh[15], vl[15];
    adjoint_sums(a, pw, lane, vh, vl);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < 15; ++k) { sh[w][k] = vh[k]; sl[w][k] = vl[k]; }
    }
  }
  __syncthreads();
  const int p = blockIdx.x * kReducePairs + threadIdx.x;
  if (threadIdx.x >= kReducePairs || p >= a.n_pair) return;
  double v[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) v[k] = (double)sh[threadIdx.x][k] + (double)sl[threadIdx.x][k];
  adjoint_tail(a, p, v);
  if (a.out_stage) {
    const size_t n = (size_t)a.n_pair;
    const double* g = a.adj_out + 14 * (size_t)p;
    double* o = a.out_stage;
    for (int k = 0; k < 6; ++k) o[6 * (size_t)p + k] = a.pair_out[p].wrench[k];
    for (int k = 0; k < 12; ++k) o[6 * n + 12 * (size_t)p + k] = g[k];
    for (int k = 0; k < 2; ++k) o[18 * n + 2 * (size_t)p + k] = g[12 + k];
  }
}
