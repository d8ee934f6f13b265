"""The soft-soft wrench reverse, restated in FP64 (tests/ss_adjoint_model.py),
against the oracle and against central differences (CPU).

The pair is the sphere-on-soft-box pair the GPU adjoint tests use
(`soft_soft_pressed(2)`, pair 1, the sphere registered first).  Its contact
boundary has vertices whose three constraint rows are linearly dependent
(an edge on one body's surface meets the other body's surface: both
pressures vanish, so the section plane and the two surface planes share a
line).  Such a vertex is not fixed by its rows and the reverse leaves it out;
in FP32 the determinant of a dependent triple is rounding noise, so the
guard must sit well above it (the device's kDetTol = 1e-4), which the FP32
emulation here shows.
"""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
from oracle import Oracle
from tests import ss_adjoint_model as M


def _rotation(w):
    th = np.linalg.norm(w)
    if th == 0:
        return np.eye(3)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


@pytest.fixture(scope="module")
def pair():
    s = scenes.soft_soft_pressed(2)
    p = 1
    ga, gb = s.g1[p], s.g2[p]
    mesh = {}
    for g in (ga, gb):
        G = s.geoms[g]
        _, v, pr, e = L.generate_mesh(G["type"], G["size"], G["cs5"], G["mesh_v"], G["mesh_f"])
        mesh[g] = (np.asarray(v, float).reshape(-1, 3), np.asarray(pr, float), np.asarray(e, int).reshape(-1, 4))
    RA, tA = s.xmat[ga].reshape(3, 3), s.xpos[ga]
    RB, tB = s.xmat[gb].reshape(3, 3), s.xpos[gb]
    vA, pA, eA = mesh[ga]
    vB0, pB, eB = mesh[gb]
    vB = ((RB @ vB0.T).T + tB - tA) @ RA          # B in A's frame
    EM, EN = s.geoms[ga]["cs5"][0], s.geoms[gb]["cs5"][0]
    dM, dN = s.geoms[ga]["cs5"][1], s.geoms[gb]["cs5"][1]
    ma, mb = s.geoms[ga]["cs5"][4], s.geoms[gb]["cs5"][4]
    wM, vM = s.vel[ga][:3], s.vel[ga][3:]
    wN, vN = s.vel[gb][:3], s.vel[gb][3:]
    # relative velocity field v_M - v_N in A's frame: lin + ang x p
    lin = RA.T @ ((vM - vN) - np.cross(wM, tA) + np.cross(wN, tB) + np.cross(wM - wN, tA))
    vf = (lin, RA.T @ (wM - wN), (EN * dM + EM * dN) / (EM + EN), 2 * ma * mb / (ma + mb))
    XA, XB = vA[eA], vB[eB]
    ov = np.all((XA.min(1)[:, None] <= XB.max(1)[None]) & (XB.min(1)[None] <= XA.max(1)[:, None]), axis=2)
    polys = {}
    for ta, tb in np.argwhere(ov):
        P = M.element_polygon(vA[eA[ta]], pA[eA[ta]], vB[eB[tb]], pB[eB[tb]])
        if P is not None:
            polys[(int(ta), int(tb))] = P

    def loss(vb, gF, gT, repr_):
        tot = 0.0
        for ta, tb in polys:   # element pairs without a polygon enter at second order
            P = M.element_polygon(vA[eA[ta]], pA[eA[ta]], vb[eB[tb]], pB[eB[tb]])
            if P is not None:
                f, t = M.polygon_wrench(P, vf, repr_)
                tot += gF @ f + gT @ t
        return tot

    def central_differences(gF, gT, repr_, h=1e-7):
        fd = np.zeros(6)
        for c in range(6):
            w, v = np.zeros(3), np.zeros(3)
            if c < 3:
                w[c] = h
            else:
                v[c - 3] = h
            lp = loss((_rotation(w) @ vB.T).T + v, gF, gT, repr_)
            lm = loss((_rotation(-w) @ vB.T).T - v, gF, gT, repr_)
            fd[c] = (lp - lm) / (2 * h)
        return fd

    def loss_moduli(fa, fb, gF, gT, repr_):
        """L with E_A scaled by fa and E_B by fb (pressures and damping)."""
        ea, eb = EM * fa, EN * fb
        vfe = (vf[0], vf[1], (eb * dM + ea * dN) / (ea + eb), vf[3])
        tot = 0.0
        for ta, tb in polys:
            P = M.element_polygon(vA[eA[ta]], pA[eA[ta]] * fa, vB[eB[tb]], pB[eB[tb]] * fb)
            if P is not None:
                f, t = M.polygon_wrench(P, vfe, repr_)
                tot += gF @ f + gT @ t
        return tot

    orc = Oracle(s)
    return dict(s=s, p=p, RA=RA, vf=vf, polys=polys, fd=central_differences, oracle=orc,
                moduli=(EM, EN), dissipation=(dM, dN), loss_moduli=loss_moduli)


@pytest.mark.parametrize("repr_", [0, 1])
def test_model_forward_matches_oracle(pair, repr_):
    F, T = np.zeros(3), np.zeros(3)
    for P in pair["polys"].values():
        f, t = M.polygon_wrench(P, pair["vf"], repr_)
        F += f
        T += t
    ref = pair["oracle"].collide(representation=repr_, pairs=[pair["p"]], sensors=False)
    assert len(pair["polys"]) == ref["n_polygons"][0]
    w = np.concatenate([pair["RA"] @ F, pair["RA"] @ T])
    assert np.linalg.norm(w - ref["wrench"][0]) <= 1e-9 * np.linalg.norm(ref["wrench"][0])


@pytest.mark.parametrize("repr_", [0, 1])
def test_reverse_matches_central_differences_and_needs_an_fp32_guard(pair, repr_):
    rng = np.random.default_rng(5)
    gF, gT = rng.normal(size=3), rng.normal(size=3) * 0.05
    fd = pair["fd"](gF, gT, repr_)
    vf = pair["vf"]
    g64 = sum(M.polygon_reverse(P, gF, gT, vf, repr_) for P in pair["polys"].values())
    err = lambda g: np.linalg.norm(g - fd) / np.linalg.norm(fd)
    assert err(g64) <= 1e-3
    vf32 = tuple(np.float32(x) for x in vf)

    def fp32(tol):
        tot = np.zeros(6)
        for P in pair["polys"].values():
            Q, anc = M.as_float32(P)
            tot += np.asarray(M.polygon_reverse(Q, np.float32(gF), np.float32(gT), vf32, repr_, anc,
                                                np.float32(tol)), np.float64)
        return tot

    # the FP64 guard lets the dependent vertices' rounding-noise determinants
    # through in FP32; the device's tolerance does not
    assert err(fp32(1e-12)) > 2e-3
    assert err(fp32(1e-4)) <= 1e-3


@pytest.mark.parametrize("repr_", [0, 1])
def test_reverse_modulus_terms(pair, repr_):
    # dL/dE_A and dL/dE_B of the reverse (the equal-pressure plane moves with
    # both moduli; the combined damping d = (E_B d_A + E_A d_B)/(E_A + E_B)
    # depends on their ratio) against central differences at relative step
    # 1e-6, and Euler's identity E_A dL/dE_A + E_B dL/dE_B = L
    rng = np.random.default_rng(6)
    gF, gT = rng.normal(size=3), rng.normal(size=3) * 0.05
    EA, EB = pair["moduli"]
    dA, dB = pair["dissipation"]
    gEa = gEb = gD = 0.0
    for P in pair["polys"].values():
        _, a, b, d = M.polygon_reverse(P, gF, gT, pair["vf"], repr_, moduli=(EA, EB))
        gEa += a
        gEb += b
        gD += d
    den = (EA + EB) ** 2
    dEa = gEa + gD * EB * (dB - dA) / den
    dEb = gEb + gD * EA * (dA - dB) / den
    h = 1e-6
    L = pair["loss_moduli"]
    ref_a = (L(1 + h, 1, gF, gT, repr_) - L(1 - h, 1, gF, gT, repr_)) / (2 * h * EA)
    ref_b = (L(1, 1 + h, gF, gT, repr_) - L(1, 1 - h, gF, gT, repr_)) / (2 * h * EB)
    got, ref = np.array([dEa, dEb]), np.array([ref_a, ref_b])
    assert np.linalg.norm(got - ref) <= 1e-3 * np.linalg.norm(ref), (got, ref)
    L0 = L(1, 1, gF, gT, repr_)
    assert abs(EA * dEa + EB * dEb - L0) <= 1e-9 * abs(L0) + 1e-12, (EA * dEa + EB * dEb, L0)


@pytest.mark.parametrize("sensor_on_b", [False, True])
def test_ray_hit_pressure_derivatives(sensor_on_b):
    # The soft-soft sample adjoint (sample_adjoint, kSS): a ray o + t D hits
    # p_A = p_B and reads p = p_A(x).  With m = g_A - g_B, ka = g_A.D / m.D and
    # kb = -g_B.D / m.D: rays on B move with it, dp = kb g_A.(w x x + v);
    # rays on A are fixed, dp = -ka g_B.(w x x + v); dp/dE_A = kb p / E_A,
    # dp/dE_B = ka p / E_B.  Central differences of the exact hit.
    rng = np.random.default_rng(31)
    EA, EB = 2e5, 3e5
    ga_u, gb_u = rng.normal(size=3), rng.normal(size=3)
    ga_u[2], gb_u[2] = 1.0 + abs(ga_u[2]), -1.0 - abs(gb_u[2])   # fields facing each other along z
    ca_u, cb_u = 0.3, 0.5
    o, D = np.array([0.01, -0.02, 0.3]), np.array([0.05, -0.03, -1.0])

    def hit(R, v, fa=1.0, fb=1.0):
        ga, ca = EA * fa * ga_u, EA * fa * ca_u
        gb, cb = EB * fb * gb_u, EB * fb * cb_u
        # B moved by (R, v): p_B'(y) = p_B(R^T (y - v))
        gbm, cbm = R @ gb, cb - (R @ gb) @ v
        oo, DD = (R @ o + v, R @ D) if sensor_on_b else (o, D)
        m, mc = ga - gbm, ca - cbm
        t = -(m @ oo + mc) / (m @ DD)
        x = oo + t * DD
        return ga @ x + ca, x

    p0, x0 = hit(np.eye(3), np.zeros(3))
    ga, gb = EA * ga_u, EB * gb_u
    mD = (ga - gb) @ D
    ka, kb = ga @ D / mD, -(gb @ D) / mD
    gv = gb * (-ka) if not sensor_on_b else ga * kb
    want = np.concatenate([np.cross(x0, gv), gv, [kb * p0 / EA, ka * p0 / EB]])
    h = 1e-7
    got = np.zeros(8)
    for c in range(6):
        w, v = np.zeros(3), np.zeros(3)
        if c < 3:
            w[c] = h
        else:
            v[c - 3] = h
        got[c] = (hit(_rotation(w), v)[0] - hit(_rotation(-w), -v)[0]) / (2 * h)
    got[6] = (hit(np.eye(3), np.zeros(3), fa=1 + h)[0] - hit(np.eye(3), np.zeros(3), fa=1 - h)[0]) / (2 * h * EA)
    got[7] = (hit(np.eye(3), np.zeros(3), fb=1 + h)[0] - hit(np.eye(3), np.zeros(3), fb=1 - h)[0]) / (2 * h * EB)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-9 * np.abs(want).max()), (got, want)


def _pair_polygons(s, p):
    """The model's polygons of pair p (A = g1, B = g2, B in A's frame)."""
    ga, gb = s.g1[p], s.g2[p]
    mesh = {}
    for g in (ga, gb):
        G = s.geoms[g]
        _, v, pr, e = L.generate_mesh(G["type"], G["size"], G["cs5"], G["mesh_v"], G["mesh_f"])
        mesh[g] = (np.asarray(v, float).reshape(-1, 3), np.asarray(pr, float), np.asarray(e, int).reshape(-1, 4))
    RA, tA = s.xmat[ga].reshape(3, 3), s.xpos[ga]
    RB, tB = s.xmat[gb].reshape(3, 3), s.xpos[gb]
    vA, pA, eA = mesh[ga]
    vB0, pB, eB = mesh[gb]
    vB = ((RB @ vB0.T).T + tB - tA) @ RA
    XA, XB = vA[eA], vB[eB]
    ov = np.all((XA.min(1)[:, None] <= XB.max(1)[None]) & (XB.min(1)[None] <= XA.max(1)[:, None]), axis=2)
    polys = [M.element_polygon(vA[eA[ta]], pA[eA[ta]], vB[eB[tb]], pB[eB[tb]]) for ta, tb in np.argwhere(ov)]
    return [P for P in polys if P is not None], RA, RA.T @ (tB - tA)


@pytest.mark.parametrize("repr_,tol", [(1, 1e-6), (0, 1e-3)])
def test_reverse_matches_oracle_differences_in_world_twist(repr_, tol):
    # The exact reverse (dependent-row vertices carried by their two face
    # rows) against central differences of the oracle in the world twist of
    # N, at rest (the model holds the velocity field fixed; the device's
    # per-pair reduction adds its pose dependence).  kPolygon is exact; with
    # kTriangle a boundary vertex whose place along the line where both
    # surfaces meet is set by rounding in the clip moves the fan quadrature,
    # which central differences see and the reverse leaves out.
    from tests.test_gpu_adjoint import perturb
    s = scenes.soft_soft_pressed(4, velocities=False)
    orc = Oracle(s)
    rng = np.random.default_rng(31)
    dLdw = rng.normal(size=(len(s.g1), 6))
    vf = (np.zeros(3), np.zeros(3), 1.0, 0.5)
    for p in range(len(s.g1)):
        polys, RA, c = _pair_polygons(s, p)
        gF, gT = RA.T @ dLdw[p][:3], RA.T @ dLdw[p][3:]
        g = sum(M.polygon_reverse(P, gF, gT, vf, repr_) for P in polys)
        world = np.concatenate([RA @ (g[:3] + np.cross(g[3:], c)), RA @ g[3:]])
        h = 1e-6
        fd = np.zeros(6)
        for k in range(6):
            lw = []
            for sgn in (1, -1):
                xp, xm = perturb(s.xpos, s.xmat, s.g2[p], k, sgn * h)
                r = orc.collide(representation=repr_, pairs=[p], xpos=xp, xmat=xm, sensors=False)
                lw.append(float(dLdw[p] @ r["wrench"][0]))
            fd[k] = (lw[0] - lw[1]) / (2 * h)
        err = np.linalg.norm(world - fd) / np.linalg.norm(fd)
        assert err <= tol, (p, err, world, fd)
    orc.close()
