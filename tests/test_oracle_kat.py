"""Known-answer tests of the FP64 oracle (CPU).

The reference ships no tests or golden data, so these anchor the oracle with
analytic answers derived from the reference's formulas
(mujoco_contact_surfaces_plugin.cpp:320-483, flat_tactile_sensor.cpp:262-402)
and the published hydroelastic model.
"""
import math

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
from mujoco_contact_surfaces_gb300.scenes import Scene, random_rotation, rot_axis, sphere_hint
from oracle import Oracle


def box_on_plane(E=1e5, d=1.0, mu=0.5, pen=1e-3, vel=(0, 0, 0, 0, 0, 0), hz=0.01):
    """Wide thin soft box resting on a rigid half-space (box registered first)."""
    s = Scene()
    b = s.add_geom(L.GEOM_BOX, [0.1, 0.1, hz], [E, d, 0.005, mu, mu])
    g = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, mu, mu])
    s.g1, s.g2 = [b], [g]
    s.xpos = np.array([[0.0, 0.0, hz - pen], [0.0, 0.0, 0.0]])
    s.xmat = np.tile(np.eye(3).reshape(1, 9), (2, 1))
    s.vel = np.zeros((2, 6))
    s.vel[0] = vel
    return s


def test_triangle_and_polygon_quadrature_agree_on_fn0():
    # centroid quadrature is exact for the linear field on each polygon
    for s in (scenes.single_pair(8), scenes.tactile(4), scenes.halfspace(4)):
        o = Oracle(s)
        a = o.collide(representation=0)["total_fn0"]
        b = o.collide(representation=1)["total_fn0"]
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-14)


def test_sphere_on_plane_converges_to_continuum():
    # p = E (1 - r/R) on a sphere pressed delta into a plane:
    # F = E [pi a^2 - 2 pi (R^3 - h^3) / (3 R)], h = R - delta, a^2 = R^2 - h^2
    R, E, delta = 0.05, 1e5, 0.004
    h = R - delta
    exact = E * (math.pi * (R * R - h * h) - 2 * math.pi * (R ** 3 - h ** 3) / (3 * R))
    errs = []
    for lev in (3, 4, 5, 6):
        s = Scene()
        g = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [E, 1.0, sphere_hint(R, lev), 0.5, 0.5])
        p = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
        s.g1, s.g2 = [g], [p]
        s.xpos = np.array([[0, 0, R - delta], [0, 0, 0.0]])
        s.xmat = np.tile(np.eye(3).reshape(1, 9), (2, 1))
        s.vel = np.zeros((2, 6))
        F = Oracle(s).collide()["wrench"][0, 2]
        errs.append(abs(F - exact) / exact)
    assert all(e2 < e1 for e1, e2 in zip(errs, errs[1:])), errs
    assert errs[-1] < 0.01, errs


@pytest.mark.parametrize("vn", [0.0, 0.05, -0.2, 0.5, 1.5])
def test_hunt_crossley_closed_form(vn):
    # uniform normal velocity: fn = max(0, 1 - d vn) (fn0 - 0.001 k vn) per
    # point, k = A g with g = E/hz on every kept face (to the FP32
    # rounding of the mesh vertices, a few 1e-8 relative in g)
    E, d, hz = 1e5, 1.0, 0.01
    s = box_on_plane(E=E, d=d, vel=(0, 0, 0, 0, 0, vn), hz=hz)
    r = Oracle(s).collide()
    fn0, A = r["total_fn0"][0], r["area"][0]
    expect = max(0.0, 1 - d * vn) * (fn0 - 0.001 * A * (E / hz) * vn)
    assert r["wrench"][0, 2] == pytest.approx(expect, rel=1e-7, abs=1e-12)
    np.testing.assert_allclose(r["wrench"][0, :2], 0, atol=1e-9 * max(1.0, abs(expect)))


@pytest.mark.parametrize("vt", [0.0, 2e-5, 5e-5, 9e-5, 1e-3, 0.1])
def test_regularised_friction_closed_form(vt):
    # uniform sliding velocity along x: f_t = -mu_reg fn, mu_reg = mu s (2 - s)
    # for s = sqrt(vt^2 + (1e-6)^2) / 1e-4 < 1
    mu = 0.5
    s = box_on_plane(mu=mu, vel=(0, 0, 0, vt, 0, 0))
    r = Oracle(s).collide()
    Fz, Fx = r["wrench"][0, 2], r["wrench"][0, 0]
    vs = math.sqrt(vt * vt + 1e-12)
    sr = vs / 1e-4
    mu_reg = mu * sr * (2 - sr) if sr < 1 else mu
    assert Fx == pytest.approx(-mu_reg * (vt / vs) * Fz, rel=1e-9, abs=1e-12)


def test_translation_invariance_and_rotation_covariance():
    s = scenes.single_pair(4, velocities=True)
    o = Oracle(s)
    w0 = o.collide()["wrench"]
    shift = np.array([0.3, -1.2, 0.7])
    w1 = o.collide(xpos=s.xpos + shift)["wrench"]
    np.testing.assert_allclose(w1, w0, rtol=1e-9, atol=1e-9)
    Rg = random_rotation(np.random.default_rng(4))
    xp = s.xpos @ Rg.T
    xm = np.array([(Rg @ m.reshape(3, 3)).reshape(9) for m in s.xmat])
    vel = s.vel.copy()
    vel[:, :3] = vel[:, :3] @ Rg.T
    vel[:, 3:] = vel[:, 3:] @ Rg.T
    w2 = o.collide(xpos=xp, xmat=xm, vel=vel)["wrench"]
    np.testing.assert_allclose(w2[:, :3], w0[:, :3] @ Rg.T, rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(w2[:, 3:], w0[:, 3:] @ Rg.T, rtol=1e-8, atol=1e-8)


def test_registration_order_sets_M():
    # M is the geom registered first: swapping the order gives the
    # force on the other body, about the other body's origin
    s = scenes.single_pair(3)
    w = Oracle(s).collide()["wrench"]
    s2 = Scene()
    for k in range(3):
        b = s.geoms[2 * k + 1]
        a = s.geoms[2 * k]
        s2.add_geom(b["type"], b["size"], b["cs5"])
        s2.add_geom(a["type"], a["size"], a["cs5"])
    s2.g1 = [2 * k + 1 for k in range(3)]
    s2.g2 = [2 * k for k in range(3)]
    idx = np.array([[2 * k + 1, 2 * k] for k in range(3)]).ravel()
    s2.xpos, s2.xmat, s2.vel = s.xpos[idx], s.xmat[idx], s.vel[idx]
    r = Oracle(s2).collide()
    assert np.array_equal(r["m"], np.array([2 * k for k in range(3)]))
    w2 = r["wrench"]
    np.testing.assert_allclose(w2[:, :3], -w[:, :3], rtol=1e-9, atol=1e-12)
    for k in range(3):
        d = s.xpos[2 * k] - s.xpos[2 * k + 1]
        np.testing.assert_allclose(w2[k, 3:], -(w[k, 3:] + np.cross(d, w[k, :3])), rtol=1e-8, atol=1e-10)


def test_uniform_pressure_taxel_map():
    # a wide soft box pressed delta into a rigid plate: the plate top carries
    # p = E delta / hz everywhere under the box, so every taxel is p
    # (25 samples x p x 1/25), to the FP32 rounding of the mesh vertices
    E, hz, delta = 2e5, 0.01, 0.002
    s = Scene()
    b = s.add_geom(L.GEOM_BOX, [0.1, 0.1, hz], [E, 1.0, 0.005, 0.5, 0.5])
    p = s.add_geom(L.GEOM_BOX, [0.0401, 0.04, 0.005], [0, 1.0, 0, 0.5, 0.5])
    s.g1, s.g2 = [b], [p]
    s.xpos = np.array([[0.003, -0.002, 0.005 - delta + hz], [0, 0, 0.0]])
    s.xmat = np.tile(np.eye(3).reshape(1, 9), (2, 1))
    s.vel = np.zeros((2, 6))
    s.sensors = [dict(geom=p, resolution=0.005, sr=5, window=L.WINDOW_NONE, sigma=-1.0)]
    r = Oracle(s).collide(taxels64=True)
    expect = E * delta / hz
    np.testing.assert_allclose(r["taxels"][0], expect, rtol=1e-5)
    np.testing.assert_allclose(r["taxels64"][0], expect, rtol=1e-6)


def test_flat_sensor_grid_size_rule():
    # cx = floor(2 xs / res + 0.1) (flat_tactile_sensor.cpp:196-197)
    import ctypes as C
    from oracle import load
    lib = load()
    cx, cy = C.c_int(), C.c_int()
    for xs, res, want in [(0.04, 0.005, 16), (0.2, 0.025, 16), (0.0401, 0.005, 16), (0.03, 0.007, 8)]:
        lib.or_sensor_grid(xs, xs, res, C.byref(cx), C.byref(cy))
        assert cx.value == want == math.floor(2 * xs / res + 0.1)


def test_no_contact_and_unsupported_pairs():
    s = box_on_plane(pen=-0.01)  # lifted 1 cm
    r = Oracle(s).collide()
    assert r["n_polygons"][0] == 0 and np.all(r["wrench"] == 0)
    s = Scene()
    a = s.add_geom(L.GEOM_BOX, [0.1, 0.1, 0.1], [0, 1, 0, 0.5, 0.5])
    b = s.add_geom(L.GEOM_BOX, [0.1, 0.1, 0.1], [0, 1, 0, 0.5, 0.5])
    s.g1, s.g2 = [a], [b]
    s.xpos = np.zeros((2, 3)); s.xmat = np.tile(np.eye(3).reshape(1, 9), (2, 1)); s.vel = np.zeros((2, 6))
    assert Oracle(s).collide()["query"][0] == 0   # rigid-rigid: default narrow phase


def test_taxel_sensor_kat():
    """Taxel-point sensor restatement (taxel_sensor.cpp:158-478): the random
    stream, the closest method's visualisation quirk, the fall-through of
    weighted and mean into squared, kept values and the empty case."""
    import oracle
    lib = oracle.load()
    # C++ [rand.predef]: the 10000th draw of a default-constructed minstd_rand0
    assert lib.or_minstd_nth(10000) == 1043618065
    R = 2147483646.0
    d1, d2 = 16807, 16807 * 16807 % 2147483647
    assert lib.or_uniform_nth(1) == ((d1 - 1) + (d2 - 1) * R) / (R * R)
    sq = dict(poly_offset=[0, 4], vert=[[0, 0, 0], [0.01, 0, 0], [0.01, 0.01, 0], [0, 0.01, 0]],
              vert_pressure=[2, 2, 2, 2], normal=[[0, 0, 1]])
    tx = [[0.005, 0.005, 0.0], [0.005, 0.005, 0.001], [0.5, 0.5, 0.5]]
    prev = [7.0, 7.0, 7.0]
    for sm, res in ((0, 0.001), (1, 0.01)):
        v = oracle.taxel_sensor(tx, 0, 0.002, res, sm, 1, [sq], values=prev)
        assert list(v) == [2.0, 2.0, 7.0]           # pressure inside, kept outside
        v = oracle.taxel_sensor(tx, 0, 0.002, res, sm, 0, [sq], values=prev)
        assert list(v) == [0.0, 0.0, 7.0]           # the else binds to the visualisation test
        w = [oracle.taxel_sensor(tx, m, 0.002, res, sm, 0, [sq], values=prev) for m in (1, 2, 3)]
        assert np.array_equal(w[0], w[1]) and np.array_equal(w[1], w[2])   # fall-through
        assert w[2][0] > w[2][1] > 0 and w[2][2] == 7.0
    assert list(oracle.taxel_sensor(tx, 3, 0.002, 0.001, 0, 0, [], values=prev)) == [0.0, 0.0, 0.0]


def test_curved_sensor_kat():
    """Curved-sensor restatement (curved_sensor.cpp): the selection's margin,
    weights and 45-degree normal test, and rays into a uniform-pressure
    square below the sensor surface (t < margin counts, t >= margin not)."""
    import oracle
    g = np.linspace(-0.004, 0.004, 9)
    pts = np.array([[x, y, 0.0] for x in g for y in g])
    pn = np.tile([0.0, 0.0, 1.0], (len(pts), 1))
    tx = np.array([[0.0, 0.0, 0.0], [0.002, 0.0, 0.0], [0.0, 0.0, 0.0], [0.1, 0.0, 0.0]])
    tn = np.array([[0, 0, 0], [0, 0, 2.0], [1.0, 0, 1.0 / np.sqrt(3.0)], [0, 0, 0]], float)
    tn_unit = tn / np.maximum(np.linalg.norm(tn, axis=1, keepdims=True), 1e-300)
    margin = 0.003
    off, pt, w = oracle.curved_select(tx, tn_unit, margin, pts, pn)
    for i in range(len(tx)):
        d = np.linalg.norm(pts - tx[i], axis=1)
        cos = tn_unit[i] @ np.array([0, 0, 1.0])
        want = np.nonzero((d < margin) & ((np.linalg.norm(tn[i]) == 0) | (np.arccos(np.clip(cos, -1, 1)) < np.pi / 4)))[0]
        assert list(pt[off[i]:off[i + 1]]) == list(want)
        np.testing.assert_allclose(w[off[i]:off[i + 1]], np.maximum(0, margin - d[want]) ** 2, rtol=1e-12, atol=1e-18)
    assert off[3] - off[2] == 0 and off[4] - off[3] == 0     # 60 degrees off; out of reach
    sq = dict(poly_offset=[0, 4], vert=[[-0.01, -0.01, -0.001], [0.01, -0.01, -0.001], [0.01, 0.01, -0.001],
                                        [-0.01, 0.01, -0.001]], vert_pressure=[5.0] * 4, normal=[[0, 0, 1]])
    v = oracle.curved_update(off, pt, w, pts, pn, margin, [sq])
    for i in range(len(tx)):
        assert v[i] == pytest.approx(5.0 * w[off[i]:off[i + 1]].sum(), rel=1e-12)
    assert v[0] > 0 and v[1] > 0
    # a surface deeper than the margin is not reached; no surface: zeros
    deep = dict(sq, vert=[[x, y, -0.004] for x, y, _ in sq["vert"]])
    assert np.all(oracle.curved_update(off, pt, w, pts, pn, margin, [deep]) == 0)
    assert np.all(oracle.curved_update(off, pt, w, pts, pn, margin, []) == 0)
    # the nearest of two surfaces along the ray counts
    sq2 = dict(sq, vert=[[x, y, -0.0005] for x, y, _ in sq["vert"]], vert_pressure=[3.0] * 4)
    v2 = oracle.curved_update(off, pt, w, pts, pn, margin, [sq, sq2])
    assert v2[0] == pytest.approx(3.0 * w[off[0]:off[1]].sum(), rel=1e-12)
