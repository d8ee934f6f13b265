"""Curved sensor (hc_add_curved_sensor) against the oracle's restatement of
CurvedSensor: the point selection at load (oracle.curved_select on the same
surface points) and the per-step rays into the engine's own contact surfaces
(hc_get_surface; the polygons are checked against the oracle by the parity
tests).  A soft icosphere mesh carries the sensor, pressed onto a ground
plane and onto a rigid plate; a second step lifts one out of contact."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
import oracle

pytestmark = pytest.mark.gpu


def icosphere(radius, level):
    t = (1 + 5 ** 0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    v = [np.array(p, float) / np.linalg.norm(p) for p in v]
    for _ in range(level):
        mid = {}

        def m(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                mid[k] = len(v) - 1
            return mid[k]
        nf = []
        for a, b, c in f:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    V = np.array(v) * radius
    F = np.array(f, np.int32)
    for k, (a, b, c) in enumerate(F):   # outward, counter-clockwise
        if np.cross(V[b] - V[a], V[c] - V[a]) @ (V[a] + V[b] + V[c]) < 0:
            F[k] = (a, c, b)
    return V, F


MARGIN = 0.005


def _taxels(Rm, radius):
    """Taxels on the sphere around the world-down direction, in the geom
    frame; radial normals on every other taxel."""
    dirs = []
    for th in np.radians([0, 12, 24, 36]):
        for ph in np.radians(np.arange(0, 360, 45 if th > 0 else 360)):
            dirs.append([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)])
    dirs = np.array(dirs)
    tx = (dirs * radius) @ Rm          # world direction -> geom frame (R^T d)
    tn = np.zeros_like(tx)
    tn[::2] = tx[::2] / radius
    return tx, tn


def _surfaces(eng, s, geom):
    out = []
    for p in range(len(s.g1)):
        if geom in (s.g1[p], s.g2[p]):
            srf = eng.surface(p)
            out.append(dict(poly_offset=srf["offset"], vert=srf["vert"], vert_pressure=srf["pressure"],
                            normal=srf["normal"]))
    return out


def test_curved_sensor_matches_oracle(gpu):
    radius = 0.03
    V, F = icosphere(radius, 3)
    pts, nrm = L.sample_surface(V, F, 3000, seed=42)
    s = scenes.Scene()
    ground = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
    ball_a = s.add_geom(L.GEOM_MESH, [0, 0, 0], [2e5, 1.0, 0, 0.5, 0.5], V, F)
    plate = s.add_geom(L.GEOM_BOX, [0.05, 0.05, 0.005], [0, 1.0, 0, 0.5, 0.5])
    ball_b = s.add_geom(L.GEOM_MESH, [0, 0, 0], [1e5, 1.0, 0, 0.5, 0.5], V, F)
    s.g1 += [ball_a, ball_b]; s.g2 += [ground, plate]; s.scene_of_pair += [0, 1]
    scenes._alloc(s)
    rng = np.random.Generator(np.random.PCG64(5))
    Ra, Rb = scenes.random_rotation(rng), scenes.random_rotation(rng)
    s.xmat[ball_a] = Ra.reshape(9)
    s.xmat[ball_b] = Rb.reshape(9)
    s.xpos[ball_a] = [0.001, -0.002, radius - 0.003]
    s.xpos[plate] = [1.0, 0.0, 0.0]
    s.xpos[ball_b] = [1.0 + 0.002, 0.001, 0.005 + radius - 0.0025]
    eng = scenes.build_engine(s)
    sensors = {}
    for geom, Rm in ((ball_a, Ra), (ball_b, Rb)):
        tx, tn = _taxels(Rm, radius)
        sensors[geom] = (eng.add_curved_sensor(geom, tx, MARGIN, pts, nrm, tn), tx, tn)
    eng.set_pairs(s.g1, s.g2)
    xpos = s.xpos.copy()
    for step in range(2):
        if step == 1:
            xpos[ball_a, 2] += 0.01                 # lifted out of contact
        eng.set_poses(xpos, s.xmat, s.vel)
        eng.step()
        for geom, (sid, tx, tn) in sensors.items():
            got = eng.curved_sensor_values(sid).astype(np.float64)
            off, pt, w = oracle.curved_select(tx, tn, MARGIN, pts, nrm)
            R = s.xmat[geom].reshape(3, 3)
            ref = oracle.curved_update(off, pt, w, pts @ R.T + xpos[geom], nrm @ R.T, MARGIN,
                                       _surfaces(eng, s, geom))
            scale = max(np.abs(ref).max(), 1e-12)
            bad = np.abs(got - ref) > 1e-4 * scale + 1e-9
            assert bad.sum() == 0, (step, geom, np.where(bad), got[bad], ref[bad], scale)
            if step == 0 or geom == ball_b:
                assert np.count_nonzero(ref) >= 8
            else:
                assert np.all(got == 0) and np.all(ref == 0)
    eng.close()


def test_disabled_curved_sensor_keeps_values(gpu):
    radius = 0.03
    V, F = icosphere(radius, 2)
    pts, nrm = L.sample_surface(V, F, 1500, seed=3)
    s = scenes.Scene()
    ground = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
    ball = s.add_geom(L.GEOM_MESH, [0, 0, 0], [2e5, 1.0, 0, 0.5, 0.5], V, F)
    s.g1.append(ball); s.g2.append(ground); s.scene_of_pair.append(0)
    scenes._alloc(s)
    s.xpos[ball] = [0, 0, radius - 0.003]
    eng = scenes.build_engine(s)
    tx, tn = _taxels(np.eye(3), radius)
    sid = eng.add_curved_sensor(ball, tx, MARGIN, pts, nrm, tn)
    eng.set_pairs(s.g1, s.g2)
    eng.step()
    v0 = eng.curved_sensor_values(sid)
    eng.set_curved_sensor_enabled(sid, False)
    xp = s.xpos.copy()
    xp[ball, 2] += 0.02
    eng.set_poses(xp, s.xmat, s.vel)
    eng.step()
    v1 = eng.curved_sensor_values(sid)
    eng.set_curved_sensor_enabled(sid, True)
    eng.step()
    v2 = eng.curved_sensor_values(sid)
    eng.close()
    assert np.count_nonzero(v0) > 0 and np.array_equal(v0, v1) and np.all(v2 == 0)
