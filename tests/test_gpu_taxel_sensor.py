"""Taxel-point sensor (hc_add_taxel_sensor) against the oracle's restatement
of TaxelSensor::internal_update, evaluated both on the engine's own contact
surfaces (hc_get_surface: the sensor alone) and on the oracle's surfaces (end
to end).  Two steps: the second moves one soft body out of contact
and shifts another, so kept values and the empty case are exercised."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
import oracle

pytestmark = pytest.mark.gpu

CONFIGS = [  # method, sample method, resolution, visualise
    (L.TAXEL_CLOSEST, L.SAMPLE_DEFAULT, 0.0015, 1),
    (L.TAXEL_SQUARED, L.SAMPLE_DEFAULT, 0.0015, 0),
    (L.TAXEL_WEIGHTED, L.SAMPLE_AREA_IMPORTANCE, 0.002, 0),
    (L.TAXEL_CLOSEST, L.SAMPLE_AREA_IMPORTANCE, 0.002, 1),
]
MARGIN = 0.002


def _taxels():
    g = np.linspace(-0.025, 0.025, 6)
    t = np.array([[x, y, 0.005] for x in g for y in g] + [[0.0, 0.0, 0.5]])
    return t


def _surfaces(eng, s, geom):
    out = []
    for p in range(len(s.g1)):
        if geom in (s.g1[p], s.g2[p]):
            srf = eng.surface(p)
            out.append(dict(poly_offset=srf["offset"], vert=srf["vert"], vert_pressure=srf["pressure"],
                            normal=srf["normal"]))
    return out


def _oracle_surfaces(orc, s, geom, xpos):
    """The oracle's own contact surfaces of the pairs that touch `geom`, in
    collision order (world frame, polygons in (soft element, other element)
    order): the sensor checked end to end, surfaces included."""
    out = []
    for p in range(len(s.g1)):
        if geom in (s.g1[p], s.g2[p]):
            srf = orc.surface(s.g1[p], s.g2[p], xpos=xpos)
            out.append(dict(poly_offset=srf["offset"], vert=srf["vert"], vert_pressure=srf["pressure"],
                            normal=srf["normal"]))
    return out


def _check(got, ref, scale, what):
    bad = np.abs(got - ref) > 1e-4 * scale + 1e-9
    assert bad.sum() == 0, (what, np.where(bad), got[bad], ref[bad], scale)


def test_taxel_sensor_matches_oracle(gpu):
    s = scenes.tactile(3, velocities=False, plate_half=(0.0401, 0.04, 0.005), min_pen=1e-3)
    eng = scenes.build_engine(s)
    tx = _taxels()
    sensors = {}
    for p in range(len(s.g1)):
        plate = s.g2[p]
        for ci, (m, sm, res, vis) in enumerate(CONFIGS):
            sensors[(plate, ci)] = eng.add_taxel_sensor(plate, tx, m, MARGIN, res, sm, bool(vis))
    eng.set_pairs(s.g1, s.g2)
    prev = {k: np.zeros(len(tx)) for k in sensors}
    prev_e2e = {k: np.zeros(len(tx)) for k in sensors}
    e2e_stats = []
    orc = oracle.Oracle(s)
    xpos = s.xpos.copy()
    for step in range(2):
        if step == 1:
            xpos[s.g1[0], 2] += 0.05          # scene 0 leaves contact
            xpos[s.g1[1], 0] += 0.004         # scene 1 slides
        eng.set_poses(xpos, s.xmat, s.vel)
        eng.step()
        for (plate, ci), sid in sensors.items():
            m, sm, res, vis = CONFIGS[ci]
            got = eng.taxel_sensor_values(sid).astype(np.float64)
            R = s.xmat[plate].reshape(3, 3)
            tw = tx @ R.T + xpos[plate]
            ref = oracle.taxel_sensor(tw, m, MARGIN, res, sm, vis, _surfaces(eng, s, plate), values=prev[(plate, ci)])
            scale = max(np.abs(ref).max(), 1e-12)
            _check(got, ref, scale, (step, plate, CONFIGS[ci]))
            prev[(plate, ci)] = ref
            # end to end: the oracle's sensor on the oracle's surfaces.  With
            # the default grid the samples of a polygon depend on its vertex
            # set and winding (each fan triangle's grid starts at the first
            # vertex of its polygon edge), which the engine's surfaces share
            # with the oracle's: every taxel within 1e-4 of the map maximum.
            # Area-importance draws walk the running area of the fan
            # triangles in order, which also depends on the vertex each
            # polygon starts at (the oracle's Sutherland-Hodgman clip of the
            # triangle starts elsewhere than the engine's clipped section),
            # so only the statistics are reported for those.
            ref2 = oracle.taxel_sensor(tw, m, MARGIN, res, sm, vis, _oracle_surfaces(orc, s, plate, xpos),
                                       values=prev_e2e[(plate, ci)])
            sc2 = max(np.abs(ref2).max(), 1e-12)
            d2 = np.abs(got - ref2) / sc2
            e2e_stats.append((step, plate, ci, float(d2.max()), float(np.mean(d2 <= 1e-4))))
            if sm == L.SAMPLE_DEFAULT:
                assert d2.max() <= 1e-4, ("oracle surfaces", e2e_stats[-1])
            prev_e2e[(plate, ci)] = ref2
            if step == 0 and plate == s.g2[0]:
                assert np.count_nonzero(ref) > 0
        # one bulk copy of every sensor equals the per-sensor reads
        each = np.concatenate([eng.taxel_sensor_values(sid) for sid in sorted(sensors.values())])
        np.testing.assert_array_equal(eng.all_taxel_sensor_values(), each)
        if step == 1:
            assert all(np.all(prev[(s.g2[0], ci)] == 0.0) for ci in range(len(CONFIGS)))
    eng.close()
    orc.close()
    for st in e2e_stats:
        print("end to end (step, plate, config, max err / map max, share within 1e-4):", st)


def test_disabled_sensor_keeps_values(gpu):
    s = scenes.tactile(1, velocities=False, plate_half=(0.0401, 0.04, 0.005), min_pen=1e-3)
    eng = scenes.build_engine(s)
    sid = eng.add_taxel_sensor(s.g2[0], _taxels(), L.TAXEL_SQUARED, MARGIN, 0.0015)
    eng.set_pairs(s.g1, s.g2)
    eng.step()
    v0 = eng.taxel_sensor_values(sid)
    eng.set_taxel_sensor_enabled(sid, False)
    xp = s.xpos.copy()
    xp[s.g1[0], 2] += 0.05
    eng.set_poses(xp, s.xmat, s.vel)
    eng.step()
    v1 = eng.taxel_sensor_values(sid)
    eng.set_taxel_sensor_enabled(sid, True)
    eng.step()
    v2 = eng.taxel_sensor_values(sid)
    eng.close()
    assert np.count_nonzero(v0) > 0 and np.array_equal(v0, v1) and np.all(v2 == 0)


def test_large_surface_and_taxel_groups(gpu):
    """One half-space contact of ~28k polygons (the polygon order is sorted in
    14 chunks and ranked across them) read by 1089 taxels (two passes of 1024
    taxels over the samples), against the oracle; area-importance samples
    depend on that order through the shared random stream."""
    s = scenes.Scene()
    ground = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
    box = s.add_geom(L.GEOM_BOX, [0.05, 0.05, 0.01], [2e5, 1.0, 0.0015, 0.5, 0.5])
    s.g1.append(box); s.g2.append(ground); s.scene_of_pair.append(0)
    scenes._alloc(s)
    s.xpos[box] = [0.0013, -0.0007, 0.01 - 0.0043]
    s.xmat[box] = scenes.rot_axis([0, 0, 1], 0.3).reshape(9)
    eng = scenes.build_engine(s)
    g = np.linspace(-0.06, 0.06, 33)
    tx = np.array([[x, y, 0.0] for x in g for y in g])
    cfgs = [(L.TAXEL_SQUARED, L.SAMPLE_DEFAULT, 0.004, 0, 0.003),
            (L.TAXEL_CLOSEST, L.SAMPLE_AREA_IMPORTANCE, 0.0005, 1, 0.004)]
    sids = [eng.add_taxel_sensor(ground, tx, m, mg, res, sm, bool(vis)) for (m, sm, res, vis, mg) in cfgs]
    eng.set_pairs(s.g1, s.g2)
    eng.step()
    srf = _surfaces(eng, s, ground)
    assert len(srf[0]["poly_offset"]) - 1 > 4 * 2048
    for sid, (m, sm, res, vis, mg) in zip(sids, cfgs):
        got = eng.taxel_sensor_values(sid).astype(np.float64)
        ref = oracle.taxel_sensor(tx, m, mg, res, sm, vis, srf, values=np.zeros(len(tx)))
        assert np.count_nonzero(ref) > 100
        _check(got, ref, max(np.abs(ref).max(), 1e-12), (m, sm))
    eng.close()
