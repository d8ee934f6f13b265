"""Taxel-point sensor (hc_add_taxel_sensor) against the oracle's restatement
of TaxelSensor::internal_update, evaluated on the engine's own contact
surfaces (hc_get_surface: the polygons are checked against the oracle by the
parity tests).  Two steps: the second moves one soft body out of contact
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
            if step == 0 and plate == s.g2[0]:
                assert np.count_nonzero(ref) > 0
        if step == 1:
            assert all(np.all(prev[(s.g2[0], ci)] == 0.0) for ci in range(len(CONFIGS)))
    eng.close()


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
