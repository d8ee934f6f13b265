"""Contact surfaces (hc_get_surface) against the oracle's, polygon by polygon
and vertex by vertex: the same element pairs in the canonical order, the same
vertex counts, and each polygon the oracle's one up to the vertex it starts
at, wound the same way (counter-clockwise about the direction in which the
section value grows, as the reference's polygons are).  The winding decides
which end of a polygon edge a taxel sensor's fan-triangle sample grid starts
from (taxel_sensor.cpp:183-249), so it is part of the surface's parity, not
only the vertex set: a polygon wound the other way gives the default grid
other samples.  Soft-rigid, soft vs half-space and soft-soft."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = 1e-6   # metres: FP32 surfaces against FP64 ones


def _dedupe(v):
    """The polygon without cyclically repeated vertices: a vertex on a clip
    plane (a near-degenerate element pair) comes out twice from the
    oracle's Sutherland-Hodgman clip, once from the device's."""
    keep = [i for i in range(len(v)) if np.abs(v[i] - v[i - 1]).max() > TOL]
    return v[keep] if keep else v[:1]


def _drop_collinear(v):
    """The polygon without vertices on the segment between their
    neighbours: where a clip plane passes through a polygon vertex (a
    near-degenerate element pair) one clip can emit a vertex on an edge that
    the other does not; the polygon, its area and its forces are the same."""
    out = list(v)
    changed = True
    while changed and len(out) > 3:
        changed = False
        for i in range(len(out)):
            a, b, c = out[i - 1], out[i], out[(i + 1) % len(out)]
            d = c - a
            L = np.linalg.norm(d)
            if L > 0 and np.linalg.norm(np.cross(b - a, d)) / L <= TOL and 0 <= (b - a) @ d <= L * L:
                del out[i]
                changed = True
                break
    return np.array(out)


def _match(ve, vo):
    """The cyclic shift of ve that equals vo within TOL, or None."""
    for r in range(len(ve)):
        if np.abs(np.roll(ve, r, axis=0) - vo).max() <= TOL:
            return r
    return None


def _check(s, min_polys):
    eng = scenes.build_engine(s)
    eng.step()
    orc = Oracle(s)
    total = collinear = 0
    for p in range(len(s.g1)):
        se = eng.surface(p)
        so = orc.surface(s.g1[p], s.g2[p])
        ke = list(zip(se["elem_a"].tolist(), se["elem_b"].tolist()))
        ko = list(zip(so["elem_a"].tolist(), so["elem_b"].tolist()))
        assert ke == ko, (p, len(ke), len(ko))
        for i in range(len(ke)):
            ve = _dedupe(se["vert"][se["offset"][i]:se["offset"][i + 1]])
            vo = _dedupe(so["vert"][so["offset"][i]:so["offset"][i + 1]])
            r = _match(ve, vo) if len(ve) == len(vo) else None
            if r is None:
                # a collinear vertex that one side has (or that the two
                # sides place at different points of the same edge)
                ve, vo = _drop_collinear(ve), _drop_collinear(vo)
                collinear += 1
                assert len(ve) == len(vo), (p, ke[i], len(ve), len(vo))
                r = _match(ve, vo)
            if r is None:
                rev = _match(ve[::-1], vo)
                dev = min(np.abs(np.roll(ve, k, axis=0) - vo).max() for k in range(len(ve)))
                size = np.ptp(vo, axis=0).max()
                raise AssertionError(f"pair {p} polygon {ke[i]}: no cyclic shift matches the oracle's "
                                     f"({'reversed winding' if rev is not None else 'different vertices'}; "
                                     f"best shift off by {dev:.3e} m, polygon size {size:.3e} m)\n"
                                     f"engine {np.round(ve, 9).tolist()}\noracle {np.round(vo, 9).tolist()}")
            # the unit normal: soft-soft's is the FP32 difference of two tet
            # gradients, normalised (FP64 only where a decision needs it)
            np.testing.assert_allclose(se["normal"][i], so["normal"][i], atol=1e-5)
        total += len(ke)
    eng.close()
    orc.close()
    print(f"{total} polygons, {collinear} compared without a collinear vertex one side has")
    assert collinear <= total // 50, (collinear, total)
    assert total >= min_polys, total


def test_soft_rigid_surfaces(gpu):
    _check(scenes.tactile(3, velocities=False, plate_half=(0.0401, 0.04, 0.005), min_pen=1e-3), 300)


def test_halfspace_surfaces(gpu):
    _check(scenes.halfspace(4, min_frac=0.03), 100)


def test_soft_soft_surfaces(gpu):
    _check(scenes.soft_soft_pressed(3, velocities=False), 100)
