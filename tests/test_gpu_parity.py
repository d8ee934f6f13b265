"""GPU (C ABI) vs FP64 oracle parity on seeded scenes.

Bars: candidate element-pair sets and polygon vertex counts equal after a
canonical sort (near-degenerate pairs reported separately); wrench and area
within 1e-5 relative; taxels within 1e-5 of the map maximum (see _parity).
"""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
from oracle import Oracle
from tests._parity import AREA_RTOL, WRENCH_RTOL, compare_candidates, taxel_check, wrench_errors

pytestmark = pytest.mark.gpu


def run_both(scene, representation=L.REPR_TRIANGLE, apply_forces=True, use_graph=True):
    eng = scenes.build_engine(scene, representation=representation, apply_forces=apply_forces, use_graph=use_graph)
    eng.set_debug(1)
    eng.step()
    out = dict(wrench=eng.wrenches(), stats=eng.pair_stats(), cand=eng.candidates(),
               taxels=[eng.taxels(k) for k in range(len(scene.sensors))], order=eng.pair_order())
    eng.close()
    orc = Oracle(scene)
    ref = orc.collide(representation=representation, apply_forces=int(apply_forces), candidates=True)
    orc.close()
    return out, ref


def check_pairs(out, ref, min_polys=1):
    q, m, n = out["order"]
    assert np.array_equal(q, ref["query"])
    assert np.array_equal(m, ref["m"]) and np.array_equal(n, ref["n"])
    bad, near, common = compare_candidates(out["cand"], ref["candidates"])
    assert not bad, f"{len(bad)} candidate mismatches (first: {bad[:5]}), {near} near-degenerate"
    assert common >= min_polys
    npoly = np.array([s.n_polygons for s in out["stats"]])
    assert np.array_equal(npoly, ref["n_polygons"]) or near > 0
    area = np.array([s.area for s in out["stats"]])
    nz = ref["area"] > 0
    assert np.all(np.abs(area[nz] - ref["area"][nz]) <= AREA_RTOL * ref["area"][nz])
    ef, et = wrench_errors(out["wrench"], ref["wrench"], ref["area"])
    assert ef.max() <= WRENCH_RTOL, f"force rel err {ef.max():.3e}"
    assert et.max() <= WRENCH_RTOL, f"torque rel err {et.max():.3e}"
    return near


@pytest.mark.parametrize("repr_", [L.REPR_TRIANGLE, L.REPR_POLYGON])
def test_single_pair(gpu, repr_):
    s = scenes.single_pair(64, velocities=True)
    out, ref = run_both(s, representation=repr_)
    check_pairs(out, ref, min_polys=1000)


def test_single_pair_no_force_mode(gpu):
    s = scenes.single_pair(16, velocities=True)
    out, ref = run_both(s, apply_forces=False)
    assert np.all(out["wrench"] == 0)
    bad, near, common = compare_candidates(out["cand"], ref["candidates"])
    assert not bad and common > 0


def test_tactile(gpu):
    s = scenes.tactile(12, velocities=True, plate_half=(0.0401, 0.04, 0.005))
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=500)
    for k in range(len(s.sensors)):
        tg, to = out["taxels"][k], ref["taxels"][k]
        assert tg.shape == (256,)
        sample = float(np.abs(to).max()) / 25.0 * 2.0
        bad, one = taxel_check(tg, to, sample)
        assert bad == 0, f"sensor {k}: {bad} taxels off"
        assert one <= 2, f"sensor {k}: {one} taxels differ by one sample"


def test_halfspace(gpu):
    s = scenes.halfspace(8)
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=50)


def test_soft_soft(gpu):
    s = scenes.soft_soft(6, tet_range=(2000, 8000))
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=50)


def test_batched_small(gpu):
    s = scenes.batched(24, tet_range=(500, 4000), tri_range=(12, 800))
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=100)
