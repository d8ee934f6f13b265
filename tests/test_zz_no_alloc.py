"""hc_step_noalloc (the forward step with its working memory in the library's
static device array) against hc_step, through the C ABI.

Two calls in a row at different poses, each compared with hc_step at the same
poses, within the parity tolerances (wrench 1e-5 relative, taxels 1e-5 of the
map maximum); hc_step's own outputs must stay untouched by the calls.  The
file runs last so the array has seen nothing else before it in a fresh
process, and everything else before it in a full run.
"""
import ctypes as C

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes
from tests._parity import WRENCH_RTOL, taxel_check, wrench_errors

pytestmark = pytest.mark.gpu


def _scenes():
    return {
        "tactile": lambda: scenes.tactile(6, velocities=True),
        "halfspace": lambda: scenes.halfspace(4),
        "soft_soft": lambda: scenes.soft_soft(3, tet_range=(2000, 6000)),
        "batched": lambda: scenes.batched(6, tet_range=(500, 3000), tri_range=(12, 800)),
    }


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _noalloc(eng, torch, xpos, xmat, vel, n_cells):
    dev = torch.device("cuda:0")
    d_xpos = torch.from_numpy(np.ascontiguousarray(xpos, np.float64)).to(dev)
    d_xmat = torch.from_numpy(np.ascontiguousarray(xmat, np.float64)).to(dev)
    d_vel = torch.from_numpy(np.ascontiguousarray(vel, np.float64)).to(dev)
    d_w = torch.full((max(1, eng.n_pair), 6), float("nan"), dtype=torch.float64, device=dev)
    d_t = torch.full((max(1, n_cells),), float("nan"), dtype=torch.float32, device=dev) if n_cells else None
    torch.cuda.synchronize()
    st = eng.lib.hc_step_noalloc(eng.ctx, xpos.shape[0], _ptr(d_xpos), _ptr(d_xmat), _ptr(d_vel), _ptr(d_w),
                                 _ptr(d_t), None)
    L.check(st)
    return d_w.cpu().numpy()[: eng.n_pair], (d_t.cpu().numpy() if n_cells else np.zeros(0, np.float32))


def _check(w_ref, t_ref, area, w, t):
    assert np.all(np.isfinite(w))
    ef, et = wrench_errors(w, w_ref, area)
    assert ef.max(initial=0) <= WRENCH_RTOL and et.max(initial=0) <= WRENCH_RTOL, (ef.max(), et.max())
    if t_ref.size:
        bad, one = taxel_check(t, t_ref, 0.0)
        assert bad == 0 and one == 0


@pytest.mark.parametrize("name", list(_scenes()))
def test_noalloc_matches_step_two_calls(gpu, name):
    torch = pytest.importorskip("torch")
    scene = _scenes()[name]()
    eng = scenes.build_engine(scene)
    try:
        rng = np.random.default_rng(7)
        poses = [(scene.xpos.copy(), scene.xmat.copy(), scene.vel.copy())]
        xp = scene.xpos + rng.normal(0, 2e-4, scene.xpos.shape)
        poses.append((xp, scene.xmat.copy(), scene.vel * 0.5))
        for xpos, xmat, vel in poses:
            eng.set_poses(xpos, xmat, vel)
            eng.step()
            w_ref = eng.wrenches()
            area = np.array([s.area for s in eng.pair_stats()])
            t_ref = eng.all_taxels() if scene.sensors else np.zeros(0, np.float32)
            assert np.any(area > 0)
            w, t = _noalloc(eng, torch, xpos, xmat, vel, t_ref.size)
            _check(w_ref, t_ref, area, w, t)
            # the context still reports hc_step's results
            assert np.array_equal(eng.wrenches(), w_ref)
            if t_ref.size:
                assert np.array_equal(eng.all_taxels(), t_ref)
    finally:
        eng.close()


def test_noalloc_rejects_oversized_step(gpu):
    torch = pytest.importorskip("torch")
    # eight 160 x 160-cell sensors at 5 x 5 rays per cell: 8 x 640,000 ray
    # samples of 8 bytes do not fit in the 32 MiB array
    scene = scenes.tactile(8, sampling_resolution=5)
    for sn in scene.sensors:
        sn["resolution"] = 0.0005
    eng = scenes.build_engine(scene)
    try:
        n_cells = 0
        for sn in scene.sensors:
            xs, ys = scene.geoms[sn["geom"]]["size"][:2]
            n_cells += int(np.floor(2 * xs / sn["resolution"] + 0.1)) * int(np.floor(2 * ys / sn["resolution"] + 0.1))
        with pytest.raises(L.HCError) as ei:
            _noalloc(eng, torch, scene.xpos, scene.xmat, scene.vel, n_cells)
        assert ei.value.status == 3 and "too small" in str(ei.value)
    finally:
        eng.close()
    # a step that fits still runs after the rejection
    scene = scenes.halfspace(2)
    eng = scenes.build_engine(scene)
    try:
        eng.step()
        w_ref = eng.wrenches()
        area = np.array([s.area for s in eng.pair_stats()])
        w, _ = _noalloc(eng, torch, scene.xpos, scene.xmat, scene.vel, 0)
        _check(w_ref, np.zeros(0), area, w, np.zeros(0))
    finally:
        eng.close()


def test_noalloc_refuses_taxel_point_and_curved_sensors(gpu):
    torch = pytest.importorskip("torch")
    # taxel-point and curved sensors read the polygons hc_step keeps; the
    # allocation-free step keeps none, so it refuses such a context instead
    # of returning with their values untouched
    scene = scenes.tactile(2, velocities=True)
    grid = np.array([[x, y, 0.005] for x in (-0.01, 0.0, 0.01) for y in (-0.01, 0.0, 0.01)])
    for kind in ("taxel", "curved"):
        eng = scenes.build_engine(scene)
        try:
            plate = scene.sensors[0]["geom"]
            if kind == "taxel":
                eng.add_taxel_sensor(plate, grid, L.TAXEL_SQUARED, 0.002, 0.0015)
            else:
                pts = grid.copy()
                nrm = np.tile([0.0, 0.0, 1.0], (len(pts), 1))
                eng.add_curved_sensor(plate, grid, 0.005, pts, nrm)
            eng.set_pairs(scene.g1, scene.g2)
            with pytest.raises(L.HCError) as ei:
                _noalloc(eng, torch, scene.xpos, scene.xmat, scene.vel, 256 * len(scene.sensors))
            assert ei.value.status == L.HC_ERR_UNSUPPORTED and "flat sensors only" in str(ei.value)
        finally:
            eng.close()
