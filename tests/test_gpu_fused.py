"""The fused forward step + adjoint (hc_step_adjoint, hc_step_adjoint_device:
one graph, one wait) against the same step run as separate calls
(hc_set_poses, hc_step, hc_get_wrenches, hc_get_taxels_all, hc_adjoint):
the same kernels on the same buffers, so the results are bit-identical, over
two steps at different poses, across a capacity overflow, and for every
query type."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scenes():
    return {
        "tactile": lambda: scenes.tactile(12, velocities=True, plate_half=(0.0401, 0.04, 0.005)),
        "soft_soft": lambda: scenes.soft_soft_pressed(2),
        "halfspace": lambda: scenes.halfspace(4),
        "batched": lambda: scenes.batched(6, tet_range=(500, 3000), tri_range=(12, 800)),
    }


def _separate(s, xpos, dLdw, dLdt, **kw):
    eng = scenes.build_engine(s, **kw)
    eng.set_adjoint_mode(True)
    eng.set_poses(xpos, s.xmat, s.vel)
    eng.step()
    w = eng.wrenches()
    t = eng.all_taxels()
    dp, dE = eng.adjoint(dLdw, dLdt)
    eng.close()
    return w, t, dp, dE


@pytest.mark.parametrize("name", list(_scenes()))
def test_fused_matches_separate_calls(gpu, name):
    s = _scenes()[name]()
    rng = np.random.default_rng(3)
    n_cells = 256 * len(s.sensors)
    eng = scenes.build_engine(s)
    try:
        for k in range(2):
            xpos = s.xpos + (rng.normal(0, 2e-4, s.xpos.shape) if k else 0.0)
            dLdw = rng.normal(size=(len(s.g1), 6))
            dLdt = rng.normal(size=n_cells).astype(np.float32) * 1e-3 if n_cells else None
            ref = _separate(s, xpos, dLdw, dLdt)
            got = eng.step_adjoint(xpos, s.xmat, s.vel, dLdw, dLdt)
            for a, b in zip(got, ref):
                assert np.array_equal(a, b)
            assert np.any(got[2] != 0)
    finally:
        eng.close()


def test_fused_grows_capacity_and_runs_again(gpu):
    # 16 kept polygons overflow at once: the call grows the records and runs
    # the whole step again before it returns
    s = _scenes()["tactile"]()
    rng = np.random.default_rng(5)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = rng.normal(size=256 * len(s.sensors)).astype(np.float32) * 1e-3
    ref = _separate(s, s.xpos, dLdw, dLdt)
    eng = scenes.build_engine(s, face_capacity=16, item_capacity=16)
    got = eng.step_adjoint(s.xpos, s.xmat, s.vel, dLdw, dLdt)
    eng.close()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


class _DevArray:
    """A view of n doubles at a device address (for torch.as_tensor)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3}


def test_fused_device_matches(gpu):
    torch = pytest.importorskip("torch")
    s = _scenes()["tactile"]()
    rng = np.random.default_rng(7)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = rng.normal(size=256 * len(s.sensors)).astype(np.float32) * 1e-3
    ref = _separate(s, s.xpos, dLdw, dLdt)
    eng = scenes.build_engine(s)
    eng.set_adjoint_mode(True)
    eng.enable_timing(True)
    gw = torch.tensor(dLdw, dtype=torch.float64, device="cuda")
    gt = torch.tensor(dLdt, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):   # the second call replays the graph
        ptr = eng.step_adjoint_device(gw.data_ptr(), gt.data_ptr())
        assert ptr
        w = eng.wrenches()       # synchronises the context stream
        t = eng.all_taxels()
        g = torch.as_tensor(_DevArray(ptr, len(s.g1) * 14), device="cuda").cpu().numpy().reshape(-1, 14)
        assert np.array_equal(w, ref[0]) and np.array_equal(t, ref[1])
        assert np.array_equal(g[:, :12].reshape(-1, 2, 6), ref[2]) and np.array_equal(g[:, 12:], ref[3])
        tm = eng.timings()
        assert tm.ms_adjoint > 0 and tm.ms_narrowphase > 0
    eng.close()
