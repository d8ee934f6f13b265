"""Engine properties on the GPU: determinism, graph vs eager launches, the
autotuner, capacity regrowth, non-finite poses, unsupported pairs and geom
resizing.  Each compares the C-ABI outputs of two runs that must agree
bit for bit."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import scenes

pytestmark = pytest.mark.gpu


def _outputs(eng, scene):
    eng.step()
    w = eng.wrenches()
    t = eng.all_taxels() if scene.sensors else np.zeros(0, np.float32)
    st = eng.pair_stats()
    return w, t, np.array([x.n_polygons for x in st]), np.array([x.area for x in st])


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_step_is_deterministic_and_graph_matches_eager(gpu):
    s = scenes.tactile(16, velocities=True)
    e1 = scenes.build_engine(s)
    e2 = scenes.build_engine(s, use_graph=False)
    a, b = _outputs(e1, s), _outputs(e2, s)
    c = _outputs(e1, s)
    e1.close(); e2.close()
    assert a[2].sum() > 0
    _same(a, b)
    _same(a, c)


def test_autotune_keeps_results(gpu):
    s = scenes.tactile(64, velocities=True)
    eng = scenes.build_engine(s)
    ref = _outputs(eng, s)
    ct, ch = eng.autotune()
    assert ct in (2, 3, 4, 6, 8) and ch in (1, 2, 4, 8)
    _same(ref, _outputs(eng, s))
    eng.close()


def test_item_and_record_overflow_regrow(gpu):
    s = scenes.batched(12, tet_range=(500, 4000), tri_range=(12, 600))
    ref_eng = scenes.build_engine(s)
    ref = _outputs(ref_eng, s)
    ref_eng.close()
    eng = scenes.build_engine(s, item_capacity=16, face_capacity=8)
    got = _outputs(eng, s)
    eng.close()
    assert ref[2].sum() > 0
    _same(ref, got)


def test_nonfinite_pose_zeroes_its_pairs_only(gpu):
    s = scenes.single_pair(6, velocities=True)
    eng = scenes.build_engine(s)
    ref = _outputs(eng, s)
    xp = s.xpos.copy()
    xp[s.g2[2], 1] = np.nan
    eng.set_poses(xp, s.xmat, s.vel)
    w, _, npoly, _ = _outputs(eng, s)
    eng.close()
    assert np.all(w[2] == 0.0) and npoly[2] == 0
    keep = [p for p in range(len(s.g1)) if p != 2]
    assert np.array_equal(w[keep], ref[0][keep])


def test_unsupported_pairs_are_reported_and_skipped(gpu):
    s = scenes.single_pair(2)
    eng = scenes.build_engine(s)
    ref = _outputs(eng, s)
    # a rigid-rigid pair and a capsule (no contact surface) next to the real ones
    k1 = eng.add_geom(100, L.GEOM_BOX, [0.1, 0.1, 0.1], [0, 1, 0, 0.5, 0.5])
    assert k1 == L.RIGID
    with pytest.raises(L.HCError) as ei:   # no capsule surface
        eng.add_geom(101, L.GEOM_CAPSULE, [0.02, 0.05, 0], [1e5, 1, 0, 0.5, 0.5])
    assert ei.value.status == L.HC_ERR_UNSUPPORTED
    g1 = list(s.g1) + [100, 101]
    g2 = list(s.g2) + [s.g2[0], s.g1[0]]
    st, q = eng.set_pairs(g1, g2)
    assert list(st[-2:]) == [L.HC_ERR_UNSUPPORTED, L.HC_ERR_UNSUPPORTED] and list(q[-2:]) == [0, 0]
    xp = np.concatenate([s.xpos, np.zeros((102 - s.n_geom, 3))])
    xm = np.concatenate([s.xmat, np.tile(np.eye(3).reshape(1, 9), (102 - s.n_geom, 1))])
    v = np.concatenate([s.vel, np.zeros((102 - s.n_geom, 6))])
    eng.set_poses(xp, xm, v)
    eng.step()
    w = eng.wrenches()
    eng.close()
    assert np.all(w[-2:] == 0.0)
    assert np.array_equal(w[:-2], ref[0])


def test_update_geom_size_matches_fresh_engine(gpu):
    s = scenes.single_pair(3)
    eng = scenes.build_engine(s)
    _outputs(eng, s)
    soft = s.g1[0]
    new = list(s.geoms[soft]["size"])
    new[0] *= 1.05
    eng.update_geom_size(soft, new)
    got = _outputs(eng, s)
    eng.close()
    s.geoms[soft]["size"] = new
    fresh = scenes.build_engine(s)
    ref = _outputs(fresh, s)
    fresh.close()
    _same(ref, got)


@pytest.mark.parametrize("which", ["soft", "rigid"])
def test_update_geom_size_matches_oracle(gpu, which):
    # hc_update_geom_size (the reference's onGeomChanged) regenerates the
    # geom's mesh, field and LBVH; the next step must equal the FP64 oracle
    # run on the resized primitive (candidates, counts, area, wrench, taxels)
    from oracle import Oracle
    from tests.test_gpu_parity import check_pairs
    from tests._parity import taxel_check
    if which == "soft":
        s = scenes.tactile(6, velocities=True, plate_half=(0.0401, 0.04, 0.005), min_pen=5e-4)
    else:
        s = scenes.single_pair(6, velocities=True)
    eng = scenes.build_engine(s)
    eng.set_debug(1)
    eng.step()
    for p in range(len(s.g1)):
        g = s.g1[p] if which == "soft" else s.g2[p]
        size = np.array(s.geoms[g]["size"], np.float64)
        if which == "soft":
            size = size * 1.04                     # every half-size and radius
        else:
            size[:2] *= 0.6 + 0.1 * p              # a smaller box top, same height
        eng.update_geom_size(g, size)
        s.geoms[g]["size"] = size
    eng.step()
    out = dict(wrench=eng.wrenches(), stats=eng.pair_stats(), cand=eng.candidates(), order=eng.pair_order(),
               taxels=[eng.taxels(k) for k in range(len(s.sensors))])
    eng.close()
    orc = Oracle(s)
    ref = orc.collide(candidates=True)
    orc.close()
    check_pairs(out, ref, min_polys=200)
    for k in range(len(s.sensors)):
        tg, to = out["taxels"][k], ref["taxels"][k]
        bad, one = taxel_check(tg, to, float(np.abs(to).max()) / 25.0 * 2.0)
        assert bad == 0 and one <= 2, (k, bad, one)


def _spread(q):
    q = q.astype(np.uint64)
    q = (q * 0x00010001) & 0xFF0000FF
    q = (q * 0x00000101) & 0x0F00F00F
    q = (q * 0x00000011) & 0xC30C30C3
    q = (q * 0x00000005) & 0x49249249
    return q


def _morton_order(v, e):
    """A stable sort of the elements by the Morton code of their centroids
    (10 bits per axis of the place in the vertices' bounding box), FP64."""
    lo, hi = v.min(0), v.max(0)
    ext = hi - lo
    c = np.zeros((len(e), 3))
    for k in range(e.shape[1]):
        c = c + v[e[:, k]] / e.shape[1]
    f = np.where(ext > 0, (c - lo) / np.where(ext > 0, ext, 1.0), 0.5)
    q = np.minimum(1023.0, np.maximum(0.0, f * 1024.0)).astype(np.uint32)
    code = (_spread(q[:, 0]) << 2) | (_spread(q[:, 1]) << 1) | _spread(q[:, 2])
    return np.argsort(code, kind="stable")


def test_device_lbvh_order_matches_morton_sort(gpu):
    # the LBVH leaf order built on the device (Morton keys, chunk sorts in
    # shared memory, ranks across chunks) against a stable sort of the same
    # codes: small rigid meshes, and soft meshes of up to ~50k tets (dozens
    # of 2048-key chunks)
    s = scenes.batched(6)
    t = scenes.soft_soft(4, tet_range=(30000, 50000))
    for sc in (s, t):
        eng = scenes.build_engine(sc)
        n_checked = 0
        for g in range(sc.n_geom):
            v, p, e = eng.geom_mesh(g)
            if len(e) == 0:
                continue
            got = eng.element_order(g)
            assert np.array_equal(got, _morton_order(v, e)), g
            n_checked += len(e)
        eng.close()
        assert n_checked > 1000
