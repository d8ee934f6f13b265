"""The batched workloads at their full sizes, through properties that do not
depend on size (the oracle checks element-level parity on the smaller
scenes of test_gpu_parity):

* 4096 independent scenes of 1-8 soft-rigid pairs, soft meshes of 500-20000
  tets and rigid meshes of 12-5000 triangles (18402 pairs, ~170M elements);
* 1024 soft-soft pairs of 2k-50k tets each.

Properties: a repeated step is bit-identical; every pair's wrench, and (soft-
rigid) its adjoint, is bit-identical to that pair computed alone in its own
context — the batch changes the scheduling, never a pair's arithmetic; the
forces are finite and the contacts non-trivial."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes

pytestmark = pytest.mark.gpu


def subscene(s, pairs):
    """The geoms, poses and pairs of the given pair indices, registered in
    their original relative order (so M/N stay as in the batch)."""
    keep = sorted({s.g1[p] for p in pairs} | {s.g2[p] for p in pairs})
    remap = {g: i for i, g in enumerate(keep)}
    t = scenes.Scene()
    for g in keep:
        d = s.geoms[g]
        t.add_geom(d["type"], d["size"], d["cs5"], d["mesh_v"], d["mesh_f"])
    scenes._alloc(t)
    for g in keep:
        t.xpos[remap[g]] = s.xpos[g]
        t.xmat[remap[g]] = s.xmat[g]
        t.vel[remap[g]] = s.vel[g]
    for p in pairs:
        t.g1.append(remap[s.g1[p]]); t.g2.append(remap[s.g2[p]]); t.scene_of_pair.append(0)
    return t


def _check(s, n_sample, adjoint, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    n_pair = len(s.g1)
    eng = scenes.build_engine(s)
    if adjoint:
        eng.set_adjoint_mode(True)
    eng.step()
    w1 = eng.wrenches()
    eng.step()
    w2 = eng.wrenches()
    assert np.array_equal(w1, w2)
    assert np.all(np.isfinite(w1))
    touching = np.linalg.norm(w1[:, :3], axis=1) > 0
    assert touching.mean() > 0.5
    if adjoint:
        up = rng.standard_normal((n_pair, 6))
        dpose, dE = eng.adjoint(up)
        assert np.all(np.isfinite(dpose)) and np.all(np.isfinite(dE))
    stats = eng.pair_stats()
    eng.close()
    # the sample: the largest contacts and random others
    npoly = np.array([st.n_polygons for st in stats])
    pick = list(np.argsort(-npoly)[:n_sample // 2]) + list(rng.choice(n_pair, n_sample - n_sample // 2,
                                                                       replace=False))
    for p in dict.fromkeys(int(x) for x in pick):
        e = scenes.build_engine(subscene(s, [p]))
        if adjoint:
            e.set_adjoint_mode(True)
        e.step()
        w = e.wrenches()[0]
        assert np.array_equal(w, w1[p]), (p, w, w1[p])
        if adjoint:
            dp, de = e.adjoint(up[p:p + 1])
            assert np.array_equal(dp[0], dpose[p]) and np.array_equal(de[0], dE[p]), p
        e.close()


def test_batched_4096_scenes(gpu):
    s = scenes.batched(4096)
    assert len(s.g1) > 16000
    _check(s, 16, adjoint=True, seed=3)


def test_soft_soft_1024_pairs(gpu):
    s = scenes.soft_soft(1024)
    _check(s, 12, adjoint=False, seed=4)
