"""The batched workloads at their full sizes against the FP64 oracle:

* 4096 independent scenes of 1-8 soft-rigid pairs, soft meshes of 500-20000
  tets and rigid meshes of 12-5000 triangles (18402 pairs, ~170M elements);
* 1024 soft-soft pairs of 2k-50k tets each, E ratio 0.1-10.

The whole batch runs as one step.  A sample of its pairs (the largest
contacts and random others) is compared with the oracle on exactly those
pairs: candidate element-pair sets and per-pair polygon counts equal after a
canonical sort (near-degenerate pairs counted and reported), area and wrench
within 1e-5 (a pair made only of near-degenerate polygons within 5e-5).  Properties that hold at any size are checked on the whole
batch: a repeated step is bit-identical, and sampled pairs computed alone in
their own context give the batch's wrench and adjoint bit for bit (the batch
changes the scheduling, never a pair's arithmetic)."""
import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes
from oracle import Oracle
from tests._parity import AREA_RTOL, WRENCH_RTOL, compare_candidates, wrench_errors

NEAR_RTOL = 5 * WRENCH_RTOL   # pairs made only of near-degenerate polygons

pytestmark = pytest.mark.gpu


def _sample(npoly, n_sample, rng):
    n_pair = len(npoly)
    big = list(np.argsort(-npoly)[:n_sample // 4])
    rest = rng.choice(n_pair, n_sample, replace=False)
    return sorted(list(dict.fromkeys(int(x) for x in big + list(rest)))[:n_sample])


def _oracle_parity(s, pairs, w, stats, cand):
    """The batch's outputs of `pairs` against the oracle on those pairs."""
    sub = scenes.subscene(s, pairs)
    orc = Oracle(sub)
    ref = orc.collide(candidates=True)
    orc.close()
    pos = {p: k for k, p in enumerate(pairs)}
    sel = np.isin(cand[:, 0], pairs)
    mine = cand[sel].copy()
    mine[:, 0] = [pos[int(p)] for p in mine[:, 0]]
    bad, near, common = compare_candidates(mine, ref["candidates"])
    assert not bad, f"{len(bad)} candidate mismatches (first: {bad[:5]}), {near} near-degenerate"
    npoly = np.array([stats[p].n_polygons for p in pairs])
    if near == 0:
        assert np.array_equal(npoly, ref["n_polygons"])
    area = np.array([stats[p].area for p in pairs])
    nz = ref["area"] > 0
    ea = np.abs(area[nz] - ref["area"][nz]) / ref["area"][nz]
    assert ea.max(initial=0) <= AREA_RTOL, f"area rel err {ea.max():.3e}"
    ef, et = wrench_errors(w[pairs], ref["wrench"], ref["area"], ref["centroid"], ref["xm"])
    for k in np.argsort(-ef)[:3]:
        print(f"pair {pairs[k]}: force rel err {ef[k]:.2e}, torque {et[k]:.2e}, |F| "
              f"{np.linalg.norm(ref['wrench'][k, :3]):.3e}, area {ref['area'][k]:.3e}, {ref['n_polygons'][k]} polygons")
    # A pair whose every polygon is near-degenerate on either side (a value
    # within 1e-12 of a clip threshold) is decided by rounding in either
    # formulation, as its candidates are: such pairs are tiny slivers (areas
    # near 1e-9 m^2) and are held to five times the bar.
    ref_c = ref["candidates"]
    all_near = np.array([
        np.all(ref_c[ref_c[:, 0] == k, 4] & 1) or np.all(mine[mine[:, 0] == k, 4] & 1) if np.any(ref_c[:, 0] == k)
        else False for k in range(len(pairs))])
    for k in np.where(all_near)[0]:
        print(f"pair {pairs[k]}: every polygon near-degenerate; force rel err {ef[k]:.2e}, torque {et[k]:.2e}")
    held = ~all_near
    assert ef[held].max(initial=0) <= WRENCH_RTOL, f"force rel err {ef[held].max():.3e}"
    assert et[held].max(initial=0) <= WRENCH_RTOL, f"torque rel err {et[held].max():.3e}"
    assert ef[all_near].max(initial=0) <= NEAR_RTOL, f"force rel err {ef[all_near].max():.3e} (near-degenerate)"
    assert et[all_near].max(initial=0) <= NEAR_RTOL, f"torque rel err {et[all_near].max():.3e} (near-degenerate)"
    print(f"{len(pairs)} pairs, {common} polygons in common, {near} near-degenerate element pairs, "
          f"max rel err: force {ef.max():.2e}, torque {et.max():.2e}, area {ea.max(initial=0):.2e}")
    return common


def _check(s, n_oracle, n_alone, adjoint, seed, min_polys):
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
    # the same step with candidate recording: the candidate list of every pair
    eng.set_debug(1)
    eng.step()
    cand = eng.candidates()
    assert np.allclose(eng.wrenches(), w1, rtol=1e-9, atol=0)
    eng.close()
    npoly = np.array([st.n_polygons for st in stats])
    pairs = _sample(npoly, n_oracle, rng)
    assert _oracle_parity(s, pairs, w1, stats, cand) >= min_polys
    # a few pairs computed alone in their own context
    for p in pairs[:n_alone // 2] + [int(x) for x in np.argsort(-npoly)[:n_alone - n_alone // 2]]:
        e = scenes.build_engine(scenes.subscene(s, [p]))
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
    _check(s, n_oracle=384, n_alone=8, adjoint=True, seed=3, min_polys=20000)


def test_soft_soft_1024_pairs(gpu):
    s = scenes.soft_soft(1024)
    _check(s, n_oracle=128, n_alone=6, adjoint=False, seed=4, min_polys=20000)
