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
    ef, et = wrench_errors(out["wrench"], ref["wrench"], ref["area"], ref["centroid"], ref["xm"])
    assert ef.max() <= WRENCH_RTOL, f"force rel err {ef.max():.3e}"
    assert et.max() <= WRENCH_RTOL, f"torque rel err {et.max():.3e}"
    return near


@pytest.mark.parametrize("repr_", [L.REPR_TRIANGLE, L.REPR_POLYGON])
def test_single_pair(gpu, repr_):
    # the soft-rigid single-pair workload at its full size: 1000 seeded poses
    s = scenes.single_pair(1000, velocities=True)
    out, ref = run_both(s, representation=repr_)
    check_pairs(out, ref, min_polys=20000)


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


def _stacked_planes_scene():
    """One item with 512 polygons: a soft sphere of 32 tets (one cluster,
    octahedral level 1, every tet apexed at the centre) sunk 2 cm into a
    rigid mesh of 32 stacked parallel triangles 0.02 mm apart (one cluster),
    each larger than the sphere.  The 16 lower-hemisphere tets cross all 32
    planes."""
    s = scenes.Scene()
    R = 0.03
    g = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [1e5, 1.0, scenes.sphere_hint(R, 1), 0.5, 0.5])
    V, F = [], []
    for k in range(32):
        z = -2e-5 * k
        V += [[-0.1, -0.1, z], [0.1, -0.1, z], [0.0, 0.1, z]]
        F.append([3 * k, 3 * k + 1, 3 * k + 2])
    m = s.add_geom(L.GEOM_MESH, [0, 0, 0], [0, 1.0, 0, 0.5, 0.5], np.array(V), np.array(F, np.int32))
    s.g1.append(g); s.g2.append(m); s.scene_of_pair.append(0)
    scenes._alloc(s)
    s.xpos[g] = [0.001, -0.002, 0.01]
    s.xmat[g] = scenes.rot_axis([0.3, 0.2, 1.0], 0.3).reshape(9)
    s.vel[g] = [0.02, -0.01, 0.03, 0.01, 0.02, -0.05]
    return s


def test_items_beyond_one_candidate_window(gpu):
    # more candidates per item than the warp's queue window holds (256): the
    # rounds refill it from the lanes' masks in the same lane-major order
    s = _stacked_planes_scene()
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=512)
    st = out["stats"][0]
    assert st.n_items == 1 and st.n_polygons == 512, (st.n_polygons, st.n_items)
    # the kept-polygon variant of the narrow kernel (adjoint mode, no debug)
    rng = np.random.default_rng(2)
    dLdw = rng.normal(size=(1, 6))
    grads = []
    for adjoint_mode in (True, False):
        eng = scenes.build_engine(s)
        eng.set_adjoint_mode(adjoint_mode)
        eng.step()
        ef, et = wrench_errors(eng.wrenches(), ref["wrench"], ref["area"], ref["centroid"], ref["xm"])
        assert ef.max() <= WRENCH_RTOL and et.max() <= WRENCH_RTOL, (adjoint_mode, ef, et)
        # the adjoint reads the kept polygons (adjoint mode) or recomputes
        # them through the same windows; the two agree to float rounding
        grads.append(eng.adjoint(dLdw, None)[0].ravel())
        eng.close()
    assert np.linalg.norm(grads[0] - grads[1]) <= 1e-5 * np.linalg.norm(grads[1])


def test_soft_soft_items_beyond_one_candidate_window(gpu):
    # a coarse soft box (1.5 cm tets) on a fine soft sphere (~2 mm tets): a
    # cluster of box tets overlaps most of a cluster of sphere tets
    s = scenes.Scene()
    b = s.add_geom(L.GEOM_BOX, [0.03, 0.03, 0.03], [2e5, 1.0, 0.015, 0.5, 0.5])
    R = 0.02
    a = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [1e5, 0.5, scenes.sphere_hint(R, 5), 0.5, 0.5])
    s.g1.append(b); s.g2.append(a); s.scene_of_pair.append(0)
    scenes._alloc(s)
    s.xpos[a] = [0.002, 0.001, 0.03 + R - 0.003]
    s.xmat[a] = scenes.random_rotation(np.random.default_rng(4)).reshape(9)
    s.vel[a] = [0.01, 0.02, -0.01, 0.02, -0.01, 0.03]
    out, ref = run_both(s)
    check_pairs(out, ref, min_polys=200)
    st = out["stats"][0]
    assert st.n_polygons > 0
    # adjoint over the same items: the wrench is homogeneous of degree 1 in
    # the two moduli, so E_M dL/dE_M + E_N dL/dE_N = L
    rng = np.random.default_rng(8)
    dLdw = rng.normal(size=(1, 6))
    eng = scenes.build_engine(s)
    eng.step()
    w = eng.wrenches()
    _, dE = eng.adjoint(dLdw, None)
    eng.close()
    L0 = float(np.dot(dLdw[0], w[0]))
    Eb, Ea = s.geoms[b]["cs5"][0], s.geoms[a]["cs5"][0]
    assert abs(Eb * dE[0, 0] + Ea * dE[0, 1] - L0) <= 1e-4 * abs(L0), (dE, L0)
