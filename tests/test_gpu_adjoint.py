"""Adjoint (C ABI, GPU) vs central finite differences of the FP64 oracle.

The gradient of L = dL/dwrench . wrench + dL/dtaxel . taxels with respect to
both geoms' world twists [dtheta; dx] (R <- exp(dtheta) R, x <- x + dx) and
the soft modulus.  Reference: central differences of the FP64 oracle at step
1e-6 (taxels from its FP64 evaluation of the same ray sampling).  Bar: 1e-3
relative error per pair (norm of the 12-vector of both twists).

Central differences only measure the derivative where the function is smooth
across the step: poses keep at least 1 mm of penetration (the force grows
with the square of the penetration near first touch), and the taxel maps,
piecewise linear in the pose with kinks where a ray crosses a tet face, are
differenced at 1e-7 so that few of the 6400 rays per sensor straddle a kink.
"""
import copy

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes
from mujoco_contact_surfaces_gb300.scenes import rot_axis
from oracle import Oracle

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-3


def perturb(xpos, xmat, g, comp, h):
    xp, xm = xpos.copy(), xmat.copy()
    if comp < 3:
        ax = np.zeros(3)
        ax[comp] = 1.0
        xm[g] = (rot_axis(ax, h) @ xm[g].reshape(3, 3)).reshape(9)
    else:
        xp[g, comp - 3] += h
    return xp, xm


def fd_gradient(orc, s, p, dLdw, dLdt, h=1e-6, representation=0):
    """Central differences of L for pair p: 12 components (M then N)."""
    m, n = orc.collide(pairs=[p], sensors=False)["m"][0], orc.collide(pairs=[p], sensors=False)["n"][0]

    def L(xp, xm):
        r = orc.collide(representation=representation, pairs=[p], xpos=xp, xmat=xm, sensors=dLdt is not None,
                        taxels64=dLdt is not None)
        v = float(np.dot(dLdw[p], r["wrench"][0]))
        if dLdt is not None:
            v += sum(float(np.dot(dLdt[k], r["taxels64"][k])) for k in range(len(s.sensors)))
        return v

    g = np.zeros(12)
    for b, geom in enumerate((m, n)):
        for c in range(6):
            xp, xm = perturb(s.xpos, s.xmat, geom, c, h)
            lp = L(xp, xm)
            xp, xm = perturb(s.xpos, s.xmat, geom, c, -h)
            lm = L(xp, xm)
            g[6 * b + c] = (lp - lm) / (2 * h)
    return g


def run_adjoint(s, dLdw, dLdt, adjoint_mode=True, **engine_kw):
    eng = scenes.build_engine(s, **engine_kw)
    if adjoint_mode:
        eng.lib.hc_set_adjoint_mode(eng.ctx, 1)
    eng.step()
    w = eng.wrenches()
    tax = eng.all_taxels() if s.sensors else None
    dt = np.concatenate(dLdt).astype(np.float32) if dLdt is not None else None
    dpose, dE = eng.adjoint(dLdw, dt)
    eng.close()
    return w, tax, dpose, dE


def test_wrench_gradient_single_pair(gpu):
    s = scenes.single_pair(6, velocities=True, min_pen=1e-3)
    rng = np.random.default_rng(7)
    dLdw = rng.normal(size=(len(s.g1), 6))
    w, _, dpose, dE = run_adjoint(s, dLdw, None)
    orc = Oracle(s)
    for p in range(len(s.g1)):
        ref = fd_gradient(orc, s, p, dLdw, None)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"


def test_wrench_and_taxel_gradient_tactile(gpu):
    s = scenes.tactile(4, velocities=True, plate_half=(0.0401, 0.04, 0.005), min_pen=1e-3)
    rng = np.random.default_rng(11)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) * 1e-3 for _ in s.sensors]
    w, tax, dpose, dE = run_adjoint(s, dLdw, dLdt)
    orc = Oracle(s)
    for p in range(len(s.g1)):
        ref = fd_gradient(orc, s, p, dLdw, dLdt, h=1e-7)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"


def _close_per_pair(d1, d2, rtol):
    for p in range(d1.shape[0]):
        a, b = d1[p].ravel(), d2[p].ravel()
        assert np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(b), 1e-30), (p, a, b)


def test_taxel_gradient_without_adjoint_mode(gpu):
    # without adjoint mode the adjoint re-runs the step to recover the ray
    # hits (the winning keys of the samples); in adjoint mode the step kept
    # them.  The two agree to float rounding.
    s = scenes.tactile(2, velocities=False, plate_half=(0.0401, 0.04, 0.005))
    rng = np.random.default_rng(3)
    dLdw = np.zeros((len(s.g1), 6))
    dLdt = [rng.normal(size=256) for _ in s.sensors]
    _, _, d1, _ = run_adjoint(s, dLdw, dLdt, adjoint_mode=False)
    _, _, d2, _ = run_adjoint(s, dLdw, dLdt, adjoint_mode=True)
    _close_per_pair(d1, d2, 1e-5)


def test_kept_polygons_match_recompute(gpu):
    # without sensors and without adjoint mode no polygons are kept and the
    # adjoint recomputes them; in adjoint mode it reads the kept polygons.
    # The two paths agree to float rounding.  The scenes hold polygons of
    # more than 4 vertices (the oracle counts them), which the kept-polygon
    # adjoint defers to turns of 8-lane groups.
    s = scenes.single_pair(6, velocities=True, min_pen=1e-3)
    cand = np.asarray(Oracle(s).collide(candidates=True)["candidates"])
    assert (cand[:, 3] > 4).sum() >= 4
    rng = np.random.default_rng(9)
    dLdw = rng.normal(size=(len(s.g1), 6))
    _, _, d1, e1 = run_adjoint(s, dLdw, None, adjoint_mode=False)
    _, _, d2, e2 = run_adjoint(s, dLdw, None, adjoint_mode=True)
    _close_per_pair(d1, d2, 1e-5)
    _close_per_pair(e1, e2, 1e-5)


def test_record_overflow_reruns_the_step(gpu):
    # A record capacity of 16 polygons overflows; the synchronising call
    # before the adjoint grows it and re-runs the step, after which forward
    # and adjoint equal those of an engine that never overflowed, bit for bit.
    s = scenes.tactile(6, velocities=True, plate_half=(0.0401, 0.04, 0.005))
    rng = np.random.default_rng(9)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dt = np.concatenate([rng.normal(size=256) * 1e-3 for _ in s.sensors]).astype(np.float32)
    ref = scenes.build_engine(s)
    ref.set_adjoint_mode(True)
    ref.step()
    w_ref, t_ref = ref.wrenches(), ref.all_taxels()
    d_ref, e_ref = ref.adjoint(dLdw, dt)
    ref.close()
    eng = scenes.build_engine(s, face_capacity=16)
    eng.set_adjoint_mode(True)
    eng.step()
    w, t = eng.wrenches(), eng.all_taxels()
    d, e = eng.adjoint(dLdw, dt)
    eng.close()
    assert np.array_equal(w, w_ref) and np.array_equal(t, t_ref)
    assert np.array_equal(d, d_ref) and np.array_equal(e, e_ref)


def test_modulus_gradient_is_linear_response(gpu):
    # soft-rigid wrench and taxels are proportional to E: dL/dE = L_E / E
    s = scenes.tactile(3, velocities=True, plate_half=(0.0401, 0.04, 0.005))
    rng = np.random.default_rng(5)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) for _ in s.sensors]
    w, tax, dpose, dE = run_adjoint(s, dLdw, dLdt)
    orc = Oracle(s)
    r = orc.collide(taxels64=True)
    for p in range(len(s.g1)):
        E = s.geoms[s.g1[p]]["cs5"][0]
        ref = (np.dot(dLdw[p], r["wrench"][p]) + np.dot(dLdt[p], r["taxels64"][p])) / E
        # the soft body is M (registered first)
        assert dE[p, 1] == 0.0
        assert abs(dE[p, 0] - ref) <= 1e-4 * abs(ref) + 1e-12, (dE[p], ref)


def test_adjoint_is_deterministic(gpu):
    s = scenes.tactile(8, velocities=True)
    rng = np.random.default_rng(1)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) for _ in s.sensors]
    a = run_adjoint(s, dLdw, dLdt)
    b = run_adjoint(s, dLdw, dLdt)
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])


def _scaled_moduli(s, geoms, f):
    st = copy.deepcopy(s)
    for g in geoms:
        st.geoms[g]["cs5"] = np.array(st.geoms[g]["cs5"], np.float64)
        st.geoms[g]["cs5"][0] *= f
    return st


def _pair_losses(s, dLdw, dLdt, representation=0):
    r = Oracle(s).collide(representation=representation, taxels64=dLdt is not None, sensors=dLdt is not None)
    return np.array([np.dot(dLdw[p], r["wrench"][p]) + (np.dot(dLdt[p], r["taxels64"][p]) if dLdt is not None else 0.0)
                     for p in range(len(s.g1))])


def test_soft_soft_gradient_poses_and_moduli(gpu):
    # soft sphere pressed into a soft box carrying the taxel grid; the box
    # is M in even scenes (sensor on the soft frame's geom) and N in odd
    # ones.  The equal-pressure surface moves with N's field and with both
    # moduli; the dissipations differ, so the combined damping depends on
    # E_M / E_N too.
    s = scenes.soft_soft_pressed(4)
    rng = np.random.default_rng(13)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) * 1e-3 for _ in s.sensors]
    w, tax, dpose, dE = run_adjoint(s, dLdw, dLdt)
    orc = Oracle(s)
    r0 = orc.collide(taxels64=True)
    assert np.all(r0["query"] == 3)
    # forward: wrenches and the soft box's taxel maps (16x16 each)
    tax = tax.reshape(len(s.sensors), -1)
    for p in range(len(s.g1)):
        assert np.linalg.norm(w[p] - r0["wrench"][p]) <= 1e-5 * np.linalg.norm(r0["wrench"][p])
        t_ref = r0["taxels64"][p]
        assert np.max(np.abs(tax[p] - t_ref)) <= 1e-4 * np.max(np.abs(t_ref))
    # poses: central differences of the oracle
    for p in range(len(s.g1)):
        ref = fd_gradient(orc, s, p, dLdw, dLdt, h=1e-7)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"
    # moduli: central differences in E_M (all pairs at once; pairs are
    # independent), then in E_N.  Mesh pressures are E x extent rounded to
    # FP32 (relative noise ~6e-8 per vertex), which swamps steps below ~1e-4;
    # at relative step 1e-3 the difference is smooth to ~1e-5.
    h = 1e-3
    ref = np.zeros((len(s.g1), 2))
    for b, geoms in enumerate((r0["m"], r0["n"])):
        lp = _pair_losses(_scaled_moduli(s, geoms, 1 + h), dLdw, dLdt)
        lm = _pair_losses(_scaled_moduli(s, geoms, 1 - h), dLdw, dLdt)
        E = np.array([s.geoms[g]["cs5"][0] for g in geoms])
        ref[:, b] = (lp - lm) / (2 * h * E)
    L0 = _pair_losses(s, dLdw, dLdt)
    for p in range(len(s.g1)):
        err = np.linalg.norm(dE[p] - ref[p]) / max(np.linalg.norm(ref[p]), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: dE rel err {err:.2e}\n{dE[p]}\n{ref[p]}"
        # wrench and taxels are homogeneous of degree 1 in (E_M, E_N)
        EM, EN = s.geoms[r0["m"][p]]["cs5"][0], s.geoms[r0["n"][p]]["cs5"][0]
        assert abs(EM * dE[p, 0] + EN * dE[p, 1] - L0[p]) <= 1e-4 * abs(L0[p]), (p, dE[p], L0[p])


def test_second_taxel_adjoint_of_a_step(gpu):
    # recomputed polygons (soft-soft) take their won ray samples once; a
    # second hc_adjoint of the same step re-runs the step and repeats the
    # first result bit for bit, and the device entry point refuses instead
    s = scenes.soft_soft_pressed(2)
    rng = np.random.default_rng(17)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dt = np.concatenate([rng.normal(size=256) for _ in s.sensors]).astype(np.float32)
    eng = scenes.build_engine(s)
    eng.set_adjoint_mode(True)
    eng.step()
    d1, e1 = eng.adjoint(dLdw, dt)
    d2, e2 = eng.adjoint(dLdw, dt)
    assert np.array_equal(d1, d2) and np.array_equal(e1, e2)
    assert np.any(e1 != 0.0)
    import torch
    gw = torch.tensor(dLdw, dtype=torch.float64, device="cuda")
    gt = torch.tensor(dt, device="cuda")
    torch.cuda.synchronize()
    with pytest.raises(RuntimeError):
        eng.adjoint_device(gw.data_ptr(), gt.data_ptr())
    eng.close()


def test_soft_soft_only_step_with_records_after_another_engine(gpu):
    # a step of soft-soft pairs alone runs no record scan (they keep no
    # polygons); its per-pair reduction must not read record offsets, which
    # then hold whatever the device memory held (here: an earlier engine's
    # records, freed before this engine allocates its own)
    t = scenes.tactile(64, velocities=True)
    eng = scenes.build_engine(t)
    eng.set_adjoint_mode(True)
    eng.step()
    eng.wrenches()
    eng.close()
    s = scenes.soft_soft_pressed(4)
    eng = scenes.build_engine(s)
    eng.set_adjoint_mode(True)
    eng.step()
    w = eng.wrenches()
    eng.close()
    ref = Oracle(s).collide()["wrench"]
    for p in range(len(s.g1)):
        assert np.linalg.norm(w[p] - ref[p]) <= 1e-5 * np.linalg.norm(ref[p]), (p, w[p], ref[p])


def test_gradient_polygon_quadrature_soft_rigid(gpu):
    # kPolygon: one quadrature point per polygon (its centroid) instead of
    # one per fan triangle; the adjoint reverses that point from the kept
    # polygons (wrench upstream: the taxel maps do not depend on the
    # quadrature)
    from mujoco_contact_surfaces_gb300 import _lib as L
    s = scenes.single_pair(4, velocities=True, min_pen=1e-3)
    rng = np.random.default_rng(23)
    dLdw = rng.normal(size=(len(s.g1), 6))
    _, _, dpose, _ = run_adjoint(s, dLdw, None, representation=L.REPR_POLYGON)
    orc = Oracle(s)
    for p in range(len(s.g1)):
        ref = fd_gradient(orc, s, p, dLdw, None, representation=1)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"


@pytest.mark.parametrize("adjoint_mode", [True, False])
def test_halfspace_gradient_poses_and_modulus(gpu, adjoint_mode):
    # soft primitives on a rigid ground plane (the half-space query).  In
    # adjoint mode the reverse reads the polygons the step kept; without it
    # (and without sensors) the half-space adjoint kernel recomputes them.
    # Poses against central differences of the oracle; the wrench is linear
    # in the soft modulus, so dL/dE = L / E.
    s = scenes.halfspace(4, min_frac=0.03)
    rng = np.random.default_rng(29)
    dLdw = rng.normal(size=(len(s.g1), 6))
    w, _, dpose, dE = run_adjoint(s, dLdw, None, adjoint_mode=adjoint_mode)
    orc = Oracle(s)
    r0 = orc.collide()
    assert np.all(r0["query"] == 2)
    for p in range(len(s.g1)):
        assert np.linalg.norm(w[p] - r0["wrench"][p]) <= 1e-5 * np.linalg.norm(r0["wrench"][p])
        ref = fd_gradient(orc, s, p, dLdw, None)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"
        soft = 0 if s.geoms[r0["m"][p]]["cs5"][0] > 0 else 1
        E = s.geoms[(r0["m"], r0["n"])[soft][p]]["cs5"][0]
        L0 = float(np.dot(dLdw[p], r0["wrench"][p]))
        assert dE[p, 1 - soft] == 0.0
        assert abs(dE[p, soft] - L0 / E) <= 1e-4 * abs(L0 / E), (p, dE[p], L0 / E)


def test_soft_soft_gradient_polygon_quadrature(gpu):
    # kPolygon on soft-soft pairs: one quadrature point per polygon, the
    # polygon recomputed in the reverse with its equal-pressure plane moving
    # with N's field and with both moduli (wrench upstream: the taxel maps do
    # not depend on the quadrature).  Poses and both moduli against central
    # differences of the oracle with the same quadrature.
    from mujoco_contact_surfaces_gb300 import _lib as L
    s = scenes.soft_soft_pressed(4)
    rng = np.random.default_rng(31)
    dLdw = rng.normal(size=(len(s.g1), 6))
    w, _, dpose, dE = run_adjoint(s, dLdw, None, representation=L.REPR_POLYGON)
    orc = Oracle(s)
    r0 = orc.collide(representation=1, sensors=False)
    for p in range(len(s.g1)):
        assert np.linalg.norm(w[p] - r0["wrench"][p]) <= 1e-5 * np.linalg.norm(r0["wrench"][p])
        ref = fd_gradient(orc, s, p, dLdw, None, representation=1)
        got = dpose[p].reshape(12)
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: rel err {err:.2e}\n{got}\n{ref}"
    h = 1e-3
    ref = np.zeros((len(s.g1), 2))
    for b, geoms in enumerate((r0["m"], r0["n"])):
        lp = _pair_losses(_scaled_moduli(s, geoms, 1 + h), dLdw, None, representation=1)
        lm = _pair_losses(_scaled_moduli(s, geoms, 1 - h), dLdw, None, representation=1)
        E = np.array([s.geoms[g]["cs5"][0] for g in geoms])
        ref[:, b] = (lp - lm) / (2 * h * E)
    for p in range(len(s.g1)):
        err = np.linalg.norm(dE[p] - ref[p]) / max(np.linalg.norm(ref[p]), 1e-30)
        assert err <= GRAD_RTOL, f"pair {p}: dE rel err {err:.2e}\n{dE[p]}\n{ref[p]}"


def _grazing_box_scene(tilt):
    """A soft box (5 layers of 4 mm) pressed into a rigid plate so that the
    plate's top plane lies on one of the box mesh's horizontal layers,
    tilted by `tilt` rad: tet edges in that layer cross the plane at about
    `tilt` rad."""
    from mujoco_contact_surfaces_gb300 import _lib as L
    s = scenes.Scene()
    b = s.add_geom(L.GEOM_BOX, [0.02, 0.02, 0.01], [1e5, 1.0, 0.004, 0.5, 0.5])
    p = s.add_geom(L.GEOM_BOX, [0.1, 0.1, 0.01], [0, 1.0, 0, 0.5, 0.5])
    s.g1.append(b); s.g2.append(p); s.scene_of_pair.append(0)
    scenes._alloc(s)
    s.xpos[b] = [0.0013, -0.0021, 0.01 + 0.01 - 0.004]
    s.xmat[b] = rot_axis([1, 0.3, 0], tilt).reshape(9)
    s.vel[b] = [0.01, -0.02, 0.01, 0.02, 0.01, -0.03]
    return s


@pytest.mark.parametrize("adjoint_mode", [True, False])
def test_soft_rigid_contraction_leaves_no_vertex_out(gpu, adjoint_mode):
    # The dependent-rows guard of the soft-rigid and half-space contractions
    # (normalised |det| below 1e-4) must not drop vertices of well-formed
    # contacts: none is left out on the test scenes, a grazing box included
    # (tet edges crossing the contact plane at 1e-3 rad)
    cases = {"single_pair": scenes.single_pair(16, velocities=True, min_pen=1e-3),
             "tactile": scenes.tactile(8, velocities=True, plate_half=(0.0401, 0.04, 0.005)),
             "halfspace": scenes.halfspace(4, min_frac=0.03),
             "grazing": _grazing_box_scene(1e-3)}
    for name, s in cases.items():
        rng = np.random.default_rng(3)
        eng = scenes.build_engine(s)
        eng.set_adjoint_mode(adjoint_mode)
        eng.set_debug(1)
        eng.step()
        assert np.any(eng.wrenches() != 0)
        eng.adjoint(rng.normal(size=(len(s.g1), 6)), None)
        n, dmin = eng.adjoint_skipped()
        eng.close()
        print(f"{name} (adjoint mode {adjoint_mode}): {n} vertices left out, smallest normalised det {dmin:.3e}")
        assert n == 0, (name, n, dmin)
