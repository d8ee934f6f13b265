"""torch.autograd wrapper (mujoco_contact_surfaces_gb300.autograd) on the GPU:
gradients of L = dL/dwrench . wrench + dL/dtaxel . taxels with respect to
geom positions, rotation vectors (R = exp(rot) R0) and soft moduli, against
central differences of the FP64 oracle (step 1e-6; poses keep 1 mm of
penetration), and modulus identification from 64 target taxel maps computed
by the oracle at random moduli in 5e4-5e5 Pa."""
import copy

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import scenes
from oracle import Oracle

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-3


def _rodrigues(r):
    th = np.linalg.norm(r)
    if th < 1e-14:
        return np.eye(3)
    k = r / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K


def _oracle_L(orc, s, xpos, rot, dLdw, dLdt):
    xm = np.array([(_rodrigues(rot[g]) @ s.xmat[g].reshape(3, 3)).reshape(9) for g in range(len(xpos))])
    r = orc.collide(xpos=xpos, xmat=xm, taxels64=True)
    v = float(np.sum(dLdw * r["wrench"]))
    v += sum(float(np.dot(dLdt[k], r["taxels64"][k])) for k in range(len(s.sensors)))
    return v, r


@pytest.mark.parametrize("rot_scale", [0.0, 0.02])
def test_autograd_matches_oracle_fd(gpu, rot_scale):
    torch = pytest.importorskip("torch")
    from mujoco_contact_surfaces_gb300.autograd import ContactModel, contact
    s = scenes.tactile(2, velocities=True, plate_half=(0.0401, 0.04, 0.005), min_pen=1e-3)
    rng = np.random.default_rng(21)
    rot0 = rng.normal(size=(s.n_geom, 3)) * rot_scale
    # the soft bodies keep their penetration when rotated about their centres
    rot0[1::2] = 0.0
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) * 1e-3 for _ in s.sensors]
    model = ContactModel.from_scene(s)
    xpos = torch.tensor(s.xpos, dtype=torch.float64, requires_grad=True)
    rot = torch.tensor(rot0, dtype=torch.float64, requires_grad=True)
    E0 = torch.tensor([g["cs5"][0] for g in s.geoms], dtype=torch.float64, requires_grad=True)
    w, t = contact(model, xpos, rot, E0)
    L = torch.sum(torch.tensor(dLdw) * w) + torch.sum(torch.tensor(np.concatenate(dLdt)) * t)
    L.backward()
    gx, gr, gE = xpos.grad.numpy(), rot.grad.numpy(), E0.grad.numpy()
    model.engine.close()

    orc = Oracle(s)
    L0, r0 = _oracle_L(orc, s, s.xpos, rot0, dLdw, dLdt)
    for g in range(s.n_geom):
        fx, fr = np.zeros(3), np.zeros(3)
        for c in range(3):
            h = 1e-6
            xp = s.xpos.copy(); xp[g, c] += h
            xm = s.xpos.copy(); xm[g, c] -= h
            fx[c] = (_oracle_L(orc, s, xp, rot0, dLdw, dLdt)[0] - _oracle_L(orc, s, xm, rot0, dLdw, dLdt)[0]) / (2 * h)
            rp = rot0.copy(); rp[g, c] += h
            rm = rot0.copy(); rm[g, c] -= h
            fr[c] = (_oracle_L(orc, s, s.xpos, rp, dLdw, dLdt)[0] - _oracle_L(orc, s, s.xpos, rm, dLdw, dLdt)[0]) / (2 * h)
        ref = np.concatenate([fx, fr])
        got = np.concatenate([gx[g], gr[g]])
        err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err <= GRAD_RTOL, f"geom {g}: rel err {err:.2e}\n{got}\n{ref}"
    # modulus: the soft-rigid wrench and taxels are linear in E
    for p in range(len(s.g1)):
        soft = s.g1[p]
        E = s.geoms[soft]["cs5"][0]
        ref = (np.dot(dLdw[p], r0["wrench"][p]) + np.dot(dLdt[p], r0["taxels64"][p])) / E
        assert abs(gE[soft] - ref) <= 1e-4 * abs(ref) + 1e-12, (gE[soft], ref)
    assert np.all(gE[[s.g2[p] for p in range(len(s.g1))]] == 0.0)


def test_modulus_identification_64_maps(gpu):
    torch = pytest.importorskip("torch")
    from mujoco_contact_surfaces_gb300.autograd import ContactModel, identify_modulus
    s = scenes.tactile(64, velocities=False, plate_half=(0.0401, 0.04, 0.005), min_pen=5e-4)
    rng = np.random.default_rng(77)
    E_true = np.array([g["cs5"][0] for g in s.geoms])
    for p in range(len(s.g1)):
        E_true[s.g1[p]] = rng.uniform(5e4, 5e5)
    # targets: the FP64 oracle's taxel maps with the true moduli
    st = copy.deepcopy(s)
    for g, d in enumerate(st.geoms):
        d["cs5"] = list(d["cs5"])
        d["cs5"][0] = E_true[g] if g in s.g1 else d["cs5"][0]
    target = np.concatenate(Oracle(st).collide(taxels64=True)["taxels64"])
    model = ContactModel.from_scene(s)
    E_init = np.array([g["cs5"][0] for g in s.geoms])
    E_init[list(s.g1)] = 2e5
    E, hist = identify_modulus(model, s.xpos, target, E_init)
    model.engine.close()
    soft = list(s.g1)
    rel = np.abs(E.numpy()[soft] - E_true[soft]) / E_true[soft]
    assert hist[-1] < 1e-8 * max(hist[0], 1e-30) + 1e-12, hist
    assert rel.max() < 1e-3, rel.max()


def test_autograd_soft_soft_pairs(gpu):
    # soft-soft pairs: the moduli move the equal-pressure surface, so the
    # wrapper keeps them at the registered values and returns the adjoint's
    # exact dL/dE_M, dL/dE_N; pose gradients map as for the other pairs.
    torch = pytest.importorskip("torch")
    from mujoco_contact_surfaces_gb300.autograd import ContactModel, contact
    s = scenes.soft_soft_pressed(2)
    rng = np.random.default_rng(5)
    dLdw = rng.normal(size=(len(s.g1), 6))
    dLdt = [rng.normal(size=256) * 1e-3 for _ in s.sensors]
    model = ContactModel.from_scene(s)
    xpos = torch.tensor(s.xpos, dtype=torch.float64, requires_grad=True)
    rot = torch.zeros(s.n_geom, 3, dtype=torch.float64, requires_grad=True)
    E0 = torch.tensor([g["cs5"][0] for g in s.geoms], dtype=torch.float64, requires_grad=True)
    w, t = contact(model, xpos, rot, E0)
    L = torch.sum(torch.tensor(dLdw) * w) + torch.sum(torch.tensor(np.concatenate(dLdt)) * t)
    L.backward()
    eng = model.engine
    dpose, dE = eng.adjoint(dLdw, np.concatenate(dLdt).astype(np.float32))
    q, m, n = eng.pair_order()
    assert np.all(np.asarray(q) == 3)
    for p in range(len(s.g1)):
        assert E0.grad[int(m[p])].item() == dE[p, 0] and E0.grad[int(n[p])].item() == dE[p, 1]
        np.testing.assert_allclose(xpos.grad[int(m[p])].numpy(), dpose[p, 0, 3:], rtol=1e-12, atol=0)
        np.testing.assert_allclose(xpos.grad[int(n[p])].numpy(), dpose[p, 1, 3:], rtol=1e-12, atol=0)
    with pytest.raises(ValueError):
        contact(model, xpos, rot, E0.detach() * 1.5)
    eng.close()
