"""torch.autograd wrapper of the contact step and its adjoint, and modulus
identification from target taxel maps.

``ContactFunction`` maps geom positions, rotation perturbations and soft
moduli to the per-pair wrenches and the taxel maps of an ``Engine``:

    R_g = exp([rot_g]x) R0_g,   x_g = xpos_g,
    wrench_p = (E_s(p) / E0_s(p)) * wrench_p(poses; E0),
    taxels of a sensor = (E_s(p) / E0_s(p)) * taxels(poses; E0)  (p: the sensor's pair).

On a soft-rigid or soft-half-space pair the wrench and the taxel pressures
are exactly linear in the soft modulus (pressure = E * extent, the damping
and stiffness terms scale with it too: mujoco_contact_surfaces_plugin.cpp:
394-402, 458), so the modulus enters as a scale of the step at the moduli
the geoms were registered with.  On a soft-soft pair the moduli move the
equal-pressure surface itself, so they are not a scale: the geoms of such
pairs keep their registered moduli (a different E raises) and the gradient
in E is the adjoint's exact dL/dE_M, dL/dE_N.  The backward pass is the engine's
hand-written adjoint (hc_adjoint): twists [dtheta; dx] of both geoms of every
pair, mapped to ``xpos`` by summing dx over the pairs a geom takes part in
and to ``rot`` through the left Jacobian of SO(3) at ``rot``.
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Engine


def _hat(w: torch.Tensor) -> torch.Tensor:
    z = torch.zeros_like(w[..., 0])
    return torch.stack([torch.stack([z, -w[..., 2], w[..., 1]], -1),
                        torch.stack([w[..., 2], z, -w[..., 0]], -1),
                        torch.stack([-w[..., 1], w[..., 0], z], -1)], -2)


def so3_exp(r: torch.Tensor) -> torch.Tensor:
    """Rodrigues' formula, batched over the leading dimensions."""
    th = torch.linalg.norm(r, dim=-1, keepdim=True)
    small = th < 1e-8
    ths = torch.where(small, torch.ones_like(th), th)
    a = torch.where(small, 1.0 - th ** 2 / 6.0, torch.sin(ths) / ths)[..., None]
    b = torch.where(small, 0.5 - th ** 2 / 24.0, (1.0 - torch.cos(ths)) / ths ** 2)[..., None]
    K = _hat(r)
    eye = torch.eye(3, dtype=r.dtype, device=r.device).expand(K.shape)
    return eye + a * K + b * (K @ K)


def so3_left_jacobian(r: torch.Tensor) -> torch.Tensor:
    """J_l(r): exp([r + dr]x) = exp([J_l(r) dr]x) exp([r]x) to first order."""
    th = torch.linalg.norm(r, dim=-1, keepdim=True)
    small = th < 1e-6
    ths = torch.where(small, torch.ones_like(th), th)
    a = torch.where(small, 0.5 - th ** 2 / 24.0, (1.0 - torch.cos(ths)) / ths ** 2)[..., None]
    b = torch.where(small, 1.0 / 6.0 - th ** 2 / 120.0, (ths - torch.sin(ths)) / ths ** 3)[..., None]
    K = _hat(r)
    eye = torch.eye(3, dtype=r.dtype, device=r.device).expand(K.shape)
    return eye + a * K + b * (K @ K)


class ContactModel:
    """An Engine plus what the autograd function needs: base orientations,
    velocities, registered moduli, and the pair / sensor bookkeeping."""

    def __init__(self, engine: Engine, xmat0, vel, E0, sensor_pair=None):
        self.engine = engine
        self.xmat0 = torch.as_tensor(np.asarray(xmat0, np.float64).reshape(-1, 3, 3))
        self.vel = None if vel is None else np.ascontiguousarray(vel, np.float64)
        self.E0 = torch.as_tensor(np.asarray(E0, np.float64))
        q, m, n = engine.pair_order()
        self.query, self.m, self.n = q, m, n
        # the soft geom of each pair (M for soft-soft)
        soft = []
        for p in range(engine.n_pair):
            km = engine.geom_info(int(m[p])).kind
            soft.append(int(m[p]) if km == 1 else int(n[p]))
        self.soft = torch.as_tensor(np.asarray(soft, np.int64))
        # soft-soft pairs: the moduli move the equal-pressure surface, so they
        # are not a scale; those geoms keep their registered modulus and the
        # adjoint gives dL/dE of both
        self.ss = torch.as_tensor(np.asarray([int(x) == 3 for x in q], bool))
        self.ss_geoms = sorted({int(g) for p in range(engine.n_pair) if self.ss[p] for g in (m[p], n[p])})
        self.n_sensor = len(engine.sensors)
        self.sensor_cells = [engine.sensors[k][0] * engine.sensors[k][1] for k in range(self.n_sensor)]
        self.sensor_pair = list(sensor_pair) if sensor_pair is not None else []
        if self.n_sensor and len(self.sensor_pair) != self.n_sensor:
            raise ValueError("sensor_pair: the pair index of every sensor is needed to scale its map by E")

    @classmethod
    def from_scene(cls, scene, **engine_kw):
        from .scenes import build_engine
        eng = build_engine(scene, **engine_kw)
        eng.set_adjoint_mode(True)
        E0 = [g["cs5"][0] for g in scene.geoms]
        # each sensor's pair: the pair that contains the sensor's geom
        sp = []
        for sn in scene.sensors:
            ps = [p for p in range(len(scene.g1)) if sn["geom"] in (scene.g1[p], scene.g2[p])]
            if len(ps) != 1:
                raise ValueError("each sensor must belong to exactly one pair")
            sp.append(ps[0])
        return cls(eng, scene.xmat, scene.vel, E0, sp)


class ContactFunction(torch.autograd.Function):
    """(xpos, rot, E) -> (wrench n_pair x 6, taxels of all sensors), float64."""

    @staticmethod
    def forward(ctx, model: ContactModel, xpos: torch.Tensor, rot: torch.Tensor, E: torch.Tensor):
        eng = model.engine
        R = so3_exp(rot.detach().cpu()) @ model.xmat0
        xp = xpos.detach().cpu().numpy().astype(np.float64)
        eng.set_poses(xp, R.reshape(-1, 9).numpy(), model.vel)
        eng.step()
        w = torch.as_tensor(eng.wrenches())
        t = torch.as_tensor(eng.all_taxels().astype(np.float64)) if model.n_sensor else torch.zeros(0, dtype=torch.float64)
        Ed = E.detach().cpu()
        if model.ss_geoms and not torch.equal(Ed[model.ss_geoms], model.E0[model.ss_geoms]):
            raise ValueError("geoms of soft-soft pairs keep their registered modulus")
        scale = torch.where(model.ss, torch.ones(()), (Ed / model.E0)[model.soft])   # per pair
        w = w * scale[:, None]
        tscale = torch.cat([scale[p].repeat(c) for p, c in zip(model.sensor_pair, model.sensor_cells)]) \
            if model.n_sensor else torch.zeros(0, dtype=torch.float64)
        t = t * tscale
        ctx.model = model
        ctx.save_for_backward(rot.detach().cpu(), scale, tscale)
        ctx.dev = xpos.device
        return w.to(xpos.device), t.to(xpos.device)

    @staticmethod
    def backward(ctx, gw: torch.Tensor, gt: torch.Tensor):
        model = ctx.model
        rot, scale, tscale = ctx.saved_tensors
        eng = model.engine
        gw = gw.detach().cpu().to(torch.float64) * scale[:, None]
        gt = gt.detach().cpu().to(torch.float64) * tscale if gt is not None and gt.numel() else None
        dpose, dE = eng.adjoint(gw.numpy(), gt.numpy().astype(np.float32) if gt is not None else None)
        n_geom = rot.shape[0]
        gx = torch.zeros(n_geom, 3, dtype=torch.float64)
        gth = torch.zeros(n_geom, 3, dtype=torch.float64)
        gE = torch.zeros(n_geom, dtype=torch.float64)
        dpose = torch.as_tensor(dpose)
        dE = torch.as_tensor(dE)
        for p in range(eng.n_pair):
            for b, g in enumerate((int(model.m[p]), int(model.n[p]))):
                gth[g] += dpose[p, b, :3]
                gx[g] += dpose[p, b, 3:]
            if model.ss[p]:   # dL/dE_M and dL/dE_N at the registered moduli
                gE[int(model.m[p])] += dE[p, 0]
                gE[int(model.n[p])] += dE[p, 1]
                continue
            # dL/dE = (dL/dout . out(E0)) / E0; the adjoint ran with the
            # upstream scaled by E/E0, so its dE carries that scale
            s = int(model.soft[p])
            side = 0 if s == int(model.m[p]) else 1
            if scale[p] != 0:
                gE[s] += dE[p, side] / scale[p]
        grot = (so3_left_jacobian(rot).transpose(-1, -2) @ gth[..., None])[..., 0]
        d = ctx.dev
        return None, gx.to(d), grot.to(d), gE.to(d)


def contact(model: ContactModel, xpos, rot, E):
    return ContactFunction.apply(model, xpos, rot, E)


def loss_and_grad(model: ContactModel, xpos, target, E):
    """Least-squares taxel misfit 0.5 |t(E) - target|^2 / |target|^2 and its
    gradient in E from the adjoint (through ContactFunction)."""
    rot = torch.zeros(xpos.shape[0], 3, dtype=torch.float64)
    Ev = E.clone().requires_grad_(True)
    _, t = contact(model, xpos, rot, Ev)
    loss = 0.5 * torch.sum((t - target) ** 2) / max(1e-30, float(torch.sum(target ** 2)))
    loss.backward()
    return float(loss.detach()), Ev.grad.detach().clone()


def identify_modulus(model: ContactModel, xpos, target_taxels, E_init, iters=4, rel_tol=1e-9):
    """Fit the soft moduli so that the taxel maps match ``target_taxels``.

    The misfit is quadratic in each soft modulus with no cross terms (every
    map scales with the modulus of its pair's soft geom), so each geom takes
    a Newton step whose curvature is the secant of two adjoint gradients;
    one or two steps converge.  Returns (E, loss history)."""
    xpos = torch.as_tensor(np.asarray(xpos, np.float64))
    target = torch.as_tensor(np.asarray(target_taxels, np.float64))
    E = torch.as_tensor(np.asarray(E_init, np.float64)).clone()
    hist = []
    for _ in range(iters):
        l1, g1 = loss_and_grad(model, xpos, target, E)
        hist.append(l1)
        E2 = E * (1.0 + 1e-3)
        _, g2 = loss_and_grad(model, xpos, target, E2)
        h = (g2 - g1) / (E2 - E)
        step = torch.where(h > 0, g1 / torch.where(h > 0, h, torch.ones_like(h)), torch.zeros_like(g1))
        E_new = torch.clamp(E - step, min=1e-3 * E)
        done = bool(torch.all(torch.abs(E_new - E) <= rel_tol * E))
        E = E_new
        if done:
            break
    hist.append(loss_and_grad(model, xpos, target, E)[0])
    return E, hist
