"""Seeded synthetic scenes for the contact-surface workloads.

Every generator uses numpy's PCG64 with seed = workload index * 1000 +
repeat.  A scene is plain data (geoms with MuJoCo geom types, sizes and the
cs:: 5-tuple [E, dissipation, resolutionHint, mu_static, mu_dynamic], poses as
geom_xpos / row-major geom_xmat, velocities [omega; v], contact pairs and flat
sensors), so the same scene feeds the engine and the oracle.

Workloads (sizes from the reference's example assets and configs):
  single_pair   soft sphere R=0.05 m at resolution 0.01 m, E=1e5 Pa, d=1 s/m,
                mu=0.5, on a rigid 0.2x0.2x0.02 m box (12 triangles); poses
                with penetration U[0,5 mm] and tilt U[-30,30] deg.
  tactile       rigid 8x8 cm plate with a 16x16 flat taxel grid (5 mm pitch,
                5x5 rays per cell) pressed by a soft sphere, ellipsoid
                (0.04/0.03/0.02) or cylinder (r=0.03, h=0.06), 2k-8k tets,
                E U[5e4,5e5], penetration U[0,4 mm], offset U[-2,2 cm]^2.
  batched       soft primitives of 500-20000 tets (log-uniform) against
                rigid meshes of 12-5000 triangles, 1-8 pairs per scene,
                penetration U[0,10%] of the soft extent, velocities U[-0.1,0.1].
  soft_soft     pairs of soft spheres/boxes, 2k-50k tets, E ratio
                log-U[0.1,10], overlap U[0,8%] of the smaller extent, random
                relative rotation.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

SEED_SINGLE, SEED_TACTILE, SEED_BATCHED, SEED_SOFTSOFT, SEED_ADJOINT = 0, 1000, 2000, 3000, 4000


@dataclass
class Scene:
    geoms: list = field(default_factory=list)      # dicts: id, type, size, cs5, mesh_v, mesh_f
    xpos: np.ndarray | None = None
    xmat: np.ndarray | None = None
    vel: np.ndarray | None = None
    g1: list = field(default_factory=list)
    g2: list = field(default_factory=list)
    sensors: list = field(default_factory=list)    # dicts: geom, resolution, sr, window, sigma
    scene_of_pair: list = field(default_factory=list)

    @property
    def n_geom(self):
        return len(self.geoms)

    def add_geom(self, gtype, size, cs5, mesh_v=None, mesh_f=None) -> int:
        gid = len(self.geoms)
        self.geoms.append(dict(id=gid, type=gtype, size=np.asarray(size, np.float64),
                               cs5=np.asarray(cs5, np.float64), mesh_v=mesh_v, mesh_f=mesh_f))
        return gid


def rot_axis(axis, ang):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * (K @ K)


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def sphere_hint(R, level):
    """Resolution hint that selects octahedral refinement `level` for radius R."""
    return math.pi * R / (2.0 * 2 ** level) * 1.0001


def _alloc(scene: Scene):
    n = scene.n_geom
    scene.xpos = np.zeros((n, 3))
    scene.xmat = np.tile(np.eye(3).reshape(1, 9), (n, 1))
    scene.vel = np.zeros((n, 6))


def single_pair(n_poses=1000, seed=SEED_SINGLE, velocities=False, min_pen=0.0) -> Scene:
    """Soft sphere on a rigid box, one pair per pose (each pose its own scene).

    min_pen > 0 draws the penetration from U[min_pen, 5 mm] (finite-difference
    checks need the contact to stay away from first touch within the step)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    R = 0.05
    for k in range(n_poses):
        gs = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [1e5, 1.0, 0.01, 0.5, 0.5])
        gb = s.add_geom(L.GEOM_BOX, [0.1, 0.1, 0.01], [0, 1.0, 0, 0.5, 0.5])
        s.g1.append(gs); s.g2.append(gb); s.scene_of_pair.append(k)
    _alloc(s)
    for k in range(n_poses):
        gs, gb = 2 * k, 2 * k + 1
        pen = rng.uniform(min_pen, 0.005)
        tilt = math.radians(rng.uniform(-30, 30))
        phi = rng.uniform(0, 2 * math.pi)
        axis = [math.cos(phi), math.sin(phi), 0.0]
        Rs = rot_axis(axis, tilt) @ rot_axis([0, 0, 1], rng.uniform(0, 2 * math.pi))
        s.xmat[gs] = Rs.reshape(9)
        s.xpos[gs] = [0.0, 0.0, 0.01 + R - pen]
        s.xpos[gb] = [0.0, 0.0, 0.0]
        if velocities:
            s.vel[gs] = rng.uniform(-0.1, 0.1, 6)
    return s


def tactile(n_scenes=16, seed=SEED_TACTILE, velocities=False, sampling_resolution=5,
            plate_half=(0.04, 0.04, 0.005), min_pen=0.0) -> Scene:
    """Rigid plate with a 16x16 taxel grid pressed by a soft primitive.

    With a square plate the top face's diagonal passes exactly through the
    samples with equal x and y indices; parity tests use a plate 0.1 mm
    wider in x so that no ray sample sits exactly on a triangle edge."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    plate_h = list(plate_half)
    kinds = []
    for k in range(n_scenes):
        kind = int(rng.integers(0, 3))
        E = rng.uniform(5e4, 5e5)
        if kind == 0:
            R = rng.uniform(0.025, 0.04)
            lev = int(rng.integers(4, 6))
            g = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [E, 1.0, sphere_hint(R, lev), 0.5, 0.5])
            low = R
        elif kind == 1:
            lev = int(rng.integers(4, 6))
            g = s.add_geom(L.GEOM_ELLIPSOID, [0.04, 0.03, 0.02], [E, 1.0, sphere_hint(0.04, lev), 0.5, 0.5])
            low = 0.02
        else:
            hint = float(rng.choice([0.01, 0.0075]))
            g = s.add_geom(L.GEOM_CYLINDER, [0.03, 0.03, 0], [E, 1.0, hint, 0.5, 0.5])
            low = 0.03   # lying on its side
        p = s.add_geom(L.GEOM_BOX, plate_h, [0, 1.0, 0, 0.5, 0.5])
        s.g1.append(g); s.g2.append(p); s.scene_of_pair.append(k)
        s.sensors.append(dict(geom=p, resolution=0.005, sr=sampling_resolution, window=L.WINDOW_NONE, sigma=-1.0))
        kinds.append((kind, low))
    _alloc(s)
    for k in range(n_scenes):
        g, p = 2 * k, 2 * k + 1
        kind, low = kinds[k]
        pen = rng.uniform(min_pen, 0.004)
        off = rng.uniform(-0.02, 0.02, 2)
        yaw = rot_axis([0, 0, 1], rng.uniform(0, 2 * math.pi))
        Rg = yaw @ rot_axis([1, 0, 0], math.pi / 2) if kind == 2 else yaw
        s.xmat[g] = Rg.reshape(9)
        s.xpos[g] = [off[0], off[1], plate_h[2] + low - pen]
        s.xpos[p] = [0, 0, 0]
        if velocities:
            s.vel[g] = rng.uniform(-0.1, 0.1, 6)
    return s


def _soft_primitive(rng, target_tets):
    """A random convex soft primitive with roughly `target_tets` tets."""
    kind = int(rng.integers(0, 4))
    ext = rng.uniform(0.02, 0.08)
    E = rng.uniform(5e4, 5e5)
    if kind == 0:
        lev = int(np.clip(round(math.log(max(target_tets, 8) / 8, 4)), 2, 6))
        return L.GEOM_SPHERE, [ext, 0, 0], [E, 1.0, sphere_hint(ext, lev), 0.5, 0.5], ext
    if kind == 1:
        ax = ext * rng.uniform(0.4, 1.0, 3)
        ax[0] = ext
        lev = int(np.clip(round(math.log(max(target_tets, 8) / 8, 4)), 2, 6))
        return L.GEOM_ELLIPSOID, list(ax), [E, 1.0, sphere_hint(ext, lev), 0.5, 0.5], float(ax.min())
    if kind == 2:
        h = ext * rng.uniform(0.3, 1.0, 3)
        vol_cells = target_tets / 6.0
        hint = (8 * h[0] * h[1] * h[2] / vol_cells) ** (1 / 3)
        return L.GEOM_BOX, list(h), [E, 1.0, hint, 0.5, 0.5], float(h.min())
    r, hl = ext, ext * rng.uniform(0.3, 1.5)
    hint = (2 * math.pi * r * r * hl * 6 / max(target_tets, 100)) ** (1 / 3) * 0.9
    return L.GEOM_CYLINDER, [r, hl, 0], [E, 1.0, hint, 0.5, 0.5], min(r, hl)


def _rigid_primitive(rng, target_tris):
    kind = int(rng.integers(0, 3))
    ext = rng.uniform(0.05, 0.2)
    if kind == 0 or target_tris <= 12:
        h = [ext, ext * rng.uniform(0.5, 1.0), ext * rng.uniform(0.1, 0.5)]
        area = 8 * (h[0] * h[1] + h[1] * h[2] + h[0] * h[2])
        hint = math.sqrt(area / max(target_tris / 2.0, 6)) if target_tris > 12 else 0.0
        return L.GEOM_BOX, h, [0, 1.0, hint, 0.5, 0.5], h[2]
    if kind == 1:
        lev = int(np.clip(round(math.log(max(target_tris, 8) / 8, 4)), 1, 5))
        return L.GEOM_SPHERE, [ext, 0, 0], [0, 1.0, sphere_hint(ext, lev), 0.5, 0.5], ext
    r, hl = ext, ext * rng.uniform(0.3, 1.0)
    hint = math.sqrt(2 * math.pi * r * 2 * hl / max(target_tris / 2.0, 12))
    return L.GEOM_CYLINDER, [r, hl, 0], [0, 1.0, hint, 0.5, 0.5], r


def batched(n_scenes=4096, seed=SEED_BATCHED, max_pairs=8, tet_range=(500, 20000), tri_range=(12, 5000)) -> Scene:
    """Independent scenes of 1-8 soft-rigid pairs with uneven mesh sizes."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    place = []
    for k in range(n_scenes):
        npair = int(rng.integers(1, max_pairs + 1))
        for _ in range(npair):
            nt = math.exp(rng.uniform(math.log(tet_range[0]), math.log(tet_range[1])))
            nr = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
            st, ssize, scs, sext = _soft_primitive(rng, nt)
            rt, rsize, rcs, rext = _rigid_primitive(rng, nr)
            gs = s.add_geom(st, ssize, scs)
            gr = s.add_geom(rt, rsize, rcs)
            s.g1.append(gs); s.g2.append(gr); s.scene_of_pair.append(k)
            place.append((gs, gr, st, ssize, rt, rsize, sext, rext))
    _alloc(s)
    for (gs, gr, st, ssize, rt, rsize, sext, rext) in place:
        # rigid body at the origin of its own scene frame, its top support
        # at z = top; the soft body above it, sunk by a fraction of its extent
        if rt == L.GEOM_BOX:
            top = rsize[2]
        elif rt == L.GEOM_SPHERE:
            top = rsize[0]
        else:
            top = rsize[1]   # cylinder cap
        Rs = random_rotation(rng)
        # lowest point of the soft body along z after rotation (support)
        if st == L.GEOM_SPHERE:
            low = ssize[0]
        elif st == L.GEOM_ELLIPSOID:
            low = float(np.sqrt(np.sum((Rs[2, :] * np.asarray(ssize)) ** 2)))
        elif st == L.GEOM_BOX:
            low = float(np.sum(np.abs(Rs[2, :]) * np.asarray(ssize)))
        else:
            r, hl = ssize[0], ssize[1]
            low = float(r * math.sqrt(max(0.0, 1 - Rs[2, 2] ** 2)) + hl * abs(Rs[2, 2]))
        pen = rng.uniform(0, 0.1) * sext
        off = rng.uniform(-0.3, 0.3, 2) * min(sext, rext)
        s.xmat[gs] = Rs.reshape(9)
        s.xpos[gs] = [off[0], off[1], top + low - pen]
        s.xpos[gr] = [0, 0, 0]
        s.vel[gs] = rng.uniform(-0.1, 0.1, 6)
        s.vel[gr] = rng.uniform(-0.1, 0.1, 6)
    return s


def soft_soft(n_pairs=1024, seed=SEED_SOFTSOFT, tet_range=(2000, 50000)) -> Scene:
    """Pairs of soft spheres/boxes meeting on the equal-pressure surface."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    place = []
    for k in range(n_pairs):
        bodies = []
        for _ in range(2):
            nt = math.exp(rng.uniform(math.log(tet_range[0]), math.log(tet_range[1])))
            E = 1e5 * math.exp(rng.uniform(math.log(0.1), math.log(10)) / 2)
            if rng.integers(0, 2) == 0:
                R = rng.uniform(0.03, 0.06)
                lev = int(np.clip(round(math.log(max(nt, 8) / 8, 4)), 3, 6))
                gid = s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [E, 1.0, sphere_hint(R, lev), 0.5, 0.5])
                bodies.append((gid, L.GEOM_SPHERE, [R, R, R], R))
            else:
                h = rng.uniform(0.02, 0.05, 3)
                hint = (8 * h[0] * h[1] * h[2] * 6 / nt) ** (1 / 3)
                gid = s.add_geom(L.GEOM_BOX, list(h), [E, 1.0, hint, 0.5, 0.5])
                bodies.append((gid, L.GEOM_BOX, list(h), float(h.min())))
        s.g1.append(bodies[0][0]); s.g2.append(bodies[1][0]); s.scene_of_pair.append(k)
        place.append(bodies)
    _alloc(s)
    for (a, b) in place:
        Ra, Rb = random_rotation(rng), random_rotation(rng)
        # b below a, its centre offset sideways; lowered until the bodies
        # touch along the vertical, then raised by the overlap
        ov = rng.uniform(0, 0.08) * min(a[3], b[3])
        off = rng.uniform(-0.2, 0.2, 2) * min(a[3], b[3])
        s.xmat[a[0]] = Ra.reshape(9)
        s.xmat[b[0]] = Rb.reshape(9)
        s.xpos[a[0]] = [0, 0, 0]
        zb = _touch_height(a, Ra, np.zeros(2), b, Rb, off)
        s.xpos[b[0]] = [off[0], off[1], zb + ov]
    return s


def soft_soft_pressed(n_pairs=4, seed=SEED_ADJOINT + 100, velocities=True, min_pen=1.5e-3) -> Scene:
    """A soft sphere pressed into the top face of a soft box that carries a
    16x16 flat taxel grid, one pair per scene (the soft-soft adjoint cases).

    Moduli E U[5e4,5e5] and dissipations 1.0 (box) / 0.4 (sphere), so the
    combined damping depends on both moduli; the box is registered first
    (M, the sensor on the soft frame's geom) in even scenes and second in odd
    ones.  Penetration U[min_pen, 4 mm] split between the bodies by the
    equal-pressure surface; the box is 0.3 mm longer in x than in y so that
    no ray sample sits exactly on a face of its tet grid."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    box_h = [0.0403, 0.04, 0.012]
    spec = []
    for k in range(n_pairs):
        R = rng.uniform(0.02, 0.03)
        Eb, Ea = rng.uniform(5e4, 5e5, 2)
        mk_box = lambda: s.add_geom(L.GEOM_BOX, box_h, [Eb, 1.0, 0.006, 0.5, 0.5])
        mk_sph = lambda: s.add_geom(L.GEOM_SPHERE, [R, 0, 0], [Ea, 0.4, sphere_hint(R, 4), 0.5, 0.5])
        if k % 2 == 0:
            b = mk_box(); a = mk_sph()
            s.g1.append(b); s.g2.append(a)
        else:
            a = mk_sph(); b = mk_box()
            s.g1.append(a); s.g2.append(b)
        s.scene_of_pair.append(k)
        s.sensors.append(dict(geom=b, resolution=0.005, sr=5, window=L.WINDOW_NONE, sigma=-1.0))
        spec.append((a, b, R))
    _alloc(s)
    for (a, b, R) in spec:
        pen = rng.uniform(min_pen, 0.004)
        off = rng.uniform(-0.015, 0.015, 2)
        s.xmat[b] = rot_axis([0, 0, 1], rng.uniform(0, 2 * math.pi)).reshape(9)
        s.xmat[a] = random_rotation(rng).reshape(9)
        s.xpos[b] = [0.0, 0.0, 0.0]
        s.xpos[a] = [off[0], off[1], box_h[2] + R - pen]
        if velocities:
            s.vel[a] = rng.uniform(-0.1, 0.1, 6)
            s.vel[b] = rng.uniform(-0.1, 0.1, 6)
    return s


def _vertical_extent(body, R, c_xy, x, y):
    """The body (centre (c_xy, 0), rotation R) along the vertical lines
    through (x, y): (z_low, z_high), NaN where the line misses it."""
    _, t, h, _ = body
    dx, dy = x - c_xy[0], y - c_xy[1]
    if t == L.GEOM_SPHERE:
        r2 = h[0] ** 2 - dx * dx - dy * dy
        hz = np.sqrt(np.where(r2 >= 0, r2, np.nan))
        return -hz, hz
    lo = np.full(x.shape, -np.inf)
    hi = np.full(x.shape, np.inf)
    for i in range(3):   # |R[:, i].(p - c)| <= h_i along p = (x, y, z)
        u = R[0, i] * dx + R[1, i] * dy
        w = R[2, i]
        if abs(w) < 1e-12:
            bad = np.abs(u) > h[i]
            lo = np.where(bad, np.nan, lo)
            continue
        z1, z2 = (-h[i] - u) / w, (h[i] - u) / w
        lo = np.maximum(lo, np.minimum(z1, z2))
        hi = np.minimum(hi, np.maximum(z1, z2))
    empty = ~(lo <= hi)
    return np.where(empty, np.nan, lo), np.where(empty, np.nan, hi)


def _touch_height(a, Ra, ca, b, Rb, cb, n=48, rounds=8):
    """Centre height of b (below a, a's centre at height 0) at which the two
    bodies touch when b rises vertically: the smallest gap between a's lower
    and b's upper envelope over vertical lines.  The gap is convex in (x, y)
    for convex bodies, so a grid is zoomed in around its minimum."""
    r = 2.0 * max(max(a[2]), max(b[2]))
    cx, cy = float(ca[0]), float(ca[1])
    best = None
    for _ in range(rounds):
        g = np.linspace(-r, r, n)
        x, y = np.meshgrid(g + cx, g + cy)
        a_lo, _ = _vertical_extent(a, Ra, ca, x, y)
        _, b_hi = _vertical_extent(b, Rb, cb, x, y)
        gap = a_lo - b_hi
        if not np.any(np.isfinite(gap)):
            break
        k = int(np.nanargmin(gap))
        v = float(gap.flat[k])
        best = v if best is None else min(best, v)
        cx, cy = float(x.flat[k]), float(y.flat[k])
        r *= 4.0 / n * 2.0   # a window of a few cells around the minimum
    return best if best is not None else -(max(a[2]) + max(b[2]))


def halfspace(n_pairs=8, seed=SEED_SINGLE + 500, min_frac=0.0) -> Scene:
    """Soft primitives resting on a rigid ground plane (plane geom), sunk by
    U[min_frac, 0.1] of their extent."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene()
    ground = s.add_geom(L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
    place = []
    for k in range(n_pairs):
        st, ssize, scs, sext = _soft_primitive(rng, rng.uniform(500, 4000))
        g = s.add_geom(st, ssize, scs)
        s.g1.append(g); s.g2.append(ground); s.scene_of_pair.append(k)
        place.append((g, st, ssize, sext))
    _alloc(s)
    for (g, st, ssize, sext) in place:
        Rs = random_rotation(rng)
        if st == L.GEOM_SPHERE:
            low = ssize[0]
        elif st == L.GEOM_ELLIPSOID:
            low = float(np.sqrt(np.sum((Rs[2, :] * np.asarray(ssize)) ** 2)))
        elif st == L.GEOM_BOX:
            low = float(np.sum(np.abs(Rs[2, :]) * np.asarray(ssize)))
        else:
            r, hl = ssize[0], ssize[1]
            low = float(r * math.sqrt(max(0.0, 1 - Rs[2, 2] ** 2)) + hl * abs(Rs[2, 2]))
        s.xmat[g] = Rs.reshape(9)
        s.xpos[g] = [rng.uniform(-1, 1), rng.uniform(-1, 1), low - rng.uniform(min_frac, 0.1) * sext]
        s.vel[g] = rng.uniform(-0.1, 0.1, 6)
    return s


def subscene(s: Scene, pairs) -> Scene:
    """The geoms, poses, sensors and pairs of the given pair indices of `s`,
    geoms registered in their original relative order (so each pair's M/N
    order is the one it has in `s`); pair k of the result is pairs[k] in
    sorted order, and a sensor is kept when its geom is."""
    pairs = sorted(int(p) for p in pairs)
    keep = sorted({s.g1[p] for p in pairs} | {s.g2[p] for p in pairs})
    remap = {g: i for i, g in enumerate(keep)}
    t = Scene()
    for g in keep:
        d = s.geoms[g]
        t.add_geom(d["type"], d["size"], d["cs5"], d["mesh_v"], d["mesh_f"])
    _alloc(t)
    for g in keep:
        t.xpos[remap[g]] = s.xpos[g]
        t.xmat[remap[g]] = s.xmat[g]
        t.vel[remap[g]] = s.vel[g]
    for p in pairs:
        t.g1.append(remap[s.g1[p]]); t.g2.append(remap[s.g2[p]])
        t.scene_of_pair.append(s.scene_of_pair[p] if s.scene_of_pair else 0)
    for sn in s.sensors:
        if sn["geom"] in remap:
            d = dict(sn)
            d["geom"] = remap[sn["geom"]]
            t.sensors.append(d)
    return t


def build_engine(scene: Scene, **engine_kw):
    """An Engine holding the scene's geoms, sensors, pairs and poses."""
    from .engine import Engine
    eng = Engine(**engine_kw)
    for g in scene.geoms:
        eng.add_geom(g["id"], g["type"], g["size"], g["cs5"], g["mesh_v"], g["mesh_f"])
    for sn in scene.sensors:
        eng.add_flat_sensor(sn["geom"], sn["resolution"], sn["sr"], sn["window"], sn["sigma"])
    eng.set_pairs(scene.g1, scene.g2)
    eng.set_poses(scene.xpos, scene.xmat, scene.vel)
    return eng
