"""ctypes wrapper of the FP64 CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, as the checker.  The product never imports it.
Parity status: unpinned (see oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


MESHGEN = [os.path.join(HERE, "..", "mujoco_contact_surfaces_gb300", "csrc", f) for f in ("meshgen.cpp", "meshgen.h")]


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, f) for f in ("oracle.c", "taxel.c", "curved.c", "oracle.h", "or_mesh.cpp", "Makefile")]
    src += MESHGEN
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        r = subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "-s"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


class or_taxel_cfg(C.Structure):
    _fields_ = [("n_taxels", C.c_int), ("taxels", C.POINTER(C.c_double)), ("method", C.c_int),
                ("include_margin", C.c_double), ("sample_resolution", C.c_double), ("sample_method", C.c_int),
                ("visualize", C.c_int)]


class or_geom(C.Structure):
    _fields_ = [("kind", C.c_int), ("is_plane", C.c_int), ("order", C.c_int), ("E", C.c_double),
                ("d", C.c_double), ("mu_s", C.c_double), ("mu_d", C.c_double), ("nv", C.c_int),
                ("v", C.POINTER(C.c_double)), ("p", C.POINTER(C.c_double)), ("ne", C.c_int),
                ("e", C.POINTER(C.c_int))]


class or_options(C.Structure):
    _fields_ = [("representation", C.c_int), ("apply_forces", C.c_int), ("n_threads", C.c_int)]


class or_pair_result(C.Structure):
    _fields_ = [("query", C.c_int), ("m", C.c_int), ("n", C.c_int), ("wrench", C.c_double * 6),
                ("n_polygons", C.c_int), ("n_faces", C.c_int), ("n_near_degenerate", C.c_int),
                ("area", C.c_double), ("total_fn0", C.c_double), ("centroid", C.c_double * 3)]


class or_candidate(C.Structure):
    _fields_ = [("pair", C.c_int32), ("elem_a", C.c_int32), ("elem_b", C.c_int32), ("n_vert", C.c_int32),
                ("flags", C.c_int32)]


class or_sensor(C.Structure):
    _fields_ = [("geom", C.c_int), ("resolution", C.c_double), ("sampling_resolution", C.c_int),
                ("window", C.c_int), ("sigma", C.c_double), ("size", C.c_double * 3), ("cx", C.c_int),
                ("cy", C.c_int), ("taxels", C.POINTER(C.c_float)), ("taxels64", C.POINTER(C.c_double))]


_lib = None


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.or_create.restype = C.c_void_p
        lib.or_create.argtypes = [C.POINTER(or_geom), C.c_int]
        lib.or_destroy.argtypes = [C.c_void_p]
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        lib.or_collide.argtypes = [C.c_void_p, dp, dp, dp, C.c_int, ip, ip, C.POINTER(or_options),
                                   C.POINTER(or_pair_result), C.POINTER(or_sensor), C.c_int,
                                   C.POINTER(or_candidate), C.c_int64, C.POINTER(C.c_int64)]
        lib.or_surface.argtypes = [C.c_void_p, dp, dp, C.c_int, C.c_int, ip, ip, ip, dp, dp, dp, ip, ip]
        lib.or_sensor_grid.argtypes = [C.c_double, C.c_double, C.c_double, ip, ip]
        lib.or_taxel_sensor.argtypes = [C.POINTER(or_taxel_cfg), C.c_int, ip, ip, dp, dp, dp, dp]
        lib.or_minstd_nth.restype = C.c_uint64
        lib.or_minstd_nth.argtypes = [C.c_int]
        lib.or_uniform_nth.restype = C.c_double
        lib.or_uniform_nth.argtypes = [C.c_int]
        lib.or_curved_select.restype = C.c_int
        lib.or_curved_select.argtypes = [C.c_int, dp, dp, C.c_double, C.c_int, dp, dp, ip, ip, dp]
        lib.or_curved_update.argtypes = [C.c_int, ip, ip, dp, C.c_int, dp, dp, C.c_double, C.c_int, ip, ip, dp,
                                         dp, dp, dp]
        lib.or_generate_mesh.restype = C.c_int
        lib.or_generate_mesh.argtypes = [C.c_int, dp, dp, dp, C.c_int, ip, C.c_int, ip, ip, ip, dp, dp, ip,
                                         C.c_char_p, C.c_int]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def generate_mesh(gtype: int, size, cs5, mesh_vert=None, mesh_face=None):
    """The scene mesh of one geom from the package's generator source,
    compiled into this library (or_mesh.cpp): (kind, verts, pressures or
    None, elems), the same arrays as the engine's hc_generate_mesh."""
    lib = load()
    size = np.ascontiguousarray(size, np.float64)
    cs5 = np.ascontiguousarray(cs5, np.float64)
    mv = np.ascontiguousarray(mesh_vert, np.float64).reshape(-1) if mesh_vert is not None else None
    mf = np.ascontiguousarray(mesh_face, np.int32).reshape(-1) if mesh_face is not None else None
    nv_in = 0 if mv is None else len(mv) // 3
    nf_in = 0 if mf is None else len(mf) // 3
    kind, nv, ne = C.c_int(), C.c_int(), C.c_int()
    err = C.create_string_buffer(256)
    if lib.or_generate_mesh(gtype, _dp(size), _dp(cs5), _dp(mv), nv_in, _ip(mf), nf_in, C.byref(kind), C.byref(nv),
                            C.byref(ne), None, None, None, err, 256):
        raise ValueError(f"mesh generation failed: {err.value.decode()}")
    npe = 4 if kind.value == 1 else 3
    v = np.zeros((nv.value, 3), np.float64)
    e = np.zeros((ne.value, npe), np.int32)
    p = np.zeros(nv.value, np.float64) if kind.value == 1 else None
    lib.or_generate_mesh(gtype, _dp(size), _dp(cs5), _dp(mv), nv_in, _ip(mf), nf_in, C.byref(kind), C.byref(nv),
                         C.byref(ne), _dp(v), _dp(p), _ip(e), err, 256)
    return kind.value, v, p, e


class Oracle:
    """FP64 oracle over a Scene (mujoco_contact_surfaces_gb300.scenes)."""

    def __init__(self, scene, meshes=None):
        from mujoco_contact_surfaces_gb300 import _lib as L
        self.lib = load()
        self.scene = scene
        self._keep = []
        n = scene.n_geom
        arr = (or_geom * n)()
        self.meshes = meshes or {}
        for i, g in enumerate(scene.geoms):
            if g["id"] not in self.meshes:
                self.meshes[g["id"]] = generate_mesh(g["type"], g["size"], g["cs5"], g["mesh_v"], g["mesh_f"])
            kind, v, p, e = self.meshes[g["id"]]
            v = np.ascontiguousarray(v, np.float64)
            e = np.ascontiguousarray(e, np.int32)
            p = np.ascontiguousarray(p, np.float64) if p is not None else None
            self._keep += [v, e, p]
            og = arr[i]
            og.kind = kind
            og.is_plane = int(g["type"] == L.GEOM_PLANE)
            og.order = i
            og.E, og.d, og.mu_s, og.mu_d = g["cs5"][0], g["cs5"][1], g["cs5"][3], g["cs5"][4]
            og.nv = len(v)
            og.v = _dp(v)
            og.p = _dp(p)
            og.ne = len(e)
            og.e = _ip(e)
        self._geoms = arr
        self.ctx = self.lib.or_create(arr, n)

    def close(self):
        if self.ctx:
            self.lib.or_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collide(self, representation=0, apply_forces=1, n_threads=0, candidates=False, pairs=None, xpos=None,
                xmat=None, vel=None, sensors=True, taxels64=False):
        s = self.scene
        xpos = np.ascontiguousarray(s.xpos if xpos is None else xpos, np.float64)
        xmat = np.ascontiguousarray(s.xmat if xmat is None else xmat, np.float64)
        vel = np.ascontiguousarray(s.vel if vel is None else vel, np.float64)
        if pairs is None:
            g1 = np.ascontiguousarray(s.g1, np.int32)
            g2 = np.ascontiguousarray(s.g2, np.int32)
        else:
            g1 = np.ascontiguousarray([s.g1[i] for i in pairs], np.int32)
            g2 = np.ascontiguousarray([s.g2[i] for i in pairs], np.int32)
        npair = len(g1)
        out = (or_pair_result * max(1, npair))()
        opt = or_options(representation, apply_forces, n_threads)
        sens = (or_sensor * max(1, len(s.sensors)))()
        taxels, t64 = [], []
        if sensors:
            for k, sn in enumerate(s.sensors):
                size = s.geoms[sn["geom"]]["size"]
                cx, cy = C.c_int(), C.c_int()
                self.lib.or_sensor_grid(size[0], size[1], sn["resolution"], C.byref(cx), C.byref(cy))
                t = np.zeros(cx.value * cy.value, np.float32)
                taxels.append(t)
                o = sens[k]
                o.geom, o.resolution, o.sampling_resolution = sn["geom"], sn["resolution"], sn["sr"]
                o.window, o.sigma = sn["window"], sn["sigma"]
                if o.window == 1 and o.sigma == -1.0:
                    o.sigma = 0.1
                if o.window == 2 and o.sigma == -1.0:
                    o.sigma = 0.3
                for a in range(3):
                    o.size[a] = size[a]
                o.taxels = t.ctypes.data_as(C.POINTER(C.c_float))
                if taxels64:
                    d = np.zeros(cx.value * cy.value, np.float64)
                    t64.append(d)
                    o.taxels64 = d.ctypes.data_as(C.POINTER(C.c_double))
        ncand = C.c_int64()
        cand = None
        cap = 0
        if candidates:
            self.lib.or_collide(self.ctx, _dp(xpos), _dp(xmat), _dp(vel), npair, _ip(g1), _ip(g2), C.byref(opt),
                                out, sens, 0, None, 0, C.byref(ncand))
            cap = ncand.value
            cand = (or_candidate * max(1, cap))()
        self.lib.or_collide(self.ctx, _dp(xpos), _dp(xmat), _dp(vel), npair, _ip(g1), _ip(g2), C.byref(opt), out,
                            sens, len(s.sensors) if sensors else 0, cand, cap,
                            C.byref(ncand) if candidates else None)
        res = dict(
            query=np.array([out[i].query for i in range(npair)]),
            m=np.array([out[i].m for i in range(npair)]),
            n=np.array([out[i].n for i in range(npair)]),
            wrench=np.array([list(out[i].wrench) for i in range(npair)]).reshape(npair, 6),
            n_polygons=np.array([out[i].n_polygons for i in range(npair)]),
            n_faces=np.array([out[i].n_faces for i in range(npair)]),
            n_near=np.array([out[i].n_near_degenerate for i in range(npair)]),
            area=np.array([out[i].area for i in range(npair)]),
            total_fn0=np.array([out[i].total_fn0 for i in range(npair)]),
            centroid=np.array([list(out[i].centroid) for i in range(npair)]).reshape(npair, 3),
            xm=xpos.reshape(-1, 3)[np.array([out[i].m for i in range(npair)], dtype=np.int64)].reshape(npair, 3),
            taxels=taxels,
            taxels64=t64,
        )
        if candidates:
            res["candidates"] = np.ctypeslib.as_array(
                C.cast(cand, C.POINTER(C.c_int32)), shape=(max(1, cap), 5))[:ncand.value].astype(np.int64)
        return res

    def surface(self, g1, g2, xpos=None, xmat=None):
        s = self.scene
        xpos = np.ascontiguousarray(s.xpos if xpos is None else xpos, np.float64)
        xmat = np.ascontiguousarray(s.xmat if xmat is None else xmat, np.float64)
        npoly, nv = C.c_int(), C.c_int()
        self.lib.or_surface(self.ctx, _dp(xpos), _dp(xmat), g1, g2, C.byref(npoly), C.byref(nv), None, None, None,
                            None, None, None)
        off = np.zeros(npoly.value + 1, np.int32)
        vert = np.zeros((nv.value, 3))
        pr = np.zeros(nv.value)
        nrm = np.zeros((npoly.value, 3))
        ea = np.zeros(npoly.value, np.int32)
        eb = np.zeros(npoly.value, np.int32)
        self.lib.or_surface(self.ctx, _dp(xpos), _dp(xmat), g1, g2, C.byref(npoly), C.byref(nv), _ip(off),
                            _dp(vert), _dp(pr), _dp(nrm), _ip(ea), _ip(eb))
        return dict(offset=off, vert=vert, pressure=pr, normal=nrm, elem_a=ea, elem_b=eb)


def taxel_sensor(taxels_world, method, include_margin, sample_resolution, sample_method, visualize, surfaces,
                 values=None):
    """Taxel-point sensor update (or_taxel_sensor) on given contact surfaces.

    surfaces: list, in collision order, of dicts with 'poly_offset' (n+1),
    'vert' (k x 3, world), 'vert_pressure' (k), 'normal' (n x 3).  values:
    the previous values (kept where nothing is sampled within the margin)."""
    lib = load()
    tx = np.ascontiguousarray(taxels_world, np.float64).reshape(-1, 3)
    n = tx.shape[0]
    out = np.zeros(n) if values is None else np.array(values, np.float64, copy=True)
    surf_off, vert_off, verts, vps, nrms = [0], [0], [], [], []
    for srf in surfaces:
        po = np.asarray(srf["poly_offset"], np.int64)
        for k in range(len(po) - 1):
            vert_off.append(vert_off[-1] + int(po[k + 1] - po[k]))
        surf_off.append(surf_off[-1] + len(po) - 1)
        verts.append(np.asarray(srf["vert"], np.float64).reshape(-1, 3))
        vps.append(np.asarray(srf["vert_pressure"], np.float64).reshape(-1))
        nrms.append(np.asarray(srf["normal"], np.float64).reshape(-1, 3))
    so = np.asarray(surf_off, np.int32)
    vo = np.asarray(vert_off, np.int32)
    V = np.ascontiguousarray(np.concatenate(verts) if verts else np.zeros((0, 3)))
    P = np.ascontiguousarray(np.concatenate(vps) if vps else np.zeros(0))
    N = np.ascontiguousarray(np.concatenate(nrms) if nrms else np.zeros((0, 3)))
    cfg = or_taxel_cfg(n, _dp(tx), int(method), float(include_margin), float(sample_resolution), int(sample_method),
                       int(visualize))
    lib.or_taxel_sensor(C.byref(cfg), len(surfaces), _ip(so), _ip(vo), _dp(V), _dp(P), _dp(N), _dp(out))
    return out


def _surface_arrays(surfaces):
    surf_off, vert_off, verts, vps, nrms = [0], [0], [], [], []
    for srf in surfaces:
        po = np.asarray(srf["poly_offset"], np.int64)
        for k in range(len(po) - 1):
            vert_off.append(vert_off[-1] + int(po[k + 1] - po[k]))
        surf_off.append(surf_off[-1] + len(po) - 1)
        verts.append(np.asarray(srf["vert"], np.float64).reshape(-1, 3))
        vps.append(np.asarray(srf["vert_pressure"], np.float64).reshape(-1))
        nrms.append(np.asarray(srf["normal"], np.float64).reshape(-1, 3))
    so = np.asarray(surf_off, np.int32)
    vo = np.asarray(vert_off, np.int32)
    V = np.ascontiguousarray(np.concatenate(verts) if verts else np.zeros((0, 3)))
    P = np.ascontiguousarray(np.concatenate(vps) if vps else np.zeros(0))
    N = np.ascontiguousarray(np.concatenate(nrms) if nrms else np.zeros((0, 3)))
    return so, vo, V, P, N


def curved_select(taxels, taxel_normals, include_margin, points, point_normals):
    """Per-taxel surface-point lists and weights (or_curved_select), all in
    the geom frame; returns (off, pt, w)."""
    lib = load()
    tx = np.ascontiguousarray(taxels, np.float64).reshape(-1, 3)
    pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
    pn = np.ascontiguousarray(point_normals, np.float64).reshape(-1, 3)
    tn = None if taxel_normals is None else np.ascontiguousarray(taxel_normals, np.float64).reshape(-1, 3)
    n, m = tx.shape[0], pts.shape[0]
    off = np.zeros(n + 1, np.int32)
    pt = np.zeros(max(1, n * m), np.int32)
    w = np.zeros(max(1, n * m))
    k = lib.or_curved_select(n, _dp(tx), _dp(tn) if tn is not None else None, float(include_margin), m, _dp(pts),
                             _dp(pn), _ip(off), _ip(pt), _dp(w))
    return off, pt[:k].copy(), w[:k].copy()


def curved_update(off, pt, w, points_world, normals_world, include_margin, surfaces):
    """Curved-sensor values (or_curved_update) for the given lists, world
    points and normals, on the given contact surfaces (as taxel_sensor)."""
    lib = load()
    off = np.ascontiguousarray(off, np.int32)
    pt = np.ascontiguousarray(pt, np.int32)
    w = np.ascontiguousarray(w, np.float64)
    pts = np.ascontiguousarray(points_world, np.float64).reshape(-1, 3)
    nrm = np.ascontiguousarray(normals_world, np.float64).reshape(-1, 3)
    so, vo, V, P, N = _surface_arrays(surfaces)
    out = np.zeros(len(off) - 1)
    lib.or_curved_update(len(off) - 1, _ip(off), _ip(pt), _dp(w), pts.shape[0], _dp(pts), _dp(nrm),
                         float(include_margin), len(surfaces), _ip(so), _ip(vo), _dp(V), _dp(P), _dp(N), _dp(out))
    return out
