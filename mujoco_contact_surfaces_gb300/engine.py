"""Host-side wrapper of one engine context (the C ABI in include/hc/hc.h).

`Engine` mirrors what the reference plugin does per model load and per step
(mujoco_contact_surfaces_plugin.cpp: load P:208-245, collision_cb
P:255-318, passiveCallback P:411-523), with numpy arrays in and out.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _out(out, shape, dtype):
    """A new zeroed array, or the caller's (right dtype and size, C-contiguous)."""
    if out is None:
        return np.zeros(shape, dtype)
    size = 1
    for s in shape:
        size *= s
    if out.dtype != dtype or out.size != size or not out.flags.c_contiguous:
        raise ValueError(f"out must be a C-contiguous {np.dtype(dtype).name} array of {size} elements")
    return out


class _Ptrs:
    """ctypes pointers of the arrays a per-step call was last given: a call
    that passes the same arrays again (a simulation loop's buffers) reuses
    them instead of converting each array again.  Holds a reference to each
    array, so an entry's pointer stays valid while it is kept."""

    def __init__(self, n):
        self.arr = [None] * n
        self.ptr = [None] * n

    def get(self, k, a, conv):
        if a is None:
            return None
        if self.arr[k] is not a:
            self.arr[k] = a
            self.ptr[k] = conv(a)
        return self.ptr[k]


class Engine:
    def __init__(self, device: int = 0, representation: int = L.REPR_TRIANGLE, apply_forces: bool = True,
                 use_graph: bool = True, item_capacity: int = 0,
                 face_capacity: int = 0):
        self.lib = L.load()
        cfg = L.hc_config()
        self.lib.hc_config_default(C.byref(cfg))
        cfg.device = device
        cfg.representation = representation
        cfg.apply_forces = int(apply_forces)
        cfg.use_graph = int(use_graph)
        cfg.item_capacity = item_capacity
        cfg.face_capacity = face_capacity
        self.ctx = C.c_void_p()
        L.check(self.lib.hc_context_create(C.byref(cfg), C.byref(self.ctx)))
        self.n_pair = 0
        self.sensors = {}   # sensor index -> (cx, cy)
        self.n_cells = 0    # taxels of all flat sensors (kept as sensors are added)
        self.n_taxel_values = 0   # taxels of all taxel-point sensors
        self.taxel_sensors = {}   # taxel sensor index -> number of taxels
        self.curved_sensors = {}  # curved sensor index -> number of taxels
        self._step_ptrs = _Ptrs(9)

    def close(self):
        if self.ctx:
            self.lib.hc_context_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- geoms ---------------------------------------------------------------
    def add_geom(self, geom_id: int, gtype: int, size, cs5, mesh_vert=None, mesh_face=None) -> int:
        size = np.ascontiguousarray(size, np.float64)
        cs5 = np.ascontiguousarray(cs5, np.float64)
        mv = np.ascontiguousarray(mesh_vert, np.float64).reshape(-1) if mesh_vert is not None else None
        mf = np.ascontiguousarray(mesh_face, np.int32).reshape(-1) if mesh_face is not None else None
        kind = C.c_int()
        L.check(self.lib.hc_add_geom(self.ctx, geom_id, gtype, L.dptr(size), L.dptr(cs5), L.dptr(mv),
                                     0 if mv is None else len(mv) // 3, L.iptr(mf), 0 if mf is None else len(mf) // 3,
                                     C.byref(kind)))
        return kind.value

    def geom_info(self, geom_id: int) -> L.hc_geom_info:
        info = L.hc_geom_info()
        L.check(self.lib.hc_get_geom_info(self.ctx, geom_id, C.byref(info)))
        return info

    def geom_mesh(self, geom_id: int):
        info = self.geom_info(geom_id)
        npe = 4 if info.kind == L.SOFT else 3
        v = np.zeros((info.n_vertices, 3), np.float64)
        e = np.zeros((info.n_elements, npe), np.int32)
        p = np.zeros(info.n_vertices, np.float64) if info.kind == L.SOFT else None
        L.check(self.lib.hc_get_geom_mesh(self.ctx, geom_id, L.dptr(v), L.dptr(p), L.iptr(e)))
        return v, p, e

    def element_order(self, geom_id: int) -> np.ndarray:
        """The geom's elements in LBVH leaf order (hc_get_element_order)."""
        out = np.zeros(self.geom_info(geom_id).n_elements, np.int32)
        L.check(self.lib.hc_get_element_order(self.ctx, geom_id, L.iptr(out)))
        return out

    def update_geom_size(self, geom_id: int, size):
        size = np.ascontiguousarray(size, np.float64)
        L.check(self.lib.hc_update_geom_size(self.ctx, geom_id, L.dptr(size)))

    def add_flat_sensor(self, geom_id: int, resolution: float, sampling_resolution: int = 5,
                        window: int = L.WINDOW_NONE, sigma: float = -1.0) -> int:
        sid, cx, cy = C.c_int(), C.c_int(), C.c_int()
        L.check(self.lib.hc_add_flat_sensor(self.ctx, geom_id, resolution, sampling_resolution, window, sigma,
                                            C.byref(sid), C.byref(cx), C.byref(cy)))
        self.sensors[sid.value] = (cx.value, cy.value)
        self.n_cells += cx.value * cy.value
        return sid.value

    def add_taxel_sensor(self, geom_id: int, taxels, method: int, include_margin: float, sample_resolution: float,
                         sample_method: int = 0, visualize: bool = False) -> int:
        t = np.ascontiguousarray(taxels, np.float64).reshape(-1, 3)
        sid = C.c_int()
        L.check(self.lib.hc_add_taxel_sensor(self.ctx, geom_id, t.shape[0], L.dptr(t), int(method),
                                             float(include_margin), float(sample_resolution), int(sample_method),
                                             int(visualize), C.byref(sid)))
        self.taxel_sensors[sid.value] = t.shape[0]
        self.n_taxel_values += t.shape[0]
        return sid.value

    def set_taxel_sensor_enabled(self, sensor: int, on: bool = True):
        L.check(self.lib.hc_set_taxel_sensor_enabled(self.ctx, sensor, int(on)))

    def taxel_sensor_values(self, sensor: int) -> np.ndarray:
        out = np.zeros(self.taxel_sensors[sensor], np.float32)
        L.check(self.lib.hc_get_taxel_sensor_values(self.ctx, sensor, L.fptr(out)))
        return out

    def add_curved_sensor(self, geom_id: int, taxels, include_margin: float, points, point_normals,
                          taxel_normals=None) -> int:
        """Curved sensor (hc_add_curved_sensor): taxels and surface points
        with unit normals in the geom frame."""
        t = np.ascontiguousarray(taxels, np.float64).reshape(-1, 3)
        tn = None if taxel_normals is None else np.ascontiguousarray(taxel_normals, np.float64).reshape(-1, 3)
        p = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        pn = np.ascontiguousarray(point_normals, np.float64).reshape(-1, 3)
        sid = C.c_int()
        L.check(self.lib.hc_add_curved_sensor(self.ctx, geom_id, t.shape[0], L.dptr(t), L.dptr(tn),
                                              float(include_margin), p.shape[0], L.dptr(p), L.dptr(pn),
                                              C.byref(sid)))
        self.curved_sensors[sid.value] = t.shape[0]
        return sid.value

    def set_curved_sensor_enabled(self, sensor: int, on: bool = True):
        L.check(self.lib.hc_set_curved_sensor_enabled(self.ctx, sensor, int(on)))

    def curved_sensor_values(self, sensor: int) -> np.ndarray:
        out = np.zeros(self.curved_sensors[sensor], np.float32)
        L.check(self.lib.hc_get_curved_sensor_values(self.ctx, sensor, L.fptr(out)))
        return out

    def all_taxel_sensor_values(self, out=None) -> np.ndarray:
        """Every taxel sensor's values, concatenated in sensor order (one copy)."""
        out = _out(out, (self.n_taxel_values,), np.float32)
        L.check(self.lib.hc_get_all_taxel_sensor_values(self.ctx, L.fptr(out), out.size))
        return out

    # -- per step --------------------------------------------------------------
    def set_poses(self, xpos, xmat, vel=None):
        xpos = np.ascontiguousarray(xpos, np.float64)
        xmat = np.ascontiguousarray(xmat, np.float64)
        n = xpos.size // 3
        v = np.ascontiguousarray(vel, np.float64) if vel is not None else None
        L.check(self.lib.hc_set_poses(self.ctx, n, L.dptr(xpos), L.dptr(xmat), L.dptr(v)))

    def set_poses_device(self, n_geom: int, d_xpos: int, d_xmat: int, d_vel: int | None):
        L.check(self.lib.hc_set_poses_device(self.ctx, n_geom, C.c_void_p(d_xpos), C.c_void_p(d_xmat),
                                             C.c_void_p(d_vel) if d_vel else None))

    def set_pairs(self, g1, g2):
        g1 = np.ascontiguousarray(g1, np.int32)
        g2 = np.ascontiguousarray(g2, np.int32)
        st = np.zeros(len(g1), np.int32)
        q = np.zeros(len(g1), np.int32)
        L.check(self.lib.hc_set_pairs(self.ctx, len(g1), L.iptr(g1), L.iptr(g2), L.iptr(st), L.iptr(q)))
        self.n_pair = len(g1)
        return st, q

    def step(self):
        L.check(self.lib.hc_step(self.ctx))

    def wrenches(self, out=None) -> np.ndarray:
        """Per-pair world wrenches (n_pair x 6).  ``out``: a caller's array to
        fill (page-locked host memory makes the read a direct copy)."""
        w = _out(out, (self.n_pair, 6), np.float64)
        L.check(self.lib.hc_get_wrenches(self.ctx, L.dptr(w)))
        return w

    def pair_order(self):
        q = np.zeros(self.n_pair, np.int32)
        m = np.zeros(self.n_pair, np.int32)
        n = np.zeros(self.n_pair, np.int32)
        L.check(self.lib.hc_get_pair_order(self.ctx, L.iptr(q), L.iptr(m), L.iptr(n)))
        return q, m, n

    def pair_stats(self):
        arr = (L.hc_pair_stats * max(1, self.n_pair))()
        L.check(self.lib.hc_get_pair_stats(self.ctx, arr))
        return [arr[i] for i in range(self.n_pair)]

    def taxels(self, sensor: int) -> np.ndarray:
        cx, cy = self.sensors[sensor]
        out = np.zeros(cx * cy, np.float32)
        L.check(self.lib.hc_get_taxels(self.ctx, sensor, L.fptr(out)))
        return out

    def all_taxels(self, out=None) -> np.ndarray:
        n = self.n_cells
        out = _out(out, (n,), np.float32)
        L.check(self.lib.hc_get_taxels_all(self.ctx, L.fptr(out), n))
        return out

    def set_debug(self, flags: int):
        L.check(self.lib.hc_set_debug(self.ctx, flags))

    def candidates(self) -> np.ndarray:
        n = C.c_int64()
        L.check(self.lib.hc_get_candidates(self.ctx, None, 0, C.byref(n)))
        buf = np.zeros((max(1, n.value), 5), np.int32)   # hc_candidate: five int32 fields
        L.check(self.lib.hc_get_candidates(self.ctx, buf.ctypes.data_as(C.POINTER(L.hc_candidate)), n.value,
                                           C.byref(n)))
        return buf[:n.value].astype(np.int64)

    def surface(self, pair: int):
        v = L.hc_surface_view()
        L.check(self.lib.hc_get_surface(self.ctx, pair, C.byref(v)))
        n, nv = v.n_poly, v.n_vert
        off = np.zeros(n + 1, np.int32)
        vert = np.zeros((nv, 3), np.float64)
        pr = np.zeros(nv, np.float64)
        nrm = np.zeros((n, 3), np.float64)
        ea = np.zeros(n, np.int32)
        eb = np.zeros(n, np.int32)
        v.poly_offset = L.iptr(off)
        v.vert = L.dptr(vert)
        v.vert_pressure = L.dptr(pr)
        v.normal = L.dptr(nrm)
        v.elem_a = L.iptr(ea)
        v.elem_b = L.iptr(eb)
        L.check(self.lib.hc_get_surface(self.ctx, pair, C.byref(v)))
        return dict(offset=off, vert=vert, pressure=pr, normal=nrm, elem_a=ea, elem_b=eb)

    def enable_timing(self, on: bool = True):
        L.check(self.lib.hc_enable_timing(self.ctx, int(on)))

    def timings(self) -> L.hc_timings:
        t = L.hc_timings()
        L.check(self.lib.hc_get_timings(self.ctx, C.byref(t)))
        return t

    def autotune(self):
        """Pick the persistent kernels' grid and the work-queue chunk on the
        current pairs and poses; returns (ctas_per_sm, chunk)."""
        ct, ch = C.c_int(), C.c_int()
        L.check(self.lib.hc_autotune(self.ctx, C.byref(ct), C.byref(ch)))
        return ct.value, ch.value

    def set_launch_shape(self, ctas_per_sm: int, chunk: int):
        """Set the persistent kernels' grid and the work-queue chunk directly."""
        L.check(self.lib.hc_set_launch_shape(self.ctx, int(ctas_per_sm), int(chunk)))

    def launch_count(self) -> int:
        n = C.c_int()
        L.check(self.lib.hc_get_launch_count(self.ctx, C.byref(n)))
        return n.value

    def stream(self) -> int:
        s = C.c_void_p()
        L.check(self.lib.hc_get_stream(self.ctx, C.byref(s)))
        return s.value or 0

    def set_adjoint_mode(self, on: bool = True):
        L.check(self.lib.hc_set_adjoint_mode(self.ctx, int(on)))

    def adjoint_device(self, d_dL_dwrench: int | None, d_dL_dtaxel: int | None) -> int:
        """Asynchronous adjoint on device buffers; returns the device pointer
        of the n_pair x 14 result ([twist M, twist N, dE_M, dE_N])."""
        out = C.c_void_p()
        L.check(self.lib.hc_adjoint_device(self.ctx, C.c_void_p(d_dL_dwrench) if d_dL_dwrench else None,
                                           C.c_void_p(d_dL_dtaxel) if d_dL_dtaxel else None, C.byref(out)))
        return out.value or 0

    def adjoint_skipped(self):
        """(vertices the last adjoint left out of its contraction, smallest
        normalised determinant it met); needs debug recording, set_debug(1)."""
        n, d = C.c_int(), C.c_float()
        L.check(self.lib.hc_get_adjoint_skipped(self.ctx, C.byref(n), C.byref(d)))
        return n.value, d.value

    def adjoint_launch_count(self) -> int:
        n = C.c_int()
        L.check(self.lib.hc_get_adjoint_launch_count(self.ctx, C.byref(n)))
        return n.value

    def step_adjoint(self, xpos, xmat, vel, dL_dwrench=None, dL_dtaxel=None, out=None):
        """Forward step and adjoint with one wait (hc_step_adjoint): returns
        (wrenches n_pair x 6, all flat taxel maps, dL/dpose n_pair x 2 x 6,
        dL/dE n_pair x 2).  ``out``: a 4-tuple of the caller's arrays."""
        xpos = np.ascontiguousarray(xpos, np.float64)
        xmat = np.ascontiguousarray(xmat, np.float64)
        v = np.ascontiguousarray(vel, np.float64) if vel is not None else None
        dw = np.ascontiguousarray(dL_dwrench, np.float64) if dL_dwrench is not None else None
        dt = np.ascontiguousarray(dL_dtaxel, np.float32) if dL_dtaxel is not None else None
        n_cells = self.n_cells
        o = out if out is not None else (None,) * 4
        w = _out(o[0], (self.n_pair, 6), np.float64)
        t = _out(o[1], (n_cells,), np.float32)
        dpose = _out(o[2], (self.n_pair, 2, 6), np.float64)
        dE = _out(o[3], (self.n_pair, 2), np.float64)
        p = self._step_ptrs
        L.check(self.lib.hc_step_adjoint(self.ctx, xpos.size // 3, p.get(0, xpos, L.dptr), p.get(1, xmat, L.dptr),
                                         p.get(2, v, L.dptr), p.get(3, dw, L.dptr), p.get(4, dt, L.fptr),
                                         p.get(5, w, L.dptr), p.get(6, t, L.fptr) if n_cells else None,
                                         p.get(7, dpose, L.dptr), p.get(8, dE, L.dptr)))
        return w, t, dpose, dE

    def step_adjoint_device(self, d_dL_dwrench: int | None, d_dL_dtaxel: int | None) -> int:
        """Forward step and adjoint as one graph on device buffers
        (hc_step_adjoint_device, asynchronous); returns the device pointer of
        the n_pair x 14 result."""
        out = C.c_void_p()
        L.check(self.lib.hc_step_adjoint_device(self.ctx, C.c_void_p(d_dL_dwrench) if d_dL_dwrench else None,
                                                C.c_void_p(d_dL_dtaxel) if d_dL_dtaxel else None, C.byref(out)))
        return out.value or 0

    def adjoint(self, dL_dwrench=None, dL_dtaxel=None, out=None):
        """(dL/dpose n_pair x 2 x 6, dL/dE n_pair x 2); ``out``: a pair of
        caller's arrays to fill."""
        dw = np.ascontiguousarray(dL_dwrench, np.float64) if dL_dwrench is not None else None
        dt = np.ascontiguousarray(dL_dtaxel, np.float32) if dL_dtaxel is not None else None
        dpose = _out(out[0] if out is not None else None, (self.n_pair, 2, 6), np.float64)
        dE = _out(out[1] if out is not None else None, (self.n_pair, 2), np.float64)
        L.check(self.lib.hc_adjoint(self.ctx, L.dptr(dw), L.fptr(dt), L.dptr(dpose), L.dptr(dE)))
        return dpose, dE
