"""ctypes bindings of the C ABI in include/hc/hc.h.

The shared library is built in-tree (mujoco_contact_surfaces_gb300/_build/
libhc.so).  Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libhc.so")

HC_OK = 0
HC_ERR_INVALID_ARG = 1
HC_ERR_UNSUPPORTED = 2
HC_ERR_OVERFLOW = 3
HC_ERR_TIMEOUT = 4
HC_ERR_CUDA = 5
HC_ERR_DEGENERATE = 6
HC_ERR_NOT_READY = 7
HC_ERR_NO_DEVICE = 8

GEOM_PLANE, GEOM_HFIELD, GEOM_SPHERE, GEOM_CAPSULE, GEOM_ELLIPSOID, GEOM_CYLINDER, GEOM_BOX, GEOM_MESH = range(8)
REPR_TRIANGLE, REPR_POLYGON = 0, 1
RIGID, SOFT = 0, 1
TAXEL_CLOSEST, TAXEL_WEIGHTED, TAXEL_MEAN, TAXEL_SQUARED = range(4)
SAMPLE_DEFAULT, SAMPLE_AREA_IMPORTANCE = 0, 1
QUERY_NONE, QUERY_SOFT_RIGID, QUERY_SOFT_HALFSPACE, QUERY_SOFT_SOFT = 0, 1, 2, 3
WINDOW_NONE, WINDOW_GAUSS, WINDOW_TUKEY, WINDOW_SQUARE = 0, 1, 2, 3


class hc_config(C.Structure):
    _fields_ = [("device", C.c_int), ("representation", C.c_int), ("apply_forces", C.c_int),
                ("use_graph", C.c_int), ("item_capacity", C.c_int64), ("face_capacity", C.c_int64)]


class hc_geom_info(C.Structure):
    _fields_ = [("kind", C.c_int), ("type", C.c_int), ("order", C.c_int), ("n_elements", C.c_int),
                ("n_vertices", C.c_int), ("E", C.c_double), ("dissipation", C.c_double),
                ("resolution_hint", C.c_double), ("mu_static", C.c_double), ("mu_dynamic", C.c_double)]


class hc_pair_stats(C.Structure):
    _fields_ = [("n_polygons", C.c_int32), ("n_faces", C.c_int32), ("n_near_degenerate", C.c_int32),
                ("n_items", C.c_int32), ("area", C.c_double), ("total_fn0", C.c_double)]


class hc_surface_view(C.Structure):
    _fields_ = [("n_poly", C.c_int), ("n_vert", C.c_int), ("poly_offset", C.POINTER(C.c_int)),
                ("vert", C.POINTER(C.c_double)), ("vert_pressure", C.POINTER(C.c_double)),
                ("normal", C.POINTER(C.c_double)), ("elem_a", C.POINTER(C.c_int)),
                ("elem_b", C.POINTER(C.c_int))]


class hc_candidate(C.Structure):
    _fields_ = [("pair", C.c_int32), ("elem_a", C.c_int32), ("elem_b", C.c_int32), ("n_vert", C.c_int32),
                ("flags", C.c_int32)]


class hc_timings(C.Structure):
    _fields_ = [("ms_setup", C.c_float), ("ms_broadphase", C.c_float), ("ms_narrowphase", C.c_float),
                ("ms_reduce", C.c_float), ("ms_taxels", C.c_float), ("ms_total", C.c_float),
                ("ms_kept_polygons", C.c_float), ("n_items", C.c_int64), ("n_polygons", C.c_int64),
                ("ms_adjoint", C.c_float)]


_P = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)

# name -> (restype, argtypes); every symbol include/hc/hc.h declares.
SIGNATURES = {
    "hc_config_default": (None, [C.POINTER(hc_config)]),
    "hc_last_error": (C.c_char_p, []),
    "hc_version": (C.c_char_p, []),
    "hc_context_create": (C.c_int, [C.POINTER(hc_config), C.POINTER(_P)]),
    "hc_context_destroy": (C.c_int, [_P]),
    "hc_reset": (C.c_int, [_P]),
    "hc_add_geom": (C.c_int, [_P, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int, _ip, C.c_int, _ip]),
    "hc_update_geom_size": (C.c_int, [_P, C.c_int, _dp]),
    "hc_get_geom_info": (C.c_int, [_P, C.c_int, C.POINTER(hc_geom_info)]),
    "hc_get_geom_mesh": (C.c_int, [_P, C.c_int, _dp, _dp, _ip]),
    "hc_get_element_order": (C.c_int, [_P, C.c_int, _ip]),
    "hc_generate_mesh": (C.c_int, [C.c_int, _dp, _dp, _dp, C.c_int, _ip, C.c_int, _ip, _ip, _ip, _dp, _dp, _ip]),
    "hc_set_poses": (C.c_int, [_P, C.c_int, _dp, _dp, _dp]),
    "hc_set_poses_device": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "hc_set_pairs": (C.c_int, [_P, C.c_int, _ip, _ip, _ip, _ip]),
    "hc_step": (C.c_int, [_P]),
    "hc_collide_pairs": (C.c_int, [_P, C.c_int, _ip, _ip, _ip]),
    "hc_get_wrenches": (C.c_int, [_P, _dp]),
    "hc_get_wrenches_device": (C.c_int, [_P, C.POINTER(_P)]),
    "hc_get_pair_order": (C.c_int, [_P, _ip, _ip, _ip]),
    "hc_get_pair_stats": (C.c_int, [_P, C.POINTER(hc_pair_stats)]),
    "hc_get_surface": (C.c_int, [_P, C.c_int, C.POINTER(hc_surface_view)]),
    "hc_set_debug": (C.c_int, [_P, C.c_int]),
    "hc_get_candidates": (C.c_int, [_P, C.POINTER(hc_candidate), C.c_int64, C.POINTER(C.c_int64)]),
    "hc_add_flat_sensor": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, _ip, _ip, _ip]),
    "hc_get_taxels": (C.c_int, [_P, C.c_int, _fp]),
    "hc_get_taxels_all": (C.c_int, [_P, _fp, C.c_int64]),
    "hc_get_taxels_device": (C.c_int, [_P, C.POINTER(_P), C.POINTER(C.c_int64)]),
    "hc_adjoint": (C.c_int, [_P, _dp, _fp, _dp, _dp]),
    "hc_set_adjoint_mode": (C.c_int, [_P, C.c_int]),
    "hc_adjoint_device": (C.c_int, [_P, _P, _P, C.POINTER(_P)]),
    "hc_get_adjoint_launch_count": (C.c_int, [_P, _ip]),
    "hc_get_adjoint_skipped": (C.c_int, [_P, _ip, _fp]),
    "hc_step_adjoint": (C.c_int, [_P, C.c_int, _dp, _dp, _dp, _dp, _fp, _dp, _fp, _dp, _dp]),
    "hc_step_adjoint_device": (C.c_int, [_P, _P, _P, C.POINTER(_P)]),
    "hc_enable_timing": (C.c_int, [_P, C.c_int]),
    "hc_get_timings": (C.c_int, [_P, C.POINTER(hc_timings)]),
    "hc_get_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "hc_get_launch_count": (C.c_int, [_P, _ip]),
    "hc_autotune": (C.c_int, [_P, _ip, _ip]),
    "hc_set_launch_shape": (C.c_int, [_P, C.c_int, C.c_int]),
    "hc_step_noalloc": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P]),
    "hc_add_taxel_sensor": (C.c_int, [_P, C.c_int, C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                      _ip]),
    "hc_set_taxel_sensor_enabled": (C.c_int, [_P, C.c_int, C.c_int]),
    "hc_get_taxel_sensor_values": (C.c_int, [_P, C.c_int, _fp]),
    "hc_get_all_taxel_sensor_values": (C.c_int, [_P, _fp, C.c_size_t]),
    "hc_sample_surface": (C.c_int, [C.c_int, _dp, C.c_int, _ip, C.c_int, C.c_uint64, C.c_int, _dp, _dp, _ip]),
    "hc_add_curved_sensor": (C.c_int, [_P, C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_int, _dp, _dp, _ip]),
    "hc_set_curved_sensor_enabled": (C.c_int, [_P, C.c_int, C.c_int]),
    "hc_get_curved_sensor_values": (C.c_int, [_P, C.c_int, _fp]),
}

_lib = None


def load(path: str | None = None):
    """Load libhc.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    p = path or _build.build()
    if not os.path.exists(p):
        raise RuntimeError(f"libhc.so missing at {p}; the CUDA extension is required")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class HCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"hc status {status}: {msg}")
        self.status = status


def check(status: int):
    if status != HC_OK:
        raise HCError(status, load().hc_last_error().decode())


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip) if a is not None else None


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_fp) if a is not None else None


def sample_surface(mesh_vert, mesh_face, n_samples: int, seed: int = 42):
    """Blue-noise points on a triangle mesh with their triangles' unit
    normals (hc_sample_surface; host only).  Returns (points, normals)."""
    lib = load()
    v = np.ascontiguousarray(mesh_vert, dtype=np.float64).reshape(-1, 3)
    f = np.ascontiguousarray(mesh_face, dtype=np.int32).reshape(-1, 3)
    cap = max(1, int(n_samples))
    pts = np.zeros((cap, 3))
    nrm = np.zeros((cap, 3))
    n = C.c_int()
    check(lib.hc_sample_surface(v.shape[0], dptr(v), f.shape[0], iptr(f), int(n_samples), int(seed), cap, dptr(pts),
                                dptr(nrm), C.byref(n)))
    return pts[:n.value].copy(), nrm[:n.value].copy()


def generate_mesh(gtype: int, size, cs5, mesh_vert=None, mesh_face=None):
    """Host-only mesh generation (no GPU needed).  Returns (kind, verts,
    pressures or None, elems)."""
    lib = load()
    size = np.ascontiguousarray(size, dtype=np.float64)
    cs5 = np.ascontiguousarray(cs5, dtype=np.float64)
    mv = np.ascontiguousarray(mesh_vert, dtype=np.float64) if mesh_vert is not None else None
    mf = np.ascontiguousarray(mesh_face, dtype=np.int32) if mesh_face is not None else None
    nv_in = 0 if mv is None else len(mv) // 3 if mv.ndim == 1 else mv.shape[0]
    nf_in = 0 if mf is None else len(mf) // 3 if mf.ndim == 1 else mf.shape[0]
    kind, nv, ne = C.c_int(), C.c_int(), C.c_int()
    check(lib.hc_generate_mesh(gtype, dptr(size), dptr(cs5), dptr(mv), nv_in, iptr(mf), nf_in, C.byref(kind),
                               C.byref(nv), C.byref(ne), None, None, None))
    npe = 4 if kind.value == SOFT else 3
    v = np.zeros((nv.value, 3), np.float64)
    e = np.zeros((ne.value, npe), np.int32)
    p = np.zeros(nv.value, np.float64) if kind.value == SOFT else None
    check(lib.hc_generate_mesh(gtype, dptr(size), dptr(cs5), dptr(mv), nv_in, iptr(mf), nf_in, C.byref(kind),
                               C.byref(nv), C.byref(ne), dptr(v), dptr(p), iptr(e)))
    return kind.value, v, p, e
