"""The C-ABI library loads and exports every symbol include/hc/hc.h declares.

No compute call runs here (no GPU on the CPU runner); context creation either
succeeds (GPU present) or returns HC_ERR_NO_DEVICE.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "hc", "hc.h")).read()
    return sorted(set(re.findall(r"HC_API\s+[\w\s\*]+?\b(hc_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported():
    lib = L.load()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    assert set(declared_symbols()) == set(L.SIGNATURES)


def test_context_create_without_device_is_clean():
    lib = L.load()
    cfg = L.hc_config()
    lib.hc_config_default(C.byref(cfg))
    assert cfg.representation == L.REPR_TRIANGLE and cfg.apply_forces == 1
    ctx = C.c_void_p()
    st = lib.hc_context_create(C.byref(cfg), C.byref(ctx))
    if st == L.HC_OK:
        lib.hc_context_destroy(ctx)
    else:
        assert st == L.HC_ERR_NO_DEVICE
        assert b"device" in lib.hc_last_error()


def test_invalid_config_rejected():
    lib = L.load()
    cfg = L.hc_config()
    lib.hc_config_default(C.byref(cfg))
    cfg.representation = 7
    ctx = C.c_void_p()
    assert lib.hc_context_create(C.byref(cfg), C.byref(ctx)) == L.HC_ERR_INVALID_ARG


def test_null_context_calls_fail_cleanly():
    lib = L.load()
    assert lib.hc_step(None) == L.HC_ERR_INVALID_ARG
    assert lib.hc_get_wrenches(None, None) == L.HC_ERR_INVALID_ARG
    assert lib.hc_context_destroy(None) == L.HC_OK


def test_generate_mesh_unsupported_types():
    # soft plane, hfield and capsule have no contact surface
    for t, E in [(L.GEOM_CAPSULE, 1e5), (L.GEOM_HFIELD, 0.0), (L.GEOM_PLANE, 1e5)]:
        try:
            L.generate_mesh(t, [0.1, 0.1, 0.1], [E, 1, 0.01, 0.5, 0.5])
        except L.HCError as e:
            assert e.status == L.HC_ERR_UNSUPPORTED
        else:
            raise AssertionError("expected HC_ERR_UNSUPPORTED")


def test_soft_cylinder_needs_hint():
    # the reference reads an uninitialised mesh for hint <= 0
    try:
        L.generate_mesh(L.GEOM_CYLINDER, [0.03, 0.03, 0], [1e5, 1, 0.0, 0.5, 0.5])
    except L.HCError as e:
        assert e.status == L.HC_ERR_INVALID_ARG
    else:
        raise AssertionError("expected HC_ERR_INVALID_ARG")


def test_generated_values_are_float_representable():
    k, v, p, e = L.generate_mesh(L.GEOM_SPHERE, [0.05, 0, 0], [1e5, 1, 0.01, 0.5, 0.5])
    assert np.array_equal(v, v.astype(np.float32).astype(np.float64))
    assert np.array_equal(p, p.astype(np.float32).astype(np.float64))


def test_caller_output_arrays_are_checked():
    # Engine outputs go into the caller's arrays (e.g. page-locked ones) when
    # given: right dtype, size and C order, else a ValueError before any call
    from mujoco_contact_surfaces_gb300.engine import _out
    a = np.zeros((4, 6))
    assert _out(a, (4, 6), np.float64) is a
    assert _out(None, (4, 6), np.float64).shape == (4, 6)
    with pytest.raises(ValueError):
        _out(np.zeros((4, 6), np.float32), (4, 6), np.float64)
    with pytest.raises(ValueError):
        _out(np.zeros((4, 5)), (4, 6), np.float64)
    with pytest.raises(ValueError):
        _out(np.zeros((6, 4)).T, (4, 6), np.float64)


def test_launch_shape_rejects_null_context():
    lib = L.load()
    assert lib.hc_set_launch_shape(None, 6, 8) == L.HC_ERR_INVALID_ARG
