"""The header-only plugin class (include/hc/contact_surfaces_plugin.hpp) over a
fake MuJoCo model: custom-field parsing on the CPU, and the collision /
passive / sensor cycle on the GPU compared with the Engine on the same scene.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _compile(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    lib = B.build()
    exe = str(tmp_path / "plugin_shim_main")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "plugin_shim_main.cpp"), "-L", os.path.dirname(lib), "-lhc",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def _run(exe, mode):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return [ln.split() for ln in r.stdout.splitlines() if ln.strip()]


def test_parse_custom_fields(tmp_path):
    out = _run(_compile(tmp_path), "parse")
    heads = [ln for ln in out if ln[0] == "repr"]
    assert heads[0] == ["repr", "0", "apply", "0", "visualize", "0", "ngeoms", "4"]
    assert heads[1] == ["repr", "0", "apply", "1", "visualize", "0", "ngeoms", "4"]
    geoms = [ln for ln in out if ln[0] == "geom"][:4]
    # numeric-field order is the registration (M/N) order; unknown geoms and
    # fields without 5 values are skipped (plugin.cpp:613-626)
    assert [g[2] for g in geoms] == ["ball", "plate", "floor", "cube"]
    assert [int(g[1]) for g in geoms] == [0, 1, 2, 4]
    assert [float(x) for x in geoms[0][3:]] == [2e5, 1.0, 0.006, 0.5, 0.5]
    assert [ln for ln in out if ln[0] == "repr2"][0][1] == "1"
    # taxels of a mesh geom with a local pose (p0, 90 degrees about z) move by
    # the inverse pose: R^T (t - p0) (taxel_sensor.cpp:121-147)
    inv = np.array([float(x) for x in [ln for ln in out if ln[0] == "invpose"][0][1:]])
    np.testing.assert_allclose(inv, [2.2, -0.9, 2.7, 0, 0, 0], atol=1e-12)
    assert [ln for ln in out if ln[0] == "identity"][0][1:] == ["1", "2", "3"]


@pytest.mark.gpu
def test_plugin_cycle_matches_engine(gpu, tmp_path):
    out = _run(_compile(tmp_path), "step")
    steps = [ln for ln in out if ln[0] == "step"]
    assert [ln[3] for ln in steps] == ["1", "1", "1"]            # step ok
    assert [ln[5] for ln in steps] == ["4", "4", "4"]            # two surface pairs x 2 bodies
    assert [ln[7] for ln in steps] == ["1", "1", "2"]            # 50 Hz sensor at t = 0, 0.01, 0.02
    assert [ln[9:11] for ln in steps] == [["1", "1"], ["1", "1"], ["2", "2"]]  # 50 Hz taxel sensors
    tv = np.array([float(x) for x in [ln for ln in out if ln[0] == "taxel_values"][0][1:]], np.float32)
    cv = np.array([float(x) for x in [ln for ln in out if ln[0] == "closest_values"][0][1:]], np.float32)
    counts = [ln for ln in out if ln[0] == "counts"][0]
    assert counts == ["counts", "default", "6", "surface", "6"]
    w = np.array([[float(x) for x in ln[2:]] for ln in out if ln[0] == "wrench"])
    body = {int(ln[1]): np.array([float(x) for x in ln[2:]]) for ln in out if ln[0] == "body"}
    tax = [ln for ln in out if ln[0] == "taxels"][0]
    resized = [ln for ln in out if ln[0] == "resized"][0]

    # the same scene through the Engine (same library, same order)
    from mujoco_contact_surfaces_gb300.engine import Engine
    eng = Engine()
    eng.add_geom(0, L.GEOM_SPHERE, [0.03, 0, 0], [2e5, 1.0, 0.006, 0.5, 0.5])
    eng.add_geom(1, L.GEOM_BOX, [0.04, 0.04, 0.005], [0, 1.0, 0, 0.4, 0.4])
    eng.add_geom(2, L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.6, 0.6])
    eng.add_geom(4, L.GEOM_BOX, [0.02, 0.02, 0.02], [1e5, 0.5, 0.01, 0.3, 0.3])
    eng.add_flat_sensor(1, 0.005, 5, L.WINDOW_NONE, -1.0)
    grid = [[-0.01 + 0.005 * i, -0.01 + 0.005 * j, 0.005] for i in range(5) for j in range(5)]
    ts = eng.add_taxel_sensor(1, grid, L.TAXEL_MEAN, 0.004, 0.002, L.SAMPLE_DEFAULT, False)
    tcl = eng.add_taxel_sensor(1, grid, L.TAXEL_CLOSEST, 0.004, 0.01, L.SAMPLE_AREA_IMPORTANCE, True)
    eng.set_pairs([1, 4], [0, 2])
    xpos = np.zeros((5, 3))
    xpos[0] = [0.004, -0.003, 0.005 + 0.03 - 0.002]
    xpos[2] = [0, 0, -0.2]
    xpos[3] = [0.5, 0.5, 0.5]
    xpos[4] = [0.3, 0.0, -0.2 + 0.02 - 0.001]
    xmat = np.tile(np.eye(3).reshape(1, 9), (5, 1))
    vel = np.zeros((5, 6))
    vel[0, 5] = -0.01
    vel[4, 3] = 0.02
    eng.set_poses(xpos, xmat, vel)
    eng.step()
    we = eng.wrenches()
    _, m, n = eng.pair_order()
    te = eng.taxels(0)
    tve, cve = eng.taxel_sensor_values(ts), eng.taxel_sensor_values(tcl)
    eng.close()
    np.testing.assert_array_equal(tv, tve)
    np.testing.assert_array_equal(cv, cve)
    assert (tv > 0).sum() >= 2 and (cv > 0).sum() >= 1
    assert list(m) == [0, 2] and list(n) == [1, 4]
    assert np.array_equal(w, we)
    assert np.linalg.norm(we[0, :3]) > 0 and np.linalg.norm(we[1, :3]) > 0
    # applied wrenches: +W on M, -W on N, torques about the world origin
    def about_origin(wr, x):
        return np.concatenate([wr[:3], wr[3:] + np.cross(x, wr[:3])])
    np.testing.assert_allclose(body[1], about_origin(we[0], xpos[0]), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(body[2], -about_origin(we[0], xpos[0]), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(body[0], about_origin(we[1], xpos[2]), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(body[4], -about_origin(we[1], xpos[2]), rtol=1e-12, atol=1e-12)
    assert int(tax[1]) == 16 and int(tax[2]) == 16
    assert float(tax[3]) == pytest.approx(float(te.sum()), rel=1e-6) and float(tax[4]) > 0
    assert resized[2] == "1" and float(resized[4]) > we[0, 2] > 0


@pytest.mark.gpu
def test_curved_sensor_plugin_matches_engine(gpu, tmp_path):
    """The CurvedSensor plugin class on a soft box mesh pressed into the
    floor: its 50 Hz gate, the (int)sample_resolution * area point count,
    and its values against the Engine given the same points."""
    out = _run(_compile(tmp_path), "curved")
    steps = [ln for ln in out if ln[0] == "cstep"]
    assert [ln[3] for ln in steps] == ["1", "1", "1"]
    assert [ln[5] for ln in steps] == ["1", "1", "2"]
    n_pts = int([ln for ln in out if ln[0] == "points"][0][1])
    vals = np.array([float(x) for x in [ln for ln in out if ln[0] == "curved_values"][0][1:]], np.float32)
    assert [ln for ln in out if ln[0] == "reject_primitive"][0][1] == "1"

    from mujoco_contact_surfaces_gb300.engine import Engine
    hx, hy, hz = np.float32(0.02), np.float32(0.02), np.float32(0.01)
    vert = np.array([[sx * hx, sy * hy, sz * hz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)],
                    np.float32).astype(np.float64)
    face = np.array([0, 1, 3, 0, 3, 2, 4, 6, 7, 4, 7, 5, 0, 4, 5, 0, 5, 1, 2, 3, 7, 2, 7, 6, 0, 2, 6, 0, 6, 4,
                     1, 5, 7, 1, 7, 3], np.int32).reshape(-1, 3)
    area = 0.0
    for a, b, c in face:
        cr = np.cross(vert[b] - vert[a], vert[c] - vert[a])
        area += 0.5 * np.sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2])
    n_want = int(200000 * area)
    assert n_pts == n_want
    pts, nrm = L.sample_surface(vert, face, n_want, seed=42)
    taxels = [[0.006 * i, 0.006 * j, -float(hz)] for i in (-1, 0, 1) for j in (-1, 0, 1)]
    tn = np.zeros((9, 3))
    tn[0] = [0, 0, -1]
    tn[2] = [0, 0, -3]
    eng = Engine()
    eng.add_geom(0, L.GEOM_PLANE, [0, 0, 1], [0, 1.0, 0, 0.5, 0.5])
    eng.add_geom(1, L.GEOM_MESH, [0, 0, 0], [1e5, 1.0, 0.004, 0.5, 0.5], vert, face)
    sid = eng.add_curved_sensor(1, taxels, 0.004, pts, nrm, tn)
    eng.set_pairs([1], [0])
    xpos = np.array([[0, 0, 0], [0.001, -0.002, float(hz) - 0.002]])
    xmat = np.tile(np.eye(3).reshape(1, 9), (2, 1))
    eng.set_poses(xpos, xmat, np.zeros((2, 6)))
    eng.step()
    ve = eng.curved_sensor_values(sid)
    eng.close()
    np.testing.assert_array_equal(vals, ve)
    assert np.count_nonzero(ve) >= 5
