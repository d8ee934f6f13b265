"""Surface sampler of the curved sensor (hc_sample_surface, host only): the
points lie on the mesh, carry their triangle's outward normal, keep a
minimum spacing, and repeat for a seed."""
import numpy as np

from mujoco_contact_surfaces_gb300 import _lib as L


def _box_mesh(h):
    v = np.array([[sx * h[0], sy * h[1], sz * h[2]] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)])
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    f = []
    for a, b, c, d in quads:
        f += [(a, b, c), (a, c, d)]
    return v, np.array(f, np.int32)


def test_samples_on_surface_with_normals_and_spacing():
    h = (0.02, 0.01, 0.005)
    v, f = _box_mesh(h)
    # outward orientation of the test mesh
    for t in f:
        n = np.cross(v[t[1]] - v[t[0]], v[t[2]] - v[t[0]])
        assert n @ (v[t].mean(0)) > 0
    area = 8 * (h[0] * h[1] + h[1] * h[2] + h[0] * h[2])
    n_want = 400
    p, nrm = L.sample_surface(v, f, n_want, seed=42)
    assert len(p) == n_want
    # on the box surface: one coordinate at +-h, the others inside
    rel = np.abs(p) / np.array(h)
    assert np.all(rel <= 1 + 1e-12)
    assert np.all(np.abs(rel.max(axis=1) - 1) < 1e-12)
    np.testing.assert_allclose(np.linalg.norm(nrm, axis=1), 1, atol=1e-12)
    face_axis = np.argmax(rel, axis=1)
    for k in range(len(p)):
        e = np.zeros(3)
        e[face_axis[k]] = np.sign(p[k, face_axis[k]])
        np.testing.assert_allclose(nrm[k], e, atol=1e-12)
    # spacing: no two points closer than a fraction of the packing spacing
    d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=2) + np.eye(len(p))
    assert d.min() > 0.4 * np.sqrt(area / n_want)
    # deterministic per seed
    p2, _ = L.sample_surface(v, f, n_want, seed=42)
    p3, _ = L.sample_surface(v, f, n_want, seed=7)
    assert np.array_equal(p, p2) and not np.array_equal(p, p3)
    # nothing asked, nothing given
    assert len(L.sample_surface(v, f, 0)[0]) == 0
