"""Mesh and pressure-field generators (load-time geometry of the soft and
rigid geoms; the reference builds these with Drake at P:648-807)."""
import math

import numpy as np
import pytest

from mujoco_contact_surfaces_gb300 import _lib as L
from mujoco_contact_surfaces_gb300.scenes import sphere_hint


def tet_vol(v, e):
    a, b, c, d = v[e[:, 0]], v[e[:, 1]], v[e[:, 2]], v[e[:, 3]]
    return np.einsum("ij,ij->i", b - a, np.cross(c - a, d - a)) / 6


def boundary_faces(e):
    faces = {}
    for t in e:
        for f in ([t[1], t[2], t[3]], [t[0], t[3], t[2]], [t[0], t[1], t[3]], [t[0], t[2], t[1]]):
            k = tuple(sorted(f))
            faces[k] = faces.get(k, 0) + 1
    return [k for k, n in faces.items() if n == 1], max(faces.values())


@pytest.mark.parametrize("gtype,size,hint,vol", [
    (L.GEOM_BOX, [0.02, 0.03, 0.01], 0.005, 8 * 0.02 * 0.03 * 0.01),
    (L.GEOM_BOX, [0.05, 0.05, 0.05], 0.0, 0.001),
    (L.GEOM_SPHERE, [0.05, 0, 0], 0.01, None),
    (L.GEOM_ELLIPSOID, [0.04, 0.03, 0.02], 0.005, None),
    (L.GEOM_CYLINDER, [0.03, 0.03, 0], 0.0075, None),
])
def test_soft_mesh_is_a_valid_tetrahedralisation(gtype, size, hint, vol):
    kind, v, p, e = L.generate_mesh(gtype, size, [1e5, 1, hint, 0.5, 0.5])
    assert kind == L.SOFT
    vols = tet_vol(v, e)
    assert vols.min() > 0, "every tet positively oriented"
    bf, maxshare = boundary_faces(e)
    assert maxshare <= 2, "a face shared by more than two tets"
    # closed boundary: every boundary edge shared by exactly two boundary faces
    edges = {}
    for f in bf:
        for i in range(3):
            k = tuple(sorted((f[i], f[(i + 1) % 3])))
            edges[k] = edges.get(k, 0) + 1
    assert set(edges.values()) == {2}
    if vol is not None:
        assert abs(vols.sum() - vol) <= 1e-6 * vol
    # pressure: 0 on the boundary, maximal (E) inside
    bverts = np.unique(np.array(bf).ravel())
    assert np.all(p[bverts] == 0)
    assert p.max() == pytest.approx(1e5, rel=1e-6)
    assert p.min() >= 0
    # every tet carries pressure: a vertex off the surface (a tet with all
    # four vertices on the surface would be a zero-pressure shell element)
    assert np.all(p[e].max(axis=1) > 0), f"{int(np.sum(p[e].max(axis=1) == 0))} tets without pressure"


def test_sphere_levels_and_tet_counts():
    for lev in range(0, 6):
        _, v, p, e = L.generate_mesh(L.GEOM_SPHERE, [0.03, 0, 0], [1e5, 1, sphere_hint(0.03, lev), 0.5, 0.5])
        assert len(e) == 8 * 4 ** lev
    # the single interior vertex (the centre) carries E
    assert np.count_nonzero(p) == 1 and np.all(v[np.argmax(p)] == 0)


def test_cylinder_volume_is_the_prism():
    _, v, p, e = L.generate_mesh(L.GEOM_CYLINDER, [0.03, 0.04, 0], [1e5, 1, 0.0075, 0.5, 0.5])
    ns = 28  # sectors chosen for r=0.03, hint 0.0075
    prism = 0.5 * ns * 0.03 ** 2 * math.sin(2 * math.pi / ns) * 0.08
    assert tet_vol(v, e).sum() == pytest.approx(prism, rel=1e-6)


def test_box_field_is_extent_times_E():
    h = np.array([0.02, 0.03, 0.01])
    _, v, p, e = L.generate_mesh(L.GEOM_BOX, h, [2e5, 1, 0.005, 0.5, 0.5])
    d = np.min(h[None, :] - np.abs(v), axis=1)
    np.testing.assert_allclose(p, 2e5 * d / h.min(), rtol=1e-6, atol=0.05)  # vertices are float-rounded


@pytest.mark.parametrize("gtype,size,hint,ntri", [
    (L.GEOM_BOX, [0.1, 0.1, 0.01], 0.0, 12),
    (L.GEOM_BOX, [0.1, 0.1, 0.01], 0.05, 2 * (2 * 4 * 4 + 2 * 4 * 1 + 2 * 4 * 1)),
])
def test_rigid_box_mesh(gtype, size, hint, ntri):
    kind, v, p, f = L.generate_mesh(gtype, size, [0, 1, hint, 0.5, 0.5])
    assert kind == L.RIGID and len(f) == ntri
    # outward orientation: divergence theorem gives +volume
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6
    assert vol == pytest.approx(8 * size[0] * size[1] * size[2], rel=1e-6)


@pytest.mark.parametrize("gtype,size,hint", [
    (L.GEOM_SPHERE, [0.05, 0, 0], 0.02), (L.GEOM_CYLINDER, [0.03, 0.05, 0], 0.01),
    (L.GEOM_ELLIPSOID, [0.04, 0.03, 0.02], 0.01)])
def test_rigid_meshes_are_closed_and_outward(gtype, size, hint):
    _, v, _, f = L.generate_mesh(gtype, size, [0, 1, hint, 0.5, 0.5])
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6
    assert vol > 0
    edges = {}
    for t in f:
        for i in range(3):
            k = (t[i], t[(i + 1) % 3])
            edges[k] = edges.get(k, 0) + 1
    assert all(edges.get((b_, a_), 0) == 1 for (a_, b_) in edges), "each directed edge has its twin"


def test_convex_mesh_soft_is_centroid_fan():
    # a unit cube as a user mesh
    _, v, _, f = L.generate_mesh(L.GEOM_BOX, [0.5, 0.5, 0.5], [0, 1, 0, 0.5, 0.5])
    kind, sv, sp, se = L.generate_mesh(L.GEOM_MESH, [0, 0, 0], [1e5, 1, 0, 0.5, 0.5], v.ravel(), f.ravel())
    assert kind == L.SOFT and len(se) == len(f)
    c = sv[np.argmax(sp)]
    np.testing.assert_allclose(c, 0, atol=1e-7)
    assert tet_vol(sv, se).sum() == pytest.approx(1.0, rel=1e-6)


def test_oracle_builds_the_same_meshes():
    # the oracle library compiles the generator source itself (so the CPU
    # baseline loads no engine library); its meshes must be the engine's,
    # bit for bit, for every primitive and kind the workloads use
    import oracle
    from mujoco_contact_surfaces_gb300 import scenes
    cases = [(L.GEOM_SPHERE, [0.05, 0, 0], [1e5, 1, 0.01, 0.5, 0.5]),
             (L.GEOM_ELLIPSOID, [0.04, 0.03, 0.02], [2e5, 1, sphere_hint(0.04, 4), 0.5, 0.5]),
             (L.GEOM_CYLINDER, [0.03, 0.03, 0], [3e5, 1, 0.0075, 0.5, 0.5]),
             (L.GEOM_BOX, [0.02, 0.03, 0.01], [1e5, 1, 0.005, 0.5, 0.5]),
             (L.GEOM_BOX, [0.1, 0.1, 0.01], [0, 1, 0, 0.5, 0.5]),
             (L.GEOM_PLANE, [0, 0, 1], [0, 1, 0, 0.5, 0.5])]
    s = scenes.batched(6)
    cases += [(g["type"], g["size"], g["cs5"]) for g in s.geoms]
    for gtype, size, cs5 in cases:
        a = L.generate_mesh(gtype, size, cs5)
        b = oracle.generate_mesh(gtype, size, cs5)
        assert a[0] == b[0]
        for x, y in zip(a[1:], b[1:]):
            assert (x is None and y is None) or np.array_equal(x, y)


def _degenerate(gtype, size, cs5, v=None, f=None):
    with pytest.raises(L.HCError) as ei:
        L.generate_mesh(gtype, size, cs5, v, f)
    assert ei.value.status == L.HC_ERR_DEGENERATE, str(ei.value)
    return str(ei.value)


def test_degenerate_meshes_are_rejected():
    # Host-side checks of the input geometry (the engine's hc_add_geom runs
    # the same generator and checks): a flat soft mesh encloses no volume, a
    # closed mesh with a zero-area face gives a zero-volume tet in its
    # centroid fan, an empty or zero-area rigid mesh has nothing to clip.
    soft, rigid = [1e5, 1.0, 0.0, 0.5, 0.5], [0, 1.0, 0.0, 0.5, 0.5]
    flat_v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], float) * 0.05
    flat_f = np.array([[0, 1, 2], [0, 2, 3], [0, 2, 1], [0, 3, 2]], np.int32)
    assert "zero volume" in _degenerate(L.GEOM_MESH, [0, 0, 0], soft, flat_v, flat_f)
    # a tetrahedron whose fourth face is split by a vertex on its edge: the
    # split leaves a zero-area sliver face
    tv = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [0.5, 0.5, 0]], float) * 0.05
    tf = np.array([[0, 2, 1], [0, 1, 3], [0, 3, 2], [1, 2, 3], [1, 4, 2]], np.int32)
    assert "zero-volume" in _degenerate(L.GEOM_MESH, [0, 0, 0], soft, tv, tf)
    rv = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0]], float)
    assert "zero-area" in _degenerate(L.GEOM_MESH, [0, 0, 0], rigid, rv, np.array([[0, 3, 1], [0, 1, 2]], np.int32))
    assert "empty" in _degenerate(L.GEOM_MESH, [0, 0, 0], rigid, rv, np.zeros((0, 3), np.int32))
    # the same rules in the oracle's copy of the generator
    import oracle
    with pytest.raises(ValueError):
        oracle.generate_mesh(L.GEOM_MESH, [0, 0, 0], soft, flat_v, flat_f)
    # well-formed meshes pass
    assert L.generate_mesh(L.GEOM_MESH, [0, 0, 0], soft, tv[:4], tf[:4])[0] == L.SOFT
