"""The isosurface oracle's own properties (CPU): planes, spheres, closure,
orientation, NaN handling."""
import numpy as np

from oracle import iso_oracle as iso


def _grid_values(n, fn, h=None):
    h = 1.0 / (n - 1) if h is None else h
    x = np.arange(n) * h
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")  # node order i fastest
    return fn(xx, yy, zz).ravel(), h


def _edges(tris_xyz):
    keys = {}
    for t in np.round(tris_xyz, 12):
        for a, b in ((0, 1), (1, 2), (2, 0)):
            e = tuple(sorted((tuple(t[a]), tuple(t[b]))))
            keys[e] = keys.get(e, 0) + 1
    return keys


def test_plane_area_and_orientation():
    n = 6
    v, h = _grid_values(n, lambda x, y, z: z + 0.0 * x)
    t = iso.isosurface(v, (n, n, n), np.zeros(3), np.full(3, h), 0.37)
    v0, v1, v2 = t[:, 0], t[:, 1], t[:, 2]
    nrm = np.cross(v1 - v0, v2 - v0)
    area = 0.5 * np.linalg.norm(nrm, axis=1).sum()
    assert abs(area - 1.0) < 1e-12
    assert np.all(nrm[:, 2] > 0)  # towards increasing f
    np.testing.assert_allclose(t[..., 2], 0.37, atol=1e-14)


def test_sphere_is_closed_and_area_converges():
    errs = []
    for n in (9, 17):
        v, h = _grid_values(n, lambda x, y, z: (x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2)
        t = iso.isosurface(v, (n, n, n), np.zeros(3), np.full(3, h), 0.3 ** 2)
        counts = _edges(t)
        assert set(counts.values()) == {2}  # closed: every edge shared by two triangles
        c = t.mean(axis=1) - 0.5
        nrm = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
        assert np.all(np.einsum("ij,ij->i", c, nrm) > 0)  # outward = increasing f
        area = 0.5 * np.linalg.norm(nrm, axis=1).sum()
        errs.append(abs(area - 4 * np.pi * 0.09) / (4 * np.pi * 0.09))
    assert errs[1] < errs[0] < 0.1


def test_no_crossing_and_nan_cells():
    n = 4
    v, h = _grid_values(n, lambda x, y, z: x + y + z)
    assert iso.isosurface(v, (n, n, n), np.zeros(3), np.full(3, h), 10.0).shape == (0, 3, 3)
    v2 = v.copy()
    v2[1 + n * (1 + n * 1)] = np.nan  # node (1, 1, 1): its 8 cells drop out
    full = iso.isosurface(v, (n, n, n), np.zeros(3), np.full(3, h), 1.1)
    part = iso.isosurface(v2, (n, n, n), np.zeros(3), np.full(3, h), 1.1)
    assert 0 < part.shape[0] < full.shape[0]


def test_isosurfacer_value_and_name_rules():
    """LoopIsosurfacer.fit's isovalue / name rules (LoopStructural/utils/_surface.py:96-133)."""
    import pytest

    from loopstructural_gb300 import surface as S

    v = np.array([0.0, np.nan, 2.0])
    assert S.isovalues_for(None, v) == [1.0]
    assert S.isovalues_for(0.5, v) == [0.5]
    assert S.isovalues_for(0, v) == [0.0]
    assert S.isovalues_for([0.2, 0.3], v) == [0.2, 0.3]
    np.testing.assert_allclose(S.isovalues_for(3, v), [0.1, 1.0, 1.9])
    with pytest.raises(ValueError):
        S.isovalues_for(-2, v)
    assert S.surface_names(None, 2) == (["surface", "surface"], False)
    assert S.surface_names("top", 1) == (["top"], True)
    assert S.surface_names("top", 2) == (["top", "top"], False)
    assert S.surface_names(["a", "b"], 2) == (["a", "b"], True)
    with pytest.raises(ValueError):
        S.LoopIsosurfacer(object())
