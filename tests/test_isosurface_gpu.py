"""GPU isosurface (ls_iso_extract / ls_iso_copy) against the oracle's
marching-tetrahedra restatement.  Tolerances: vertex coordinates 1e-10
absolute (snapped to the oracle's points), then the triangle sets equal
exactly (orientation included); unit normals along +grad f."""
import numpy as np
import pytest
from scipy.spatial import cKDTree

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import _lib, fd  # noqa: E402
from oracle import iso_oracle as iso  # noqa: E402

pytestmark = pytest.mark.gpu


def _field(n, fn):
    x = np.arange(n) / (n - 1)
    zz, yy, xx = np.meshgrid(x, x, x, indexing="ij")
    return fn(xx, yy, zz).ravel()


def _check(grid, values, level):
    d = torch.from_numpy(values).to(_lib.device())
    verts, tris, nrm = fd.isosurface(grid, d, level)
    ref = iso.isosurface(values, grid.nsteps, grid.origin, grid.step_vector, level)
    assert tris.shape[0] == ref.shape[0]
    if ref.shape[0] == 0:
        assert verts.shape[0] == 0
        return verts, tris, nrm
    pts = ref.reshape(-1, 3)
    dist, idx = cKDTree(pts).query(verts)
    assert dist.max() <= 1e-10
    assert iso.canonical(pts[idx][tris]) == iso.canonical(ref)
    # every vertex is used (one per crossing edge of an emitted cell)
    assert np.array_equal(np.unique(tris), np.arange(verts.shape[0]))
    np.testing.assert_allclose(np.linalg.norm(nrm, axis=1), 1.0, atol=1e-12)
    return verts, tris, nrm


@pytest.mark.parametrize("n", [9, 24])
def test_sphere_matches_oracle(n):
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.array([n - 1] * 3), step_vector=np.ones(3) / (n - 1))
    vals = _field(n, lambda x, y, z: (x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2 + 0.05 * np.sin(5 * x))
    verts, tris, nrm = _check(grid, vals, 0.09)
    # normals point outwards (towards increasing f)
    c = verts - np.array([0.5, 0.45, 0.55])
    assert np.mean(np.einsum("ij,ij->i", c, nrm) > 0) > 0.99


def test_nan_nodes_plane_and_empty():
    n = 12
    grid = L.StructuredGrid(origin=np.array([1.0, -2.0, 0.5]), nsteps=np.array([n - 1, n - 2, n - 3]),
                            step_vector=np.array([0.1, 0.2, 0.05]))
    nx, ny, nz = grid.nsteps
    k = np.arange(grid.n_nodes) // (nx * ny)
    vals = 0.5 + 0.05 * k.astype(float)
    vals[[5, 300, 777]] = np.nan
    _check(grid, vals, 0.5 + 0.05 * 3.3)
    _check(grid, vals, 100.0)  # no crossing: empty


def test_interpolator_surfaces():
    n = 20
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.array([n - 1] * 3), step_vector=np.ones(3) / (n - 1))
    interp = L.FiniteDifferenceInterpolator(grid)
    rng = np.random.default_rng(0)
    vp = rng.uniform(0, 1, size=(200, 3))
    interp.set_value_constraints(np.column_stack([vp, vp[:, 2] + 0.1 * np.sin(3 * vp[:, 0]), np.ones(200)]))
    interp.setup_interpolator(regularisation=0.1)
    interp.solve_system("cg", solver_kwargs={"rtol": 1e-12})
    surfs = interp.surfaces([0.3, 0.6, 50.0])
    assert len(surfs) == 2 and surfs[0].values[0] == 0.3
    for s, level in zip(surfs, (0.3, 0.6)):
        ref = iso.isosurface(interp.c, grid.nsteps, grid.origin, grid.step_vector, level)
        assert s.triangles.shape[0] == ref.shape[0]
        # the trilinear field at the vertices is close to the level (piecewise-linear vs trilinear: O(h^2))
        v = interp.evaluate_value(s.vertices)
        assert np.max(np.abs(v - level)) < 0.02
        assert abs(s.area - 1.0) < 0.2  # a near-horizontal layer across the unit box


def test_isosurfacer_on_a_callable():
    """LoopIsosurfacer (utils/_surface.py API) samples the callable on the box's
    regular grid and extracts each level with the GPU kernel."""
    from types import SimpleNamespace

    from loopstructural_gb300.surface import LoopIsosurfacer

    box = SimpleNamespace(origin=np.array([-1.0, -1.0, -1.0]), maximum=np.array([1.0, 1.0, 1.0]),
                          nsteps=np.array([21, 17, 19]))

    def fn(p):
        return np.sum(p * p, axis=1)

    surfs = LoopIsosurfacer(box, callable=fn).fit([0.25, 0.64, 9.0], name="shell")
    assert [s.name for s in surfs] == ["shell_0.25", "shell_0.64"]
    for s, level in zip(surfs, (0.25, 0.64)):
        grid = L.StructuredGrid(origin=box.origin, nsteps=box.nsteps - 1,
                                step_vector=(box.maximum - box.origin) / (box.nsteps - 1))
        ref = iso.isosurface(fn(grid.nodes), grid.nsteps, grid.origin, grid.step_vector, level)
        assert s.triangles.shape[0] == ref.shape[0]
        r = np.linalg.norm(s.vertices, axis=1)
        assert np.max(np.abs(r - np.sqrt(level))) < 0.05
        assert np.all(s.values == level)
