"""GPU adjoint (value constraints -> field at query points) against the dense
FP64 oracle gradient and against central finite differences of GPU solves.
Tolerance: 1e-6 relative to max |gradient|."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300.adjoint import ValueFieldAdjoint, _trilinear_norm2  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu


def _case(cells, nv, nn, nq, seed=0):
    rng = np.random.default_rng(seed)
    vp = rng.uniform(0, 1, size=(nv, 3))
    vals = np.column_stack([vp, np.sin(3 * vp[:, 0]) + vp[:, 2], rng.uniform(0.5, 2.0, nv)])
    npnt = rng.uniform(0, 1, size=(nn, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(nn, 3)), np.ones(nn)])
    q = rng.uniform(0, 1, size=(nq, 3))
    return np.asarray(cells), vals, nrm, q, q[:, 2] + 0.05 * np.cos(4 * q[:, 1])


def _gpu(cells, vals, nrm, setup):
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(vals)
    interp.set_normal_constraints(nrm)
    interp.setup_interpolator(**setup)
    return interp


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_matches_dense_oracle_gradient(precision):
    cells, vals, nrm, q, target = _case((9, 8, 10), 120, 20, 200)
    setup = dict(regularisation=0.1, cpw=1.3, npw=1.0)
    f = ValueFieldAdjoint(_gpu(cells, vals, nrm, setup), q, precision=precision, rtol=1e-13)
    v = torch.tensor(vals[:, 3], device="cuda", dtype=torch.float64, requires_grad=True)
    t = torch.tensor(target, device="cuda", dtype=torch.float64)
    loss = ((f(v) - t) ** 2).mean()
    loss.backward()
    got = v.grad.cpu().numpy()
    # dense FP64 reference
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    weights = fdo.resolve_weights(**setup)
    A, b = fdo.assemble(grid, {"value": vals, "normal": nrm}, weights).matrix()
    N, rhs = fdo.normal_equations(A, b)
    c = np.linalg.solve(N.toarray(), rhs)
    Eq = np.stack([fdo.evaluate_value_local(grid, q, e) for e in np.eye(grid.n_nodes)], axis=1)
    Ev = np.stack([fdo.evaluate_value_local(grid, vals[:, :3], e) for e in np.eye(grid.n_nodes)], axis=1)
    u = Eq @ c
    np.testing.assert_allclose(float(loss), np.mean((u - target) ** 2), rtol=1e-8)
    lam = np.linalg.solve(N.toarray(), Eq.T @ (2.0 / q.shape[0] * (u - target)))
    w = weights["cpw"] * vals[:, 4]
    ref = w * w / _trilinear_norm2(grid_support(cells), vals) * (Ev @ lam)
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(np.abs(ref)), (np.max(np.abs(got - ref)), np.max(np.abs(ref)))
    f.close()


def grid_support(cells):
    return L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))


def test_adjoint_matches_central_differences_of_gpu_solves():
    """The loss is quadratic in v, so a central difference is exact for any h;
    h = 1e-3 keeps the solve tolerance far below the difference."""
    cells, vals, nrm, q, target = _case((24, 20, 26), 600, 120, 1000, seed=3)
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    f = ValueFieldAdjoint(_gpu(cells, vals, nrm, setup), q, precision="mixed", rtol=1e-13)
    t = torch.tensor(target, device="cuda", dtype=torch.float64)
    v0 = torch.tensor(vals[:, 3], device="cuda", dtype=torch.float64)
    v = v0.clone().requires_grad_(True)
    ((f(v) - t) ** 2).mean().backward()
    grad = v.grad.clone()
    rng = np.random.default_rng(7)
    h = 1e-3
    scale = float(grad.abs().max())
    for i in rng.choice(vals.shape[0], size=12, replace=False):
        e = torch.zeros_like(v0)
        e[i] = h
        lp = float(((f.solve_field(v0 + e)[1] - t) ** 2).mean())
        lm = float(((f.solve_field(v0 - e)[1] - t) ** 2).mean())
        fd = (lp - lm) / (2 * h)
        assert abs(fd - float(grad[i])) <= 1e-6 * scale + 1e-9, (i, fd, float(grad[i]))
    f.close()
