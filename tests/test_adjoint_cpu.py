"""The adjoint formula used by loopstructural_gb300.adjoint, checked on the
oracle (CPU, dense FP64): dL/dv from one adjoint solve equals central finite
differences of the loss through the full reference assembly + solve.
Tolerance: 1e-6 relative (the FD check bar for gradients)."""
import numpy as np

from loopstructural_gb300.adjoint import _trilinear_norm2
from oracle import fd_oracle as fdo


class _Support:
    def __init__(self, cells):
        self.origin = np.zeros(3)
        self.nsteps_cells = np.asarray(cells)
        self.step_vector = 1.0 / np.asarray(cells, dtype=float)


def _setup(seed=0):
    cells = np.array([6, 5, 7])
    rng = np.random.default_rng(seed)
    vp = rng.uniform(0, 1, size=(40, 3))
    vals = np.column_stack([vp, np.sin(3 * vp[:, 0]) + vp[:, 2], rng.uniform(0.5, 2.0, 40)])
    npnt = rng.uniform(0, 1, size=(8, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(8, 3)), np.ones(8)])
    q = rng.uniform(0, 1, size=(60, 3))
    target = q[:, 2]
    return cells, vals, nrm, q, target


def _loss_and_field(cells, vals, nrm, q, target, weights):
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    A, b = fdo.assemble(grid, {"value": vals, "normal": nrm}, weights).matrix()
    c = fdo.solve_direct(A, b)
    u = fdo.evaluate_value_local(grid, q, c)
    return np.mean((u - target) ** 2), u, grid, A


def test_value_gradient_formula_matches_finite_differences():
    cells, vals, nrm, q, target = _setup()
    weights = fdo.resolve_weights(regularisation=0.1, cpw=1.3, npw=1.0)
    L0, u, grid, A = _loss_and_field(cells, vals, nrm, q, target, weights)
    N, _ = fdo.normal_equations(A, np.zeros(A.shape[0]))
    # adjoint: lambda = N^-1 E_q^T dL/du ; dL/dv = w^2/|t|^2 * E_v lambda
    Eq = np.stack([fdo.evaluate_value_local(grid, q, e) for e in np.eye(grid.n_nodes)], axis=1)
    Ev = np.stack([fdo.evaluate_value_local(grid, vals[:, :3], e) for e in np.eye(grid.n_nodes)], axis=1)
    lam = np.linalg.solve(N.toarray(), Eq.T @ (2.0 / q.shape[0] * (u - target)))
    w = weights["cpw"] * vals[:, 4]
    grad = w * w / _trilinear_norm2(_Support(cells), vals) * (Ev @ lam)
    h = 1e-6
    for i in range(0, vals.shape[0], 3):
        vp, vm = vals.copy(), vals.copy()
        vp[i, 3] += h
        vm[i, 3] -= h
        fd = (_loss_and_field(cells, vp, nrm, q, target, weights)[0] -
              _loss_and_field(cells, vm, nrm, q, target, weights)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 * max(1e-3, np.max(np.abs(grad))), (i, fd, grad[i])
