"""Gradients through the FD solve (hand-written adjoint).

The field evaluated at query points q is u = E_q c with c the solution of the
normal equations N c = A^T W b (N = A^T W A + ridge^2 I, symmetric).  The value
constraints enter only the right-hand side: a value row of point i has
a_i = t_i / |t_i| and b_i = v_i / |t_i| (t_i the 8 trilinear weights, rows
normalised as the reference does, DI:316-389) and weight w_i = cpw * weight_i,
so their share of A^T W b is E_v^T (w^2 v / |t|^2).  Hence, for a loss L(u),

    dL/dv = (w^2 / |t|^2) * (E_v lambda),   N lambda = E_q^T dL/du,

one extra solve with the same operator (the adjoint solve) and two evaluation
kernels.  The reference has no gradient path; this is the GPU-side addition
that lets a model's field be fitted to data by gradient descent.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _trilinear_norm2(support, pts: np.ndarray) -> np.ndarray:
    """|t|^2 of the trilinear weights at each point (0 outside the support)."""
    origin = np.asarray(support.origin, dtype=float)
    step = np.asarray(support.step_vector, dtype=float)
    cells = np.asarray(support.nsteps_cells, dtype=int)
    x = (pts[:, :3] - origin) / step
    k = np.clip(np.floor(x), 0, cells - 1)
    loc = np.clip(x - k, 0.0, 1.0)
    s = np.ones(pts.shape[0])
    for d in range(3):
        s *= loc[:, d] ** 2 + (1.0 - loc[:, d]) ** 2
    extent = np.maximum(np.abs(cells * step), 1.0)
    tol = np.finfo(float).eps * 32.0 * extent
    inside = np.all((pts[:, :3] >= origin - tol) & (pts[:, :3] <= origin + cells * step + tol), axis=1)
    return np.where(inside, s, 0.0)


class ValueFieldAdjoint:
    """u(v): the field at `query` as a differentiable function of the value
    constraints' values v (the 4th column of the value array) of a set-up
    FiniteDifferenceInterpolator; every other constraint stays fixed.

        f = ValueFieldAdjoint(interp, query)
        v = torch.tensor(values, device="cuda", requires_grad=True)
        loss = ((f(v) - target) ** 2).mean(); loss.backward()   # v.grad
    """

    def __init__(self, interp, query: np.ndarray, precision: str = "mixed", rtol: float = 1e-12,
                 maxiter: int | None = None):
        import torch

        self.interp = interp
        self.support = interp.support
        self.system = interp._build_system()
        self.precision, self.rtol, self.maxiter = precision, rtol, maxiter
        dev = _lib.device()
        vals = np.asarray(interp.get_value_constraints(), dtype=float)
        self.n_values = vals.shape[0]
        w = interp.interpolation_weights["cpw"] * vals[:, 4]
        n2 = _trilinear_norm2(self.support, vals)
        scale = np.where(n2 > 0, w * w / np.where(n2 > 0, n2, 1.0), 0.0)
        self.vpts = torch.from_numpy(np.ascontiguousarray(vals[:, :3])).to(dev)
        self.scale = torch.from_numpy(scale).to(dev)
        self.qpts = torch.from_numpy(np.ascontiguousarray(np.asarray(query, dtype=float)[:, :3])).to(dev)
        v0 = torch.from_numpy(vals[:, 3].copy()).to(dev)
        # the right-hand side without the value rows' share
        self.rhs_fixed = self.system.rhs() - self._spread(self.vpts, self.scale * v0)
        self.last_stats = {}

    # E^T g for points pts (device): node vector
    def _spread(self, pts, g):
        import torch

        out = torch.zeros(self.system.n, dtype=torch.float64, device=pts.device)
        grid = self.support.grid3()
        _lib.check(_lib.load().ls_fd_eval_adjoint(C.byref(grid), _lib.ptr(pts), pts.shape[0], 3,
                                                  _lib.ptr(g.contiguous()), None, _lib.ptr(out), _lib.stream_ptr()))
        return out

    # E c at points pts (device); 0 outside the support
    def _gather(self, pts, c):
        import torch

        v = torch.empty(pts.shape[0], dtype=torch.float64, device=pts.device)
        grid = self.support.grid3()
        _lib.check(_lib.load().ls_fd_eval_points(C.byref(grid), _lib.ptr(c.contiguous()), _lib.ptr(pts),
                                                 pts.shape[0], 3, _lib.ptr(v), None, _lib.stream_ptr()))
        return torch.nan_to_num(v, nan=0.0)

    def _solve(self, rhs, key):
        _lib.check(_lib.load().ls_fd_set_rhs(self.system.handle, _lib.ptr(rhs.contiguous()), _lib.stream_ptr()))
        x, st = self.system.solve(atol=0.0, rtol=self.rtol, precision=self.precision, maxiter=self.maxiter)
        self.last_stats[key] = st
        return x

    def solve_field(self, v):
        """(c, u) for values v (device FP64 tensor, no autograd)."""
        c = self._solve(self.rhs_fixed + self._spread(self.vpts, self.scale * v), "forward")
        return c, self._gather(self.qpts, c)

    def value_gradient(self, grad_u):
        """dL/dv for dL/du = grad_u (device FP64 tensor)."""
        lam = self._solve(self._spread(self.qpts, grad_u), "adjoint")
        return self.scale * self._gather(self.vpts, lam)

    def __call__(self, v):
        import torch

        outer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, values):
                _c, u = outer.solve_field(values.detach().to(torch.float64))
                return u

            @staticmethod
            def backward(ctx, grad_u):
                return outer.value_gradient(grad_u.detach().to(torch.float64).contiguous())

        return _Fn.apply(v)

    def close(self):
        self.system.close()
