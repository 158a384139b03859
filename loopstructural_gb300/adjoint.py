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


class ConstraintAdjoint:
    """u(theta) = E_q c(theta): the field at `query` points as a differentiable
    function of an FD interpolator's data -- the value constraints' values
    and positions, the normal constraints' vectors and positions -- and of the
    isotropic regularisation weight.

        f = ConstraintAdjoint(grid, query, value_weights, normal_weights, cpw=1.0, npw=1.0)
        u = f(values, value_points, normals, normal_points, reg)   # FP64 CUDA tensors
        loss(u).backward()                                        # .grad on every input

    Each forward call assembles the rows (ls_fd_point_rows) and solves the
    normal equations N c = A^T W b; backward runs one adjoint solve
    N lam = E_q^T dL/du with the same handle and then, per data row r with
    a = row coefficients, b = target, w = weight (rows normalised as the
    reference does, DI:361-366):

        dL/db_r = w^2 (lam . a),   dL/da_r = w^2 ((b - a.c) lam - (lam . a) c),

    chained through a = t/|t|, b = v/|t| (value rows, t the trilinear weights)
    and a = T_d/|T_d|, b = n_d/|T_d| (normal rows, T_d the shape-function
    derivatives along axis d), using the jets (value, gradient, mixed second
    derivatives) of c and lam at the points (ls_fd_eval_jets).  The
    regularisation weight scales every interior family's row weight, so
    dL/dreg = -(2/reg) lam^T N_int c with N_int the interior regularisation
    operator (a second handle without data rows, borders or ridge).
    Positions move rows inside their cell; a point crossing a cell face changes
    the row's columns, where the field is continuous but its derivative is not.
    The reference has no gradient path; iterates are not stored (the backward
    solve recomputes what it needs)."""

    def __init__(self, support, query, value_weights, normal_weights, cpw=1.0, npw=1.0, precision="fp64",
                 rtol=1e-13, maxiter=None):
        import torch

        self.support = support
        self.dev = _lib.device()
        self.qpts = torch.as_tensor(np.ascontiguousarray(np.asarray(query, dtype=float)[:, :3])).to(self.dev)
        self.value_w = np.asarray(value_weights, dtype=float)
        self.normal_w = np.asarray(normal_weights, dtype=float)
        self.cpw, self.npw = float(cpw), float(npw)
        self.precision, self.rtol, self.maxiter = precision, rtol, maxiter
        self.step = torch.as_tensor(np.asarray(support.step_vector, dtype=float)).to(self.dev)
        self.last_stats = {}

    # -- device helpers ---------------------------------------------------------
    def _jets(self, pts, c):
        import torch

        out = torch.empty((pts.shape[0], 11), dtype=torch.float64, device=self.dev)
        if pts.shape[0]:
            grid = self.support.grid3()
            _lib.check(_lib.load().ls_fd_eval_jets(C.byref(grid), _lib.ptr(c.contiguous()), _lib.ptr(pts.contiguous()),
                                                   pts.shape[0], 3, _lib.ptr(out), _lib.stream_ptr()))
        return out

    def _spread(self, pts, g):
        import torch

        out = torch.zeros(self.support.n_nodes, dtype=torch.float64, device=self.dev)
        grid = self.support.grid3()
        _lib.check(_lib.load().ls_fd_eval_adjoint(C.byref(grid), _lib.ptr(pts), pts.shape[0], 3,
                                                  _lib.ptr(g.contiguous()), None, _lib.ptr(out), _lib.stream_ptr()))
        return out

    def _interp(self, values, vpts, normals, npts, reg):
        from .interpolators import FiniteDifferenceInterpolator

        it = FiniteDifferenceInterpolator(self.support)
        if values.shape[0]:
            it.set_value_constraints(np.column_stack([vpts, values, self.value_w]))
        if normals.shape[0]:
            it.set_normal_constraints(np.column_stack([npts, normals, self.normal_w]))
        it.setup_interpolator(regularisation=reg, cpw=self.cpw, npw=self.npw)
        return it

    def solve(self, values, vpts, normals, npts, reg):
        """(c, u, system) for the given data (host or device tensors; no autograd)."""
        cpu = [np.asarray(t.detach().cpu().numpy() if hasattr(t, "detach") else t, dtype=float)
               for t in (values, vpts, normals, npts)]
        it = self._interp(*cpu, float(reg))
        system = it._build_system()
        c, st = system.solve(atol=0.0, rtol=self.rtol, precision=self.precision, maxiter=self.maxiter)
        self.last_stats["forward"] = st
        u = self._jets(self.qpts, c)[:, 0]
        return c, u, system, it

    # -- gradients ---------------------------------------------------------------
    def gradients(self, system, interp, c, grad_u, values, vpts, normals, npts, reg):
        """dL/d(values, value points, normals, normal points, reg) for
        dL/du = grad_u, at the solution c of `system`."""
        import torch

        _lib.check(_lib.load().ls_fd_set_rhs(system.handle, _lib.ptr(self._spread(self.qpts, grad_u)),
                                             _lib.stream_ptr()))
        lam, st = system.solve(atol=0.0, rtol=self.rtol, precision=self.precision, maxiter=self.maxiter)
        self.last_stats["adjoint"] = st
        h = self.step

        def axis_terms(J):
            loc = J[:, 7:10]
            s = loc * loc + (1.0 - loc) ** 2            # per-axis |weights|^2
            ds = 2.0 * (2.0 * loc - 1.0) / h            # d s / d p (per axis)
            return s, ds

        # value rows ------------------------------------------------------------
        v = values.to(torch.float64)
        gv = torch.zeros_like(v)
        gvp = torch.zeros((v.shape[0], 3), dtype=torch.float64, device=self.dev)
        if v.shape[0]:
            Jc, Jl = self._jets(vpts, c), self._jets(vpts, lam)
            inside = Jc[:, 10] > 0
            s, ds = axis_terms(Jc)
            n2 = s.prod(dim=1)
            w2 = (self.cpw * torch.as_tensor(self.value_w, device=self.dev)) ** 2
            U, gU, L0, gL = Jc[:, 0], Jc[:, 1:4], Jl[:, 0], Jl[:, 1:4]
            safe = torch.where(inside, n2, torch.ones_like(n2))
            f = torch.where(inside, w2 / safe, torch.zeros_like(n2))
            gv = f * L0
            res = v - U
            gn_over_n = 0.5 * ds / s                   # (d|t|/dp) / |t|
            gvp = f[:, None] * (res[:, None] * gL - L0[:, None] * gU - 2.0 * (res * L0)[:, None] * gn_over_n)
        # normal rows -----------------------------------------------------------
        nv = normals.to(torch.float64)
        gn = torch.zeros_like(nv)
        gnp = torch.zeros((nv.shape[0], 3), dtype=torch.float64, device=self.dev)
        if nv.shape[0]:
            Jc, Jl = self._jets(npts, c), self._jets(npts, lam)
            inside = Jc[:, 10] > 0
            s, ds = axis_terms(Jc)
            w2 = (self.npw / 3.0 * torch.as_tensor(self.normal_w, device=self.dev)) ** 2
            # mixed second derivatives, symmetric: index (d, e) -> column
            mix = {(0, 1): 4, (1, 0): 4, (0, 2): 5, (2, 0): 5, (1, 2): 6, (2, 1): 6}
            for d in range(3):
                others = [e for e in range(3) if e != d]
                m2 = 2.0 * s[:, others[0]] * s[:, others[1]] / (h[d] * h[d])   # |T_d|^2
                safe = torch.where(inside, m2, torch.ones_like(m2))
                f = torch.where(inside, w2 / safe, torch.zeros_like(m2))
                dU, dL = Jc[:, 1 + d], Jl[:, 1 + d]
                gn[:, d] = f * dL
                res = nv[:, d] - dU
                for e in others:
                    gm_over_m = 0.5 * ds[:, e] / s[:, e]  # (d|T_d|/dp_e) / |T_d|
                    gnp[:, e] += f * (res * Jl[:, mix[(d, e)]] - dL * Jc[:, mix[(d, e)]] - 2.0 * res * dL * gm_over_m)
        # regularisation weight ------------------------------------------------------
        greg = torch.zeros((), dtype=torch.float64, device=self.dev)
        if reg != 0.0:
            from .fd import FdSystem

            wint = {k: float(val) for k, val in interp._reg_weights().items()}
            for k in ("dx", "dy", "dz"):
                wint[k] = 0.0
            interior = FdSystem(self.support, wint, [], 0.0)
            try:
                greg = -(2.0 / float(reg)) * torch.dot(lam, interior.apply(c))
            finally:
                interior.close()
        return gv, gvp, gn, gnp, greg

    def __call__(self, values, value_points, normals, normal_points, reg):
        import torch

        outer = self

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, v, vp, n, np_, r):
                c, u, system, it = outer.solve(v, vp, n, np_, float(r))
                ctx.saved = (c, system, it, v.detach().to(torch.float64), vp.detach().to(torch.float64).contiguous(),
                             n.detach().to(torch.float64), np_.detach().to(torch.float64).contiguous(), float(r))
                return u

            @staticmethod
            def backward(ctx, grad_u):
                c, system, it, v, vp, n, np_, r = ctx.saved
                try:
                    gv, gvp, gn, gnp, greg = outer.gradients(system, it, c, grad_u.detach().to(torch.float64).contiguous(),
                                                             v, vp, n, np_, r)
                finally:
                    system.close()
                return gv, gvp, gn, gnp, greg

        return _Fn.apply(values, value_points, normals, normal_points, torch.as_tensor(reg, dtype=torch.float64,
                                                                                       device=self.dev))
