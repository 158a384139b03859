"""Inequality-constrained solve (``solve_system('admm')``) on the GPU.

Reference: packages/loop_interpolation/src/loop_interpolation/
  loopsolver/admm_solver.py  admm_solve :59-463 (the major iteration :375-463)
  loopsolver/admm_method.py  ADMM.admm_method_iterate_admm_array :12-25
  _solver_strategy.py        extract_admm_kwargs :139-177, solve_with_admm :180-217
  _discrete_interpolator.py  _solve_with_admm :1171-1219

The reference solves, in the column-scaled variable y (c = S y, S = diag of
the reciprocal column norms of [A; ridge I]),

    y_{k+1} = argmin |A S y - b|^2 + rho^2 |Q y - (z_k - u_k)|^2

once per major iteration (as an increment dx from y_k, with an inner
least-squares solver), with z the projection of Q y + u onto the bounds and u
the scaled dual.  In the node values c that is

    (N + rho^2 Q'^T Q') c = A^T W b + rho^2 Q'^T (z - u),   Q' = Q S^-1,

so the inequality rows become extra data rows (coefficients Q', weight rho)
of one matrix-free operator: the projection and the new right-hand side are
one kernel pass (ls_fd_admm_step), the solve is the multigrid-preconditioned
CG warm-started from the previous c.  The inner solves are run to a tight
relative tolerance, so the iterates follow the reference's with an exact
inner solver.

Supported: constant rho (``admm_weight``), rho schedules
(``admm_weight_final``, linear or geometric), adaptive rho, the primal/dual
stopping test, ``model_update_tol``, ``min_iterations``, ``x0``,
``return_history``.  The active-set variant and the constant-norm polish
raise NotImplementedError.

Two properties of the reference kept here: the bounds constrain Q y (the
scaled variable), not Q c; and a rho changed by the adaptive rule is set back
to the schedule's value at the start of the next major iteration (u is
rescaled there and back), so the handle is only rebuilt for a step that runs
at a new rho.
"""
from __future__ import annotations

import logging
import math

import numpy as np

from . import _lib

logger = logging.getLogger(__name__)

# options the reference reads for its inner least-squares solver; the GPU
# inner solve is the CG of the handle, so they carry no meaning here
_INNER_SOLVER_ONLY = ("linsys_solver", "reuse_inner_solve", "cg_preconditioner", "cg_preconditioner_shift",
                      "matrix_free", "inner_rtol_start", "inner_rtol_end", "inner_atol_start", "inner_atol_end",
                      "inner_maxiter_start", "inner_maxiter_end", "batch_size", "batch_fraction", "random_seed",
                      "btol", "show", "conlim", "damp", "iter_lim", "M", "callback")


def admm_options(solver_kwargs: dict | None):
    """Splits the solver kwargs into the ADMM options (the reference's names
    and defaults, SS:139-217 and admm_solve's signature) and the options of
    the inner GPU solve; raises as the reference does on bad values."""
    kw = dict(solver_kwargs or {})
    kw.pop("backend", None)
    iterations = max(0, int(kw.pop("constant_norm_iterations", 0)))
    weight = float(kw.pop("constant_norm_weight", 0.0))
    kw.pop("constant_norm_target", None)
    if iterations > 0 and weight > 0.0:
        raise NotImplementedError("the constant-norm polish after ADMM is not part of the GPU path")
    if bool(kw.pop("active_set", False)):
        raise NotImplementedError("the active-set ADMM variant is not part of the GPU path")
    for k in ("active_set_padding", "active_set_min_size", "active_set_max_size", "active_set_hysteresis",
              "active_set_refresh_interval"):
        kw.pop(k, None)
    o = {
        "rho": float(kw.pop("admm_weight", 0.01)),
        "nmajor": int(kw.pop("nmajor", 200)),
        "rho_final": kw.pop("admm_weight_final", None),
        "schedule": kw.pop("admm_weight_schedule", "geometric"),
        "adaptive": bool(kw.pop("adaptive_rho", False)),
        "mu": float(kw.pop("adaptive_rho_mu", 10.0)),
        "tau": float(kw.pop("adaptive_rho_tau", 2.0)),
        "rho_min": float(kw.pop("adaptive_rho_min", 1e-4)),
        "rho_max": float(kw.pop("adaptive_rho_max", 1e3)),
        "abs_tol": float(kw.pop("admm_abs_tol", 1e-4)),
        "rel_tol": float(kw.pop("admm_rel_tol", 1e-3)),
        "model_update_tol": float(kw.pop("model_update_tol", 0.0)),
        "min_iterations": int(kw.pop("min_iterations", 5)),
        "return_history": bool(kw.pop("return_history", False)),
        "x0": kw.pop("x0", None),
    }
    inner_schedule = kw.pop("inner_maxiter_schedule", "linear")
    if o["nmajor"] <= 0:
        raise ValueError("nmajor must be positive")
    if o["model_update_tol"] < 0:
        raise ValueError("model_update_tol must be >= 0")
    if inner_schedule not in ("linear", "geometric"):
        raise ValueError("inner_maxiter_schedule must be 'linear' or 'geometric'")
    if o["rho_final"] is not None:
        if o["rho_final"] <= 0:
            raise ValueError("admm_weight_final must be > 0")
        if o["rho"] <= 0:
            raise ValueError("admm_weight must be > 0")
    for k in _INNER_SOLVER_ONLY:
        if k in kw:
            logger.info("ADMM option %s ignored: the inner solve is the GPU CG", k)
            kw.pop(k)
    inner = {
        "rtol": float(kw.pop("rtol", 1e-10)),
        "atol": float(kw.pop("atol", 0.0)),
        "maxiter": kw.pop("maxiter", None),
        "precision": kw.pop("precision", "mixed"),
        "preconditioner": kw.pop("preconditioner", "mg"),
    }
    for k in kw:
        logger.info("solver kwarg %s ignored by the GPU ADMM", k)
    return o, inner


def rho_schedule(o) -> np.ndarray:
    """rho of every major iteration (admm_solve :139-148)."""
    n = o["nmajor"]
    if o["rho_final"] is None:
        return np.full(n, o["rho"], dtype=float)
    if o["schedule"] == "linear":
        return np.linspace(o["rho"], float(o["rho_final"]), n)
    return np.geomspace(o["rho"], float(o["rho_final"]), n)


class InequalityRows:
    """The inequality rows of one solve, concatenated on the device: column
    indices (m x k, -1 padding), raw coefficients Q, and bounds."""

    def __init__(self, families):
        import torch

        width = max(int(f.idc.shape[1]) for f in families)
        idc, a, lo, hi = [], [], [], []
        for f in families:
            k = int(f.idc.shape[1])
            fi, fa = f.idc, f.a
            if k < width:
                fi = torch.cat([fi, torch.full((fi.shape[0], width - k), -1, dtype=fi.dtype, device=fi.device)], 1)
                fa = torch.cat([fa, torch.zeros((fa.shape[0], width - k), dtype=fa.dtype, device=fa.device)], 1)
            idc.append(fi)
            a.append(fa)
            lo.append(f.bounds[:, 0])
            hi.append(f.bounds[:, 1])
        self.idc = torch.cat(idc).contiguous()
        self.a = torch.cat(a).contiguous()
        self.lo = torch.cat(lo).contiguous()
        self.hi = torch.cat(hi).contiguous()
        self.m = int(self.idc.shape[0])

    def scaled(self, d):
        """Q' = Q diag(d): the rows acting on node values when Q acts on the
        column-scaled variable."""
        import torch

        valid = self.idc >= 0
        dd = torch.where(valid, d[self.idc.clamp(min=0)], torch.zeros_like(self.a))
        return (self.a * dd).contiguous()


def solve_admm(interp, o, inner, timing) -> bool:
    """Runs the ADMM major iterations for ``interp`` (an FD interpolator with
    its constraint families and inequality families set up); stores c and
    returns True, or logs the reference's error and returns False when there
    is no inequality row."""
    import torch

    families = [f for f in interp.ineq_constraints.values() if f.rows > 0]
    if not families:
        # the reference's ADMM(0) raises ValueError, which _solve_with_admm logs
        logger.error("ADMM solver failed: nelements must be greater than 0")
        return False
    ineq = InequalityRows(families)
    dev = _lib.device()
    base_rows = interp._data_rows()
    base = interp._make_system(base_rows)
    try:
        if interp.apply_scaling_matrix:
            d = torch.sqrt(base.diagonal())
            d = torch.where(d > 0, d, torch.ones_like(d))
        else:
            d = torch.ones(interp.dof, dtype=torch.float64, device=dev)
    finally:
        base.close()
    qa = ineq.scaled(d)
    row0 = sum(int(r[0].shape[0]) for r in base_rows)
    zero_b = torch.zeros(ineq.m, dtype=torch.float64, device=dev)

    def build(rho):
        w = torch.full((ineq.m,), float(rho), dtype=torch.float64, device=dev)
        return interp._make_system(base_rows + [(ineq.idc, qa, zero_b, w)])

    x0 = o["x0"]
    if callable(x0):
        x0 = x0(interp.support)
    if x0 is not None:
        y0 = torch.as_tensor(np.asarray(x0, dtype=float).reshape(-1)).to(dev)
        if y0.shape[0] != interp.dof:
            logger.error("ADMM solver failed: Number of columns in interpolation matrix does not match x0")
            return False
        c = (y0 / d).contiguous()
    else:
        c = torch.zeros(interp.dof, dtype=torch.float64, device=dev)
    z = torch.zeros(ineq.m, dtype=torch.float64, device=dev)
    u = torch.zeros(ineq.m, dtype=torch.float64, device=dev)
    sched = rho_schedule(o)
    adaptive = o["adaptive"] and o["rho_final"] is None
    rho = float(sched[0])
    system = build(rho)
    built = rho  # the handle is rebuilt only when a step runs at another rho
    history = []
    inner_iterations = 0
    builds = 1
    sqrt_m = math.sqrt(ineq.m)
    try:
        for i in range(o["nmajor"]):
            target = float(sched[i])
            if target != rho:
                if rho > 0:
                    u.mul_(rho / target)
                rho = target
            if rho != built:
                system.close()
                system = build(rho)
                built = rho
                builds += 1
            sums = system.admm_step(row0, ineq.lo, ineq.hi, z, u, c)
            c_prev = c
            c, stats = system.solve(x=c, **inner)
            inner_iterations += int(stats["iterations"])
            if stats["status"] == _lib.LS_NOT_CONVERGED:
                logger.warning("ADMM inner solve %d reached its iteration limit", i)
            elif stats["status"] in (_lib.LS_NAN, _lib.LS_BREAKDOWN):
                logger.warning("ADMM inner solve %d stopped early (status %d)", i, int(stats["status"]))
            primal = math.sqrt(sums[0])
            dual = rho * math.sqrt(sums[1])
            qx_norm, z_norm, u_norm = math.sqrt(sums[2]), math.sqrt(sums[3]), rho * math.sqrt(sums[4])
            eps_pri = sqrt_m * o["abs_tol"] + o["rel_tol"] * max(qx_norm, z_norm)
            eps_dual = sqrt_m * o["abs_tol"] + o["rel_tol"] * u_norm
            history.append({"iteration": i + 1, "primal_norm": primal, "dual_norm": dual, "eps_pri": eps_pri,
                            "eps_dual": eps_dual, "rho": rho, "active_count": ineq.m,
                            "inner_iterations": int(stats["iterations"])})
            if i + 1 >= o["min_iterations"] and primal <= eps_pri and dual <= eps_dual:
                break
            if o["model_update_tol"] > 0.0 and i + 1 >= o["min_iterations"]:
                dx_norm = float(torch.linalg.vector_norm(d * (c - c_prev)))
                model_norm = float(torch.linalg.vector_norm(d * c_prev))
                if dx_norm <= o["model_update_tol"] * max(model_norm, 1.0):
                    history[-1].update({"stopped_on_model_update": True, "dx_norm": dx_norm,
                                        "model_norm": model_norm})
                    break
            if adaptive and i + 1 >= o["min_iterations"]:
                new = rho
                if primal > o["mu"] * dual:
                    new = min(rho * o["tau"], o["rho_max"])
                elif dual > o["mu"] * primal:
                    new = max(rho / o["tau"], o["rho_min"])
                if new != rho:
                    # as in the reference, the schedule sets rho back at the
                    # start of the next major iteration (constant schedule)
                    if rho > 0:
                        u.mul_(rho / new)
                    rho = float(new)
    finally:
        system.close()
    interp._c_dev = c
    from . import fd

    interp._c = fd.to_host(c)
    interp.solver_history = history if o["return_history"] else None
    timing.update({"admm_iterations": len(history), "inner_iterations": inner_iterations, "rho": rho,
                   "inequality_rows": ineq.m, "system_builds": builds, "precision": inner["precision"],
                   "preconditioner": inner["preconditioner"]})
    return True
