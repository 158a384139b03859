"""Ensembles of independent FD models solved together on one GPU.

Each model is an ordinary FiniteDifferenceInterpolator (its own grid, data
and weights); the solves of all models run concurrently, `concurrency` of them
in flight at a time, each on its own CUDA stream (ls_fd_solve_batched).  The
reference builds and solves such ensembles one model after another through
the same interpolator API; results here are those of the individual solves.
"""
from __future__ import annotations

from time import perf_counter

import numpy as np

from . import _lib, fd
from .interpolators import FiniteDifferenceInterpolator


class FdEnsemble:
    """models: iterable of dicts with keys ``grid`` (StructuredGrid), optional
    ``value`` / ``normal`` / ``gradient`` / ``tangent`` / ``interface``
    constraint arrays and ``setup`` (setup_interpolator keyword arguments)."""

    SETTERS = {"value": "set_value_constraints", "normal": "set_normal_constraints",
               "gradient": "set_gradient_constraints", "tangent": "set_tangent_constraints",
               "interface": "set_interface_constraints"}

    def __init__(self, models):
        self.interpolators = []
        t0 = perf_counter()
        for m in models:
            interp = FiniteDifferenceInterpolator(m["grid"])
            for key, setter in self.SETTERS.items():
                arr = m.get(key)
                if arr is not None and len(arr) > 0:
                    getattr(interp, setter)(np.asarray(arr, dtype=float))
            interp.setup_interpolator(**m.get("setup", {}))
            self.interpolators.append(interp)
        self.setup_seconds = perf_counter() - t0
        self.stats = []

    def __len__(self):
        return len(self.interpolators)

    def solve(self, concurrency=8, solver_kwargs=None):
        """Solves every model; returns the per-model solver statistics."""
        import torch

        kw = dict(solver_kwargs or {})
        opts = dict(atol=float(kw.pop("atol", 0.0)), rtol=float(kw.pop("rtol", 1e-5)), maxiter=kw.pop("maxiter", None),
                    precision=kw.pop("precision", "mixed"), preconditioner=kw.pop("preconditioner", "mg"),
                    reliable_delta=float(kw.pop("reliable_delta", 0.1)), check_every=int(kw.pop("check_every", 64)))
        if kw:
            raise TypeError(f"unknown solver options {sorted(kw)}")
        systems = []
        for interp in self.interpolators:
            interp._release_system()
            interp._system = interp._build_system()
            systems.append(interp._system)
        torch.cuda.synchronize()
        results = fd.solve_batched(systems, concurrency=concurrency, **opts)
        self.stats = []
        for interp, (x, st) in zip(self.interpolators, results):
            interp._c_dev = x
            interp._c = x.cpu().numpy()
            interp.up_to_date = True
            interp.latest_solve_timing = {"solver": "cg", "backend": "gb300", "iterations": int(st["iterations"]),
                                          "device_ms": st["device_ms"], "status": int(st["status"]),
                                          "preconditioner": st["preconditioner"], "batched": True}
            if st["status"] != _lib.LS_OK:
                interp.latest_solve_timing["warning"] = "solver status %d" % st["status"]
            self.stats.append(st)
        return self.stats

    def evaluate_value(self, i, locations):
        return self.interpolators[i].evaluate_value(locations)

    def evaluate_gradient(self, i, locations):
        return self.interpolators[i].evaluate_gradient(locations)

    def close(self):
        for interp in self.interpolators:
            interp._release_system()
