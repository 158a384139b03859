"""Batched ensemble solves: every model's solution equals its own single
solve (same handle code path, concurrent streams) -- bit-identical for the
deterministic mixed/FP64 solvers -- and matches the oracle's direct solve."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300.ensemble import FdEnsemble  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu


def _models(k, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for m in range(k):
        n = int(rng.choice([6, 9, 12, 26]))
        cells = np.array([n, n + 1, n - 1])
        s = rng.uniform(0.5, 2.0)
        nv, nn = int(rng.integers(30, 200)), int(rng.integers(5, 40))
        vp = rng.uniform(0, 1, size=(nv, 3))
        val = np.column_stack([vp, vp[:, 2] / s + 0.1 * np.sin(6 * vp[:, 0]), np.ones(nv)])
        npnt = rng.uniform(0, 1, size=(nn, 3))
        g = np.tile([0.0, 0.0, 1.0 / s], (nn, 1)) + rng.normal(0, 0.05, size=(nn, 3))
        nrm = np.column_stack([npnt, g, np.ones(nn)])
        grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells)
        out.append({"grid": grid, "cells": cells, "value": val, "normal": nrm,
                    "setup": {"regularisation": 0.1, "cpw": 1.0, "npw": 1.0}})
    return out


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batched_solves_equal_single_solves(precision):
    models = _models(10)
    ens = FdEnsemble(models)
    kw = {"rtol": 1e-12, "atol": 0.0, "precision": precision, "maxiter": 200000}
    stats = ens.solve(concurrency=4, solver_kwargs=kw)
    assert all(st["status"] == 0 for st in stats)
    batched = [it.c.copy() for it in ens.interpolators]
    for it, cb in zip(ens.interpolators, batched):
        assert it.solve_system("cg", solver_kwargs=dict(kw))
        np.testing.assert_array_equal(it.c, cb)
    ens.close()


def test_batched_solutions_match_direct_solves():
    models = _models(6, seed=1)
    ens = FdEnsemble(models)
    ens.solve(concurrency=6, solver_kwargs={"rtol": 1e-13, "atol": 0.0, "precision": "mixed", "maxiter": 200000})
    for m, it in zip(models, ens.interpolators):
        grid = fdo.Grid(np.zeros(3), m["cells"], 1.0 / m["cells"])
        cs = fdo.assemble(grid, {"value": m["value"], "normal": m["normal"]}, fdo.resolve_weights(**m["setup"]))
        A, b = cs.matrix()
        ref = fdo.solve_direct(A, b)
        assert np.linalg.norm(it.c - ref) <= 1e-8 * np.linalg.norm(ref)
    ens.close()


def test_empty_and_single_model_ensembles():
    assert FdEnsemble([]).solve() == []
    ens = FdEnsemble(_models(1, seed=2))
    (st,) = ens.solve(concurrency=16, solver_kwargs={"rtol": 1e-10})
    assert st["status"] == 0
    ens.close()
