"""The TMA-staged finest-level FP32 apply (fd_apply_tma.cuh).

Grids whose x extent is a multiple of 4 (and every axis >= 8 nodes) run every
FP32 operator apply of the finest level through it: the outer CG product
(STORE), the multigrid smoother (CHEB) and residual (RESID) epilogues, with
and without directional terms.  Checked through the C ABI against the
oracle's explicit normal matrix (FP64, 2e-5 relative to max |N x| in FP32, as
the other FP32 operator tests), against the cp.async tile kernels on the same
system (LS_GB300_STAGED_APPLY=tiles at handle creation), through one V-cycle,
and by whole multigrid solves landing on the same solution."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu

KW = dict(dxx=1.0, dyy=0.8, dzz=1.3, dxy=0.5, dxz=0.4, dyz=0.6, dx=0.7, dy=0.9, dz=1.1)


def _data(rng, npts, nnrm):
    vp = rng.uniform(0, 1, size=(npts, 3))
    val = np.column_stack([vp, vp[:, 2] + 0.1 * np.sin(2 * np.pi * vp[:, 0]), np.ones(npts)])
    npnt = rng.uniform(0, 1, size=(nnrm, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(nnrm, 3)), np.ones(nnrm)])
    return val, nrm


def _interp(cells, val, nrm, setup, tiles=False, directional=None, step=None):
    cells = np.asarray(cells)
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
    it = L.FiniteDifferenceInterpolator(grid)
    it.set_value_constraints(val)
    it.set_normal_constraints(nrm)
    kw = dict(setup)
    if directional is not None:
        kw["regularisation"] = {"isotropic": kw.pop("regularisation", 0.1), "directional": directional}
    it.setup_interpolator(**kw)
    env = {"LS_GB300_STAGED_APPLY": "tiles" if tiles else None,
           "LS_GB300_TMA_STEP": None if step is None else str(step)}
    old = {k: os.environ.get(k) for k in env}
    try:
        for k, v in env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        system = it._build_system()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return it, system


@pytest.mark.parametrize("cells, step", [((71, 69, 65), 1), ((75, 68, 64), 2), ((71, 69, 62), 2)])
def test_staged_apply_matches_explicit_operator(cells, step):
    """x extent a multiple of 4 (72 / 76 nodes), y / z not multiples of the
    8-row tile; data rows near every face; one and two planes per step (an odd
    segment length for the two-plane variant)."""
    rng = np.random.default_rng(21)
    val, nrm = _data(rng, 3000, 600)
    setup = dict(cpw=1.0, npw=1.0, **KW)
    it, system = _interp(cells, val, nrm, setup, step=step)
    assert system.staged_apply and (cells[0] + 1) % 4 == 0
    grid = fdo.Grid(np.zeros(3), np.asarray(cells), 1.0 / np.asarray(cells, dtype=float))
    cs = fdo.assemble(grid, {"value": val, "normal": nrm}, fdo.resolve_weights(**setup))
    A, _ = cs.matrix()
    N, _ = fdo.normal_equations(A, np.zeros(A.shape[0]))
    for seed in (1, 2):
        x = np.random.default_rng(seed).normal(size=system.n)
        ref = N @ x
        got = system.apply(torch.from_numpy(x).float()).cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - ref)) <= 2e-5 * np.max(np.abs(ref)), seed
    system.close()


def test_staged_apply_matches_tile_kernels():
    """The same FP32 operator through the TMA kernel and through the cp.async
    deep-box + shell kernels: equal to FP32 rounding of the data totals."""
    cells = (79, 72, 70)
    rng = np.random.default_rng(22)
    val, nrm = _data(rng, 5000, 1000)
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    _, s_tma = _interp(cells, val, nrm, setup)
    _, s_tile = _interp(cells, val, nrm, setup, tiles=True)
    assert s_tma.staged_apply and not s_tile.staged_apply
    x = torch.from_numpy(np.random.default_rng(3).normal(size=s_tma.n)).float()
    a = s_tma.apply(x)
    b = s_tile.apply(x)
    torch.cuda.synchronize()
    scale = float(b.abs().max())
    assert float((a - b).abs().max()) <= 1e-6 * scale
    s_tma.close()
    s_tile.close()


@pytest.mark.parametrize("directional, step", [(False, 1), (True, 2), (False, 2)])
def test_multigrid_solve_with_staged_apply(directional, step):
    """Whole mixed multigrid solves (every level-0 epilogue through the TMA
    kernel) reach the same solution as with the tile kernels and as the FP64
    Jacobi solve, at 1e-8."""
    cells = (71, 67, 63)
    rng = np.random.default_rng(23)
    val, nrm = _data(rng, 4000, 800)
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    terms = None
    if directional:
        grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.asarray(cells),
                                step_vector=1.0 / np.asarray(cells, dtype=float))
        ang = 2.0 * np.pi * grid.nodes[:, 0]
        across = np.column_stack([np.cos(ang), np.zeros(len(ang)), np.sin(ang)])
        terms = [L.DirectionalRegularisation(0.05, across, "fold regularisation 1")]
    sols = {}
    for mode in ("tiles", "tma", "fp64"):
        it, system = _interp(cells, val, nrm, setup, tiles=(mode == "tiles"), directional=terms, step=step)
        assert system.staged_apply == (mode != "tiles")
        if mode == "fp64":
            x, st = system.solve(rtol=1e-12, precision="fp64", preconditioner="jacobi", maxiter=400000)
        else:
            x, st = system.solve(rtol=1e-11, precision="mixed", preconditioner="mg", maxiter=5000)
            assert st["preconditioner"] == "mg", st
        assert st["status"] == 0, (mode, st)
        sols[mode] = (x.cpu().numpy(), st["iterations"])
        system.close()
    ref = sols["fp64"][0]
    for mode in ("tma", "tiles"):
        err = np.linalg.norm(sols[mode][0] - ref) / np.linalg.norm(ref)
        assert err <= 1e-8, (mode, err)
    assert abs(sols["tma"][1] - sols["tiles"][1]) <= max(2, sols["tiles"][1] // 20), {k: v[1] for k, v in sols.items()}


@pytest.mark.parametrize("step", [1, 2])
def test_vcycle_with_staged_apply_matches_tile_kernels(step):
    """One multigrid V-cycle (the CHEB and RESID epilogues of every level-0
    smoothing step) through the TMA kernel and through the tile kernels; the
    preconditioner stays symmetric and positive."""
    from loopstructural_gb300 import fd

    cells = (75, 71, 66)
    rng = np.random.default_rng(24)
    val, nrm = _data(rng, 3000, 600)
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    _, s_tma = _interp(cells, val, nrm, setup, step=step)
    _, s_tile = _interp(cells, val, nrm, setup, tiles=True)
    assert s_tma.staged_apply and not s_tile.staged_apply
    r = torch.from_numpy(rng.normal(size=s_tma.n)).float()
    y = torch.from_numpy(rng.normal(size=s_tma.n)).float()
    za = fd.mg_vcycle(s_tma, r).double()
    zb = fd.mg_vcycle(s_tile, r).double()
    assert float((za - zb).norm() / zb.norm()) <= 1e-5
    vy = fd.mg_vcycle(s_tma, y).double()
    lhs, rhs = float(torch.dot(y.double().cuda(), za)), float(torch.dot(r.double().cuda(), vy))
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs))
    assert float(torch.dot(r.double().cuda(), za)) > 0 and float(torch.dot(y.double().cuda(), vy)) > 0
    s_tma.close()
    s_tile.close()
