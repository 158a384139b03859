"""GPU adjoint of the field at query points with respect to every input of an
FD interpolator's data (ConstraintAdjoint): value constraints' values and
positions, normal constraints' vectors and positions, and the isotropic
regularisation weight.  Loss: mean squared misfit of the field at held-out
points.  Bar: 1e-6 relative to the largest gradient entry of each group.

* Small grid: central differences of dense FP64 solves of the oracle's
  system.  Values and normals enter the right-hand side only, so the loss is
  quadratic in them and a central difference is exact for any step: h = 1e-2
  keeps FP64 rounding of the solves (~1e-10 of the loss here) far below the
  bar.  Positions and the regularisation weight use the 4-point stencil with
  h = 1e-3 (truncation O(h^4)), at points at least 3h from any cell face.
* 24^3 nodes: an FP64 direct-solve reference gradient: c and the adjoint lam
  from one sparse LU factorisation of the oracle's normal matrix, and each
  component as the derivative of the oracle's own row assembly at fixed c and
  lam, F(theta) = sum_rows w^2 (a.lam)(b - a.c), by central differences
  (dL/dtheta = dF/dtheta), so that neither the GPU jets nor the chain rule of
  the adjoint are used by the reference."""
import numpy as np
import pytest
from scipy import sparse
from scipy.sparse.linalg import splu

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300.adjoint import ConstraintAdjoint  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu

SETUP = dict(cpw=1.3, npw=0.9)


def _case(cells, nv, nn, nq, seed):
    rng = np.random.default_rng(seed)
    vp = rng.uniform(0.02, 0.98, size=(nv, 3))
    vals = np.column_stack([vp, np.sin(3 * vp[:, 0]) + vp[:, 2], rng.uniform(0.5, 2.0, nv)])
    npnt = rng.uniform(0.02, 0.98, size=(nn, 3))
    g = np.column_stack([0.3 * np.cos(3 * npnt[:, 0]), 0.1 * np.ones(nn), np.ones(nn)])
    nrm = np.column_stack([npnt, g + rng.normal(0, 0.05, size=g.shape), rng.uniform(0.5, 2.0, nn)])
    q = rng.uniform(0, 1, size=(nq, 3))
    return np.asarray(cells), vals, nrm, q, q[:, 2] + 0.05 * np.cos(4 * q[:, 1])


def _gpu_grads(cells, vals, nrm, q, target, reg, precision="fp64"):
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
    f = ConstraintAdjoint(grid, q, vals[:, 4], nrm[:, 6], precision=precision, rtol=1e-13, **SETUP)
    dev = "cuda"
    args = [torch.tensor(a, device=dev, dtype=torch.float64, requires_grad=True)
            for a in (vals[:, 3], vals[:, :3], nrm[:, 3:6], nrm[:, :3])]
    r = torch.tensor(reg, device=dev, dtype=torch.float64, requires_grad=True)
    t = torch.tensor(target, device=dev, dtype=torch.float64)
    loss = ((f(*args, r) - t) ** 2).mean()
    loss.backward()
    return float(loss.detach()), [a.grad.cpu().numpy() for a in args] + [float(r.grad)]


def _oracle_loss(cells, vals, nrm, q, target, reg):
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    w = fdo.resolve_weights(regularisation=reg, **SETUP)
    A, b = fdo.assemble(grid, {"value": vals, "normal": nrm}, w).matrix()
    N, rhs = fdo.normal_equations(A, b)
    c = np.linalg.solve(N.toarray(), rhs)
    u = np.nan_to_num(fdo.evaluate_value_local(grid, q, c))
    return float(np.mean((u - target) ** 2))


def _away_from_faces(p, cells, h):
    loc = p * cells - np.floor(p * cells)
    return np.all((loc > 3 * h * cells) & (loc < 1 - 3 * h * cells))


def test_constraint_adjoint_matches_central_differences_of_dense_solves():
    cells, vals, nrm, q, target = _case((7, 6, 8), 60, 15, 80, seed=5)
    reg = 0.1
    loss, grads = _gpu_grads(cells, vals, nrm, q, target, reg)
    assert abs(loss - _oracle_loss(cells, vals, nrm, q, target, reg)) <= 1e-10 * loss
    gv, gvp, gn, gnp, greg = grads
    rng = np.random.default_rng(8)

    def fd_check(name, ref_scale, idx_list, perturb, h, four_point):
        for idx in idx_list:
            def at(step):
                v2, n2, r2 = vals.copy(), nrm.copy(), reg
                v2, n2, r2 = perturb(v2, n2, r2, idx, step)
                return _oracle_loss(cells, v2, n2, q, target, r2)
            if four_point:
                d = (-at(2 * h) + 8 * at(h) - 8 * at(-h) + at(-2 * h)) / (12 * h)
            else:
                d = (at(h) - at(-h)) / (2 * h)
            got = {"value": gv, "normal": gn, "vpos": gvp, "npos": gnp, "reg": np.array([greg])}[name][idx]
            assert abs(d - got) <= 1e-6 * ref_scale, (name, idx, d, got)

    def p_value(v, n, r, i, s):
        v[i, 3] += s
        return v, n, r

    def p_normal(v, n, r, idx, s):
        n[idx[0], 3 + idx[1]] += s
        return v, n, r

    def p_vpos(v, n, r, idx, s):
        v[idx[0], idx[1]] += s
        return v, n, r

    def p_npos(v, n, r, idx, s):
        n[idx[0], idx[1]] += s
        return v, n, r

    def p_reg(v, n, r, idx, s):
        return v, n, r + s

    fd_check("value", np.abs(gv).max(), list(rng.choice(len(vals), 8, replace=False)), p_value, 1e-2, False)
    pick = [(int(i), int(d)) for i, d in zip(rng.choice(len(nrm), 8), rng.integers(0, 3, 8))]
    fd_check("normal", np.abs(gn).max(), pick, p_normal, 1e-2, False)
    h = 1e-3
    vs = [i for i in rng.permutation(len(vals)) if _away_from_faces(vals[i, :3], cells, h)][:6]
    fd_check("vpos", np.abs(gvp).max(), [(int(i), int(d)) for i in vs for d in range(3)][:12], p_vpos, h, True)
    ns = [i for i in rng.permutation(len(nrm)) if _away_from_faces(nrm[i, :3], cells, h)][:6]
    fd_check("npos", np.abs(gnp).max(), [(int(i), int(d)) for i in ns for d in range(3)][:12], p_npos, h, True)
    fd_check("reg", abs(greg), [0], p_reg, 1e-3 * reg, True)


def _row_functional(grid, rows_fn, c, lam):
    """F = sum_rows w^2 (a.lam)(b - a.c) of the oracle's rows for one point."""
    cs = fdo.ConstraintSet(grid.n_nodes)
    rows_fn(cs)
    F = 0.0
    for fam in cs.families.values():
        la = np.sum(fam["A"] * lam[fam["idc"]], axis=1)
        ca = np.sum(fam["A"] * c[fam["idc"]], axis=1)
        F += float(np.sum(fam["w"] ** 2 * la * (fam["B"] - ca)))
    return F


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_constraint_adjoint_matches_direct_solve_reference_at_24(precision):
    cells, vals, nrm, q, target = _case((23, 23, 23), 1000, 200, 2000, seed=6)
    reg = 0.1
    loss, (gv, gvp, gn, gnp, greg) = _gpu_grads(cells, vals, nrm, q, target, reg, precision)
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    w = fdo.resolve_weights(regularisation=reg, **SETUP)
    A, b = fdo.assemble(grid, {"value": vals, "normal": nrm}, w).matrix()
    N, rhs = fdo.normal_equations(A, b)
    lu = splu(N.tocsc())
    c = lu.solve(rhs)
    idc, inside = grid.position_to_cell_corners(q)
    Eq = sparse.csr_matrix((grid.dof_coefs(q[inside]).ravel(),
                            (np.repeat(np.nonzero(inside)[0], 8), idc[inside].ravel())), shape=(len(q), grid.n_nodes))
    u = Eq @ c
    assert abs(loss - float(np.mean((u - target) ** 2))) <= 1e-9 * loss
    lam = lu.solve(Eq.T @ (2.0 / len(q) * (u - target)))
    rng = np.random.default_rng(9)
    h = 1e-4

    def deriv(fn, step, four=True):
        if four:
            return (-fn(2 * step) + 8 * fn(step) - 8 * fn(-step) + fn(-2 * step)) / (12 * step)
        return (fn(step) - fn(-step)) / (2 * step)

    def value_rows(p):
        return lambda cs: fdo.add_value_constraints(grid, cs, p[None, :], w["cpw"])

    def normal_rows(p):
        return lambda cs: fdo.add_norm_constraints(grid, cs, p[None, :], w["npw"])

    checks = []
    for i in rng.choice(len(vals), 12, replace=False):
        def F(s, i=i):
            p = vals[i].copy()
            p[3] += s
            return _row_functional(grid, value_rows(p), c, lam)
        checks.append(("value", deriv(F, 1e-2, four=False), gv[i], np.abs(gv).max()))
    for i, d in zip(rng.choice(len(nrm), 12), rng.integers(0, 3, 12)):
        def F(s, i=i, d=d):
            p = nrm[i].copy()
            p[3 + d] += s
            return _row_functional(grid, normal_rows(p), c, lam)
        checks.append(("normal", deriv(F, 1e-2, four=False), gn[i, d], np.abs(gn).max()))
    for i in [k for k in rng.permutation(len(vals)) if _away_from_faces(vals[k, :3], cells, h)][:6]:
        for d in range(3):
            def F(s, i=i, d=d):
                p = vals[i].copy()
                p[d] += s
                return _row_functional(grid, value_rows(p), c, lam)
            checks.append(("vpos", deriv(F, h), gvp[i, d], np.abs(gvp).max()))
    for i in [k for k in rng.permutation(len(nrm)) if _away_from_faces(nrm[k, :3], cells, h)][:6]:
        for d in range(3):
            def F(s, i=i, d=d):
                p = nrm[i].copy()
                p[d] += s
                return _row_functional(grid, normal_rows(p), c, lam)
            checks.append(("npos", deriv(F, h), gnp[i, d], np.abs(gnp).max()))

    def Freg(s):
        cs = fdo.ConstraintSet(grid.n_nodes)
        fdo.add_regularisation(grid, cs, fdo.resolve_weights(regularisation=reg + s, **SETUP))
        Ar, _ = cs.matrix()
        return -float(lam @ (Ar.T @ (Ar @ c)))
    checks.append(("reg", deriv(Freg, 1e-3 * reg, four=False), greg, abs(greg)))
    for name, ref, got, scale in checks:
        assert abs(ref - got) <= 1e-6 * scale, (name, ref, got, scale)
