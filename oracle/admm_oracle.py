"""ADMM oracle: numpy/scipy restatement of the reference's
inequality-constrained solve with an exact inner solver.  TEST
INFRASTRUCTURE ONLY: imported by tests/ and nowhere in the product.

Reference (packages/loop_interpolation/src/loop_interpolation/):
  _discrete_interpolator.py  add_inequality_constraints_to_matrix :467-507,
                             add_value_inequality_constraints :509-518,
                             add_inequality_pairs_constraints :520-593,
                             add_inequality_feature :595-632,
                             build_inequality_matrix :874-884
  _finite_difference_interpolator.py  setup_interpolator :214-219
  loopsolver/admm_solver.py  admm_solve :59-463
  loopsolver/admm_method.py  ADMM :4-25
Pinned by tests/test_oracle_admm.py against fixtures recorded from the
reference (tests/golden/make_golden.py --admm, run with an exact inner
least-squares solver).

Two properties of the reference that this restatement keeps:
  * Q acts on the column-scaled variable y (c = S y): the bounds constrain
    Q y, not Q c;
  * a rho raised or lowered by the adaptive rule is set back to the
    schedule's value at the start of the next major iteration (the schedule
    is constant without ``admm_weight_final``), so adaptive rho only rescales
    u there and back.
"""
from __future__ import annotations

import numpy as np
from scipy import sparse
from scipy.sparse.linalg import splu

from .fd_oracle import RIDGE, Grid


def value_inequality_rows(grid: Grid, points):  # DI:509-518
    """(idc, raw trilinear weights, bounds) of the points inside the grid."""
    idc, inside = grid.position_to_cell_corners(points[:, :3])
    a = grid.dof_coefs(points[inside, :3])
    return idc[inside], a, points[inside, 3:5]


def pair_rows(grid: Grid, points, pairs=None, upper_bound=np.finfo(float).eps, lower_bound=-np.inf):
    """[(name, idc, a, bounds)] of the inequality pairs (DI:520-593)."""
    out = []
    ids = points[:, 3]
    if not pairs:
        u = np.unique(ids)
        pairs = [(u[i], u[j]) for i in range(len(u)) for j in range(i + 1, len(u))]
    for p0, p1 in pairs:
        up, lo = points[ids == p0], points[ids == p1]
        iu, in_u = grid.position_to_cell_corners(up[:, :3])
        il, in_l = grid.position_to_cell_corners(lo[:, :3])
        au = grid.dof_coefs(up[in_u, :3])
        al = grid.dof_coefs(lo[in_l, :3])
        ju, jl = np.meshgrid(np.arange(int(in_u.sum())), np.arange(int(in_l.sum())))
        ju, jl = ju.ravel(), jl.ravel()
        a = np.hstack([au[ju], -al[jl]])
        idc = np.hstack([iu[in_u][ju], il[in_l][jl]])
        bounds = np.column_stack([np.full(len(ju), lower_bound), np.full(len(ju), upper_bound)])
        out.append((f"inequality_pairs_{p0}_{p1}", idc, a, bounds))
    return out


def p1_value_inequality_rows(mesh, points):  # DI:509-518 on the TetMesh
    """(idc, barycentric weights, bounds) of the points inside the mesh."""
    _, bc, tet, inside = mesh.element_for_location(points[:, :3])
    return mesh.elements[tet[inside]], bc[inside], points[inside, 3:5]


def p1_pair_rows(mesh, points, pairs=None, upper_bound=1.0, lower_bound=-np.inf):  # DI:520-593 on the TetMesh
    """[(name, idc, a, bounds)]: the P1 setup passes no bounds, so the DI
    defaults [-inf, 1.0] apply (P1:244)."""
    out = []
    ids = points[:, 3]
    if not pairs:
        u = np.unique(ids)
        pairs = [(u[i], u[j]) for i in range(len(u)) for j in range(i + 1, len(u))]
    for p0, p1 in pairs:
        up, lo = points[ids == p0], points[ids == p1]
        _, bu, tu, in_u = mesh.element_for_location(up[:, :3])
        _, bl, tl, in_l = mesh.element_for_location(lo[:, :3])
        ju, jl = np.meshgrid(np.arange(int(in_u.sum())), np.arange(int(in_l.sum())))
        ju, jl = ju.ravel(), jl.ravel()
        a = np.hstack([bu[in_u][ju], -bl[in_l][jl]])
        idc = np.hstack([mesh.elements[tu[in_u]][ju], mesh.elements[tl[in_l]][jl]])
        bounds = np.column_stack([np.full(len(ju), lower_bound), np.full(len(ju), upper_bound)])
        out.append((f"inequality_pairs_{p0}_{p1}", idc, a, bounds))
    return out


def feature_rows(grid: Grid, value, lower=True, mask=None):  # DI:595-632
    n = grid.n_nodes
    if mask is None:
        mask = np.ones(n, dtype=bool)
    lo, hi = np.full(n, -np.inf), np.full(n, np.inf)
    mask = mask & ~np.isnan(value)
    if lower:
        lo[mask] = value[mask]
    else:
        hi[mask] = value[mask]
    return np.arange(n)[:, None], np.ones((n, 1)), np.column_stack([lo, hi])


def inequality_matrix(dof, families):
    """Stack (idc, a, bounds) families into (Q csr, bounds) (DI:874-884)."""
    mats, bounds = [], []
    for idc, a, b in families:
        n, k = idc.shape
        rows = np.repeat(np.arange(n), k)
        mats.append(sparse.coo_matrix((a.ravel(), (rows, idc.ravel())), shape=(n, dof)).tocsr())
        bounds.append(b)
    return sparse.vstack(mats).tocsr(), np.vstack(bounds)


def admm_solve(A, b, Q, bounds, x0, rho=0.01, nmajor=200, rho_final=None, schedule="geometric",
               adaptive=False, mu=10.0, tau=2.0, rho_min=1e-4, rho_max=1e3, abs_tol=1e-4, rel_tol=1e-3,
               model_update_tol=0.0, min_iterations=5):
    """admm_solve :59-463 with an exact inner solve (sparse LU of the normal
    equations of [A; rho Q]); returns (y, history)."""
    nA = A.shape[0]
    m = Q.shape[0]
    xmin, xmax = bounds[:, 0], bounds[:, 1]
    model = np.array(x0, dtype=float)
    z = np.zeros(m)
    u = np.zeros(m)
    if rho_final is None:
        sched = np.full(nmajor, float(rho))
    elif schedule == "linear":
        sched = np.linspace(float(rho), float(rho_final), nmajor)
    else:
        sched = np.geomspace(float(rho), float(rho_final), nmajor)
    adaptive = adaptive and rho_final is None
    cur = float(sched[0])

    def system(r):
        M = sparse.vstack([A, Q * r]).tocsr()
        return M, splu((M.T @ M).tocsc())

    M, lu = system(cur)
    history = []
    for i in range(nmajor):
        if float(sched[i]) != cur:
            old, cur = cur, float(sched[i])
            if old > 0:
                u = u * (old / cur)
            M, lu = system(cur)
        z_prev = z.copy()
        Mx = M @ model
        rhs = np.zeros(nA + m)
        rhs[:nA] = b - Mx[:nA]
        qx = Mx[nA:] / cur
        # ADMM.admm_method_iterate_admm_array
        arg = qx + u
        inside = (arg >= xmin) & (arg <= xmax)
        z[inside] = arg[inside]
        below = (arg < xmin) & ~inside
        above = (arg > xmax) & ~inside
        z[below] = xmin[below]
        z[above] = xmax[above]
        u = u + qx - z
        rhs[nA:] = -cur * (qx - (z - u))
        dx = lu.solve(M.T @ rhs)
        model_norm = float(np.linalg.norm(model))
        model = model + dx
        primal = float(np.linalg.norm(qx - z))
        dual = float(cur * np.linalg.norm(z - z_prev))
        eps_pri = np.sqrt(m) * abs_tol + rel_tol * max(float(np.linalg.norm(qx)), float(np.linalg.norm(z)))
        eps_dual = np.sqrt(m) * abs_tol + rel_tol * float(np.linalg.norm(cur * u))
        history.append({"primal_norm": primal, "dual_norm": dual, "eps_pri": eps_pri, "eps_dual": eps_dual,
                        "rho": cur})
        if i + 1 >= min_iterations and primal <= eps_pri and dual <= eps_dual:
            break
        if model_update_tol > 0.0 and i + 1 >= min_iterations:
            if float(np.linalg.norm(dx)) <= model_update_tol * max(model_norm, 1.0):
                break
        if adaptive and i + 1 >= min_iterations:
            new = cur
            if primal > mu * dual:
                new = min(cur * tau, rho_max)
            elif dual > mu * primal:
                new = max(cur / tau, rho_min)
            if new != cur:
                if cur > 0:
                    u = u * (cur / new)
                cur = float(new)
                M, lu = system(cur)
    return model, history


def solve(A, b, Q, bounds, ridge=RIDGE, x0=None, **kw):
    """The reference's preprocessing (ridge rows, column scaling S) around
    admm_solve; returns (c = S y, history)."""
    Af = sparse.vstack([A, sparse.eye(A.shape[1]) * ridge]).tocsr()
    bf = np.hstack([b, np.zeros(A.shape[1])])
    cn = sparse.linalg.norm(Af, axis=0)
    s = np.ones(Af.shape[1])
    s[cn > 0] = 1.0 / cn[cn > 0]
    As = (Af @ sparse.diags(s)).tocsr()
    y0 = np.zeros(A.shape[1]) if x0 is None else np.asarray(x0, dtype=float)
    y, hist = admm_solve(As, bf, Q, bounds, y0, **kw)
    return s * y, hist
