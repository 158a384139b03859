"""Pin the ADMM oracle against the fixtures recorded from the reference's
``solve_system('admm')`` with an exact inner solver (make_golden.py --admm):
the inequality rows (value inequalities, inequality pairs, an inequality
feature) as the reference's build_inequality_matrix returns them, and the
solution and primal/dual history of the major iterations.  Cases: constant
rho, a geometric rho schedule, adaptive rho, and loose bounds from an x0 that
stop on the primal/dual test.  CPU only."""
import numpy as np
import pytest
from scipy import sparse

from conftest import ADMM_CASES, admm_kwargs
from oracle import admm_oracle as ao
from oracle import fd_oracle as fdo


def oracle_case(g, name):
    cells = g[f"{name}_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    cs = fdo.assemble(grid, {"value": g[f"{name}_value"], "normal": g[f"{name}_normal"]},
                      fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0))
    A, b = cs.matrix()
    fams = [ao.value_inequality_rows(grid, g[f"{name}_ineq"])]
    fams += [(i, a, bd) for _n, i, a, bd in ao.pair_rows(grid, g[f"{name}_pairs"])]
    feat = float(g[f"{name}_feature"][0])
    if not np.isnan(feat):
        nodes = grid.nodes
        fams.append(ao.feature_rows(grid, nodes[:, 2] - feat, lower=True, mask=nodes[:, 0] > 0.5))
    Q, bounds = ao.inequality_matrix(grid.n_nodes, fams)
    return grid, A, b, Q, bounds


def _fixture_q(g, name, dof):
    return sparse.coo_matrix((g[f"{name}_Q_val"], (g[f"{name}_Q_row"], g[f"{name}_Q_col"])),
                             shape=(g[f"{name}_bounds"].shape[0], dof)).tocsr()


@pytest.mark.parametrize("name", ADMM_CASES)
def test_inequality_rows_match_reference(agolden, name):
    grid, _A, _b, Q, bounds = oracle_case(agolden, name)
    ref = _fixture_q(agolden, name, grid.n_nodes)
    assert Q.shape == ref.shape
    assert abs(Q - ref).max() <= 1e-15
    np.testing.assert_array_equal(bounds, agolden[f"{name}_bounds"])


@pytest.mark.parametrize("name", ADMM_CASES)
def test_admm_solution_and_history_match_reference(agolden, name):
    grid, A, b, Q, bounds = oracle_case(agolden, name)
    kw = admm_kwargs(agolden, name)
    x0 = grid.nodes[:, 2].copy() if kw.pop("x0", None) == "nodes_z" else None
    opts = {"rho": kw.pop("admm_weight", 0.01), "nmajor": kw.pop("nmajor", 200),
            "rho_final": kw.pop("admm_weight_final", None), "schedule": kw.pop("admm_weight_schedule", "geometric"),
            "adaptive": kw.pop("adaptive_rho", False), "min_iterations": kw.pop("min_iterations", 5)}
    assert not kw
    c, hist = ao.solve(A, b, Q, bounds, x0=x0, **opts)
    assert len(hist) == int(agolden[f"{name}_iterations"])
    ref = agolden[f"{name}_c"]
    np.testing.assert_allclose(c, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    for k in ("primal_norm", "dual_norm", "eps_pri", "eps_dual", "rho"):
        got = np.array([h[k] for h in hist])
        exp = agolden[f"{name}_hist_{k}"]
        np.testing.assert_allclose(got, exp, rtol=1e-7, atol=1e-9 * np.abs(exp).max(), err_msg=k)
    # the inequalities changed the solution: the case exercises them
    assert np.abs(ref - agolden[f"{name}_c_unconstrained"]).max() > 1e-3


def test_p1_admm_rows_and_solution(agolden):
    """P1 (P1:243-244): barycentric inequality rows, pair bounds [-inf, 1]."""
    from oracle import p1_oracle as p1o

    g = agolden
    cells = g["admm_p1_cells"]
    mesh = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))
    cs = p1o.assemble(mesh, {"value": g["admm_p1_value"], "normal": g["admm_p1_normal"]},
                      p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0))
    A, b = cs.matrix()
    fams = [ao.p1_value_inequality_rows(mesh, g["admm_p1_ineq"])]
    fams += [(i, a, bd) for _n, i, a, bd in ao.p1_pair_rows(mesh, g["admm_p1_pairs"])]
    Q, bounds = ao.inequality_matrix(mesh.n_nodes, fams)
    ref = _fixture_q(g, "admm_p1", mesh.n_nodes)
    assert abs(Q - ref).max() <= 1e-15
    np.testing.assert_array_equal(bounds, g["admm_p1_bounds"])
    c, hist = ao.solve(A, b, Q, bounds, rho=1.0, nmajor=60)
    assert len(hist) == int(g["admm_p1_iterations"])
    np.testing.assert_allclose(c, g["admm_p1_c"], rtol=0, atol=1e-9 * np.abs(g["admm_p1_c"]).max())
