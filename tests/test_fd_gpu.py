"""GPU parity of the FD hot path against the oracle and the reference's golden
vectors.  Every compute call goes through the C ABI (libls_gb300.so).

Tolerances (written per test):
  indices                 bit-exact int64
  row values A, b, w      1e-15 relative (ulp-level; the kernels follow numpy's
                          evaluation order)
  normal operator (FP64)  1e-12 relative to max |N x|
  solution, FP64 CG       1e-6 relative (vs the FP64 direct solve)
  solution, mixed         1e-8 relative (vs the FP64 direct solve)
  evaluation              1e-13 relative given the same coefficients
"""
import numpy as np
import pytest
from scipy import sparse

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import _lib, fd  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu

SETUP = {
    "fd_small": dict(regularisation=0.1, cpw=1.0, npw=1.0, gpw=1.0, tpw=1.0, ipw=1.0),
    "fd_cfg1_20": dict(regularisation=0.1, cpw=1.0, npw=1.0),
}


def _grid(cells, step=None):
    cells = np.asarray(cells)
    step = 1.0 / cells.astype(float) if step is None else np.asarray(step, dtype=float)
    return L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=step)


def _interp(golden, name):
    interp = L.FiniteDifferenceInterpolator(_grid(golden[f"{name}_cells"]))
    setters = {"value": interp.set_value_constraints, "normal": interp.set_normal_constraints,
               "gradient": interp.set_gradient_constraints, "tangent": interp.set_tangent_constraints,
               "interface": interp.set_interface_constraints}
    for k, fn in setters.items():
        arr = golden[f"{name}_data_{k}"]
        if arr.shape[0] > 0:
            fn(arr)
    interp.setup_interpolator(**SETUP[name])
    return interp


def _oracle_system(golden, name):
    cells = golden[f"{name}_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {k: golden[f"{name}_data_{k}"] for k in ("value", "normal", "gradient", "tangent", "interface")}
    w = fdo.resolve_weights(**SETUP[name])
    return grid, fdo.assemble(grid, data, w)


def _csr(idc, A, dof):
    n, k = A.shape
    m = sparse.coo_matrix((A.ravel(), (np.repeat(np.arange(n), k), idc.ravel())), shape=(n, dof)).tocsr()
    m.sort_indices()
    return m


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_assembly_matches_reference(golden, name):
    interp = _interp(golden, name)
    names = [str(s) for s in golden[f"{name}_family_names"]]
    assert list(interp.constraints) + list(interp.regularisation_families) == names
    for nm in names:
        got = interp.regularisation_rows(nm) if nm in interp.regularisation_families else interp.constraints[nm].numpy()
        np.testing.assert_array_equal(got["idc"], golden[f"{name}_fam_{nm}_idc"], err_msg=nm)
        m = _csr(got["idc"], got["A"], interp.dof)
        np.testing.assert_array_equal(m.indptr, golden[f"{name}_fam_{nm}_indptr"], err_msg=nm)
        np.testing.assert_array_equal(m.indices, golden[f"{name}_fam_{nm}_indices"], err_msg=nm)
        np.testing.assert_allclose(m.data, golden[f"{name}_fam_{nm}_data"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["B"], golden[f"{name}_fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["w"], golden[f"{name}_fam_{nm}_w"], rtol=1e-15, atol=0, err_msg=nm)


@pytest.mark.parametrize("cells", [(5, 5, 5), (3, 4, 2), (2, 5, 6)])
def test_regularisation_indices_match_reference(golden, cells):
    grid = _grid(cells, np.ones(3))
    prefix = "reg_" + "x".join(str(c) for c in cells) + "_"
    for nm in [str(s) for s in golden[f"{prefix}family_names"]]:
        idc = fd.reg_rows(grid, nm).cpu().numpy()
        np.testing.assert_array_equal(idc, golden[f"{prefix}fam_{nm}_idc"], err_msg=nm)


def _check_operator(system, A, x_seed=0):
    N, rhs = fdo.normal_equations(A, np.zeros(A.shape[0]) if A.shape[0] else np.zeros(0))
    rng = np.random.default_rng(x_seed)
    x = rng.normal(size=A.shape[1])
    ref = N @ x
    got = system.apply(torch.from_numpy(x)).cpu().numpy()
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale
    got32 = system.apply(torch.from_numpy(x).float()).cpu().numpy()
    assert np.max(np.abs(got32 - ref)) <= 2e-5 * scale
    # symmetric operator
    y = rng.normal(size=A.shape[1])
    ny = system.apply(torch.from_numpy(y)).cpu().numpy()
    assert abs(np.dot(got, y) - np.dot(x, ny)) <= 1e-10 * max(1.0, abs(np.dot(got, y)))


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_normal_operator_rhs_diagonal_match_oracle(golden, name):
    interp = _interp(golden, name)
    system = interp._build_system()
    _, cs = _oracle_system(golden, name)
    A, b = cs.matrix()
    _check_operator(system, A)
    N, rhs = fdo.normal_equations(A, b)
    np.testing.assert_allclose(system.rhs().cpu().numpy(), rhs, rtol=1e-13, atol=1e-13 * np.max(np.abs(rhs)))
    np.testing.assert_allclose(system.diagonal().cpu().numpy(), fdo.jacobi_diagonal(A), rtol=1e-13)
    system.close()


@pytest.mark.parametrize("cells", [(5, 5, 5), (8, 6, 12), (14, 14, 14), (1, 4, 5), (2, 2, 9), (23, 23, 23),
                                   (26, 24, 33)])
def test_regularisation_operator_matches_explicit_gram_everywhere(cells):
    """The reference's fused-operator test (every DOF, non-uniform family weights)."""
    kw = dict(dxx=1.0, dyy=0.8, dzz=1.3, dxy=0.5, dxz=0.4, dyz=0.6, dx=0.7, dy=0.9, dz=1.1,
              cpw=0.0, gpw=0.0, npw=0.0, tpw=0.0, ipw=0.0)
    interp = L.FiniteDifferenceInterpolator(_grid(cells, np.ones(3)))
    interp.setup_interpolator(**kw)
    system = interp._build_system()
    grid = fdo.Grid(np.zeros(3), cells, np.ones(3))
    cs = fdo.ConstraintSet(grid.n_nodes)
    fdo.add_regularisation(grid, cs, fdo.resolve_weights(**kw))
    A, _ = cs.matrix()
    _check_operator(system, A, x_seed=11)
    system.close()


def test_operator_on_large_thin_grid():
    """Grids of more than 300,000 nodes with an axis under 24 nodes run the staged
    full-grid kernel (exact shell sum at every boundary node)."""
    cells = np.array([640, 520, 2])
    kw = dict(dxx=1.0, dyy=0.8, dzz=1.3, dxy=0.5, dxz=0.4, dyz=0.6, dx=0.7, dy=0.9, dz=1.1,
              cpw=0.0, gpw=0.0, npw=0.0, tpw=0.0, ipw=0.0)
    interp = L.FiniteDifferenceInterpolator(_grid(cells, np.ones(3)))
    interp.setup_interpolator(**kw)
    system = interp._build_system()
    assert system.n > 300_000
    grid = fdo.Grid(np.zeros(3), cells, np.ones(3))
    cs = fdo.ConstraintSet(grid.n_nodes)
    fdo.add_regularisation(grid, cs, fdo.resolve_weights(**kw))
    A, _ = cs.matrix()
    x = np.random.default_rng(4).normal(size=A.shape[1])
    N, _ = fdo.normal_equations(A, np.zeros(A.shape[0]))
    ref = N @ x
    got = system.apply(torch.from_numpy(x)).cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    got32 = system.apply(torch.from_numpy(x).float()).cpu().numpy()
    assert np.max(np.abs(got32 - ref)) <= 2e-5 * np.max(np.abs(ref))
    system.close()


def test_normal_operator_with_data_on_split_grid():
    """Grids of >= 24 nodes per axis run the deep-box kernel plus the boundary-shell
    kernel; the data term must land on both."""
    cells = np.array([25, 24, 27])
    rng = np.random.default_rng(5)
    vp = rng.uniform(0, 1, size=(400, 3))
    val = np.column_stack([vp, vp[:, 2] + 0.1 * vp[:, 0], np.ones(400)])
    npnt = rng.uniform(0, 1, size=(80, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(80, 3)), np.ones(80)])
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.setup_interpolator(**setup)
    system = interp._build_system()
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    cs = fdo.assemble(grid, {"value": val, "normal": nrm}, fdo.resolve_weights(**setup))
    A, _ = cs.matrix()
    _check_operator(system, A, x_seed=3)
    system.close()


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-6), ("mixed", 1e-8)])
def test_solution_matches_direct_solve(golden, name, precision, tol):
    interp = _interp(golden, name)
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-14, "atol": 0.0, "precision": precision,
                                                    "maxiter": 200000})
    ref = golden[f"{name}_c_direct"]
    err = np.linalg.norm(interp.c - ref) / np.linalg.norm(ref)
    assert err <= tol, (precision, err, interp.get_last_solve_timing())
    q = golden[f"{name}_query"]
    v = interp.evaluate_value(q)
    vr = golden[f"{name}_eval_value"]
    ok = np.isfinite(vr)
    assert np.max(np.abs(v[ok] - vr[ok])) <= tol * np.max(np.abs(vr[ok])) * 10


def test_default_tolerance_follows_reference_iteration(golden):
    """Same algorithm as the reference's column-scaled scipy cg: the FP64 GPU
    iteration count at the reference defaults (tol=1e-10, rtol=1e-5) matches
    the oracle's scipy run up to rounding-path differences."""
    name = "fd_cfg1_20"
    interp = _interp(golden, name)
    interp.solve_system("cg", tol=1e-10, solver_kwargs={"precision": "fp64"})
    t = interp.get_last_solve_timing()
    _, cs = _oracle_system(golden, name)
    A, b = cs.matrix()
    c_ref, flag, it_ref = fdo.solve_reference_cg(A, b, tol=1e-10)
    assert flag == 0
    assert abs(t["iterations"] - it_ref) <= max(3, 0.05 * it_ref), (t["iterations"], it_ref)
    res, bn = fdo.pcg_scaled_residual(A, b, interp.c)
    assert res < max(1e-10, 1e-5 * bn) * 1.01
    # both answers are equally (un)converged: compare at the level rtol implies
    assert np.linalg.norm(interp.c - c_ref) <= 0.05 * np.linalg.norm(c_ref)


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_evaluation_matches_reference(golden, name):
    cells = golden[f"{name}_cells"]
    grid = _grid(cells)
    q = golden[f"{name}_query"]
    c = golden[f"{name}_c_direct"]
    v, g = fd.eval_points(grid, c, q)
    np.testing.assert_allclose(v, golden[f"{name}_eval_value"], rtol=1e-13, atol=1e-13, equal_nan=True)
    np.testing.assert_allclose(g, golden[f"{name}_eval_gradient"], rtol=1e-13, atol=1e-13, equal_nan=True)


def test_lattice_evaluation_matches_oracle():
    cells = np.array([9, 7, 11])
    grid = _grid(cells)
    ref = fdo.Grid(np.zeros(3), cells, 1.0 / cells)
    rng = np.random.default_rng(3)
    c = rng.normal(size=grid.n_nodes)
    origin, step, counts = (-0.05, 0.0, 0.02), (0.011, 0.013, 0.0097), (100, 80, 104)
    v, g = fd.eval_lattice(grid, torch.from_numpy(c).cuda(), origin, step, counts)
    i, j, k = np.meshgrid(*[np.arange(n) for n in counts], indexing="ij")
    pts = np.stack([origin[0] + step[0] * i.ravel(order="F"), origin[1] + step[1] * j.ravel(order="F"),
                    origin[2] + step[2] * k.ravel(order="F")], axis=1)
    np.testing.assert_allclose(v.cpu().numpy(), fdo.evaluate_value_local(ref, pts, c), rtol=1e-13, atol=1e-13,
                               equal_nan=True)
    np.testing.assert_allclose(g.cpu().numpy(), fdo.evaluate_gradient_local(ref, pts, c), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("cells, origin, step, counts", [
    # a lattice far coarser than the grid in x: the chunk's node span exceeds the
    # row-collapse buffer, so every point gathers its 8 coefficients
    ((700, 3, 4), (-0.01, 0.05, 0.1), (0.0251, 0.3, 0.2), (41, 4, 5)),
    # a reversed lattice (negative steps), partly outside the grid
    ((13, 9, 6), (1.02, 0.97, 0.99), (-0.0173, -0.0211, -0.0197), (70, 50, 53)),
])
def test_lattice_evaluation_paths(cells, origin, step, counts):
    cells = np.array(cells)
    grid = _grid(cells)
    ref = fdo.Grid(np.zeros(3), cells, 1.0 / cells)
    c = np.random.default_rng(4).normal(size=grid.n_nodes)
    v, g = fd.eval_lattice(grid, torch.from_numpy(c).cuda(), origin, step, counts)
    i, j, k = np.meshgrid(*[np.arange(n) for n in counts], indexing="ij")
    pts = np.stack([origin[0] + step[0] * i.ravel(order="F"), origin[1] + step[1] * j.ravel(order="F"),
                    origin[2] + step[2] * k.ravel(order="F")], axis=1)
    vr = fdo.evaluate_value_local(ref, pts, c)
    gr = fdo.evaluate_gradient_local(ref, pts, c)
    assert np.isnan(vr).any() and np.isfinite(vr).any()
    np.testing.assert_allclose(v.cpu().numpy(), vr, rtol=1e-13, atol=1e-13, equal_nan=True)
    scale = np.abs(gr).max()
    np.testing.assert_allclose(g.cpu().numpy(), gr, rtol=1e-12, atol=1e-12 * scale)


def test_mixed_solve_is_deterministic(golden):
    a = _interp(golden, "fd_cfg1_20")
    a.solve_system("cg", solver_kwargs={"rtol": 1e-12, "atol": 0.0})
    b = _interp(golden, "fd_cfg1_20")
    b.solve_system("cg", solver_kwargs={"rtol": 1e-12, "atol": 0.0})
    np.testing.assert_array_equal(a.c, b.c)


def test_edge_cases():
    grid = _grid((4, 4, 4))
    # no data: zero right-hand side, zero solution
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.setup_interpolator(regularisation=0.1)
    assert interp.solve_system("cg")
    assert np.all(interp.c == 0)
    # every point outside: no rows are added
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(np.array([[2.0, 2.0, 2.0, 1.0], [-1.0, 0.5, 0.5, 1.0]]))
    rep = interp.setup_interpolator(regularisation=0.1)
    assert "value" not in rep
    # maxiter=1: the last iterate is returned (reference warns, still True)
    interp = L.FiniteDifferenceInterpolator(grid)
    pts = np.random.default_rng(5).uniform(0, 1, size=(20, 3))
    interp.set_value_constraints(np.column_stack([pts, pts[:, 2]]))
    interp.setup_interpolator(regularisation=0.1)
    assert interp.solve_system("cg", solver_kwargs={"maxiter": 1, "rtol": 1e-14, "precision": "fp64"})
    t = interp.get_last_solve_timing()
    assert t["iterations"] == 1 and t["status"] == _lib.LS_NOT_CONVERGED
    # a single-cell-thick grid has no interior rows
    interp = L.FiniteDifferenceInterpolator(_grid((1, 5, 5)))
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0], [0.5, 0.1, 0.9, 0.0]]))
    rep = interp.setup_interpolator(regularisation=0.1)
    assert "dxx" not in rep and "dyy" not in rep and "dy_lower" in rep
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-10})
    # empty evaluation
    assert interp.evaluate_value(np.zeros((0, 3))).shape == (0,)
    assert interp.evaluate_gradient(np.zeros((0, 3))).shape == (0, 3)


def _synthetic(n_nodes, n_val, n_nrm, seed=0):
    rng = np.random.default_rng(seed)
    cells = np.array([n_nodes - 1] * 3)
    vp = rng.uniform(0, 1, size=(n_val, 3))
    val = np.column_stack([vp, vp[:, 2] + 0.1 * np.sin(2 * np.pi * vp[:, 0]) + 0.2 * (vp[:, 0] > 0.5), np.ones(n_val)])
    npnt = rng.uniform(0, 1, size=(n_nrm, 3))
    g = np.column_stack([0.2 * np.pi * np.cos(2 * np.pi * npnt[:, 0]), np.zeros(n_nrm), np.ones(n_nrm)])
    nrm = np.column_stack([npnt, g + rng.normal(0, 0.02, g.shape), np.ones(n_nrm)])
    return cells, val, nrm


@pytest.mark.parametrize("n_nodes", [21, 34])
def test_multigrid_matches_jacobi_solution_with_fewer_iterations(n_nodes):
    """The MG preconditioner changes only the iteration path: the FP32+FP64
    MG solve lands on the FP64 Jacobi solve (1e-8) in far fewer iterations."""
    cells, val, nrm = _synthetic(n_nodes, 400, 100)
    out = {}
    for prec, pc in (("fp64", "jacobi"), ("mixed", "mg"), ("mixed", "jacobi")):
        interp = L.FiniteDifferenceInterpolator(_grid(cells))
        interp.set_value_constraints(val)
        interp.set_normal_constraints(nrm)
        interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "precision": prec,
                                                 "preconditioner": pc, "maxiter": 500000})
        t = interp.get_last_solve_timing()
        assert t["status"] == 0 and t["preconditioner"] == (pc if prec == "mixed" else "jacobi")
        out[(prec, pc)] = (interp.c.copy(), t["iterations"])
    ref = out[("fp64", "jacobi")][0]
    for key in (("mixed", "mg"), ("mixed", "jacobi")):
        err = np.linalg.norm(out[key][0] - ref) / np.linalg.norm(ref)
        assert err <= 1e-8, (key, err)
    assert out[("mixed", "mg")][1] * 5 < out[("fp64", "jacobi")][1], {k: v[1] for k, v in out.items()}


def test_multigrid_falls_back_to_jacobi_on_thin_grids():
    cells = np.array([30, 30, 2])
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    rng = np.random.default_rng(1)
    vp = rng.uniform(0, 1, size=(100, 3))
    interp.set_value_constraints(np.column_stack([vp, vp[:, 0]]))
    interp.setup_interpolator(regularisation=0.1)
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-10, "preconditioner": "mg"})
    t = interp.get_last_solve_timing()
    assert t["preconditioner"] == "jacobi" and t["status"] == 0


def _prolong_1d(nf):
    nc = nf // 2 + 1
    P = sparse.lil_matrix((nf, nc))
    for i in range(nf):
        if i % 2 == 0:
            P[i, i // 2] = 1.0
        else:
            P[i, i // 2] = P[i, i // 2 + 1] = 0.5
    return P.tocsr(), nc


@pytest.mark.parametrize("cells", [(24, 23, 26), (40, 38, 42)])
def test_coarse_levels_are_galerkin(cells):
    """Every coarse multigrid level applies P^T A_fine P exactly (regularisation
    by the tensor-product Galerkin operator, data rows by the 27-point form)."""
    cells = np.array(cells)
    rng = np.random.default_rng(9)
    vp = rng.uniform(0, 1, size=(300, 3))
    val = np.column_stack([vp, vp[:, 2], np.ones(300)])
    npnt = rng.uniform(0, 1, size=(60, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(60, 3)), np.ones(60)])
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.setup_interpolator(**setup)
    system = interp._build_system()
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    A, _ = fdo.assemble(grid, {"value": val, "normal": nrm}, fdo.resolve_weights(**setup)).matrix()
    G, _ = fdo.normal_equations(A, np.zeros(A.shape[0]))
    nf = cells + 1
    level = 0
    while True:
        ps = [_prolong_1d(n) for n in nf]
        P = sparse.kron(sparse.kron(ps[2][0], ps[1][0]), ps[0][0]).tocsr()
        G = (P.T @ G @ P).tocsr()
        nf = np.array([p[1] for p in ps])
        level += 1
        nodes, _ = fd.mg_apply_level(system, level)
        assert nodes == G.shape[0]
        if nodes <= 200:  # the coarsest level (of grids this small) is solved densely, not applied
            break
        x = np.random.default_rng(level).normal(size=nodes)
        _, y = fd.mg_apply_level(system, level, torch.from_numpy(x))
        ref = G @ x
        assert np.max(np.abs(y.cpu().numpy() - ref)) <= 2e-5 * np.max(np.abs(ref)), level
    system.close()


def _prolong_axes(x, ps, shape_c):
    """P x for P = Pz (x) Py (x) Px applied axis by axis (x: coarse, z-major)."""
    t = x.reshape(shape_c[::-1])
    t = np.tensordot(t, ps[0].toarray(), axes=([2], [1]))
    t = np.moveaxis(np.tensordot(t, ps[1].toarray(), axes=([1], [1])), 2, 1)
    t = np.moveaxis(np.tensordot(t, ps[2].toarray(), axes=([0], [1])), 2, 0)
    return t.ravel()


def _restrict_axes(y, ps, shape_f):
    """P^T y axis by axis (y: fine, z-major)."""
    t = y.reshape(shape_f[::-1])
    t = np.tensordot(t, ps[0].toarray(), axes=([2], [0]))
    t = np.moveaxis(np.tensordot(t, ps[1].toarray(), axes=([1], [0])), 2, 1)
    t = np.moveaxis(np.tensordot(t, ps[2].toarray(), axes=([0], [0])), 2, 0)
    return t.ravel()


@pytest.mark.parametrize("cells", [(240, 80, 90), (200, 150, 120)])
def test_large_coarse_levels_are_galerkin_of_the_finer_level(cells):
    """Levels too large for explicit stencils (boundary faces, edges and
    corners from their own tables: 121 x 41 x 46, 101 x 76 x 61 and
    51 x 39 x 31) and an explicit level (61 x 21 x 24, one warp per node)
    apply P^T A_finer P, with A_finer the level above's own FP32 apply."""
    cells = np.array(cells)
    assert int(np.prod(cells // 2 + 1)) > 200000  # level 1 holds no explicit stencils
    rng = np.random.default_rng(11)
    vp = rng.uniform(0, 1, size=(3000, 3))
    val = np.column_stack([vp, vp[:, 2] + 0.1 * vp[:, 0], np.ones(3000)])
    npnt = rng.uniform(0, 1, size=(600, 3))
    nrm = np.column_stack([npnt, rng.normal(size=(600, 3)), np.ones(600)])
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
    system = interp._build_system()
    nf = cells + 1
    for level in (1, 2):
        ps = [_prolong_1d(int(n)) for n in nf]
        nc = np.array([p[1] for p in ps])
        nodes, _ = fd.mg_apply_level(system, level)
        assert nodes == int(np.prod(nc))
        x = np.random.default_rng(level).normal(size=nodes)
        fine = torch.from_numpy(_prolong_axes(x, [p[0] for p in ps], nc))
        _, yf = fd.mg_apply_level(system, level - 1, fine)
        ref = _restrict_axes(yf.cpu().numpy().astype(np.float64), [p[0] for p in ps], nf)
        _, y = fd.mg_apply_level(system, level, torch.from_numpy(x))
        assert np.max(np.abs(y.cpu().numpy() - ref)) <= 5e-5 * np.max(np.abs(ref)), level
        nf = nc
    system.close()


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_build_matrix_and_custom_solver_match_reference(golden, name):
    """The explicit system (DI:684-755) in the reference's family order, and a
    custom solver callable on it (DI:1283-1313)."""
    from scipy.sparse.linalg import spsolve

    interp = _interp(golden, name)
    _g, cs = _oracle_system(golden, name)
    assert interp.family_order == [str(s) for s in golden[f"{name}_family_names"]]
    A, b = interp.build_matrix()
    Ar, br = cs.matrix()
    assert A.shape == Ar.shape
    assert abs(A - Ar).max() <= 1e-15 * abs(Ar).max()
    np.testing.assert_allclose(b, br, rtol=1e-15, atol=1e-15 * np.max(np.abs(br)))
    assert interp.solve_system(lambda M, rhs: spsolve((M.T @ M).tocsc(), M.T @ rhs))
    ref = golden[f"{name}_c_direct"]
    assert np.linalg.norm(interp.c - ref) <= 1e-8 * np.linalg.norm(ref)
    res = interp.calculate_residual_for_constraints()
    assert set(res) == set(cs.families)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_rows_give_nan_status(caplog, precision):
    """A data row with a NaN coefficient that reaches ls_fd_create (the
    interpolator's own checks drop such families, as the reference does, so
    the row is planted in the device tensor after setup): the solve stops with
    LS_NAN instead of iterating to maxiter, and solve_system warns."""
    import logging

    rng = np.random.default_rng(31)
    grid = _grid((12, 10, 9))
    interp = L.FiniteDifferenceInterpolator(grid)
    vp = rng.uniform(0, 1, size=(50, 3))
    interp.set_value_constraints(np.column_stack([vp, vp[:, 2], np.ones(50)]))
    interp.setup_interpolator(regularisation=0.1, cpw=1.0)
    interp.constraints["value"].a[3, 2] = float("nan")
    with caplog.at_level(logging.WARNING):
        assert interp.solve_system("cg", solver_kwargs={"precision": precision, "maxiter": 5000,
                                                        "preconditioner": "jacobi"})
    t = interp.get_last_solve_timing()
    assert t["status"] == _lib.LS_NAN, t
    assert t["iterations"] < 5000
    assert "nan" in caplog.text
