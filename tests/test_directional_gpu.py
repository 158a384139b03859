"""GPU parity of directional regularisation (FD:1207-1337 matrix-free, P1
directional face rows) and gradient-orthogonal rows with a target
(FD:478-539) against the reference's fixtures and the oracle.  Every compute
call goes through the C ABI.

Tolerances (written per test):
  indices                    bit-exact int64
  row values A, b, w         1e-15 relative
  normal operator (FP64)     1e-12 relative to max |N x|; FP32 2e-5
  diagonal                   1e-13 relative
  solution, FP64 CG          1e-6 relative (vs the FP64 direct solve)
  solution, mixed            1e-8 relative (vs the FP64 direct solve)
"""
import numpy as np
import pytest
from scipy import sparse

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import _lib, fd  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

from test_fd_gpu import _check_operator, _csr, _grid  # noqa: E402
from test_oracle_directional import fd_dir_case, fd_fold_oracle, p1_dir_case  # noqa: E402
from golden.make_golden import SyntheticFold, fold_case_weights  # noqa: E402

pytestmark = pytest.mark.gpu


def _fd_dir_interp(g):
    """The fd_dir fixture's calls on the GPU class: the regularisation dict
    with an array term and a callable term, then a gradient-orthogonal family
    with a target."""
    cells = g["fd_dir_cells"]
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    interp.set_value_constraints(g["fd_dir_value_in"])
    interp.set_normal_constraints(g["fd_dir_normal_in"])
    dir_b = g["fd_dir_dir_b"]

    def v2(p):
        return np.column_stack([np.zeros(len(p)), np.ones(len(p)), p[:, 2]])

    reg = {"isotropic": 0.1,
           "directional": [L.DirectionalRegularisation(weight=0.5, direction=g["fd_dir_dir_a"], name="fold a"),
                           {"weight": 0.2, "direction": v2, "name": "fold b"}]}
    report = interp.setup_interpolator(regularisation=reg, cpw=1.0, npw=1.0)
    np.testing.assert_allclose(v2(interp.get_regularisation_sample_points()), dir_b, rtol=0, atol=1e-15)
    interp.add_gradient_orthogonal_constraints(g["fd_dir_orth_points"], g["fd_dir_orth_vectors"].copy(), w=2.0, b=0.3,
                                               name="fold normalisation")
    return interp, report


def _rows(interp, nm):
    if nm in interp.regularisation_families:
        return interp.regularisation_rows(nm)
    if nm in interp.directional_families:
        return interp.directional_rows(nm)
    return interp.constraints[nm].numpy()


def test_fd_directional_families_match_reference(dgolden):
    interp, report = _fd_dir_interp(dgolden)
    names = [str(s) for s in dgolden["fd_dir_family_names"]]
    assert set(report) | {"fold normalisation"} == set(names)
    for nm in names:
        got = _rows(interp, nm)
        np.testing.assert_array_equal(got["idc"], dgolden[f"fd_dir_fam_{nm}_idc"], err_msg=nm)
        m = _csr(got["idc"], got["A"], interp.dof)
        np.testing.assert_array_equal(m.indices, dgolden[f"fd_dir_fam_{nm}_indices"], err_msg=nm)
        np.testing.assert_allclose(m.data, dgolden[f"fd_dir_fam_{nm}_data"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["B"], dgolden[f"fd_dir_fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["w"], dgolden[f"fd_dir_fam_{nm}_w"], rtol=1e-15, atol=0, err_msg=nm)
        assert got["idc"].shape[0] == (report[nm] if nm in report else got["idc"].shape[0])


def test_fd_directional_operator_and_diagonal_match_oracle(dgolden):
    interp, _ = _fd_dir_interp(dgolden)
    system = interp._build_system()
    _grid_o, cs = fd_dir_case(dgolden)
    A, b = cs.matrix()
    _check_operator(system, A, x_seed=7)
    N, rhs = fdo.normal_equations(A, b)
    np.testing.assert_allclose(system.diagonal().cpu().numpy(), fdo.jacobi_diagonal(A), rtol=1e-13)
    np.testing.assert_allclose(system.rhs().cpu().numpy(), rhs, rtol=1e-13, atol=1e-13 * np.max(np.abs(rhs)))
    system.close()


@pytest.mark.parametrize("precision,preconditioner,tol", [("fp64", "jacobi", 1e-6), ("mixed", "jacobi", 1e-8),
                                                          ("mixed", "mg", 1e-8)])
def test_fd_directional_solution_matches_reference(dgolden, precision, preconditioner, tol):
    interp, _ = _fd_dir_interp(dgolden)
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-14, "atol": 0.0, "precision": precision,
                                                    "preconditioner": preconditioner, "maxiter": 200000})
    ref = dgolden["fd_dir_c_direct"]
    err = np.linalg.norm(interp.c - ref) / np.linalg.norm(ref)
    assert err <= tol, (precision, preconditioner, err, interp.get_last_solve_timing())


def _fold_like(n_nodes, seed=0):
    """A grid with data and three directional terms of a fold-like geometry
    (axis, axial-plane and across-fold directions varying over the grid)."""
    rng = np.random.default_rng(seed)
    cells = np.array([n_nodes - 1] * 3)
    grid = _grid(cells)
    nodes = grid.nodes
    ang = 2.0 * np.pi * nodes[:, 0]
    across = np.column_stack([np.cos(ang), np.zeros(len(ang)), np.sin(ang)])
    axis = np.tile([0.0, 1.0, 0.0], (len(ang), 1))
    plane = np.cross(across, axis)
    vp = rng.uniform(0, 1, size=(300, 3))
    val = np.column_stack([vp, np.sin(2 * np.pi * vp[:, 0]) * 0.1 + vp[:, 2], np.ones(300)])
    terms = [L.DirectionalRegularisation(0.1, across, "fold regularisation 1"),
             L.DirectionalRegularisation(0.01, plane, "fold regularisation 2"),
             L.DirectionalRegularisation(0.01, axis, "fold regularisation 3")]
    return cells, val, terms


@pytest.mark.parametrize("n_nodes", [21, 41])
def test_fd_directional_multigrid_matches_jacobi(n_nodes):
    """Multigrid with the averaged directional coarse term lands on the FP64
    Jacobi solution (1e-8) in fewer iterations."""
    cells, val, terms = _fold_like(n_nodes)
    out = {}
    for prec, pc in (("fp64", "jacobi"), ("mixed", "mg")):
        interp = L.FiniteDifferenceInterpolator(_grid(cells))
        interp.set_value_constraints(val)
        interp.setup_interpolator(regularisation={"isotropic": 0.01, "directional": terms}, cpw=1.0)
        assert len(interp.directional_families) > 0
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "precision": prec,
                                                 "preconditioner": pc, "maxiter": 500000})
        t = interp.get_last_solve_timing()
        assert t["status"] == 0 and t["preconditioner"] == pc, t
        out[pc] = (interp.c.copy(), t["iterations"])
    err = np.linalg.norm(out["mg"][0] - out["jacobi"][0]) / np.linalg.norm(out["jacobi"][0])
    assert err <= 1e-8, err
    assert out["mg"][1] * 3 < out["jacobi"][1], {k: v[1] for k, v in out.items()}


def test_fd_directional_coarse_levels_are_symmetric_positive():
    cells, val, terms = _fold_like(41)
    interp = L.FiniteDifferenceInterpolator(_grid(cells))
    interp.set_value_constraints(val)
    interp.setup_interpolator(regularisation={"isotropic": 0.01, "directional": terms}, cpw=1.0)
    interp.solve_system("cg", solver_kwargs={"rtol": 1e-6, "preconditioner": "mg"})
    system = interp._system
    rng = np.random.default_rng(2)
    for level in (1, 2):
        n, _ = fd.mg_apply_level(system, level)
        u = torch.from_numpy(rng.normal(size=n)).float()
        v = torch.from_numpy(rng.normal(size=n)).float()
        au = fd.mg_apply_level(system, level, u)[1].double().cpu()
        av = fd.mg_apply_level(system, level, v)[1].double().cpu()
        lhs, rhs = float(v.double() @ au), float(u.double() @ av)
        assert abs(lhs - rhs) <= 1e-4 * (abs(lhs) + abs(rhs)), (level, lhs, rhs)
        assert float(u.double() @ au) > 0


def test_directional_config_errors_follow_reference():
    interp = L.FiniteDifferenceInterpolator(_grid((4, 4, 4)))
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0, 1.0]]))
    with pytest.raises(TypeError):
        interp.setup_interpolator(regularisation={"directional": [0.1, 0.2]})
    with pytest.raises(ValueError):
        interp.setup_interpolator(directional_regularisation={"weight": 1.0})
    # wrong shape: warned and skipped; zero weight: skipped
    rep = interp.setup_interpolator(directional_regularisation=[{"weight": 1.0, "direction": np.ones((3, 3))},
                                                               {"weight": 0.0, "direction": np.ones((125, 3))}])
    assert not interp.directional_families and "dxx" in rep
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-10})


def test_p1_directional_matches_reference(dgolden):
    cells = dgolden["p1_dir_cells"]
    mesh = L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))
    interp = L.P1Interpolator(mesh)
    interp.set_value_constraints(dgolden["p1_dir_value_in"])
    vec = dgolden["p1_dir_dir"]
    interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0,
                              directional_regularisation={"weight": 0.3, "direction": vec, "name": "fold p1"})
    names = [str(s) for s in dgolden["p1_dir_family_names"]]
    assert list(interp.constraints) == names
    for nm in names:
        got = interp.constraints[nm].numpy()
        np.testing.assert_array_equal(got["idc"], dgolden[f"p1_dir_fam_{nm}_idc"], err_msg=nm)
        ref = dgolden[f"p1_dir_fam_{nm}_data"]
        m = _csr(got["idc"], got["A"], interp.dof)
        data = m.data
        if nm in ("edge jump",):  # the face normal's sign follows the shared-node order
            sign = np.sign(np.add.reduceat(data * ref, m.indptr[:-1]))
            data = data * np.repeat(sign, np.diff(m.indptr))
        np.testing.assert_allclose(data, ref, rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["w"], dgolden[f"p1_dir_fam_{nm}_w"], rtol=1e-15, atol=0, err_msg=nm)
    # the face centres are the reference's regularisation sample points
    from golden.make_golden import _direction_field
    np.testing.assert_allclose(_direction_field(interp.get_regularisation_sample_points()), vec, rtol=1e-12,
                               atol=1e-12)
    _m, cs = p1_dir_case(dgolden)
    A, _b = cs.matrix()
    system = interp._build_system()
    _check_operator(system, A, x_seed=5)
    system.close()
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-14, "atol": 0.0, "maxiter": 200000})
    ref = dgolden["p1_dir_c_direct"]
    assert np.linalg.norm(interp.c - ref) <= 1e-8 * np.linalg.norm(ref)


def test_noalloc_rejects_directional_systems():
    """The no-allocation apply has no handle for the directional weights."""
    import ctypes as C

    lib = _lib.load()
    s = _lib.FdSystem()
    s.grid = _grid((4, 4, 4)).grid3()
    w = torch.zeros((6, 125), dtype=torch.float64, device=_lib.device())
    s.d_dir = _lib.ptr(w)
    x = torch.zeros(125, dtype=torch.float64, device=_lib.device())
    assert lib.ls_fd_apply_noalloc(C.byref(s), _lib.ptr(x), _lib.ptr(x), None, None) == -1


def _fold_interp(g):
    cells = g["fd_fold_cells"]
    interp = L.FDFoldInterpolator(_grid(cells), fold=SyntheticFold())
    interp.set_value_constraints(g["fd_fold_value_in"])
    interp.set_normal_constraints(g["fd_fold_normal_in"])
    report = interp.setup_interpolator(regularisation=0.05, cpw=1.0, npw=1.0, fold_weights=fold_case_weights())
    return interp, report


def test_fd_fold_interpolator_matches_reference(dgolden):
    interp, report = _fold_interp(dgolden)
    names = [str(s) for s in dgolden["fd_fold_family_names"]]
    assert set(report) == set(names)
    for nm in names:
        got = _rows(interp, nm)
        np.testing.assert_array_equal(got["idc"], dgolden[f"fd_fold_fam_{nm}_idc"], err_msg=nm)
        m = _csr(got["idc"], got["A"], interp.dof)
        np.testing.assert_allclose(m.data, dgolden[f"fd_fold_fam_{nm}_data"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["B"], dgolden[f"fd_fold_fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["w"], dgolden[f"fd_fold_fam_{nm}_w"], rtol=1e-15, atol=0, err_msg=nm)
        assert report[nm] == got["idc"].shape[0], nm
    system = interp._build_system()
    _g, cs = fd_fold_oracle(dgolden)
    A, _b = cs.matrix()
    _check_operator(system, A, x_seed=9)
    system.close()
    for prec, pc, tol in (("mixed", "mg", 1e-8), ("fp64", "jacobi", 1e-6)):
        assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-14, "atol": 0.0, "precision": prec,
                                                        "preconditioner": pc, "maxiter": 400000})
        ref = dgolden["fd_fold_c_direct"]
        err = np.linalg.norm(interp.c - ref) / np.linalg.norm(ref)
        assert err <= tol, (prec, err, interp.get_last_solve_timing())


def test_fd_fold_needs_a_fold():
    interp = L.FDFoldInterpolator(_grid((4, 4, 4)))
    with pytest.raises(RuntimeError):
        interp.setup_interpolator()
    interp.fold = SyntheticFold()
    with pytest.raises(ValueError):
        interp.setup_interpolator(fold_weights={"dgz_alignment": "sideways"})
