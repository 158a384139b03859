"""``use_regularisation_weight_scale`` on the GPU against fixtures recorded
from the reference (make_golden.py --weight-scale): the per-node scale
(ls_fd_weight_scale: exact nearest normal constraint, numpy linspace node
coordinates), every regularisation family's rows and per-row weights, the
operator against the oracle's explicit system, and the solution against the
reference's direct solve (FP64 CG 1e-6, mixed multigrid 1e-8 of the largest
coefficient).  FD with the default sigma and with a small one; P1."""
import numpy as np
import pytest
from scipy import sparse

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wgolden():
    import os

    root = os.path.dirname(os.path.abspath(__file__))
    return np.load(os.path.join(root, "golden", "weight_scale_golden.npz"), allow_pickle=False)


def _fd(g, name):
    cells = g[f"{name}_cells"]
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
    it = L.FiniteDifferenceInterpolator(grid)
    it.set_value_constraints(g[f"{name}_value"])
    it.set_normal_constraints(g[f"{name}_normal"])
    kw = dict(regularisation=0.1, cpw=1.0, npw=1.0, use_regularisation_weight_scale=True)
    sig = float(g[f"{name}_sigma"][0])
    if not np.isnan(sig):
        kw["regularisation_weight_sigma"] = sig
    it.setup_interpolator(**kw)
    return it


def _csr(idc, A, w, dof):
    n, k = A.shape
    keep = idc.reshape(-1) >= 0
    m = sparse.coo_matrix(((A * w[:, None]).reshape(-1)[keep], (np.repeat(np.arange(n), k)[keep],
                                                                idc.reshape(-1)[keep])), shape=(n, dof))
    return m.tocsr()


@pytest.mark.parametrize("name", ["ws_fd_default", "ws_fd_sigma"])
def test_fd_scale_rows_operator_and_solution(wgolden, name):
    g = wgolden
    it = _fd(g, name)
    np.testing.assert_allclose(it.regularisation_scale_array(), g[f"{name}_scale"], rtol=1e-14, atol=0)
    names = [str(s) for s in g[f"{name}_family_names"]]
    assert it.family_order == names
    for nm in names:
        fam = it._family_rows(nm)
        np.testing.assert_array_equal(fam["idc"], g[f"{name}_fam_{nm}_idc"].reshape(fam["idc"].shape), err_msg=nm)
        np.testing.assert_allclose(fam["w"], g[f"{name}_fam_{nm}_w"], rtol=1e-14, atol=0, err_msg=nm)
    # operator: the GPU normal matrix (matrix-free, scaled interior families in
    # the weight planes, scaled borders as data rows) against the explicit one
    A, b = it.build_matrix()
    N, rhs = fdo.normal_equations(A, b)
    sys_ = it._build_system()
    try:
        x = torch.from_numpy(np.random.default_rng(1).normal(size=it.dof)).cuda()
        y = sys_.apply(x).cpu().numpy()
        ref = N @ x.cpu().numpy()
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
        np.testing.assert_allclose(sys_.rhs().cpu().numpy(), rhs, rtol=1e-12, atol=1e-12 * np.abs(rhs).max())
    finally:
        sys_.close()
    c_ref = g[f"{name}_c_direct"]
    for kw, tol in ((dict(precision="fp64", preconditioner="jacobi"), 1e-6), (dict(precision="mixed"), 1e-8)):
        assert it.solve_system("cg", solver_kwargs=dict(rtol=1e-13, atol=0.0, maxiter=200000, **kw))
        assert np.abs(it.c - c_ref).max() <= tol * np.abs(c_ref).max(), kw


def test_p1_scale_rows_and_solution(wgolden):
    g = wgolden
    cells = g["ws_p1_cells"]
    mesh = L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))
    it = L.P1Interpolator(mesh)
    it.set_value_constraints(g["ws_p1_value"])
    it.set_normal_constraints(g["ws_p1_normal"])
    it.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0, use_regularisation_weight_scale=True,
                          regularisation_weight_sigma=0.2)
    np.testing.assert_allclose(it.regularisation_scale_array(), g["ws_p1_scale"], rtol=1e-14, atol=0)
    fam = it.constraints["edge jump"].numpy()
    np.testing.assert_allclose(fam["w"], g["ws_p1_fam_edge jump_w"], rtol=1e-14, atol=0)
    assert it.solve_system("cg", solver_kwargs=dict(rtol=1e-13, atol=0.0, maxiter=200000, precision="fp64"))
    c_ref = g["ws_p1_c_direct"]
    assert np.abs(it.c - c_ref).max() <= 1e-6 * np.abs(c_ref).max()


def test_fd_scale_at_96_cubed_nearest_point_exact():
    """96^3 nodes, 3,000 normal points: the GPU scale equals the reference's
    KD-tree weighting evaluated by the oracle (exact nearest point)."""
    rng = np.random.default_rng(4)
    n = 95
    grid = L.StructuredGrid(origin=np.array([10.0, -3.0, 2.5]), nsteps=np.array([n, n, n]),
                            step_vector=np.array([0.7, 0.5, 0.3]))
    it = L.FiniteDifferenceInterpolator(grid)
    lo, hi = grid.origin, grid.maximum
    pts = lo + (hi - lo) * rng.uniform(0, 1, size=(3000, 3))
    g = np.column_stack([np.zeros((3000, 2)), np.ones(3000)])
    it.set_normal_constraints(np.column_stack([pts, g]))
    it.set_value_constraints(np.column_stack([pts[:10], np.zeros(10)]))
    it.setup_interpolator(regularisation=0.1, use_regularisation_weight_scale=True, regularisation_weight_sigma=2.0)
    og = fdo.Grid(grid.origin, grid.nsteps_cells, grid.step_vector)
    ref = fdo.regularisation_scale(og, it.get_norm_constraints(), 2.0)
    np.testing.assert_allclose(it.regularisation_scale_array(), ref, rtol=1e-14, atol=0)


def test_p1_tangent_and_orthogonal_rows(wgolden):
    """P1 tangent constraints and gradient-orthogonal rows with a target
    (LS_ROWS_TANGENT / LS_ROWS_ORTHOGONAL on the TetMesh): rows, volume
    weights and the solution against the reference."""
    from test_oracle_golden import _family_csr

    g = wgolden
    cells = g["p1_orth_cells"]
    mesh = L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))
    it = L.P1Interpolator(mesh)
    it.set_value_constraints(g["p1_orth_value"])
    it.set_tangent_constraints(g["p1_orth_tangent"])
    it.setup_interpolator(cgw=0.1, cpw=1.0, tpw=2.0)
    vec = g["p1_orth_orth_vectors"].copy()
    it.add_gradient_orthogonal_constraints(g["p1_orth_orth_points"], vec, w=0.7, b=0.3, name="orth")
    np.testing.assert_array_equal(vec, g["p1_orth_orth_vectors"])  # the caller's array is left alone
    assert list(it.constraints) == [str(s) for s in g["p1_orth_family_names"]]
    for nm in it.constraints:
        fam = it.constraints[nm].numpy()
        np.testing.assert_array_equal(fam["idc"], g[f"p1_orth_fam_{nm}_idc"].reshape(fam["idc"].shape), err_msg=nm)
        m = _family_csr(fam, it.dof)
        ref = g[f"p1_orth_fam_{nm}_data"]
        if nm == "edge jump":  # face rows agree up to the row sign (the shared-node order)
            m.data, ref = np.abs(m.data), np.abs(ref)
        np.testing.assert_allclose(m.data, ref, rtol=1e-13, atol=1e-13, err_msg=nm)
        np.testing.assert_allclose(fam["B"], g[f"p1_orth_fam_{nm}_b"], rtol=1e-13, atol=1e-13, err_msg=nm)
        np.testing.assert_allclose(fam["w"], g[f"p1_orth_fam_{nm}_w"], rtol=1e-13, atol=0, err_msg=nm)
    # the diagonal (the reference's column scaling): face rows hold the shared
    # nodes twice, summed before squaring
    A, b = it.build_matrix()
    N, _rhs = fdo.normal_equations(A, b)
    sys_ = it._build_system()
    try:
        np.testing.assert_allclose(sys_.diagonal().cpu().numpy(), N.diagonal(), rtol=1e-12, atol=0)
    finally:
        sys_.close()
    assert it.solve_system("cg", solver_kwargs=dict(rtol=1e-13, atol=0.0, maxiter=200000, precision="fp64"))
    c_ref = g["p1_orth_c_direct"]
    assert np.abs(it.c - c_ref).max() <= 1e-6 * np.abs(c_ref).max()
