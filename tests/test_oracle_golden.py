"""Pin the CPU oracle against golden vectors recorded from the reference
implementation (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest
from scipy import sparse

from oracle import fd_oracle as fdo
from oracle import p1_oracle as p1o


def _weights(g, name):
    keys = [str(k) for k in g[f"{name}_weights_keys"]]
    vals = g[f"{name}_weights_vals"]
    return {k: float(v) for k, v in zip(keys, vals)}


def _fd_case(g, name):
    cells = g[f"{name}_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {k: g[f"{name}_data_{k}"] for k in ("value", "normal", "gradient", "tangent", "interface")}
    cs = fdo.assemble(grid, data, _weights(g, name))
    return grid, cs


def _family_csr(fam, dof):
    n, k = fam["A"].shape
    rows = np.repeat(np.arange(n), k)
    m = sparse.coo_matrix((fam["A"].ravel(), (rows, fam["idc"].ravel())), shape=(n, dof)).tocsr()
    m.sort_indices()
    return m


def _check_families(g, prefix, cs, dof, sign_free=()):
    names = [str(s) for s in g[f"{prefix}family_names"]]
    assert list(cs.families.keys()) == names
    for nm in names:
        fam = cs.families[nm]
        idc = g[f"{prefix}fam_{nm}_idc"]
        assert fam["idc"].dtype == np.int64
        np.testing.assert_array_equal(fam["idc"], idc, err_msg=nm)  # bit-exact indices
        m = _family_csr(fam, dof)
        np.testing.assert_array_equal(m.indptr, g[f"{prefix}fam_{nm}_indptr"], err_msg=nm)
        np.testing.assert_array_equal(m.indices, g[f"{prefix}fam_{nm}_indices"], err_msg=nm)
        ref = g[f"{prefix}fam_{nm}_data"]
        got = m.data
        if nm in sign_free:  # face rows: the sign follows the face node order
            rowsign = np.sign(np.add.reduceat(got * ref, m.indptr[:-1])) if got.size else got
            got = got * np.repeat(rowsign, np.diff(m.indptr))
        np.testing.assert_allclose(got, ref, rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(fam["B"], g[f"{prefix}fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_array_equal(fam["w"], g[f"{prefix}fam_{nm}_w"], err_msg=nm)


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_fd_families_match_reference(golden, name):
    grid, cs = _fd_case(golden, name)
    _check_families(golden, f"{name}_", cs, grid.n_nodes)


@pytest.mark.parametrize("cells", [(5, 5, 5), (3, 4, 2), (2, 5, 6)])
def test_regularisation_indices_match_reference(golden, cells):
    grid = fdo.Grid(np.zeros(3), cells, np.ones(3))
    w = fdo.resolve_weights(dxy=1.0, dyz=0.8, dxz=1.3, dxx=0.5, dyy=0.4, dzz=0.6, dx=0.7, dy=0.9, dz=1.1,
                            cpw=0.0, gpw=0.0, npw=0.0, tpw=0.0, ipw=0.0)
    cs = fdo.ConstraintSet(grid.n_nodes)
    fdo.add_regularisation(grid, cs, w)
    _check_families(golden, "reg_" + "x".join(str(c) for c in cells) + "_", cs, grid.n_nodes)


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_fd_direct_solution_matches_reference(golden, name):
    grid, cs = _fd_case(golden, name)
    A, b = cs.matrix()
    c = fdo.solve_direct(A, b)
    ref = golden[f"{name}_c_direct"]
    assert np.linalg.norm(c - ref) <= 1e-10 * np.linalg.norm(ref)
    # the reference's own tightly converged CG agrees with the direct solve
    cg = golden[f"{name}_c_cg_tight"]
    assert np.linalg.norm(cg - ref) <= 1e-6 * np.linalg.norm(ref)


@pytest.mark.parametrize("name", ["fd_small", "fd_cfg1_20"])
def test_fd_evaluation_matches_reference(golden, name):
    cells = golden[f"{name}_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    q = golden[f"{name}_query"]
    c = golden[f"{name}_c_direct"]
    v = fdo.evaluate_value_local(grid, q, c)
    gr = fdo.evaluate_gradient_local(grid, q, c)
    np.testing.assert_allclose(v, golden[f"{name}_eval_value"], rtol=1e-14, atol=1e-14, equal_nan=True)
    np.testing.assert_allclose(gr, golden[f"{name}_eval_gradient"], rtol=1e-13, atol=1e-13, equal_nan=True)


def test_fd_reference_cg_restatement_converges_like_reference(golden):
    grid, cs = _fd_case(golden, "fd_small")
    A, b = cs.matrix()
    c, flag, _ = fdo.solve_reference_cg(A, b, tol=0.0, rtol=1e-13, maxiter=200000)
    assert flag == 0
    ref = golden["fd_small_c_cg_tight"]
    assert np.linalg.norm(c - ref) <= 1e-8 * np.linalg.norm(ref)


def _p1_mesh(g):
    cells = g["p1_small_cells"]
    return p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))


def test_p1_geometry_matches_reference(golden):
    mesh = _p1_mesh(golden)
    np.testing.assert_array_equal(mesh.elements, golden["p1_small_elements"])
    np.testing.assert_array_equal(mesh.neighbours(), golden["p1_small_neighbours"])
    rel, shared = mesh.face_table()
    np.testing.assert_array_equal(rel, golden["p1_small_shared_rel"])
    # the three shared nodes of each face, as a set
    np.testing.assert_array_equal(np.sort(shared, axis=1), np.sort(golden["p1_small_shared_nodes"], axis=1))


def test_p1_families_match_reference(golden):
    mesh = _p1_mesh(golden)
    data = {"value": golden["p1_small_value_in"], "normal": golden["p1_small_normal_in"]}
    cs = p1o.assemble(mesh, data, p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0))
    _check_families(golden, "p1_small_", cs, mesh.n_nodes, sign_free=("edge jump",))


def test_p1_location_and_evaluation_match_reference(golden):
    mesh = _p1_mesh(golden)
    q = golden["p1_small_query"]
    _, bc, tet, inside = mesh.element_for_location(q[:-1])
    np.testing.assert_array_equal(inside, golden["p1_small_loc_inside"])
    np.testing.assert_array_equal(tet, golden["p1_small_loc_tet"])
    np.testing.assert_allclose(bc, golden["p1_small_loc_bc"], rtol=1e-14, atol=1e-14, equal_nan=True)
    c = golden["p1_small_c_direct"]
    np.testing.assert_allclose(mesh.evaluate_value(q[:-1], c), golden["p1_small_eval_value"][:-1], rtol=1e-13,
                               atol=1e-13, equal_nan=True)
    np.testing.assert_allclose(mesh.evaluate_gradient(q[:-1], c), golden["p1_small_eval_gradient"][:-1],
                               rtol=1e-12, atol=1e-12, equal_nan=True)


def test_p1_direct_solution_matches_reference(golden):
    mesh = _p1_mesh(golden)
    data = {"value": golden["p1_small_value_in"], "normal": golden["p1_small_normal_in"]}
    cs = p1o.assemble(mesh, data, p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0))
    A, b = cs.matrix()
    c = fdo.solve_direct(A, b)
    ref = golden["p1_small_c_direct"]
    assert np.linalg.norm(c - ref) <= 1e-9 * np.linalg.norm(ref)
