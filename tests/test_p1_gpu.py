"""GPU parity of the P1 (TetMesh) path against the reference's golden vectors
and the oracle.  Tolerances: indices bit-exact; row values 1e-15 relative
(face rows up to the row sign: the normal's orientation follows the order of
the three shared nodes, which the reference takes from an unstable sort; the
sign does not change A^T W A); evaluation 1e-12; solutions 1e-8 (mixed) /
1e-6 (FP64) vs the FP64 direct solve."""
import numpy as np
import pytest
from scipy import sparse

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import p1  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402
from oracle import p1_oracle as p1o  # noqa: E402

pytestmark = pytest.mark.gpu


def _mesh(golden):
    cells = golden["p1_small_cells"]
    return L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))


def _interp(golden):
    interp = L.P1Interpolator(_mesh(golden))
    interp.set_value_constraints(golden["p1_small_value_in"])
    interp.set_normal_constraints(golden["p1_small_normal_in"])
    interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0)
    return interp


def _csr(idc, A, dof):
    n, k = A.shape
    m = sparse.coo_matrix((A.ravel(), (np.repeat(np.arange(n), k), idc.ravel())), shape=(n, dof)).tocsr()
    m.sort_indices()
    return m


def test_face_table_matches_reference(golden):
    mesh = _mesh(golden)
    idc, a, b, w, pairs, shared = p1.face_rows(mesh, 0.1, with_topology=True)
    np.testing.assert_array_equal(pairs.cpu().numpy(), golden["p1_small_shared_rel"])
    np.testing.assert_array_equal(np.sort(shared.cpu().numpy(), axis=1), np.sort(golden["p1_small_shared_nodes"], axis=1))


def test_p1_families_match_reference(golden):
    interp = _interp(golden)
    names = [str(s) for s in golden["p1_small_family_names"]]
    assert list(interp.constraints) == names
    for nm in names:
        got = interp.constraints[nm].numpy()
        np.testing.assert_array_equal(got["idc"], golden[f"p1_small_fam_{nm}_idc"], err_msg=nm)
        m = _csr(got["idc"], got["A"], interp.dof)
        np.testing.assert_array_equal(m.indptr, golden[f"p1_small_fam_{nm}_indptr"], err_msg=nm)
        np.testing.assert_array_equal(m.indices, golden[f"p1_small_fam_{nm}_indices"], err_msg=nm)
        ref = golden[f"p1_small_fam_{nm}_data"]
        data = m.data
        if nm == "edge jump":
            sign = np.sign(np.add.reduceat(data * ref, m.indptr[:-1]))
            data = data * np.repeat(sign, np.diff(m.indptr))
        np.testing.assert_allclose(data, ref, rtol=1e-14, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["B"], golden[f"p1_small_fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_array_equal(got["w"], golden[f"p1_small_fam_{nm}_w"], err_msg=nm)


def test_p1_location_matches_reference(golden):
    q = golden["p1_small_query"][:-1]
    tet, bc = p1.locate(_mesh(golden), q)
    np.testing.assert_array_equal(tet, golden["p1_small_loc_tet"])
    np.testing.assert_array_equal(tet >= 0, golden["p1_small_loc_inside"])
    np.testing.assert_allclose(bc, golden["p1_small_loc_bc"], rtol=1e-14, atol=1e-14, equal_nan=True)


def test_p1_evaluation_matches_reference(golden):
    mesh = _mesh(golden)
    q = golden["p1_small_query"]
    c = golden["p1_small_c_direct"]
    v, g = p1.eval_points(mesh, c, q)
    np.testing.assert_allclose(v, golden["p1_small_eval_value"], rtol=1e-13, atol=1e-13, equal_nan=True)
    np.testing.assert_allclose(g[:-1], golden["p1_small_eval_gradient"][:-1], rtol=1e-12, atol=1e-12, equal_nan=True)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-6), ("mixed", 1e-8)])
def test_p1_solution_matches_direct_solve(golden, precision, tol):
    interp = _interp(golden)
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-14, "atol": 0.0, "precision": precision,
                                                    "maxiter": 200000})
    ref = golden["p1_small_c_direct"]
    err = np.linalg.norm(interp.c - ref) / np.linalg.norm(ref)
    assert err <= tol, (precision, err, interp.get_last_solve_timing())


def test_p1_operator_matches_oracle():
    cells = np.array([6, 5, 7])
    mesh = L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells)
    rng = np.random.default_rng(2)
    vp = rng.uniform(0, 1, size=(50, 3))
    val = np.column_stack([vp, vp[:, 2], np.ones(50)])
    interp = L.P1Interpolator(mesh)
    interp.set_value_constraints(val)
    interp.setup_interpolator(cgw=0.1, cpw=1.0)
    system = interp._build_system()
    om = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells)
    cs = p1o.assemble(om, {"value": val}, p1o.resolve_weights(cgw=0.1, cpw=1.0))
    A, b = cs.matrix()
    N, rhs = fdo.normal_equations(A, b)
    x = rng.normal(size=om.n_nodes)
    ref = N @ x
    got = system.apply(torch.from_numpy(x)).cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    np.testing.assert_allclose(system.rhs().cpu().numpy(), rhs, rtol=1e-12, atol=1e-12 * np.max(np.abs(rhs)))
    system.close()
