"""GPU parity at the benchmark configurations' sizes, through the mirror of
the reference's interpolator API (setters, setup_interpolator, solve_system,
evaluate_value / evaluate_gradient), against fixtures recorded from the
unmodified reference (make_golden.py --configs):

* configuration 1 exactly: 50^3 nodes, 200 values, 50 noisy normals,
  regularisation 0.1;
* an FD interpolator whose support the reference's factory built from a
  BoundingBox with a shifted origin (local frame, non-unit cells), the data and
  queries given in world coordinates and projected by the box;
* a StructuredGrid with a shifted origin and a different cell size per axis;
* P1 on a TetMesh of 16^3 cells.

Bars: indices bit-exact; row values 1e-15 relative; evaluation of the
reference's solution 1e-12; the solved field against the reference's tight CG
solution 1e-6 (FP64 Jacobi-CG) and 1e-8 (mixed FP32 + FP64 refinement),
relative 2-norm over the evaluation points."""
import numpy as np
import pytest
from scipy import sparse

torch = pytest.importorskip("torch")

import bench  # noqa: E402
import loopstructural_gb300 as L  # noqa: E402
from conftest import AffineBox  # noqa: E402

pytestmark = pytest.mark.gpu

FIELD_TOL = {"fp64": 1e-6, "mixed": 1e-8}


def _csr(idc, A, dof):
    n, k = A.shape
    m = sparse.coo_matrix((A.ravel(), (np.repeat(np.arange(n), k), idc.ravel())), shape=(n, dof)).tocsr()
    m.sort_indices()
    return m


def _check_point_families(g, prefix, interp):
    for nm in [str(s) for s in g[f"{prefix}point_family_names"]]:
        got = interp.constraints[nm].numpy()
        np.testing.assert_array_equal(got["idc"], g[f"{prefix}fam_{nm}_idc"], err_msg=nm)
        m = _csr(got["idc"], got["A"], interp.dof)
        np.testing.assert_array_equal(m.indptr, g[f"{prefix}fam_{nm}_indptr"], err_msg=nm)
        np.testing.assert_array_equal(m.indices, g[f"{prefix}fam_{nm}_indices"], err_msg=nm)
        np.testing.assert_allclose(m.data, g[f"{prefix}fam_{nm}_data"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(got["B"], g[f"{prefix}fam_{nm}_b"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_array_equal(got["w"], g[f"{prefix}fam_{nm}_w"], err_msg=nm)


def _field_error(v, ref):
    ok = np.isfinite(ref)
    return float(np.linalg.norm(v[ok] - ref[ok]) / np.linalg.norm(ref[ok]))


def _solve_kw(precision, rtol):
    kw = {"rtol": rtol, "atol": 0.0, "precision": precision, "maxiter": 400000}
    if precision == "fp64":
        kw["preconditioner"] = "jacobi"
    return kw


def _cfg1_interp():
    cells, val, nrm = bench.cfg1_workload()
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.setup_interpolator(regularisation=bench.REGULARISATION, cpw=1.0, npw=1.0)
    return interp


def _cfg1_points(g):
    n = bench.CFG1_LATTICE
    ax = np.linspace(0.0, 1.0, n)
    i, j, k = np.unravel_index(g["cfg1_lattice_pick"], (n, n, n), order="F")
    return np.column_stack([ax[i], ax[j], ax[k]])


def test_cfg1_families_and_evaluation(cgolden):
    interp = _cfg1_interp()
    _check_point_families(cgolden, "cfg1_", interp)
    names = [str(s) for s in cgolden["cfg1_all_family_names"]]
    assert list(interp.family_order) == names
    rows = dict(zip(names, cgolden["cfg1_all_family_rows"]))
    for nm in names:
        got = interp.constraints[nm].n_rows if nm in interp.constraints else interp.regularisation_families[nm][0]
        assert got == rows[nm], nm
    # evaluation of the reference's solution on the 100^3 lattice sample (the
    # interpolator is marked solved, so that evaluate does not re-solve)
    interp.c = cgolden["cfg1_c_tight"]
    interp.up_to_date = True
    q = _cfg1_points(cgolden)
    np.testing.assert_allclose(interp.evaluate_value(q), cgolden["cfg1_eval_value"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(interp.evaluate_gradient(q), cgolden["cfg1_eval_gradient"], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cfg1_solution_matches_reference(cgolden, precision):
    interp = _cfg1_interp()
    assert interp.solve_system("cg", solver_kwargs=_solve_kw(precision, 1e-12))
    t = interp.get_last_solve_timing()
    assert t["status"] == 0, t
    err = _field_error(interp.evaluate_value(_cfg1_points(cgolden)), cgolden["cfg1_eval_value"])
    assert err <= FIELD_TOL[precision], (precision, err, t["iterations"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_factory_bounding_box_case(cgolden, precision):
    g = cgolden
    grid = L.StructuredGrid(origin=g["fac_origin"], nsteps=g["fac_nsteps"] - 1, step_vector=g["fac_step"])
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.bounding_box = AffineBox(g["fac_world_to_local"], g["fac_local_to_world"], g["fac_local_rotation"])
    interp.set_value_constraints(g["fac_value_in"])
    interp.set_normal_constraints(g["fac_normal_in"])
    interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
    np.testing.assert_allclose(interp.data["value"], g["fac_data_value"], rtol=1e-14, atol=1e-12)
    np.testing.assert_allclose(interp.data["normal"], g["fac_data_normal"], rtol=1e-14, atol=1e-12)
    _check_point_families(g, "fac_", interp)
    assert interp.solve_system("cg", solver_kwargs=_solve_kw(precision, 1e-13))
    err = _field_error(interp.evaluate_value(g["fac_query"]), g["fac_eval_value"])
    assert err <= FIELD_TOL[precision], (precision, err)
    # world-frame evaluation of the reference's solution (projection, then the
    # gradient reprojected)
    interp.c = g["fac_c_tight"]
    np.testing.assert_allclose(interp.evaluate_value(g["fac_query"]), g["fac_eval_value"], rtol=1e-12, atol=1e-12,
                               equal_nan=True)
    ref = g["fac_eval_gradient"]
    np.testing.assert_allclose(interp.evaluate_gradient(g["fac_query"]), ref, rtol=1e-12,
                               atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_anisotropic_grid_case(cgolden, precision):
    g = cgolden
    grid = L.StructuredGrid(origin=g["ani_origin"], nsteps=g["ani_cells"], step_vector=g["ani_step"])
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(g["ani_value_in"])
    interp.set_normal_constraints(g["ani_normal_in"])
    interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
    _check_point_families(g, "ani_", interp)
    assert interp.solve_system("cg", solver_kwargs=_solve_kw(precision, 1e-13))
    err = _field_error(interp.evaluate_value(g["ani_query"]), g["ani_eval_value"])
    assert err <= FIELD_TOL[precision], (precision, err)
    interp.c = g["ani_c_tight"]
    np.testing.assert_allclose(interp.evaluate_value(g["ani_query"]), g["ani_eval_value"], rtol=1e-12, atol=1e-12,
                               equal_nan=True)
    np.testing.assert_allclose(interp.evaluate_gradient(g["ani_query"]), g["ani_eval_gradient"], rtol=1e-12,
                               atol=1e-12)


def test_p1_config_case(cgolden):
    g = cgolden
    cells = g["p1c_cells"]
    mesh = L.TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))
    interp = L.P1Interpolator(mesh)
    interp.set_value_constraints(g["p1c_value_in"])
    interp.set_normal_constraints(g["p1c_normal_in"])
    interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0)
    _check_point_families(g, "p1c_", interp)
    face = interp.constraints["edge jump"].numpy()
    idc, A = face["idc"], face["A"]
    assert idc.shape[0] == int(g["p1c_face_rows"])
    rw = (np.arange(idc.shape[0], dtype=np.int64) % 1009) + 1
    assert int(np.sum(idc * (np.arange(idc.shape[1]) + 1)[None, :] * rw[:, None])) == int(g["p1c_face_idc_checksum"])
    sub = g["p1c_face_sub_rows"]
    si = idc[sub]
    np.testing.assert_array_equal(si, g["p1c_face_sub_idc"])
    vals = np.einsum("rkj,rj->rk", (si[:, :, None] == si[:, None, :]).astype(float), A[sub])
    ref = g["p1c_face_sub_vals"]
    sign = np.sign(np.sum(vals * ref, axis=1))[:, None]  # the face normal's orientation
    np.testing.assert_allclose(vals * sign, ref, rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(face["w"][sub], g["p1c_face_w"])
    assert interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "precision": "mixed",
                                                    "maxiter": 400000})
    err = _field_error(interp.evaluate_value(g["p1c_query"]), g["p1c_eval_value"])
    assert err <= FIELD_TOL["mixed"], err
    interp.c = g["p1c_c_tight"]
    np.testing.assert_allclose(interp.evaluate_value(g["p1c_query"]), g["p1c_eval_value"], rtol=1e-12, atol=1e-12,
                               equal_nan=True)
    np.testing.assert_allclose(interp.evaluate_gradient(g["p1c_query"]), g["p1c_eval_gradient"], rtol=1e-12,
                               atol=1e-12)
