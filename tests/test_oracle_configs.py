"""Pin the CPU oracle against the fixtures recorded from the reference at the
benchmark configurations' sizes (make_golden.py --configs): configuration 1
(50^3 nodes), an FD interpolator built by the reference's factory from a
BoundingBox with a shifted origin, a grid with a different cell size per axis,
and P1 at 16^3 cells.  Point families bit-exact in their indices and 1e-15 in
their values; evaluation of the reference's solution 1e-13 (value) / 1e-12
(gradient).  CPU only."""
import numpy as np

from conftest import AffineBox
from oracle import fd_oracle as fdo
from oracle import p1_oracle as p1o
from test_oracle_golden import _family_csr


def _check_point_families(g, prefix, cs, dof, tol=1e-15):
    for nm in [str(s) for s in g[f"{prefix}point_family_names"]]:
        fam = cs.families[nm]
        np.testing.assert_array_equal(fam["idc"], g[f"{prefix}fam_{nm}_idc"], err_msg=nm)
        m = _family_csr(fam, dof)
        np.testing.assert_array_equal(m.indptr, g[f"{prefix}fam_{nm}_indptr"], err_msg=nm)
        np.testing.assert_array_equal(m.indices, g[f"{prefix}fam_{nm}_indices"], err_msg=nm)
        np.testing.assert_allclose(m.data, g[f"{prefix}fam_{nm}_data"], rtol=tol, atol=tol, err_msg=nm)
        np.testing.assert_allclose(fam["B"], g[f"{prefix}fam_{nm}_b"], rtol=tol, atol=tol, err_msg=nm)
        np.testing.assert_array_equal(fam["w"], g[f"{prefix}fam_{nm}_w"], err_msg=nm)


def _lattice_points(g, n=100):
    ax = np.linspace(0.0, 1.0, n)
    i, j, k = np.unravel_index(g["cfg1_lattice_pick"], (n, n, n), order="F")
    return np.column_stack([ax[i], ax[j], ax[k]])


def test_cfg1_point_families_and_evaluation(cgolden):
    import bench

    cells, val, nrm = bench.cfg1_workload()
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    cs = fdo.assemble(grid, {"value": val, "normal": nrm}, fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0))
    _check_point_families(cgolden, "cfg1_", cs, grid.n_nodes)
    assert list(cs.families.keys()) == [str(s) for s in cgolden["cfg1_all_family_names"]]
    assert [cs.families[k]["A"].shape[0] for k in cs.families] == list(cgolden["cfg1_all_family_rows"])
    q = _lattice_points(cgolden)
    c = cgolden["cfg1_c_tight"]
    np.testing.assert_allclose(fdo.evaluate_value_local(grid, q, c), cgolden["cfg1_eval_value"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(fdo.evaluate_gradient_local(grid, q, c), cgolden["cfg1_eval_gradient"], rtol=1e-12,
                               atol=1e-12)


def test_factory_case_projection_families_and_evaluation(cgolden):
    g = cgolden
    box = AffineBox(g["fac_world_to_local"], g["fac_local_to_world"], g["fac_local_rotation"])
    val = g["fac_value_in"].copy()
    val[:, :3] = box.project(val[:, :3])
    nrm = g["fac_normal_in"].copy()
    nrm[:, :3] = box.project(nrm[:, :3])
    nrm[:, 3:6] = box.project_vectors(nrm[:, 3:6])
    np.testing.assert_allclose(val, g["fac_data_value"], rtol=1e-14, atol=1e-12)
    np.testing.assert_allclose(nrm, g["fac_data_normal"], rtol=1e-14, atol=1e-12)
    assert np.all(g["fac_step"] > 1.0) and np.any(g["fac_origin"] != 0.0)  # non-unit cells, shifted origin
    grid = fdo.Grid(g["fac_origin"], g["fac_nsteps"] - 1, g["fac_step"])
    cs = fdo.assemble(grid, {"value": g["fac_data_value"], "normal": g["fac_data_normal"]},
                      fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0))
    _check_point_families(g, "fac_", cs, grid.n_nodes)
    q = box.project(g["fac_query"])
    c = g["fac_c_tight"]
    np.testing.assert_allclose(fdo.evaluate_value_local(grid, q, c), g["fac_eval_value"], rtol=1e-13, atol=1e-13,
                               equal_nan=True)
    grad = box.reproject_vectors(fdo.evaluate_gradient_local(grid, q, c))
    np.testing.assert_allclose(grad, g["fac_eval_gradient"], rtol=1e-12, atol=1e-12 * np.abs(grad).max())


def test_anisotropic_grid_families_and_evaluation(cgolden):
    g = cgolden
    grid = fdo.Grid(g["ani_origin"], g["ani_cells"], g["ani_step"])
    cs = fdo.assemble(grid, {"value": g["ani_value_in"], "normal": g["ani_normal_in"]},
                      fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0))
    _check_point_families(g, "ani_", cs, grid.n_nodes)
    q, c = g["ani_query"], g["ani_c_tight"]
    np.testing.assert_allclose(fdo.evaluate_value_local(grid, q, c), g["ani_eval_value"], rtol=1e-13, atol=1e-13,
                               equal_nan=True)
    np.testing.assert_allclose(fdo.evaluate_gradient_local(grid, q, c), g["ani_eval_gradient"], rtol=1e-12,
                               atol=1e-12)


def _summed_by_column(idc, A):
    """Row coefficients summed over duplicate columns (as a stored sparse
    matrix holds them), indexed like idc."""
    return np.einsum("rkj,rj->rk", (idc[:, :, None] == idc[:, None, :]).astype(float), A)


def test_p1_config_families(cgolden):
    g = cgolden
    cells = g["p1c_cells"]
    mesh = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))
    cs = p1o.assemble(mesh, {"value": g["p1c_value_in"], "normal": g["p1c_normal_in"]},
                      p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0))
    _check_point_families(g, "p1c_", cs, mesh.n_nodes)
    face = cs.families["edge jump"]
    idc = face["idc"]
    assert idc.shape[0] == int(g["p1c_face_rows"])
    rw = (np.arange(idc.shape[0], dtype=np.int64) % 1009) + 1
    assert int(np.sum(idc * (np.arange(idc.shape[1]) + 1)[None, :] * rw[:, None])) == int(g["p1c_face_idc_checksum"])
    sub = g["p1c_face_sub_rows"]
    np.testing.assert_array_equal(idc[sub], g["p1c_face_sub_idc"])
    vals = _summed_by_column(idc[sub], face["A"][sub])
    ref = g["p1c_face_sub_vals"]
    sign = np.sign(np.sum(vals * ref, axis=1))[:, None]  # the face normal's orientation
    np.testing.assert_allclose(vals * sign, ref, rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(face["w"][sub], g["p1c_face_w"])
