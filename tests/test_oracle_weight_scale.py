"""Pin the oracle's ``use_regularisation_weight_scale`` against fixtures
recorded from the reference (make_golden.py --weight-scale): the per-node
scale (KD-tree distances to the normal constraints inside the support),
every family's rows and per-row weights, and the direct solution, for FD with
the default sigma and with a small one, and for P1.  CPU only."""
import numpy as np
import pytest

from oracle import fd_oracle as fdo
from oracle import p1_oracle as p1o
from test_oracle_golden import _family_csr


@pytest.fixture(scope="module")
def wgolden():
    import os

    root = os.path.dirname(os.path.abspath(__file__))
    return np.load(os.path.join(root, "golden", "weight_scale_golden.npz"), allow_pickle=False)


def _check(g, prefix, cs, dof):
    assert list(cs.families) == [str(s) for s in g[f"{prefix}_family_names"]]
    for nm in cs.families:
        fam = cs.families[nm]
        np.testing.assert_array_equal(fam["idc"], g[f"{prefix}_fam_{nm}_idc"].reshape(fam["idc"].shape), err_msg=nm)
        m = _family_csr(fam, dof)
        np.testing.assert_allclose(m.data, g[f"{prefix}_fam_{nm}_data"], rtol=1e-15, atol=1e-15, err_msg=nm)
        np.testing.assert_allclose(fam["w"], g[f"{prefix}_fam_{nm}_w"], rtol=1e-14, atol=0, err_msg=nm)


@pytest.mark.parametrize("name", ["ws_fd_default", "ws_fd_sigma"])
def test_fd_weight_scale(wgolden, name):
    g = wgolden
    cells = g[f"{name}_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    sig = float(g[f"{name}_sigma"][0])
    sigma = None if np.isnan(sig) else sig
    data = {"value": g[f"{name}_value"], "normal": g[f"{name}_normal"]}
    np.testing.assert_allclose(fdo.regularisation_scale(grid, data["normal"], sigma), g[f"{name}_scale"],
                               rtol=1e-15, atol=0)
    cs = fdo.assemble(grid, data, fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0), weight_scale=True,
                      weight_sigma=sigma)
    _check(g, name, cs, grid.n_nodes)
    np.testing.assert_allclose(fdo.solve_direct(*cs.matrix()), g[f"{name}_c_direct"], rtol=0,
                               atol=1e-9 * np.abs(g[f"{name}_c_direct"]).max())


def test_p1_weight_scale(wgolden):
    g = wgolden
    cells = g["ws_p1_cells"]
    mesh = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {"value": g["ws_p1_value"], "normal": g["ws_p1_normal"]}
    np.testing.assert_allclose(p1o.regularisation_scale(mesh, data["normal"], 0.2), g["ws_p1_scale"], rtol=1e-15,
                               atol=0)
    cs = p1o.assemble(mesh, data, p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0), weight_scale=True,
                      weight_sigma=0.2)
    _check(g, "ws_p1", cs, mesh.n_nodes)
    np.testing.assert_allclose(fdo.solve_direct(*cs.matrix()), g["ws_p1_c_direct"], rtol=0,
                               atol=1e-9 * np.abs(g["ws_p1_c_direct"]).max())


def test_p1_tangent_and_orthogonal_rows(wgolden):
    """P1 tangent constraints and gradient-orthogonal rows with a target
    (P1:248-296): weight = w x the tetrahedron's volume."""
    g = wgolden
    cells = g["p1_orth_cells"]
    mesh = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {"value": g["p1_orth_value"], "tangent": g["p1_orth_tangent"]}
    cs = p1o.assemble(mesh, data, p1o.resolve_weights(cgw=0.1, cpw=1.0, tpw=2.0))
    p1o.add_gradient_orthogonal_constraints(mesh, cs, g["p1_orth_orth_points"], g["p1_orth_orth_vectors"], w=0.7,
                                            b=0.3, name="orth")
    # the reference's family order: edge jumps, value, tangent, then "orth"
    order = ["edge jump", "value", "undefined gradient orthogonal constraint", "orth"]
    assert list(cs.families) == order == [str(s) for s in g["p1_orth_family_names"]]
    _check(g, "p1_orth", cs, mesh.n_nodes)
    np.testing.assert_allclose(fdo.solve_direct(*cs.matrix()), g["p1_orth_c_direct"], rtol=0,
                               atol=1e-9 * np.abs(g["p1_orth_c_direct"]).max())
