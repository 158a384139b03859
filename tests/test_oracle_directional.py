"""Pin the oracle's directional regularisation (FD:1207-1337, P1:115-178) and
gradient-orthogonal rows with a target (FD:478-539) against fixtures recorded
from the reference (tests/golden/make_golden.py --directional).  CPU only."""
import numpy as np

from oracle import fd_oracle as fdo
from oracle import p1_oracle as p1o

from golden.make_golden import SyntheticFold, _direction_field, fold_case_weights
from test_oracle_golden import _check_families


def fd_dir_case(g):
    """The fd_dir fixture's constraint set, built by the oracle."""
    cells = g["fd_dir_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {"value": g["fd_dir_value_in"], "normal": g["fd_dir_normal_in"]}
    w = fdo.resolve_weights(regularisation=0.1, cpw=1.0, npw=1.0)
    directional = [(0.5, g["fd_dir_dir_a"], "fold a"), (0.2, g["fd_dir_dir_b"], "fold b")]
    cs = fdo.assemble(grid, data, w, directional)
    fdo.add_gradient_orthogonal_constraints(grid, cs, g["fd_dir_orth_points"], g["fd_dir_orth_vectors"], 2.0, b=0.3,
                                            name="fold normalisation")
    return grid, cs


def p1_dir_case(g):
    cells = g["p1_dir_cells"]
    mesh = p1o.TetMesh(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {"value": g["p1_dir_value_in"]}
    cs = p1o.assemble(mesh, data, p1o.resolve_weights(cgw=0.1, cpw=1.0, npw=1.0), [(0.3, g["p1_dir_dir"], "fold p1")])
    return mesh, cs


def test_fd_directional_families_match_reference(dgolden):
    grid, cs = fd_dir_case(dgolden)
    # families with every row weight zero are absent (fold b has vx = 0)
    assert "fold b_dxx" not in cs.families and "fold b_dyy" in cs.families
    _check_families(dgolden, "fd_dir_", cs, grid.n_nodes)


def test_fd_directional_solution_matches_reference(dgolden):
    grid, cs = fd_dir_case(dgolden)
    A, b = cs.matrix()
    c = fdo.solve_direct(A, b)
    ref = dgolden["fd_dir_c_direct"]
    assert np.linalg.norm(c - ref) <= 1e-10 * np.linalg.norm(ref)


def test_p1_directional_families_match_reference(dgolden):
    mesh, cs = p1_dir_case(dgolden)
    # the recorded per-face vectors are a function of the reference's face
    # centres (P1:169-170): the oracle's centres reproduce them in face order
    np.testing.assert_allclose(_direction_field(p1o.face_centres(mesh)), dgolden["p1_dir_dir"], rtol=1e-14, atol=1e-15)
    _check_families(dgolden, "p1_dir_", cs, mesh.n_nodes, sign_free=("edge jump", "fold p1"))
    A, b = cs.matrix()
    c = fdo.solve_direct(A, b)
    ref = dgolden["p1_dir_c_direct"]
    assert np.linalg.norm(c - ref) <= 1e-9 * np.linalg.norm(ref)


def fd_fold_oracle(g):
    cells = g["fd_fold_cells"]
    grid = fdo.Grid(np.zeros(3), cells, 1.0 / cells.astype(float))
    data = {"value": g["fd_fold_value_in"], "normal": g["fd_fold_normal_in"]}
    cs = fdo.assemble(grid, data, fdo.resolve_weights(regularisation=0.05, cpw=1.0, npw=1.0))
    fdo.add_fold_constraints(grid, cs, SyntheticFold(), g["fd_fold_normal_in"], **fold_case_weights())
    return grid, cs


def test_fd_fold_families_and_solution_match_reference(dgolden):
    grid, cs = fd_fold_oracle(dgolden)
    _check_families(dgolden, "fd_fold_", cs, grid.n_nodes)
    A, b = cs.matrix()
    c = fdo.solve_direct(A, b)
    ref = dgolden["fd_fold_c_direct"]
    assert np.linalg.norm(c - ref) <= 1e-10 * np.linalg.norm(ref)
