"""Host-side logic of the drop-in interpolators (no GPU): validation,
geometry and weight handling, mirroring the reference's tests
(test_input_validation.py, test_discrete_supports.py, test_regularisation_api.py)."""
import numpy as np
import pytest

import loopstructural_gb300 as L
from loopstructural_gb300 import constraints as cons
from oracle import fd_oracle as fdo


def test_value_array_contract():
    arr = cons.value_array(np.array([[0.1, 0.2, 0.3, 1.0]]))
    assert arr.shape == (1, 5) and arr[0, 4] == 1.0
    arr = cons.value_array(np.array([[0.1, 0.2, 0.3, 1.0, np.nan], [0.1, np.nan, 0.3, 1.0, 2.0]]))
    assert arr.shape == (1, 5) and arr[0, 4] == 1.0  # NaN weight -> 1, NaN row dropped
    with pytest.raises(cons.ShapeError):
        cons.value_array(np.zeros((3, 7)))
    with pytest.raises(cons.DtypeError):
        cons.value_array([["a", "b", "c", "d"]])
    with pytest.raises(ValueError):
        cons.value_array(np.zeros(5))


def test_gradient_array_contract():
    arr = cons.gradient_array(np.array([[0, 0, 0, 0, 0, 1.0], [0, 0, 0, 0, 0, 0.0]]), is_normal=True)
    assert arr.shape == (1, 7)  # zero-magnitude vector dropped, weight appended
    with pytest.raises(cons.ShapeError):
        cons.gradient_array(np.zeros((2, 5)))


def test_setters_store_validated_arrays():
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.array([4, 4, 4]), step_vector=np.ones(3) * 0.25)
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0], [np.nan, 0.5, 0.5, 1.0]]))
    assert interp.get_value_constraints().shape == (1, 5)
    interp.set_normal_constraints(np.array([[0.5, 0.5, 0.5, 0, 0, 1.0, 2.0]]))
    assert interp.get_norm_constraints()[0, 6] == 2.0
    with pytest.raises(L.ValidationError):
        interp.set_value_constraints(np.zeros((2, 9)))
    assert interp.interpolation_weights["npw"] == 10.0  # FD default (reference FD:115)


def test_grid_geometry_matches_oracle():
    grid = L.StructuredGrid(origin=np.array([0.1, -0.2, 0.3]), nsteps=np.array([5, 3, 4]),
                            step_vector=np.array([0.5, 0.25, 1.0]))
    ref = fdo.Grid(np.array([0.1, -0.2, 0.3]), (5, 3, 4), np.array([0.5, 0.25, 1.0]))
    assert grid.n_nodes == ref.n_nodes == 6 * 4 * 5
    np.testing.assert_array_equal(grid.nodes, ref.nodes)
    np.testing.assert_array_equal(grid.maximum, ref.maximum)
    rng = np.random.default_rng(0)
    p = rng.uniform(-1, 3, size=(500, 3))
    np.testing.assert_array_equal(grid.inside(p), ref.inside(p))


def test_support_rejects_bad_geometry():
    with pytest.raises(L.supports.LoopException):
        L.StructuredGrid(nsteps=np.array([0, 3, 3]))
    with pytest.raises(L.supports.LoopException):
        L.StructuredGrid(nsteps=np.array([-1, 3, 3]))


def test_no_gpu_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    grid = L.StructuredGrid(nsteps=np.array([4, 4, 4]))
    interp = L.FiniteDifferenceInterpolator(grid)
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0]]))
    with pytest.raises(L.ExtensionUnavailable):
        interp.setup_interpolator(regularisation=0.1)


def test_solver_option_mapping():
    grid = L.StructuredGrid(nsteps=np.array([4, 4, 4]))
    interp = L.FiniteDifferenceInterpolator(grid)
    s, o = interp._solver_options("cg", 1e-10, {})
    assert s == "cg" and o["atol"] == 1e-10 and o["rtol"] == 1e-5
    s, o = interp._solver_options("cg", 1e-10, {"atol": 1.0, "rtol": 1e-3})
    assert o["atol"] == 1.0 and o["rtol"] == 1e-3  # both given: tol ignored (reference SS:58)
    s, o = interp._solver_options("cg", 1e-10, {"atol": 1.0})
    assert o["atol"] == 1e-10  # reference quirk: tol overrides atol unless rtol is also given
    s, o = interp._solver_options("bogus", None, None)
    assert s == "cg"
    s, o = interp._solver_options("lsmr", 1e-8, None)
    assert s == "lsmr" and o["rtol"] == 1e-8
    s, (o, inner) = interp._solver_options("admm", None, {"admm_weight": 0.2, "nmajor": 7})
    assert s == "admm" and o["rho"] == 0.2 and o["nmajor"] == 7 and inner["preconditioner"] == "mg"
