"""Inequality data setters of the interpolator API (GI:464-522,
constraints.py:289-407): shapes, defaults and the reference's errors.  CPU
only (no device work happens in the setters)."""
import numpy as np
import pytest

import loopstructural_gb300 as L
from loopstructural_gb300 import constraints


def _interp():
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.array([4, 4, 4]), step_vector=np.full(3, 0.25))
    return L.FiniteDifferenceInterpolator(grid)


def test_value_inequality_shapes_and_weights():
    it = _interp()
    it.set_value_inequality_constraints(np.array([[0.1, 0.2, 0.3, 0.0, 1.0]]))
    np.testing.assert_array_equal(it.get_inequality_value_constraints(), [[0.1, 0.2, 0.3, 0.0, 1.0, 1.0]])
    it.set_value_inequality_constraints(np.array([[0.1, 0.2, 0.3, 0.0, 1.0, np.nan]]))
    assert it.get_inequality_value_constraints()[0, 5] == 1.0
    assert it.up_to_date is False


@pytest.mark.parametrize("arr, cause, msg", [
    (np.array([[0.1, 0.2, 0.3, 1.0, 1.0]]), constraints.ValidationError, "lower_bound >= upper_bound"),
    (np.array([[0.1, 0.2, np.nan, 0.0, 1.0]]), constraints.FiniteValueError, "Position (X, Y, Z)"),
    (np.array([[0.1, 0.2, 0.3, 0.0, np.inf]]), constraints.FiniteValueError, "Bound values"),
    (np.array([[0.1, 0.2, 0.3, 0.0]]), constraints.ShapeError, "must have 5 or 6 columns"),
    (np.array([0.1, 0.2, 0.3, 0.0, 1.0]), constraints.ShapeError, "must be 2D"),
])
def test_value_inequality_errors(arr, cause, msg):
    """The setter re-raises every validation error as ValidationError with a
    prefix; the original exception is the cause (GI:491-493)."""
    with pytest.raises(constraints.ValidationError) as e:
        _interp().set_value_inequality_constraints(arr)
    assert msg in str(e.value)
    assert str(e.value).startswith("Failed to set inequality value constraints: ")
    assert type(e.value.__cause__) is cause


def test_inequality_pairs_shapes_and_errors():
    it = _interp()
    it.set_inequality_pairs_constraints(np.array([[0.1, 0.2, 0.3, 0.0], [0.4, 0.5, 0.6, 1.0]]))
    assert it.get_inequality_pairs_constraints().shape == (2, 5)
    with pytest.raises(constraints.ValidationError) as e:
        it.set_inequality_pairs_constraints(np.array([[0.1, 0.2, 0.3, np.nan]]))
    assert "Pair id column" in str(e.value) and type(e.value.__cause__) is constraints.FiniteValueError
    with pytest.raises(constraints.ValidationError) as e:
        it.set_inequality_pairs_constraints(np.zeros((2, 7)))
    assert "must have 4 or 5 columns" in str(e.value)
    assert str(e.value).startswith("Failed to set inequality pairs constraints: ")


def test_add_inequality_constraints_to_matrix_checks():
    it = _interp()
    with pytest.raises(ValueError, match="same shape"):
        it.add_inequality_constraints_to_matrix(np.ones((2, 3)), np.zeros((2, 2)), np.zeros((2, 2), dtype=int))
    with pytest.raises(ValueError, match="bounds must have shape"):
        it.add_inequality_constraints_to_matrix(np.ones((2, 2)), np.zeros((3, 2)), np.zeros((2, 2), dtype=int))
    with pytest.raises(ValueError, match="out of range"):
        it.add_inequality_constraints_to_matrix(np.ones((1, 1)), np.zeros((1, 2)), np.array([[it.dof]]))


def test_admm_option_errors():
    from loopstructural_gb300 import admm

    with pytest.raises(ValueError, match="nmajor must be positive"):
        admm.admm_options({"nmajor": 0})
    with pytest.raises(ValueError, match="admm_weight_final must be > 0"):
        admm.admm_options({"admm_weight_final": -1.0})
    with pytest.raises(NotImplementedError):
        admm.admm_options({"active_set": True})
    o, inner = admm.admm_options({"admm_weight": 0.5, "linsys_solver": "cg", "rtol": 1e-9})
    assert o["rho"] == 0.5 and o["nmajor"] == 200 and inner["rtol"] == 1e-9
    np.testing.assert_allclose(admm.rho_schedule(dict(o, rho_final=2.0, nmajor=3)), [0.5, 1.0, 2.0])
