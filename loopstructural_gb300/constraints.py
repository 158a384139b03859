"""Constraint-array validation with the reference's contract.

Mirrors ``constraints.py`` / ``_validation.py`` of loop_interpolation
(ValueConstraint.from_array :128-188, GradientConstraint.from_array :191-287,
the NaN handling contract of _validation.py:1-15):
  * value / interface arrays have 4 or 5 columns  [x, y, z, v|id, (w)]
  * gradient / normal / tangent arrays have 6 or 7 [x, y, z, gx, gy, gz, (w)]
  * a NaN weight becomes 1.0 (warning); rows with NaN/inf position or data are
    dropped (warning); gradient-type rows with |g| < 1e-14 are dropped.
  * inequality arrays [x, y, z, lower, upper, (w)] and inequality pair arrays
    [x, y, z, pair_id, (w)] (InequalityConstraint :289-350, InequalityPair
    :352-407) must be finite instead (FiniteValueError), with lower < upper.
Errors raise the reference's exception types (all subclasses of ValueError).
"""
from __future__ import annotations

import logging

import numpy as np

logger = logging.getLogger(__name__)


class ValidationError(ValueError):
    """Base exception for constraint validation errors."""


class ShapeError(ValidationError):
    pass


class DtypeError(ValidationError):
    pass


class FiniteValueError(ValidationError):
    pass


class VectorError(ValidationError):
    pass


def _as_float(points, name):
    try:
        arr = np.asarray(points, dtype=float)
    except (TypeError, ValueError) as e:
        raise DtypeError(f"{name} could not be converted to float64. Error: {e}") from e
    if arr.ndim != 2:
        raise ShapeError(f"{name} must be 2D")
    return arr


def _fill_weights(arr, col):
    bad = ~np.isfinite(arr[:, col])
    if np.any(bad):
        logger.warning("%d NaN weight value(s) replaced with 1.0 (default weight).", int(bad.sum()))
        arr = arr.copy()
        arr[bad, col] = 1.0
    return arr


def _drop_bad_rows(arr, ncols_data, name):
    bad = ~np.isfinite(arr[:, :ncols_data]).all(axis=1)
    if np.any(bad):
        logger.warning("%d %s row(s) dropped: position or data columns contain NaN or inf.", int(bad.sum()), name)
        arr = arr[~bad]
    return arr


def value_array(points, dimensions: int = 3, name: str = "Value constraint") -> np.ndarray:
    """[x, y, z, v, w] (weight 1.0 appended when absent)."""
    arr = _as_float(points, f"{name} array")
    if arr.shape[1] == dimensions + 1:
        arr = np.hstack([arr, np.ones((arr.shape[0], 1))])
    elif arr.shape[1] != dimensions + 2:
        raise ShapeError(f"{name} array must have {dimensions + 1} or {dimensions + 2} columns")
    arr = _fill_weights(arr, dimensions + 1)
    arr = _drop_bad_rows(arr, dimensions + 1, name.lower())
    return np.ascontiguousarray(arr)


def gradient_array(points, dimensions: int = 3, is_normal: bool = False, name: str | None = None) -> np.ndarray:
    """[x, y, z, gx, gy, gz, w] (weight 1.0 appended when absent)."""
    label = name or ("Normal" if is_normal else "Gradient")
    arr = _as_float(points, f"{label} constraint array")
    if arr.shape[1] == 2 * dimensions:
        arr = np.hstack([arr, np.ones((arr.shape[0], 1))])
    elif arr.shape[1] != 2 * dimensions + 1:
        raise ShapeError(f"Gradient constraint array must have {2 * dimensions} or {2 * dimensions + 1} columns")
    arr = _fill_weights(arr, 2 * dimensions)
    arr = _drop_bad_rows(arr, 2 * dimensions, f"{label.lower()} constraint")
    mag = np.linalg.norm(arr[:, dimensions:2 * dimensions], axis=1)
    zero = mag < 1e-14
    if np.any(zero):
        logger.warning("Dropping %d %s constraints with zero or near-zero magnitude vectors.", int(zero.sum()),
                       label.lower())
        arr = arr[~zero]
    return np.ascontiguousarray(arr)


def _check_finite(arr, name):
    bad = ~np.isfinite(arr)
    if np.any(bad):
        raise FiniteValueError(f"{name} contains {int(bad.sum())} non-finite values (NaN or inf). "
                               f"All constraint values must be finite. Found at indices: {np.where(bad)}")


def _weights(col, label):
    w = np.array(col, dtype=float)
    bad = ~np.isfinite(w)
    if np.any(bad):
        logger.warning("%d NaN weight value(s) replaced with 1.0 (default weight). Provide explicit finite weights to "
                       "suppress this warning.", int(bad.sum()))
        w[bad] = 1.0
    _check_finite(w, f"{label} weights")
    return w


def inequality_array(points, dimensions: int = 3) -> np.ndarray:
    """[x, y, z, lower, upper, w] (constraints.py:289-350 InequalityConstraint):
    every position and bound finite, lower < upper on every row."""
    arr = _as_float(points, "Inequality constraint array")
    d = dimensions
    if arr.shape[1] == d + 2:
        w = np.ones(arr.shape[0])
    elif arr.shape[1] == d + 3:
        w = _weights(arr[:, d + 2], "Inequality constraint")
    else:
        raise ShapeError(f"Inequality constraint array must have {d + 2} or {d + 3} columns")
    pts, bounds = arr[:, :d], arr[:, d:d + 2]
    _check_finite(pts, "Position (X, Y, Z)")
    _check_finite(bounds, "Bound values")
    invalid = bounds[:, 0] >= bounds[:, 1]
    if np.any(invalid):
        raise ValidationError(
            f"Found {int(invalid.sum())} inequality constraints with lower_bound >= upper_bound. "
            "For each constraint, lower_bound must be strictly less than upper_bound. "
            f"Invalid constraints at indices: {np.where(invalid)[0]}")
    return np.ascontiguousarray(np.column_stack([pts, bounds, w]))


def inequality_pair_array(points, dimensions: int = 3) -> np.ndarray:
    """[x, y, z, pair_id, w] (constraints.py:352-407 InequalityPair)."""
    arr = _as_float(points, "Inequality pair constraint array")
    d = dimensions
    if arr.shape[1] == d + 1:
        w = np.ones(arr.shape[0])
    elif arr.shape[1] == d + 2:
        w = _weights(arr[:, d + 1], "Inequality pairs constraint")
    else:
        raise ShapeError(f"Inequality pair array must have {d + 1} or {d + 2} columns")
    _check_finite(arr[:, :d], "Position (X, Y, Z)")
    _check_finite(arr[:, d], "Pair id column")
    return np.ascontiguousarray(np.column_stack([arr[:, :d + 1], w]))
