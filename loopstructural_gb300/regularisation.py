"""Regularisation configuration: an isotropic weight plus directional terms.

Mirrors the reference's ``loop_interpolation/_regularisation.py``
(``DirectionalRegularisation``, ``RegularisationConfig``,
``coerce_regularisation_config``): the same accepted forms and the same
errors, so that ``setup_interpolator(regularisation=..., directional_regularisation=...)``
takes exactly what the reference takes.  Objects of the reference's own
classes are accepted too (anything with ``weight`` / ``direction`` / ``name``
attributes, or ``isotropic`` / ``directional`` for a whole configuration).
"""
from __future__ import annotations

from collections.abc import Sequence
from dataclasses import dataclass
from typing import Callable, Union

import numpy as np

DirectionProvider = Union[np.ndarray, Callable[[np.ndarray], np.ndarray]]


@dataclass(frozen=True)
class DirectionalRegularisation:
    """One directional term: ``direction`` is an (n, 3) array sampled at the
    interpolator's regularisation sample points, or a callable that returns
    one from those points."""

    weight: float
    direction: DirectionProvider
    name: str = "directional regularisation"


@dataclass(frozen=True)
class RegularisationConfig:
    isotropic: float | None = None
    directional: tuple = ()


def _is_term(value) -> bool:
    return all(hasattr(value, k) for k in ("weight", "direction", "name"))


def _is_config(value) -> bool:
    return hasattr(value, "isotropic") and hasattr(value, "directional")


def _is_directional_mapping(value) -> bool:
    return isinstance(value, dict) and any(k in value for k in ("direction", "vector", "weight", "name"))


def _coerce_term(value, index: int = 0, default_name: str = "directional regularisation"):
    if isinstance(value, DirectionalRegularisation) or _is_term(value):
        return value
    if isinstance(value, dict):
        direction = value.get("direction", value.get("vector", None))
        if direction is None:
            raise ValueError("Directional regularisation entries require 'direction' or 'vector'")
        weight = value.get("weight", None)
        if weight is None:
            raise ValueError("Directional regularisation entries require 'weight'")
        return DirectionalRegularisation(weight=float(weight), direction=direction,
                                         name=value.get("name", f"{default_name} {index + 1}"))
    raise TypeError("Directional regularisation must be a DirectionalRegularisation or dict entry")


def coerce_directional_regularisation(value, default_name: str = "directional regularisation") -> tuple:
    if value is None:
        return ()
    if isinstance(value, (DirectionalRegularisation, dict)) or _is_term(value):
        return (_coerce_term(value, default_name=default_name),)
    if isinstance(value, Sequence) and not isinstance(value, (str, bytes, np.ndarray)):
        if len(value) == 0:
            return ()
        if all(np.isscalar(item) for item in value):
            raise TypeError("A sequence of scalars is not a valid directional regularisation config")
        return tuple(_coerce_term(item, index=i, default_name=default_name) for i, item in enumerate(value))
    raise TypeError("Unsupported directional regularisation configuration")


def coerce_regularisation_config(regularisation=None, directional_regularisation=None) -> RegularisationConfig:
    """Isotropic weight and directional terms from the forms the reference
    accepts: a scalar, a config object, a single directional mapping, or a
    dict with ``isotropic`` / ``weight`` and ``directional`` keys; plus the
    separate ``directional_regularisation`` argument (appended)."""
    isotropic = None
    directional = ()
    if isinstance(regularisation, RegularisationConfig) or _is_config(regularisation):
        isotropic = regularisation.isotropic
        directional = tuple(regularisation.directional)
    elif np.isscalar(regularisation) and regularisation is not None:
        isotropic = float(regularisation)
    elif _is_directional_mapping(regularisation):
        directional = coerce_directional_regularisation(regularisation)
    elif isinstance(regularisation, dict):
        iso = regularisation.get("isotropic", regularisation.get("weight", None))
        if iso is not None and "direction" not in regularisation and "vector" not in regularisation:
            isotropic = float(iso)
        directional = coerce_directional_regularisation(regularisation.get("directional", ()))
    elif regularisation is not None:
        raise TypeError("Unsupported regularisation configuration")
    if directional_regularisation is not None:
        directional = directional + coerce_directional_regularisation(directional_regularisation)
    return RegularisationConfig(isotropic=isotropic, directional=directional)
