"""Regularisation configuration: an isotropic weight plus directional terms.

``setup_interpolator(regularisation=..., directional_regularisation=...)``
accepts the forms the reference's ``loop_interpolation/_regularisation.py``
accepts, and rejects the others with the same exception types and messages:

* ``regularisation``: ``None``; a number (the isotropic weight); a
  configuration object (``isotropic`` + ``directional``); one directional
  entry written as a mapping (keys ``direction``/``vector``, ``weight``,
  ``name``); or a mapping with ``isotropic`` (alias ``weight``) and
  ``directional`` keys.
* ``directional_regularisation`` (appended to the terms above): ``None``; one
  term (object or mapping); or a sequence of terms.

Objects of the reference's own classes are accepted as well: a term is
anything carrying ``weight``, ``direction`` and ``name``, a configuration
anything carrying ``isotropic`` and ``directional``.

Here each input is first given a *form* (``_form_of``), and one table per
entry point maps a form to the routine that reads it.
"""
from __future__ import annotations

from collections.abc import Sequence
from typing import Callable, NamedTuple, Optional, Union

import numpy as np

DirectionProvider = Union[np.ndarray, Callable[[np.ndarray], np.ndarray]]


class DirectionalRegularisation(NamedTuple):
    """One directional term: ``direction`` is an (n, 3) array sampled at the
    interpolator's regularisation sample points, or a callable returning one
    from those points; ``weight`` scales the term's rows."""

    weight: float
    direction: DirectionProvider
    name: str = "directional regularisation"


class RegularisationConfig(NamedTuple):
    """The isotropic weight (``None``: the interpolator's default) and the
    directional terms of one setup."""

    isotropic: Optional[float] = None
    directional: tuple = ()


_TERM_ATTRS = ("weight", "direction", "name")
_TERM_KEYS = ("direction", "vector", "weight", "name")

_MSG_NEED_DIRECTION = "Directional regularisation entries require 'direction' or 'vector'"
_MSG_NEED_WEIGHT = "Directional regularisation entries require 'weight'"
_MSG_BAD_TERM = "Directional regularisation must be a DirectionalRegularisation or dict entry"
_MSG_SCALARS = "A sequence of scalars is not a valid directional regularisation config"
_MSG_BAD_DIRECTIONAL = "Unsupported directional regularisation configuration"
_MSG_BAD_CONFIG = "Unsupported regularisation configuration"


def _form_of(value) -> str:
    """The form of a configuration input: 'none', 'term', 'config',
    'term-mapping' (a mapping with a term key), 'mapping', 'scalar',
    'sequence' or 'other'.  Terms and configurations are recognised by their
    attributes first, so the tuple types above never count as sequences."""
    if value is None:
        return "none"
    if all(hasattr(value, a) for a in _TERM_ATTRS):
        return "term"
    if hasattr(value, "isotropic") and hasattr(value, "directional"):
        return "config"
    if isinstance(value, dict):
        return "term-mapping" if any(k in value for k in _TERM_KEYS) else "mapping"
    if np.isscalar(value):
        return "scalar"
    if isinstance(value, Sequence) and not isinstance(value, (bytes, np.ndarray)):
        return "sequence"
    return "other"


def _term_from_mapping(entry: dict, index: int, default_name: str) -> DirectionalRegularisation:
    direction = entry.get("direction", entry.get("vector"))
    if direction is None:
        raise ValueError(_MSG_NEED_DIRECTION)
    if entry.get("weight") is None:
        raise ValueError(_MSG_NEED_WEIGHT)
    label = entry["name"] if "name" in entry else f"{default_name} {index + 1}"
    return DirectionalRegularisation(float(entry["weight"]), direction, label)


def _one_term(value, index: int, default_name: str):
    form = _form_of(value)
    if form == "term":
        return value
    if form in ("term-mapping", "mapping"):
        return _term_from_mapping(value, index, default_name)
    raise TypeError(_MSG_BAD_TERM)


def _terms_from_sequence(items, default_name: str) -> tuple:
    if len(items) == 0:
        return ()
    if all(np.isscalar(item) for item in items):
        raise TypeError(_MSG_SCALARS)
    return tuple(_one_term(item, i, default_name) for i, item in enumerate(items))


def coerce_directional_regularisation(value, default_name: str = "directional regularisation") -> tuple:
    """The directional terms described by ``value`` (see the module notes)."""
    form = _form_of(value)
    if form == "none":
        return ()
    if form in ("term", "term-mapping", "mapping"):
        return (_one_term(value, 0, default_name),)
    if form == "sequence":
        return _terms_from_sequence(value, default_name)
    raise TypeError(_MSG_BAD_DIRECTIONAL)


def _config_from_mapping(entry: dict) -> RegularisationConfig:
    iso = entry.get("isotropic", entry.get("weight"))
    if iso is not None:
        iso = float(iso)
    return RegularisationConfig(iso, coerce_directional_regularisation(entry.get("directional", ())))


# form of ``regularisation`` -> (isotropic weight, directional terms)
_READERS = {
    "none": lambda v: RegularisationConfig(),
    "config": lambda v: RegularisationConfig(v.isotropic, tuple(v.directional)),
    "scalar": lambda v: RegularisationConfig(float(v), ()),
    "term-mapping": lambda v: RegularisationConfig(None, coerce_directional_regularisation(v)),
    "mapping": _config_from_mapping,
}


def coerce_regularisation_config(regularisation=None, directional_regularisation=None) -> RegularisationConfig:
    """Isotropic weight and directional terms from the forms listed in the
    module notes; the separate ``directional_regularisation`` terms are
    appended after those of ``regularisation``."""
    form = _form_of(regularisation)
    if form == "term":
        # a term object on its own is not a whole configuration
        raise TypeError(_MSG_BAD_CONFIG)
    reader = _READERS.get(form)
    if reader is None:
        raise TypeError(_MSG_BAD_CONFIG)
    cfg = reader(regularisation)
    extra = coerce_directional_regularisation(directional_regularisation)
    return RegularisationConfig(cfg.isotropic, tuple(cfg.directional) + extra)
