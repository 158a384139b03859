"""FD interpolator with fold constraints on the GPU.

Mirrors the reference's ``FDFoldInterpolator``
(packages/loop_interpolation/src/loop_interpolation/_fd_fold_interpolator.py,
FF below) with its helpers ``setup_with_fold_constraints`` (_fold_setup.py)
and ``resolve_fold_norm_target`` (_fold_norm_alignment.py, FN).  The fold
geometry comes from any object with the reference ``FoldEvent`` contract
``get_deformed_orientation(points) -> (deformed_orientation, fold_axis, dgz)``
(a reference FoldEvent works as is).  The fold families are ordinary GPU
families: gradient-orthogonal rows at every active node (three families,
ls_fd_point_rows) and three matrix-free directional regularisation terms.
"""
from __future__ import annotations

import logging

import numpy as np

from .interpolators import FiniteDifferenceInterpolator
from .regularisation import DirectionalRegularisation

logger = logging.getLogger(__name__)

_DEFAULT = object()
_ALIGNMENT_MODES = {"none", "warn", "correct"}


def _dgz_normal_agreement(fold, normals):
    """Median cosine between the fold's dgz direction and the normal vectors
    of the normal constraints (rows x y z nx ny nz ...), over the rows where
    both are finite and non-zero; None when it cannot be measured (no usable
    rows, or a fold that cannot evaluate dgz at the points)."""
    table = np.asarray(normals, dtype=float)
    if table.ndim != 2 or table.shape[1] < 6 or len(table) == 0:
        return None
    try:
        dgz = np.asarray(fold.get_deformed_orientation(table[:, :3])[2], dtype=float)
    except (AttributeError, TypeError, ValueError, RuntimeError) as exc:
        logger.warning("dgz could not be evaluated at the normal constraints (%s); fold_norm left as given.", exc)
        return None
    if dgz.ndim != 2 or dgz.shape[1] != 3:
        logger.warning("dgz has shape %s, expected (n, 3); fold_norm left as given.", getattr(dgz, "shape", None))
        return None
    rows = min(len(dgz), len(table))
    if rows != len(dgz) or rows != len(table):
        logger.warning("dgz has %d rows and the normals %d; comparing the first %d.", len(dgz), len(table), rows)
    a, b = dgz[:rows], table[:rows, 3:6]
    la, lb = np.linalg.norm(a, axis=1), np.linalg.norm(b, axis=1)
    usable = np.isfinite(a).all(axis=1) & np.isfinite(b).all(axis=1) & (la > 1e-12) & (lb > 1e-12)
    if not usable.any():
        return None
    cosines = np.sum(a[usable] * b[usable], axis=1) / (la[usable] * lb[usable])
    return float(np.median(cosines))


def resolve_fold_norm_target(*, fold, normal_constraints, fold_norm, dgz_alignment, default_fold_norm=-1.0):
    """Target of grad(f) . dgz for the fold-normalisation rows (FN:9-118).

    It is ``fold_norm`` (``default_fold_norm`` when None).  With
    ``dgz_alignment`` 'warn' (the default) or 'correct', the fold's dgz is
    compared with the normal constraints: a median cosine below -0.2 means dgz
    points against the data, which is logged, and under 'correct' the target's
    sign is flipped.  'none' skips the comparison; any other mode raises
    ValueError."""
    target = float(default_fold_norm if fold_norm is None else fold_norm)
    mode = "warn" if dgz_alignment is None else str(dgz_alignment).strip().lower()
    if mode not in _ALIGNMENT_MODES:
        raise ValueError(f"dgz_alignment must be one of {{{', '.join(sorted(_ALIGNMENT_MODES))}}}, got {dgz_alignment!r}")
    agreement = None if mode == "none" else _dgz_normal_agreement(fold, normal_constraints)
    if agreement is None or agreement >= -0.2:
        return target
    flipped = mode == "correct"
    logger.warning("dgz points opposite to the normal constraints (median cosine %.3f); %s", agreement,
                   f"fold_norm sign flipped to {-target:.3f}." if flipped else "fold_norm may need the opposite sign.")
    return -target if flipped else target


class FDFoldInterpolator(FiniteDifferenceInterpolator):
    """FD interpolator with fold orientation, fold axis, fold normalisation and
    anisotropic fold regularisation constraints (FF:26-237)."""

    def __init__(self, grid, fold=None, data=None):
        super().__init__(grid, data=data)
        self.fold = fold

    def setup_interpolator(self, **kwargs):
        """The FD setup, then ``add_fold_constraints(**fold_weights)`` (FF:62-87,
        _fold_setup.py)."""
        if self.fold is None:
            raise RuntimeError(f"{self.__class__.__name__}: no fold event set. "
                               "Assign self.fold before calling setup_interpolator.")
        kw = dict(kwargs)
        fold_weights = kw.pop("fold_weights", {})
        report = super().setup_interpolator(**kw)
        self.add_fold_constraints(**fold_weights)
        for name, fam in self.constraints.items():
            report[name] = fam.n_rows
        for name, (rows, _t, _f) in self.directional_families.items():
            report[name] = rows
        return report

    def add_fold_constraints(self, fold_orientation=10.0, fold_axis_w=10.0, fold_regularisation=_DEFAULT,
                             fold_normalisation=1.0, fold_norm=-1.0, dgz_alignment="warn", mask_fn=None):
        """FF:93-237: at every node not excluded by ``mask_fn``,
        grad(f) . deformed_orientation = 0 (weight fold_orientation),
        grad(f) . fold_axis = 0 (fold_axis_w), grad(f) . dgz = fold_norm
        (fold_normalisation); then directional regularisation along dgz,
        the deformed orientation and the fold axis with the three weights of
        ``fold_regularisation`` (default [0.1, 0.01, 0.01])."""
        if fold_regularisation is _DEFAULT:
            fold_regularisation = [0.1, 0.01, 0.01]
        nodes = self.support.nodes
        deformed, axis, dgz = self.fold.get_deformed_orientation(nodes)
        weight = np.ones(self.support.n_nodes)
        if mask_fn is not None:
            weight[mask_fn(nodes)] = 0.0
        active = weight > 0.0
        pos = nodes[active]
        if fold_orientation is not None:
            self.add_gradient_orthogonal_constraints(pos, np.array(deformed)[active], w=fold_orientation,
                                                     name="fold orientation")
        if fold_axis_w is not None:
            self.add_gradient_orthogonal_constraints(pos, np.array(axis)[active], w=fold_axis_w, name="fold axis")
        if fold_normalisation is not None:
            target = resolve_fold_norm_target(fold=self.fold, normal_constraints=self.get_norm_constraints(),
                                              fold_norm=fold_norm, dgz_alignment=dgz_alignment)
            self.add_gradient_orthogonal_constraints(pos, np.array(dgz)[active], w=fold_normalisation, b=target,
                                                     name="fold normalisation")
        if fold_regularisation is not None:

            def masked(v):
                v = np.asarray(v, dtype=float).copy()
                v[~active] = 0.0
                return v

            self.add_directional_regularisation((
                DirectionalRegularisation(fold_regularisation[0], masked(dgz), "fold regularisation 1"),
                DirectionalRegularisation(fold_regularisation[1], masked(deformed), "fold regularisation 2"),
                DirectionalRegularisation(fold_regularisation[2], masked(axis), "fold regularisation 3"),
            ))
        self.up_to_date = False
