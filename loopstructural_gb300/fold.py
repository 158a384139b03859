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


def resolve_fold_norm_target(*, fold, normal_constraints, fold_norm, dgz_alignment, default_fold_norm=-1.0):
    """Target of grad(f) . dgz (FN:9-118): ``fold_norm`` (default -1), its sign
    flipped under ``dgz_alignment='correct'`` when dgz points against the
    normal constraints (median unit dot product below -0.2); ``'warn'`` only
    logs, ``'none'`` skips the check."""
    target = float(default_fold_norm if fold_norm is None else fold_norm)
    mode = "warn" if dgz_alignment is None else str(dgz_alignment).strip().lower()
    if mode not in _ALIGNMENT_MODES:
        raise ValueError(f"dgz_alignment must be one of {{{', '.join(sorted(_ALIGNMENT_MODES))}}}, got {dgz_alignment!r}")
    if mode == "none":
        return target
    normals = np.asarray(normal_constraints, dtype=float)
    if normals.ndim != 2 or normals.shape[0] == 0 or normals.shape[1] < 6:
        return target
    vec = normals[:, 3:6]
    try:
        _, _, dgz = fold.get_deformed_orientation(normals[:, :3])
    except (AttributeError, TypeError, ValueError, RuntimeError) as exc:
        logger.warning("Could not evaluate dgz for alignment check (%s).", exc)
        return target
    dgz = np.asarray(dgz, dtype=float)
    if dgz.ndim != 2 or dgz.shape[1] != vec.shape[1]:
        logger.warning("Skipping dgz alignment check due to unexpected dgz shape %s.", getattr(dgz, "shape", None))
        return target
    if dgz.shape[0] != vec.shape[0]:
        n = min(dgz.shape[0], vec.shape[0])
        logger.warning("dgz alignment check received mismatched rows (dgz=%d, normals=%d); using first %d.",
                       dgz.shape[0], vec.shape[0], n)
        if n == 0:
            return target
        dgz, vec = dgz[:n], vec[:n]
    nn = np.linalg.norm(vec, axis=1)
    dn = np.linalg.norm(dgz, axis=1)
    ok = np.all(np.isfinite(vec), axis=1) & np.all(np.isfinite(dgz), axis=1) & (nn > 1e-12) & (dn > 1e-12)
    if not np.any(ok):
        return target
    med = float(np.median(np.einsum("ij,ij->i", dgz[ok] / dn[ok, None], vec[ok] / nn[ok, None])))
    if med < -0.2:
        logger.warning("Detected dgz opposite to normal constraints (median dot %.3f). "
                       "fold_norm may need sign inversion.", med)
        if mode == "correct":
            target *= -1.0
            logger.warning("Auto-correcting fold_norm sign to %.3f using dgz_alignment='correct'.", target)
    return target


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
