"""Host logic of the fold interpolator (CPU): the fold-normalisation target
and its dgz / normal alignment check, against the oracle's restatement of
_fold_norm_alignment.py."""
import logging

import numpy as np
import pytest

from golden.make_golden import SyntheticFold
from loopstructural_gb300.fold import resolve_fold_norm_target
from oracle import fd_oracle as fdo


def _normals(sign, n=40, seed=0):
    rng = np.random.default_rng(seed)
    p = rng.uniform(0, 1, size=(n, 3))
    _, _, dgz = SyntheticFold().get_deformed_orientation(p)
    v = sign * dgz + rng.normal(0, 0.05, size=dgz.shape)
    return np.column_stack([p, v, np.ones(n)])


@pytest.mark.parametrize("mode", ["none", "warn", "correct", None, " Correct "])
@pytest.mark.parametrize("sign", [1.0, -1.0])
@pytest.mark.parametrize("fold_norm", [-1.0, 2.5, None])
def test_target_matches_oracle(mode, sign, fold_norm):
    nrm = _normals(sign)
    got = resolve_fold_norm_target(fold=SyntheticFold(), normal_constraints=nrm, fold_norm=fold_norm,
                                   dgz_alignment=mode)
    ref = fdo.fold_norm_target(SyntheticFold(), nrm, fold_norm, mode)
    assert got == ref
    base = -1.0 if fold_norm is None else fold_norm
    flip = sign < 0 and mode is not None and mode.strip().lower() == "correct"
    assert got == (-base if flip else base)


def test_warns_and_rejects(caplog):
    with caplog.at_level(logging.WARNING):
        resolve_fold_norm_target(fold=SyntheticFold(), normal_constraints=_normals(-1.0), fold_norm=-1.0,
                                 dgz_alignment="warn")
    assert "opposite" in caplog.text
    with pytest.raises(ValueError):
        resolve_fold_norm_target(fold=SyntheticFold(), normal_constraints=_normals(1.0), fold_norm=-1.0,
                                 dgz_alignment="sideways")
    # no normals, or a fold that cannot evaluate: the requested target
    assert resolve_fold_norm_target(fold=SyntheticFold(), normal_constraints=np.zeros((0, 7)), fold_norm=3.0,
                                    dgz_alignment="correct") == 3.0

    class Broken:
        def get_deformed_orientation(self, p):
            raise ValueError("no fold frame")

    assert resolve_fold_norm_target(fold=Broken(), normal_constraints=_normals(-1.0), fold_norm=-1.0,
                                    dgz_alignment="correct") == -1.0
