"""The explicit-matrix side of the interpolator API on the CPU:
add_constraints_to_least_squares (DI:316-389), build_matrix (DI:684-755),
calculate_residual_for_constraints (DI:453-465), clear_constraints and
solve_system with a custom solver callable (DI:1283-1313, SS:32-45), checked
against the oracle's restatement.  Families live in torch tensors; the test
keeps them on the CPU (no kernels are involved in these methods)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import _lib  # noqa: E402
from loopstructural_gb300.interpolators import normalise_rows  # noqa: E402
from oracle import fd_oracle as fdo  # noqa: E402


@pytest.fixture
def cpu_device(monkeypatch):
    monkeypatch.setattr(_lib, "device", lambda: torch.device("cpu"))


def _families(rng, dof):
    fams = []
    A = rng.normal(size=(30, 8))
    idc = rng.integers(0, dof, size=(30, 8))
    fams.append((A, rng.normal(size=30), idc, 1.5, "value"))
    A3 = rng.normal(size=(10, 3, 8))  # a 3-D block (three rows per point) with per-point weights
    fams.append((A3, rng.normal(size=(10, 3)), rng.integers(0, dof, size=(10, 3, 8)), rng.uniform(1, 2, 10), "norm"))
    fams.append((rng.normal(size=(5, 4)), np.zeros(5), rng.integers(0, dof, size=(5, 4)), 0.7, "value"))  # -> value_0
    return fams


def test_normalise_rows_matches_oracle():
    rng = np.random.default_rng(0)
    cs = fdo.ConstraintSet(50)
    for A, B, idc, w, name in _families(rng, 50):
        got = normalise_rows(A, B, idc, w, name)
        cs.add(A, B, idc, w=w, name=name)
        ref = list(cs.families.values())[-1]
        np.testing.assert_array_equal(got[0], ref["A"])
        np.testing.assert_array_equal(got[1], ref["B"])
        np.testing.assert_array_equal(got[2], ref["idc"])
        np.testing.assert_array_equal(got[3], ref["w"])
    assert normalise_rows(np.ones((2, 3)), np.zeros(2), np.ones((2, 4), dtype=int)) is None  # shape mismatch
    assert normalise_rows(np.array([[np.nan, 1.0]]), np.zeros(1), np.zeros((1, 2), dtype=int)) is None
    with pytest.raises(ValueError):
        normalise_rows(np.ones((2, 2)), np.zeros(2), np.zeros((2, 2), dtype=int), w=np.ones(3))
    with pytest.raises(TypeError):
        normalise_rows(np.ones((2, 2)), np.zeros(2), np.zeros((2, 2), dtype=int), w=[1.0, 2.0])


def test_build_matrix_residuals_and_callable_solve(cpu_device):
    from scipy.sparse.linalg import spsolve

    rng = np.random.default_rng(1)
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=np.array([3, 3, 2]), step_vector=np.ones(3))
    interp = L.FiniteDifferenceInterpolator(grid)
    dof = interp.dof
    cs = fdo.ConstraintSet(dof)
    for A, B, idc, w, name in _families(rng, dof):
        interp.add_constraints_to_least_squares(A, B, idc, w=w, name=name)
        cs.add(A, B, idc, w=w, name=name)
    assert interp.family_order == list(cs.families) == ["value", "norm", "value_0"]
    A, b = interp.build_matrix()
    Ar, br = cs.matrix()
    np.testing.assert_allclose(A.toarray(), Ar.toarray(), rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(b, br, rtol=1e-14, atol=1e-14)
    # a custom solver on the explicit, ridge-augmented, column-scaled system
    assert interp.solve_system(lambda M, rhs: spsolve((M.T @ M).tocsc(), M.T @ rhs))
    ref = fdo.solve_direct(Ar, br)
    assert np.linalg.norm(interp.c - ref) <= 1e-8 * np.linalg.norm(ref)
    assert interp.get_last_solve_timing()["solver"] == "callable"
    res = interp.calculate_residual_for_constraints()
    for name, fam in cs.families.items():
        m = np.zeros((fam["A"].shape[0], dof))
        for r in range(m.shape[0]):
            np.add.at(m[r], fam["idc"][r], fam["A"][r])
        np.testing.assert_allclose(res[name], m @ interp.c - fam["B"], rtol=1e-12, atol=1e-12)
    interp.clear_constraints()
    assert not interp.constraints and interp.family_order == []
    A0, b0 = interp.build_matrix()
    assert A0.shape == (0, dof) and b0.size == 0
