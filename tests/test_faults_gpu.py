"""Faulted-feature evaluation on the GPU (loopstructural_gb300.faults, the
ls_fault_apply and ls_tetra_gradient kernels) against fixtures recorded from
the reference (make_golden.py --faults): points restored through fault slip
events (base profile, BaseFault3D, a custom cubic / composite profile), the
values of a feature displaced by two faults in order, its gradient from the
regular-tetrahedron steps, and the unfaulted gradient.  Bars: 1e-11 absolute
for coordinates and values (ten integration steps in FP64), 1e-9 for the
tetrahedron gradients (value differences over tetrahedra of ~2e-3)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import faults as F  # noqa: E402

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fg():
    return np.load(os.path.join(HERE, "golden", "fault_golden.npz"), allow_pickle=False)


def _interp(g, name):
    grid = L.StructuredGrid(origin=g[f"{name}_origin"], nsteps=g[f"{name}_cells"], step_vector=g[f"{name}_step"])
    it = L.FiniteDifferenceInterpolator(grid)
    it.c = g[f"{name}_c"]
    it.up_to_date = True
    return it


def _fault(g, k):
    feats = [F.GeologicalFeature(f"fault{k}_{n}", _interp(g, f"f{k}_{n}")) for n in ("gx", "gy", "gz")]
    return F.FaultSegment(f"fault{k}", feats, displacement=float(g[f"f{k}_displacement"]))


def test_restoration_matches_reference(fg):
    pts = fg["points"]
    for k in (0, 1):
        np.testing.assert_allclose(_fault(fg, k).apply_to_points(pts), fg[f"restored_f{k}_base"], rtol=0, atol=1e-11)
    f0 = _fault(fg, 0)
    f0.faultfunction = "BaseFault3D"
    np.testing.assert_allclose(f0.apply_to_points(pts), fg["restored_f0_base3d"], rtol=0, atol=1e-11)
    hw, fw = F.CubicFunction(), F.CubicFunction()
    for f, s in ((hw, 1.0), (fw, -1.0)):
        f.add_cstr(0, s)
        f.add_grad(0, 0)
        f.add_cstr(s, 0)
        f.add_grad(s, 0)
        f.set_lim(*((0, 1) if s > 0 else (-1, 0)))
    gy = F.CubicFunction()
    gy.add_cstr(-1, 0)
    gy.add_cstr(1, 0)
    gy.add_cstr(0, 1)
    gy.add_grad(0, 0)
    gy.add_min(-1)
    gy.add_max(1)
    f0.faultfunction = F.FaultDisplacement(hw=hw, fw=fw, gy=gy, gz=F.Ones(), scale=0.7)
    np.testing.assert_allclose(f0.apply_to_points(pts), fg["restored_f0_custom"], rtol=0, atol=1e-11)
    with pytest.raises(ValueError):
        f0.faultfunction = "no such profile"


def test_faulted_feature_values_and_gradients(fg):
    pts = fg["points"]
    strat = _interp(fg, "strat")
    feat = F.GeologicalFeature("strat", strat, faults=[_fault(fg, 0), _fault(fg, 1)])
    np.testing.assert_allclose(feat.evaluate_value(pts), fg["faulted_value"], rtol=0, atol=1e-11, equal_nan=True)
    g = feat.evaluate_gradient(pts, element_scale_parameter=0.01)
    np.testing.assert_allclose(g, fg["faulted_gradient_reference_steps"], rtol=1e-9, atol=1e-9, equal_nan=True)
    plain = F.GeologicalFeature("strat", strat)
    np.testing.assert_allclose(plain.evaluate_gradient(pts), fg["plain_gradient"], rtol=0, atol=1e-12)
    # regions mask points out (NaN), as the reference's _calculate_mask
    region = F.GeologicalFeature("strat", strat, faults=feat.faults, regions=[lambda p: p[:, 0] < 0.5])
    v = region.evaluate_value(pts)
    assert np.all(np.isnan(v[pts[:, 0] >= 0.5]))
    np.testing.assert_allclose(v[pts[:, 0] < 0.5], fg["faulted_value"][pts[:, 0] < 0.5], atol=1e-11, equal_nan=True)
