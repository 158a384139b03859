"""Pin the fault oracle against fixtures recorded from the reference
(make_golden.py --faults): restoration of points through fault slip events
with the base displacement profile, BaseFault3D and a custom cubic / composite
profile; the faulted feature's values through two faults in order; its
gradient from the regular-tetrahedron steps (the reference's own functions);
the unfaulted gradient.  1e-12 absolute (coordinates and values of order 1).
CPU only."""
import os

import numpy as np
import pytest

from oracle import fault_oracle as fo
from oracle import fd_oracle as fdo

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fg():
    return np.load(os.path.join(HERE, "golden", "fault_golden.npz"), allow_pickle=False)


def field(g, name):
    return fo.Field(fdo.Grid(g[f"{name}_origin"], g[f"{name}_cells"], g[f"{name}_step"]), g[f"{name}_c"])


def frame(g, k):
    return tuple(field(g, f"f{k}_{n}") for n in ("gx", "gy", "gz"))


def custom_profile():
    hw = fo.Cubic(cstr=[(0, 1), (1, 0)], grad=[(0, 0), (1, 0)], lim=(0, 1))
    fw = fo.Cubic(cstr=[(0, -1), (-1, 0)], grad=[(0, 0), (-1, 0)], lim=(-1, 0))
    gy = fo.Cubic(cstr=[(-1, 0), (1, 0), (0, 1)], grad=[(0, 0)], min_v=-1, max_v=1)
    return fo.displacement(fo.composite(hw, fw), gy, fo.ones, scale=0.7)


def test_restoration_matches_reference(fg):
    pts = fg["points"]
    for k in (0, 1):
        got = fo.apply_to_points(frame(fg, k), pts, float(fg[f"f{k}_displacement"]), fo.base_fault())
        np.testing.assert_allclose(got, fg[f"restored_f{k}_base"], rtol=0, atol=1e-12)
    got = fo.apply_to_points(frame(fg, 0), pts, float(fg["f0_displacement"]), fo.base_fault_3d())
    np.testing.assert_allclose(got, fg["restored_f0_base3d"], rtol=0, atol=1e-12)
    got = fo.apply_to_points(frame(fg, 0), pts, float(fg["f0_displacement"]), custom_profile())
    np.testing.assert_allclose(got, fg["restored_f0_custom"], rtol=0, atol=1e-12)


def test_faulted_value_and_gradient_match_reference(fg):
    faults = [(frame(fg, k), float(fg[f"f{k}_displacement"]), fo.base_fault()) for k in (0, 1)]
    strat = field(fg, "strat")
    v = fo.faulted_value(strat, faults, fg["points"])
    np.testing.assert_allclose(v, fg["faulted_value"], rtol=0, atol=1e-12, equal_nan=True)
    assert str(fg["faulted_gradient_error"]).startswith("ValueError")  # the reference's own call raises
    g, scale = fo.faulted_gradient(strat, faults, fg["points"], 0.01)
    assert scale == float(fg["faulted_gradient_scale"])
    np.testing.assert_allclose(g, fg["faulted_gradient_reference_steps"], rtol=1e-9, atol=1e-9, equal_nan=True)
    np.testing.assert_allclose(strat.gradient(fg["points"]), fg["plain_gradient"], rtol=0, atol=1e-12)
