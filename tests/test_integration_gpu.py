"""The drop-in route on the GPU: ``integration.register(li)`` and then the
reference's own factory, setters, ``setup_interpolator``, ``solve_system``
and ``evaluate_value`` / ``evaluate_gradient`` (the FD case that the
factory builds from a BoundingBox with a shifted origin and an anisotropic
extent), compared with the fixture recorded through the same calls on the
unmodified reference (make_golden.py --configs, ``fac_*``).

The reference is looked up in LOOPSTRUCTURAL_REFERENCE (a source tree) or
in ``baseline/_ref`` (a ``pip install --target`` of it).  Where neither
imports, the test skips and says why: the reference's constraint layer
needs pydantic, whose compiled core is not installed for aarch64."""
import os
import sys
import types

import numpy as np
import pytest

from test_configs_gpu import FIELD_TOL, _field_error, _solve_kw

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference():
    for name in ("pyvista", "yaml"):
        if name not in sys.modules:
            try:
                __import__(name)
            except Exception:
                sys.modules[name] = types.ModuleType(name)
    src = os.environ.get("LOOPSTRUCTURAL_REFERENCE", "")
    paths = []
    if src:
        paths += [os.path.join(src, "packages", sub, "src") for sub in ("loop_common", "loop_interpolation")]
    paths.append(os.path.join(ROOT, "baseline", "_ref"))
    for p in paths:
        if os.path.isdir(p) and p not in sys.path:
            sys.path.append(p)
    try:
        import loop_interpolation
        from loop_common.geometry import BoundingBox
    except Exception as e:  # noqa: BLE001 - any import failure means the route cannot run here
        pytest.skip(f"the reference does not import on this machine ({type(e).__name__}: {e}); neither "
                    "LOOPSTRUCTURAL_REFERENCE nor baseline/_ref provides it with its pydantic dependency")
    return loop_interpolation, BoundingBox


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_factory_route_on_the_gpu(cgolden, precision):
    li, BoundingBox = _reference()
    from loopstructural_gb300 import integration

    g = cgolden
    saved = dict(li.interpolator_map)
    try:
        gpu_cls, _ = integration.register(li)
        origin = np.array([100.0, -50.0, 20.0])
        bb = BoundingBox(origin=origin, maximum=np.array([600.0, 250.0, 120.0]))
        interp = li.InterpolatorFactory.create_interpolator("FDI", boundingbox=bb, nelements=3000)
        assert isinstance(interp, gpu_cls)
        np.testing.assert_array_equal(np.asarray(interp.support.nsteps), g["fac_nsteps"])
        interp.set_value_constraints(g["fac_value_in"])
        interp.set_normal_constraints(g["fac_normal_in"])
        interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
        assert interp.solve_system("cg", solver_kwargs=_solve_kw(precision, 1e-13))
        err = _field_error(interp.evaluate_value(g["fac_query"]), g["fac_eval_value"])
        assert err <= FIELD_TOL[precision], (precision, err)
        gr = interp.evaluate_gradient(g["fac_query"])
        ref = g["fac_eval_gradient"]
        ok = np.isfinite(ref).all(axis=1)
        assert np.linalg.norm(gr[ok] - ref[ok]) <= 1e-5 * np.linalg.norm(ref[ok])
    finally:
        li.interpolator_map.clear()
        li.interpolator_map.update(saved)
