"""Registration of the GPU interpolator into the reference's own factory.

Needs the reference's loop_interpolation package importable (only where the
reference source is available); the compute path itself needs a GPU and is
covered by the -m gpu tests, so here it must fail loudly."""
import os
import sys
import types

import numpy as np
import pytest

REF = os.environ.get("LOOPSTRUCTURAL_REFERENCE", "")


@pytest.fixture(scope="module")
def li():
    if not REF or not os.path.isdir(os.path.join(REF, "packages", "loop_interpolation")):
        pytest.skip("reference source not available: set LOOPSTRUCTURAL_REFERENCE to the LoopStructural source root")
    for name in ("pyvista", "yaml"):
        if name not in sys.modules:
            try:
                __import__(name)
            except Exception:
                sys.modules[name] = types.ModuleType(name)
    for sub in ("loop_common", "loop_interpolation"):
        p = os.path.join(REF, "packages", sub, "src")
        if p not in sys.path:
            sys.path.append(p)
    import loop_interpolation

    return loop_interpolation


def test_factory_builds_gpu_subclass(li):
    from loop_common.geometry import BoundingBox

    from loopstructural_gb300 import integration

    saved = dict(li.interpolator_map)
    try:
        gpu_cls, gpu_p1 = integration.register(li)
        assert issubclass(gpu_p1, li.P1Interpolator)
        assert li.interpolator_map[li.InterpolatorType.PIECEWISE_LINEAR] is gpu_p1
        assert issubclass(gpu_cls, li.FiniteDifferenceInterpolator)
        bb = BoundingBox(origin=np.zeros(3), maximum=np.ones(3))
        interp = li.InterpolatorFactory.create_interpolator("FDI", boundingbox=bb, nelements=1000)
        assert isinstance(interp, gpu_cls)
        # the reference setters, projection and weights are inherited unchanged
        interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0], [0.2, 0.3, 0.4, 0.0]]))
        assert interp.get_value_constraints().shape == (2, 5)
        assert interp.interpolation_weights["npw"] == 10.0
    finally:
        li.interpolator_map.clear()
        li.interpolator_map.update(saved)


def test_gpu_subclass_fails_loudly_without_gpu(li):
    import torch

    import loopstructural_gb300 as L
    from loopstructural_gb300 import integration

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    gpu_cls, _ = integration.gpu_interpolator_classes(li)
    grid = li.StructuredGrid(origin=np.zeros(3), nsteps=np.array([5, 5, 5]), step_vector=np.ones(3) * 0.2)
    interp = gpu_cls(grid)
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0]]))
    with pytest.raises(L.ExtensionUnavailable):
        interp.setup_interpolator(regularisation=0.1)
    # surfaces go to the engine (the reference's own contours through pyvista)
    assert gpu_cls.surfaces is not li.FiniteDifferenceInterpolator.surfaces
    # so do the explicit-matrix methods (a family added through the reference's
    # own method would otherwise never reach the GPU solve)
    for meth in ("add_constraints_to_least_squares", "build_matrix", "calculate_residual_for_constraints",
                 "clear_constraints"):
        assert meth in gpu_cls.__dict__, meth
    with pytest.raises(L.ExtensionUnavailable):
        interp.surfaces(0.5)


def test_gpu_p1_subclass_keeps_reference_api_and_fails_loudly_without_gpu(li):
    import torch

    import loopstructural_gb300 as L
    from loopstructural_gb300 import integration

    _, gpu_p1 = integration.gpu_interpolator_classes(li)
    mesh = li.TetMesh(origin=np.zeros(3), nsteps_cells=np.array([3, 3, 3]), step_vector=np.ones(3) / 3)
    interp = gpu_p1(mesh)
    assert interp.interpolation_weights["cgw"] == 0.1
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0]]))
    assert interp.get_value_constraints().shape == (1, 5)
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    with pytest.raises(L.ExtensionUnavailable):
        interp.setup_interpolator(cgw=0.1)


def test_gpu_fold_subclass_routes_fold_families_to_the_engine(li):
    import torch

    import loopstructural_gb300 as L
    from loopstructural_gb300 import integration

    gpu_fold = integration.gpu_fold_interpolator_class(li)
    from loop_interpolation._fd_fold_interpolator import FDFoldInterpolator

    assert issubclass(gpu_fold, FDFoldInterpolator)
    gpu_fd = gpu_fold.__mro__[2]
    # the reference fold code reaches the GPU setup and add_* methods
    for meth in ("setup_interpolator", "add_gradient_orthogonal_constraints", "add_directional_regularisation",
                 "solve_system", "_evaluate_value_local"):
        assert getattr(gpu_fold, meth) is getattr(FDFoldInterpolator, meth) or meth in gpu_fd.__dict__, meth
    assert gpu_fold.add_gradient_orthogonal_constraints is gpu_fd.add_gradient_orthogonal_constraints
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    grid = li.StructuredGrid(origin=np.zeros(3), nsteps=np.array([5, 5, 5]), step_vector=np.ones(3) * 0.2)
    interp = gpu_fold(grid, fold=object())
    interp.set_value_constraints(np.array([[0.5, 0.5, 0.5, 1.0]]))
    with pytest.raises(L.ExtensionUnavailable):
        interp.setup_interpolator(regularisation=0.1)
