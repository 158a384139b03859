"""Drop-in registration into the reference's loop_interpolation package.

    import loop_interpolation as li
    from loopstructural_gb300.integration import gpu_interpolator_classes, register
    register(li)   # FINITE_DIFFERENCE now builds GPU interpolators

``gpu_interpolator_classes(li)`` returns subclasses of the reference's own
``FiniteDifferenceInterpolator`` and ``P1Interpolator`` that keep every setter,
getter, weight dictionary, bounding-box projection and serialisation method of
the reference and override only the hot path, delegating to the GB300 engine:

  setup_interpolator     (_finite_difference_interpolator.py:132-224, _p1interpolator.py:180-246)
  solve_system           (_discrete_interpolator.py:1221-1319)
  _evaluate_value_local / _evaluate_gradient_local (_discrete_interpolator.py:1342-1379)

The reference setters have already projected the data into the local frame,
so the engine receives ``self.data`` as is.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from . import interpolators, p1, supports


def _grid_of(support, cls=supports.StructuredGrid):
    return cls(origin=np.asarray(support.origin, dtype=float),
               nsteps_cells=np.asarray(support.nsteps_cells, dtype=int),
               step_vector=np.asarray(support.step_vector, dtype=float))


def _engine_for(obj, support_cls, engine_cls):
    eng = getattr(obj, "_gb300_engine", None)
    grid = _grid_of(obj.support, support_cls)
    if eng is None or eng.support.n_nodes != grid.n_nodes or not np.array_equal(
            eng.support.origin, grid.origin) or not np.array_equal(eng.support.step_vector, grid.step_vector):
        eng = engine_cls(grid)
        obj._gb300_engine = eng
    return eng


def gpu_interpolator_classes(li):
    """Subclasses of the reference interpolators with the GPU hot path:
    (FiniteDifferenceInterpolator, P1Interpolator)."""
    base = li.FiniteDifferenceInterpolator

    class GpuFiniteDifferenceInterpolator(base):
        """Reference FiniteDifferenceInterpolator with GB300 assembly, solve and evaluation."""

        def _engine(self):
            return _engine_for(self, supports.StructuredGrid, interpolators.FiniteDifferenceInterpolator)

        def setup_interpolator(self, **kwargs):
            eng = self._engine()
            eng.data = {k: np.array(v, dtype=float) for k, v in self.data.items()}
            eng.interpolation_weights = dict(self.interpolation_weights)
            for attr in ("interface_pair_mode", "interface_pair_threshold", "interface_pair_fallback"):
                if hasattr(self, attr):
                    setattr(eng, attr, getattr(self, attr))
            eng.ridge_factor = self.ridge_factor
            eng.add_ridge_regulatisation = self.add_ridge_regulatisation
            eng.setup_interpolator(**kwargs)
            self.interpolation_weights = dict(eng.interpolation_weights)
            self._mirror_families(eng)
            self.up_to_date = False
            return self.finalize_setup_diagnostics_report()

        def _mirror_families(self, eng):
            """Row counts for the reference's diagnostics report (matrix shape only)."""
            self.constraints = {}
            for name, fam in eng.constraints.items():
                self.constraints[name] = {"matrix": SimpleNamespace(shape=(fam.n_rows, self.dof)), "b": None,
                                          "w": fam.w.cpu().numpy()}
            for name, (rows, w) in getattr(eng, "regularisation_families", {}).items():
                self.constraints[name] = {"matrix": SimpleNamespace(shape=(rows, self.dof)), "b": None,
                                          "w": np.full(rows, w)}
            for name, (rows, _t, _f) in getattr(eng, "directional_families", {}).items():
                self.constraints[name] = {"matrix": SimpleNamespace(shape=(rows, self.dof)), "b": None,
                                          "w": None}

        # families added after setup (fold constraints, FF:93-237) go to the engine
        def add_gradient_orthogonal_constraints(self, points, vectors, w=1.0, b=0, name="gradient orthogonal"):
            eng = self._engine()
            eng.add_gradient_orthogonal_constraints(points, vectors, w=w, b=b, name=name)
            self._mirror_families(eng)
            self.up_to_date = False

        def minimise_directional_gradient_change(self, w, vector, name="directional regularisation"):
            eng = self._engine()
            eng.minimise_directional_gradient_change(w, vector, name=name)
            self._mirror_families(eng)
            self.up_to_date = False

        def add_directional_regularisation(self, directional_regularisation):
            eng = self._engine()
            terms = eng.add_directional_regularisation(directional_regularisation)
            self._mirror_families(eng)
            self.up_to_date = False
            return terms

        # the explicit-matrix API works on the engine's families
        def add_constraints_to_least_squares(self, A, B, idc, w=1.0, name="undefined"):
            eng = self._engine()
            eng.add_constraints_to_least_squares(A, B, idc, w=w, name=name)
            self._mirror_families(eng)
            self.up_to_date = False

        def build_matrix(self):
            return self._engine().build_matrix()

        def calculate_residual_for_constraints(self):
            eng = self._engine()
            eng.c = np.array(self.c, dtype=float)
            return eng.calculate_residual_for_constraints()

        def clear_constraints(self):
            eng = self._engine()
            eng.clear_constraints()
            self._mirror_families(eng)
            self.ineq_constraints = {}
            self.equal_constraints = {}

        def solve_system(self, solver=None, tol=None, solver_kwargs=None):
            eng = self._engine()
            ok = eng.solve_system(solver, tol, solver_kwargs)
            self.c = np.array(eng.c)
            self.latest_solve_timing = eng.get_last_solve_timing()
            self.up_to_date = bool(ok)
            return self.up_to_date

        def _sync_engine_c(self, eng):
            if eng._c is not self.c and (eng._c.shape != np.shape(self.c) or not np.array_equal(eng._c, self.c)):
                eng.c = np.array(self.c, dtype=float)
            eng.up_to_date = True

        def _evaluate_value_local(self, locations):
            self.update()
            eng = self._engine()
            self._sync_engine_c(eng)
            return eng._evaluate_value_local(np.asarray(locations, dtype=float))

        def _evaluate_gradient_local(self, locations):
            self.update()
            eng = self._engine()
            self._sync_engine_c(eng)
            return eng._evaluate_gradient_local(np.asarray(locations, dtype=float))

        def surfaces(self, value, **kwargs):
            """Isosurfaces of the solved field on the GPU (the reference
            contours through pyvista, _discrete_interpolator.py:1395-1405);
            returns loopstructural_gb300 Surface objects."""
            self.update()
            eng = self._engine()
            self._sync_engine_c(eng)
            return eng.surfaces(value, **kwargs)

    class GpuP1Interpolator(_p1_mixin(GpuFiniteDifferenceInterpolator), li.P1Interpolator):
        """Reference P1Interpolator with GB300 face rows, point rows, solve and evaluation."""

        def _engine(self):
            return _engine_for(self, supports.TetMesh, p1.P1Interpolator)

    return GpuFiniteDifferenceInterpolator, GpuP1Interpolator


def _p1_mixin(fd_cls):
    """The engine-delegating methods of the FD subclass, for the P1 subclass
    (same delegation; the P1 engine keeps no regularisation families)."""

    class _Delegate:
        solve_system = fd_cls.solve_system
        _sync_engine_c = fd_cls._sync_engine_c
        _evaluate_value_local = fd_cls._evaluate_value_local
        _evaluate_gradient_local = fd_cls._evaluate_gradient_local
        _mirror_families = fd_cls._mirror_families
        add_constraints_to_least_squares = fd_cls.add_constraints_to_least_squares
        build_matrix = fd_cls.build_matrix
        calculate_residual_for_constraints = fd_cls.calculate_residual_for_constraints
        clear_constraints = fd_cls.clear_constraints

        def setup_interpolator(self, **kwargs):
            eng = self._engine()
            eng.data = {k: np.array(v, dtype=float) for k, v in self.data.items()}
            eng.interpolation_weights = dict(self.interpolation_weights)
            eng.ridge_factor = self.ridge_factor
            eng.add_ridge_regulatisation = self.add_ridge_regulatisation
            eng.setup_interpolator(**kwargs)
            self.interpolation_weights = dict(eng.interpolation_weights)
            self.constraints = {}
            for name, fam in eng.constraints.items():
                self.constraints[name] = {"matrix": SimpleNamespace(shape=(fam.n_rows, self.dof)), "b": None,
                                          "w": fam.w.cpu().numpy()}
            self.up_to_date = False
            return self.finalize_setup_diagnostics_report()

    return _Delegate


def gpu_fold_interpolator_class(li):
    """Subclass of the reference's FDFoldInterpolator (_fd_fold_interpolator.py)
    whose base setup, fold families, solve and evaluation run on the GPU: its
    own setup_interpolator / add_fold_constraints (reference code) call the
    GPU FD class's setup and add_* methods through the method order."""
    from loop_interpolation._fd_fold_interpolator import FDFoldInterpolator

    gpu_fd, _ = gpu_interpolator_classes(li)

    class GpuFDFoldInterpolator(FDFoldInterpolator, gpu_fd):
        """Reference FDFoldInterpolator on the GB300 engine."""

    return GpuFDFoldInterpolator


def register(li):
    """Point the reference factory's FINITE_DIFFERENCE and PIECEWISE_LINEAR
    entries at the GPU classes."""
    gpu_fd, gpu_p1 = gpu_interpolator_classes(li)
    li.interpolator_map[li.InterpolatorType.FINITE_DIFFERENCE] = gpu_fd
    li.interpolator_map[li.InterpolatorType.PIECEWISE_LINEAR] = gpu_p1
    return gpu_fd, gpu_p1
