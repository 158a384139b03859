"""Interpolation supports: StructuredGrid (FD) and TetMesh (P1).

Host-side geometry with the reference constructor semantics
(packages/loop_common/src/loop_common/supports/_3d_base_structured.py:24-75,
_3d_structured_grid.py:21-60, _3d_structured_tetra.py:19-44): ``nsteps`` /
``nsteps_cells`` are CELL counts, nodes = cells + 1, F-order node numbering
gi = i + nx*j + nx*ny*k.  Field evaluation runs on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import _lib


class LoopException(Exception):
    """Invalid support geometry."""


class _StructuredSupport:
    dimension = 3

    def __init__(self, origin=None, nsteps_cells=None, step_vector=None, nsteps=None):
        origin = np.zeros(3) if origin is None else np.array(origin, dtype=float)
        step_vector = np.ones(3) if step_vector is None else np.array(step_vector, dtype=float)
        if nsteps_cells is None:
            nsteps_cells = np.array([10, 10, 10]) if nsteps is None else np.array(nsteps)
        nsteps_cells = np.array(nsteps_cells)
        if np.any(nsteps_cells == 0):
            raise LoopException("nsteps cannot be zero")
        if np.any(nsteps_cells < 0):
            raise LoopException("nsteps cannot be negative")
        self._nsteps = np.array(nsteps_cells, dtype=int) + 1
        self._step_vector = step_vector
        self._origin = origin

    # -- geometry ---------------------------------------------
    @property
    def nsteps(self):
        return self._nsteps

    @property
    def nsteps_cells(self):
        return self.nsteps - 1

    @property
    def step_vector(self):
        return self._step_vector

    @property
    def origin(self):
        return self._origin

    @property
    def maximum(self):
        return self.origin + self.nsteps_cells * self.step_vector

    @property
    def n_nodes(self):
        return int(np.prod(self.nsteps))

    @property
    def nodes(self):
        mx = self.maximum
        axes = [np.linspace(self.origin[d], mx[d], self.nsteps[d]) for d in range(3)]
        xx, yy, zz = np.meshgrid(*axes, indexing="ij")
        return np.array([xx.flatten(order="F"), yy.flatten(order="F"), zz.flatten(order="F")]).T

    @property
    def element_size(self):
        return np.prod(self.step_vector)

    def grid3(self) -> _lib.Grid3:
        return _lib.Grid3.make(self.nsteps, self.origin, self.step_vector)

    def to_dict(self):
        return {"origin": self.origin, "nsteps": self.nsteps_cells, "step_vector": self.step_vector}


class StructuredGrid(_StructuredSupport):
    """Regular grid of trilinear cells (FD support)."""

    def __init__(self, origin=None, nsteps_cells=None, step_vector=None, nsteps=None, rotation_xy=None,
                 properties=None, cell_properties=None, name="StructuredGrid"):
        super().__init__(origin, nsteps_cells, step_vector, nsteps)
        self.name = name

    @property
    def n_elements(self):
        return int(np.prod(self.nsteps_cells))

    @property
    def barycentre(self):
        ci = np.arange(self.n_elements)
        cx, cy = self.nsteps_cells[0], self.nsteps_cells[1]
        idx = np.stack([ci % cx, ci // cx % cy, ci // cx // cy], axis=1)
        return self.origin[None, :] + self.step_vector[None, :] * idx + self.step_vector[None, :] * 0.5

    def inside(self, pos):
        """S:287-293 (eps * 32 * extent tolerance)."""
        pos = np.asarray(pos, dtype=float)
        extent = np.maximum(np.abs(self.maximum - self.origin), 1.0)
        tol = np.finfo(float).eps * 32.0 * extent
        return np.all((pos >= (self.origin - tol)) & (pos <= (self.maximum + tol)), axis=1)

    # -- evaluation on the GPU (G:295-391) --------------------------------
    def evaluate_value(self, evaluation_points, property_array):
        from . import fd

        pos = np.asarray(evaluation_points, dtype=float)
        out = fd.eval_points(self, property_array, pos, value=True, gradient=False)[0]
        out[np.any(np.isnan(pos), axis=1)] = np.nan  # support level: NaN input is outside
        return out

    def evaluate_gradient(self, evaluation_points, property_array):
        from . import fd

        return fd.eval_points(self, property_array, np.asarray(evaluation_points, dtype=float), value=False,
                              gradient=True)[1]


class TetMesh(_StructuredSupport):
    """Structured tetrahedral mesh: 5 tetrahedra per cell (P1 support)."""

    def __init__(self, origin=None, nsteps_cells=None, step_vector=None, nsteps=None):
        if nsteps_cells is None and nsteps is None:
            nsteps_cells = np.ones(3) * 10
        super().__init__(origin, nsteps_cells, step_vector, nsteps)

    @property
    def n_cells(self):
        return int(np.prod(self.nsteps_cells))

    @property
    def ntetra(self):
        return self.n_cells * 5

    @property
    def n_elements(self):
        return self.ntetra

    def inside(self, pos):
        """T:264-272 strict inside."""
        pos = np.asarray(pos, dtype=float)
        ok = np.ones(pos.shape[0], dtype=bool)
        for i in range(3):
            ok &= pos[:, i] > self.origin[i]
            ok &= pos[:, i] < self.origin[i] + self.step_vector[i] * self.nsteps_cells[i]
        return ok
