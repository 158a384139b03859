"""Triangulated isosurfaces of a solved field.

``Surface`` carries the fields of the reference's ``loop_common.geometry.Surface``
that ``DiscreteInterpolator.surfaces`` fills (DI:1395-1405): vertices (V, 3),
triangles (T, 3), plus the vertex normals, the name and the isovalue.
``LoopIsosurfacer`` mirrors the reference's ``LoopStructural/utils/_surface.py``
(LI below): sample a field on a bounding box's regular grid, then extract
isosurfaces -- here with the GPU kernel of ``ls_iso_extract``.
"""
from __future__ import annotations

from collections.abc import Iterable
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Surface:
    vertices: np.ndarray
    triangles: np.ndarray
    normals: np.ndarray | None = None
    name: str = "surface"
    values: np.ndarray | None = field(default=None)

    @property
    def area(self) -> float:
        v = self.vertices[self.triangles]
        return float(0.5 * np.linalg.norm(np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0]), axis=1).sum())


def isovalues_for(values, all_values):
    """The isovalues LI:96-121 derives from ``values``: None -> the middle of
    the sampled range; a float -> [value]; 0 -> [0.0]; an int n >= 1 -> n
    values evenly spaced inside the range less 5% at either end; any other
    iterable as given (ints < 1 other than 0 raise ValueError)."""
    lo, hi = float(np.nanmin(all_values)), float(np.nanmax(all_values))
    if values is None:
        values = [(hi - lo) / 2 + lo]
    if isinstance(values, Iterable):
        return list(values)
    if isinstance(values, float):
        return [values]
    if isinstance(values, int) and values == 0:
        return [0.0]
    if isinstance(values, int) and values < 1:
        raise ValueError("Number of isosurfaces must be greater than 1. Either use a positive integer or provide "
                         "a list or float for a specific isovalue.")
    if isinstance(values, int):
        buffer = (hi - lo) * 0.05
        return list(np.linspace(lo + buffer, hi - buffer, values))
    raise TypeError("values must be None, a number or an iterable of numbers")


def surface_names(name, n):
    """(names, individual) as LI:123-133: one name per isovalue, and whether
    the names are used as given (else ``name_isovalue``)."""
    if name is None:
        return ["surface"] * n, False
    if isinstance(name, str):
        return [name] * n, n == 1
    names = list(name)
    return names, len(names) == n


class LoopIsosurfacer:
    """Isosurfaces of an interpolator or a callable on a bounding box's regular
    grid (LI:23-175).  ``bounding_box`` needs ``origin``, ``maximum`` and
    ``nsteps`` (nodes per axis), as the reference's BoundingBox has."""

    def __init__(self, bounding_box, interpolator=None, callable=None):  # noqa: A002 - the reference's keyword
        self.bounding_box = bounding_box
        if interpolator is None and callable is None:
            raise ValueError("Must specify either interpolator or callable")
        if interpolator is not None and callable is not None:
            raise ValueError("Must specify either interpolator or callable")
        self.callable = interpolator.evaluate_value if interpolator is not None else callable

    def _grid(self):
        from .supports import StructuredGrid

        origin = np.asarray(self.bounding_box.origin, dtype=float)
        maximum = np.asarray(self.bounding_box.maximum, dtype=float)
        nsteps = np.asarray(self.bounding_box.nsteps, dtype=int)
        step = (maximum - origin) / (nsteps - 1)
        return StructuredGrid(origin=origin, nsteps=nsteps - 1, step_vector=step)

    def fit(self, values=None, name=None, colours=None):
        """A Surface per isovalue the sampled field crosses (LI:63-175)."""
        import torch

        from . import _lib, fd

        if not callable(self.callable):
            raise TypeError("No interpolator of callable function set")
        grid = self._grid()
        nodes = grid.nodes  # node order: x fastest, the order of the isosurface kernel
        all_values = np.asarray(self.callable(nodes), dtype=float).reshape(-1)
        isovalues = isovalues_for(values, all_values)
        names, individual = surface_names(name, len(isovalues))
        colours = [None] * len(isovalues) if colours is None else list(colours)
        d_values = torch.from_numpy(np.ascontiguousarray(all_values)).to(_lib.device())
        out = []
        for surface_name, iso, colour in zip(names, isovalues, colours):
            verts, tris, nrm = fd.isosurface(grid, d_values, float(iso))
            if verts.shape[0] == 0:
                continue
            s = Surface(vertices=verts, triangles=tris, normals=nrm,
                        name=surface_name if individual else f"{surface_name}_{iso}",
                        values=np.zeros(verts.shape[0]) + iso)
            s.colour = colour
            out.append(s)
        return out
