"""Triangulated isosurfaces of a solved field.

``Surface`` carries the fields of the reference's ``loop_common.geometry.Surface``
that ``DiscreteInterpolator.surfaces`` fills (DI:1395-1405): vertices (V, 3),
triangles (T, 3), plus the vertex normals, the name and the isovalue.
"""
from __future__ import annotations

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
