"""Isosurface oracle: the level set {f = iso} of node values on a structured
grid under the piecewise-linear interpolant on the Freudenthal triangulation
(6 tetrahedra per cell along the main diagonal).  TEST INFRASTRUCTURE ONLY.

The reference extracts isosurfaces with VTK's contour filter
(DiscreteInterpolator.surfaces, packages/loop_interpolation/src/
loop_interpolation/_discrete_interpolator.py:1395-1405, through pyvista) or
skimage's marching_cubes (LoopStructural/utils/_surface.py:82); neither
library is installed, so this restatement is the definition the GPU kernel is
checked against, and parity with the reference's own surfaces is unpinned.
Properties the tests add: vertices on the level set of the interpolant, a
closed surface for a closed level set, normals along +grad f, areas of planes
and spheres.

Plain Python loops: for grids of a few thousand cells.
"""
from __future__ import annotations

import numpy as np

# the 6 tetrahedra of a cell as corner bitmasks (bit 0: +x, bit 1: +y, bit 2: +z)
TETS = ((0, 1, 3, 7), (0, 1, 5, 7), (0, 2, 3, 7), (0, 2, 6, 7), (0, 4, 5, 7), (0, 4, 6, 7))


def isosurface(values, nsteps, origin, step, iso):
    """Triangles (T, 3, 3) of coordinates, each wound with its normal along
    +grad f of its tetrahedron.  ``values``: one per node, node order
    i + nx * (j + ny * k)."""
    nx, ny, nz = (int(v) for v in nsteps)
    f = np.asarray(values, dtype=float).reshape(nz, ny, nx)
    origin = np.asarray(origin, dtype=float)
    step = np.asarray(step, dtype=float)
    tris = []
    for k in range(nz - 1):
        for j in range(ny - 1):
            for i in range(nx - 1):
                c = [f[k + ((b >> 2) & 1), j + ((b >> 1) & 1), i + (b & 1)] for b in range(8)]
                if any(np.isnan(c)):
                    continue
                for tet in TETS:
                    up = [v for v in tet if c[v] > iso]
                    dn = [v for v in tet if not c[v] > iso]
                    if not up or not dn:
                        continue

                    def point(u, w):
                        lo, hi = min(u, w), max(u, w)
                        t = (iso - c[lo]) / (c[hi] - c[lo])
                        base = np.array([i + (lo & 1), j + ((lo >> 1) & 1), k + ((lo >> 2) & 1)], dtype=float)
                        d = np.array([(hi & ~lo) & 1, ((hi & ~lo) >> 1) & 1, ((hi & ~lo) >> 2) & 1], dtype=float)
                        return origin + step * (base + t * d)

                    grad = np.zeros(3)
                    for s in range(3):
                        a, b = tet[s], tet[s + 1]
                        ax = {1: 0, 2: 1, 4: 2}[b & ~a]
                        grad[ax] = (c[b] - c[a]) / step[ax]
                    if len(up) == 1 or len(dn) == 1:
                        apex, other = (up[0], dn) if len(up) == 1 else (dn[0], up)
                        polys = [[point(apex, other[0]), point(apex, other[1]), point(apex, other[2])]]
                    else:
                        q = [point(up[0], dn[0]), point(up[0], dn[1]), point(up[1], dn[1]), point(up[1], dn[0])]
                        polys = [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
                    for p0, p1, p2 in polys:
                        if np.dot(np.cross(p1 - p0, p2 - p0), grad) < 0.0:
                            p1, p2 = p2, p1
                        tris.append([p0, p1, p2])
    return np.array(tris).reshape(-1, 3, 3)


def canonical(tris, decimals=None):
    """Sorted list of triangles, each rotated (orientation kept) to start at
    its lexicographically smallest vertex (coordinates rounded when asked)."""
    out = []
    tris = np.asarray(tris, dtype=float)
    if decimals is not None:
        tris = np.round(tris, decimals)
    for t in tris:
        keys = [tuple(v) for v in t]
        r = min(range(3), key=lambda m: keys[m])
        out.append(tuple(keys[(r + m) % 3] for m in range(3)))
    return sorted(out)
