"""CPU oracle (test infrastructure only) of faulted-feature evaluation: a
numpy restatement of the reference's fault displacement and the evaluation
of a faulted feature, used by tests/ and nowhere in the product.

Reference (LoopStructural/modelling/features/):
  fault/_fault_function.py  smooth_peak :12-16, CubicFunction :40-150,
                            Composite :197-230, FaultDisplacement :310-361,
                            BaseFault :397-424, BaseFault3D :427-456
  fault/_fault_segment.py   FaultSegment.apply_to_points :315-423
  _geological_feature.py    evaluate_value :116-157, evaluate_gradient :159-235
  LoopStructural/utils/maths.py  regular_tetraherdron_for_points :354-386,
                                 gradient_from_tetrahedron :388-424
Pinned by tests/test_oracle_faults.py against fixtures recorded from the
reference (tests/golden/make_golden.py --faults).  The reference's faulted
gradient raises (it stores the (N, 3) gradients into the (N, 4) array of the
straddle check); the fixture records the same steps assembled from the
reference's own functions into an (N, 3) array, and this oracle follows them.
"""
from __future__ import annotations

import numpy as np

from .fd_oracle import Grid, evaluate_gradient_local, evaluate_value_local


def smooth_peak(x):  # FF:12-16
    v = np.zeros(x.shape)
    m = (x >= -1) & (x <= 1)
    v[m] = x[m] ** 4 - 2 * x[m] ** 2 + 1
    return v


class Cubic:  # FF:40-150 (fitted on first use)
    def __init__(self, cstr=(), grad=(), lim=(-1, 1), min_v=-99999, max_v=999999):
        self.A = [[x ** 3, x ** 2, x, 1.0] for x, _ in cstr] + [[3 * x ** 2, 2 * x, 1.0, 0.0] for x, _ in grad]
        self.B = [y for _, y in cstr] + [g for _, g in grad]
        self.lim, self.min_v, self.max_v = list(lim), min_v, max_v
        A, B = np.array(self.A), np.array(self.B)
        self.w = np.linalg.lstsq(A.T @ A, A.T @ B, rcond=None)[0]

    def __call__(self, v):
        w = self.w
        e = w[0] * v ** 3 + w[1] * v ** 2 + w[2] * v + w[3]
        e[v > self.lim[1]] = w[0] * self.lim[1] ** 3 + w[1] * self.lim[1] ** 2 + w[2] * self.lim[1] + w[3]
        e[v < self.lim[0]] = w[0] * self.lim[0] ** 3 + w[1] * self.lim[0] ** 2 + w[2] * self.lim[0] + w[3]
        e[e > self.max_v] = self.max_v
        e[e < self.min_v] = self.min_v
        return e


def composite(pos, neg):  # FF:197-230
    def f(v):
        r = np.zeros(v.shape)
        r[v > 0] = pos(v[v > 0])
        r[v < 0] = neg(v[v < 0])
        return r
    return f


def ones(v):
    return np.ones(v.shape)


def displacement(gxf, gyf, gzf, scale=0.5):  # FF:310-361
    return lambda gx, gy, gz: scale * gxf(gx) * gyf(gy) * gzf(gz)


def base_fault():  # FF:397-424
    hw = Cubic(cstr=[(0, 1), (1, 0)], grad=[(0, 0), (1, 0)], lim=(0, 1))
    fw = Cubic(cstr=[(0, -1), (-1, 0)], grad=[(0, 0), (-1, 0)], lim=(-1, 0))
    return displacement(composite(hw, fw), ones, smooth_peak)


def base_fault_3d():  # FF:427-456
    hw = Cubic(cstr=[(0, 1), (1, 0)], grad=[(0, 0), (1, 0)], max_v=1)
    fw = Cubic(cstr=[(0, -1), (-1, 0)], grad=[(0, 0), (-1, 0)], min_v=-1)
    return displacement(composite(hw, fw), smooth_peak, smooth_peak)


class Field:
    """A solved FD field (node values c on `grid`) in world coordinates."""

    def __init__(self, grid: Grid, c):
        self.grid, self.c = grid, np.asarray(c, dtype=float)

    def value(self, p):
        return evaluate_value_local(self.grid, p, self.c)

    def gradient(self, p):
        return evaluate_gradient_local(self.grid, p, self.c)


def apply_to_points(frame, points, disp, fn, steps=10):  # FS:315-423
    """frame = (gx, gy, gz) Fields; fn = displacement function or None."""
    newp = np.array(points, dtype=float)
    gx, gy, gz = (f.value(newp) for f in frame)
    d = np.zeros(gx.shape)
    ok = ~np.isnan(gx) & ~np.isnan(gy) & ~np.isnan(gz)
    d[ok & (np.nan_to_num(gx) > 0)] = 1.0
    if fn is not None:
        d[ok] = fn(gx[ok], gy[ok], gz[ok])
    mask = np.abs(d) > 0.0
    for i in range(steps):
        if i == 0:
            gx_m, gy_m, gz_m = gx[mask], gy[mask], gz[mask]
        else:
            gx_m, gy_m, gz_m = (f.value(newp[mask]) for f in frame)
        g = frame[1].gradient(newp[mask])
        d = np.zeros(gx_m.shape)
        ok = ~np.isnan(gx_m) & ~np.isnan(gy_m) & ~np.isnan(gz_m)
        d[ok & (np.nan_to_num(gx_m) > 0)] = 1.0
        if fn is not None:
            d[ok] = fn(gx_m[ok], gy_m[ok], gz_m[ok])
        d *= disp
        mag = np.zeros(g.shape[0])
        mag[ok] = np.linalg.norm(g[ok], axis=1)
        g[mag > 0] /= mag[mag > 0, None]
        g *= (1.0 / steps) * d[:, None]
        newp[mask] += g
    return newp


REGULAR_TETRA = np.array([[np.sqrt(8 / 9), 0, -1 / 3], [-np.sqrt(2 / 9), np.sqrt(2 / 3), -1 / 3],
                          [-np.sqrt(2 / 9), -np.sqrt(2 / 3), -1 / 3], [0, 0, 1]])


def tetrahedra(p, scale):
    return p[:, None, :] + scale * REGULAR_TETRA[None]


def tetra_gradient(tet, val):
    """Gradient of the linear interpolant over each tetrahedron: solves
    (v_k - v_0) . g = f_k - f_0."""
    M = tet[:, 1:, :] - tet[:, :1, :]
    r = val[:, 1:] - val[:, :1]
    return np.linalg.solve(M, r[:, :, None])[:, :, 0]


def faulted_value(field, faults, pts):
    """faults = [(frame, disp, fn)] applied in order, then the field."""
    p = np.array(pts, dtype=float)
    for frame, disp, fn in faults:
        p = apply_to_points(frame, p, disp, fn)
    return field.value(p)


def faulted_gradient(field, faults, pts, scale):
    tet = tetrahedra(pts, scale)
    while True:
        resolved = True
        for frame, _d, _f in faults:
            gx = frame[0].value(tet.reshape(-1, 3))
            bad = np.isnan(gx)
            if bad.any() and not bad.all():
                from scipy import spatial

                flat = tet.reshape(-1, 3)
                _dist, i = spatial.cKDTree(flat[~bad]).query(flat[bad])
                gx[bad] = gx[~bad][i]
            gx = gx.reshape(-1, 4)
            if not np.all(np.all(gx > 0, axis=1) | np.all(gx < 0, axis=1)):
                scale *= 0.5
                tet = tetrahedra(pts, scale)
                resolved = False
        if resolved:
            break
    vals = faulted_value(field, faults, tet.reshape(-1, 3)).reshape(-1, 4)
    return tetra_gradient(tet, vals), scale
