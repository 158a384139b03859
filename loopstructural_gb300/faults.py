"""Faulted features on the GPU: points restored through fault slip events,
then the feature's field evaluated (the caller of the evaluation kernels).

Reference (LoopStructural/modelling/features/):
  fault/_fault_function.py (FF)  profile functions and FaultDisplacement
  fault/_fault_segment.py  (FS)  FaultSegment.apply_to_points :315-423
  _geological_feature.py   (GF)  GeologicalFeature.evaluate_value :116-157,
                                 evaluate_gradient :159-235
  _base_geological_feature.py    _calculate_mask :229-250, _apply_faults :252-270
  LoopStructural/utils/maths.py  regular_tetraherdron_for_points :354-386,
                                 gradient_from_tetrahedron :388-424

The restoration of a point through one fault (frame evaluation, displacement
profile, `steps` integration steps along the slip direction) runs in one CUDA
thread per point (ls_fault_apply); the field and the tetrahedron gradients
run on the evaluation kernels.  Frame fields are solved FD interpolators of
this package (their c on the device) or anything with ``interpolator``
attributes pointing at one; frame features that are themselves faulted are
not supported (NotImplementedError).

Profile functions accept this module's classes and, duck-typed, the
reference's own objects (a CubicFunction has ``solve``/``w``/``lim``/
``max_v``/``min_v``; a Composite ``positive``/``negative``).
"""
from __future__ import annotations

import ctypes as C
import logging

import numpy as np

from . import _lib

logger = logging.getLogger(__name__)


# ---------------------------------------------------------------------------
# profile functions (FF)
# ---------------------------------------------------------------------------
def smooth_peak(x):
    """x^4 - 2 x^2 + 1 on [-1, 1], 0 elsewhere (FF:12-16)."""
    x = np.asarray(x, dtype=float)
    inside = (x >= -1) & (x <= 1)
    return np.where(inside, x ** 4 - 2 * x ** 2 + 1, 0.0)


class Ones:
    """Unit displacement for every coordinate value."""

    def __call__(self, v):
        return np.ones(np.shape(v))


class Zeros:
    """No displacement."""

    def __call__(self, v):
        return np.zeros(np.shape(v))


class CubicFunction:
    """a v^3 + b v^2 + c v + d fitted (least squares on the normal equations)
    to value and slope conditions; outside [lim_lo, lim_hi] it keeps its value
    at the nearer limit, and the result is clamped to [min_v, max_v]."""

    def __init__(self):
        self._rows, self._rhs = [], []
        self.w = np.zeros(4)
        self.lim = [-1.0, 1.0]
        self.max_v, self.min_v = 999999.0, -99999.0
        self.up_to_date = False

    def add_cstr(self, x, y):
        self._rows.append([x ** 3, x ** 2, x, 1.0])
        self._rhs.append(y)
        self.up_to_date = False

    def add_grad(self, x, g):
        self._rows.append([3 * x ** 2, 2 * x, 1.0, 0.0])
        self._rhs.append(g)
        self.up_to_date = False

    def add_max(self, v):
        self.max_v = v

    def add_min(self, v):
        self.min_v = v

    def set_lim(self, lo, hi):
        self.lim = [lo, hi]

    def solve(self):
        if self.up_to_date:
            return
        if len(self._rhs) < 3:
            raise ValueError("Underdetermined")
        A, b = np.array(self._rows, dtype=float), np.array(self._rhs, dtype=float)
        self.w = np.linalg.lstsq(A.T @ A, A.T @ b, rcond=None)[0]
        self.up_to_date = True

    def _poly(self, v):
        return self.w[0] * v ** 3 + self.w[1] * v ** 2 + self.w[2] * v + self.w[3]

    def __call__(self, v):
        self.solve()
        v = np.asarray(v, dtype=float)
        e = self._poly(v)
        e = np.where(v > self.lim[1], self._poly(self.lim[1]), e)
        e = np.where(v < self.lim[0], self._poly(self.lim[0]), e)
        e = np.where(e > self.max_v, self.max_v, e)
        return np.where(e < self.min_v, self.min_v, e)


class Composite:
    """`positive` for coordinates > 0, `negative` for < 0, 0 at 0."""

    def __init__(self, positive, negative):
        self.positive, self.negative = positive, negative

    def __call__(self, v):
        v = np.asarray(v, dtype=float)
        out = np.zeros(v.shape)
        out[v > 0] = self.positive(v[v > 0])
        out[v < 0] = self.negative(v[v < 0])
        return out


class FaultDisplacement:
    """scale * gx(gx) * gy(gy) * gz(gz); hw / fw form the composite gx
    profile; missing profiles are Ones (FF:310-361)."""

    def __init__(self, hw=None, fw=None, gx=None, gy=None, gz=None, scale=0.5):
        self.gx = Composite(hw, fw) if (hw is not None and fw is not None) else gx
        self.gx = Ones() if self.gx is None else self.gx
        self.gy = Ones() if gy is None else gy
        self.gz = Ones() if gz is None else gz
        self.scale = scale

    def __call__(self, gx, gy, gz):
        return self.scale * self.gx(gx) * self.gy(gy) * self.gz(gz)


def _wall_cubic(sign, bounded):
    """The hanging-wall (sign +1) / footwall (-1) cubic of the base faults:
    +-1 at 0 with zero slope, 0 with zero slope at +-1."""
    f = CubicFunction()
    f.add_cstr(0, float(sign))
    f.add_grad(0, 0)
    f.add_cstr(float(sign), 0)
    f.add_grad(float(sign), 0)
    if bounded:
        if sign > 0:
            f.add_max(1)
        else:
            f.add_min(-1)
    else:
        f.set_lim(*((0, 1) if sign > 0 else (-1, 0)))
    return f


def base_fault_displacement():
    """The default displacement of a fault slip event (FF:397-424, BaseFault)."""
    return FaultDisplacement(gx=Composite(_wall_cubic(1, False), _wall_cubic(-1, False)), gy=Ones(), gz=smooth_peak)


def base_fault_3d_displacement():
    """FF:427-456, BaseFault3D: bounded walls, a smooth peak along slip too."""
    return FaultDisplacement(gx=Composite(_wall_cubic(1, True), _wall_cubic(-1, True)), gy=smooth_peak,
                             gz=smooth_peak)


def _cubic_parts(f):
    f.solve()
    return (np.asarray(f.w, dtype=float), [float(f.lim[0]), float(f.lim[1])],
            [float(f.min_v), float(f.max_v)])


def profile_spec(p) -> "_lib.FaultProfile":
    """ls_fault_profile of one profile function (this module's or, duck-typed,
    the reference's)."""
    spec = _lib.FaultProfile()
    name = getattr(p, "__name__", type(p).__name__)
    if hasattr(p, "positive") and hasattr(p, "negative"):
        spec.kind = _lib.PROFILE_COMPOSITE
        parts = [_cubic_parts(p.positive), _cubic_parts(p.negative)]
    elif hasattr(p, "solve") and hasattr(p, "w"):
        spec.kind = _lib.PROFILE_CUBIC
        parts = [_cubic_parts(p)]
    elif name == "smooth_peak":
        spec.kind = _lib.PROFILE_SMOOTH_PEAK
        parts = []
    elif name == "Zeros":
        spec.kind = _lib.PROFILE_ZEROS
        parts = []
    elif name == "Ones":
        spec.kind = _lib.PROFILE_ONES
        parts = []
    else:
        raise NotImplementedError(f"fault profile {p!r} has no GPU form (ones, zeros, smooth_peak, cubic, composite)")
    for k, (w, lim, clamp) in enumerate(parts):
        for j in range(4):
            spec.w[k][j] = float(w[j])
        spec.lim[k][0], spec.lim[k][1] = lim
        spec.clamp[k][0], spec.clamp[k][1] = clamp
    return spec


# ---------------------------------------------------------------------------
# features
# ---------------------------------------------------------------------------
def _affine_of(box):
    """(to_local 3x4, to_world 3x3) of an interpolator's bounding box (identity
    without one), read from its matrices or probed from project()."""
    if box is None:
        return np.hstack([np.eye(3), np.zeros((3, 1))]), np.eye(3)
    if hasattr(box, "world_to_local_matrix") and hasattr(box, "local_to_world_matrix"):
        w2l, l2w = np.asarray(box.world_to_local_matrix), np.asarray(box.local_to_world_matrix)
        return w2l[:3, :4].copy(), l2w[:3, :3].copy()
    o = np.asarray(box.project(np.zeros((1, 3))), dtype=float)[0]
    cols = np.asarray(box.project(np.eye(3)), dtype=float) - o
    rot = np.asarray(box.reproject_vectors(np.eye(3)), dtype=float).T
    return np.hstack([cols.T, o[:, None]]), rot


def _interpolator_of(feature):
    return getattr(feature, "interpolator", feature)


class GeologicalFeature:
    """A scalar field (a solved FD / P1 interpolator of this package) that may
    be displaced by faults and limited to regions (callables returning a
    boolean mask of the points), with the reference's evaluation semantics:
    values NaN where masked out, points restored through every fault in order
    before the field is read, gradients of faulted features from a regular
    tetrahedron around each point (GF:159-235)."""

    def __init__(self, name, interpolator, faults=None, regions=None, model=None):
        self.name = name
        self.interpolator = interpolator
        self.faults = list(faults) if faults else []
        self.regions = list(regions) if regions else []
        self.model = model
        self.faults_enabled = True

    def _calculate_mask(self, pos, ignore_regions=False):
        mask = np.ones(pos.shape[0], dtype=bool)
        if not ignore_regions:
            for r in self.regions:
                mask = np.logical_and(mask, r(pos))
        return mask

    def _apply_faults(self, pts):
        if not self.faults_enabled or not self.faults:
            return pts
        return apply_faults(self.faults, pts)

    def evaluate_value(self, pos, ignore_regions=False, fillnan=None):
        pos = np.asarray(pos, dtype=float)
        if pos.ndim != 2 or pos.shape[1] != 3:
            raise ValueError("Need Nx3 array of xyz points to evaluate value")
        v = np.full(pos.shape[0], np.nan)
        mask = self._calculate_mask(pos, ignore_regions)
        pts = self._apply_faults(pos)
        if np.any(mask):
            v[mask] = self.interpolator.evaluate_value(pts[mask])
        if fillnan == "nearest":
            from scipy import spatial

            bad = np.isnan(v)
            if np.any(bad) and not np.all(bad):
                _d, i = spatial.cKDTree(pts[~bad]).query(pts[bad])
                v[bad] = v[~bad][i]
        return v

    def evaluate_gradient(self, pos, ignore_regions=False, element_scale_parameter=None):
        pos = np.asarray(pos, dtype=float)
        if pos.ndim != 2 or pos.shape[1] != 3:
            raise ValueError("Need Nx3 array of xyz points to evaluate gradient")
        if element_scale_parameter is None:
            box = getattr(self.model, "bounding_box", None) if self.model is not None else None
            element_scale_parameter = np.min(box.step_vector) / 10 if box is not None else 1.0
        else:
            element_scale_parameter = float(element_scale_parameter)
        v = np.full(pos.shape, np.nan)
        mask = self._calculate_mask(pos, ignore_regions)
        if self.faults and self.faults_enabled:
            return tetrahedron_gradient(self, pos, mask, element_scale_parameter)
        if np.any(mask):
            v[mask] = self.interpolator.evaluate_gradient(pos[mask])
        return v


class FaultSegment:
    """A fault slip event: the three fault-frame features (gx normal to the
    fault surface, gy along slip, gz along the fault's extent), a
    displacement magnitude and `steps` integration steps (FS:25-60).  As in
    the reference, the constructor keeps the base displacement profile
    (BaseFault); assign ``faultfunction`` (a FaultDisplacement, a profile
    object, or "BaseFault" / "BaseFault3D") to change it."""

    def __init__(self, name, features, faultfunction=None, steps=10, displacement=1.0):
        self.name = name
        self.features = list(features)
        if len(self.features) != 3:
            raise ValueError("a fault needs its three frame features")
        self.displacement = displacement
        self.steps = steps
        self._faultfunction = base_fault_displacement()
        self.faults_enabled = True

    def __getitem__(self, i):
        return self.features[i]

    @property
    def faultfunction(self):
        return self._faultfunction

    @faultfunction.setter
    def faultfunction(self, value):
        if isinstance(value, FaultDisplacement) or (hasattr(value, "gx") and hasattr(value, "scale")):
            self._faultfunction = value
        elif isinstance(value, str) and value == "BaseFault":
            self._faultfunction = base_fault_displacement()
        elif isinstance(value, str) and value == "BaseFault3D":
            self._faultfunction = base_fault_3d_displacement()
        else:
            raise ValueError("Fault function must be a function or BaseFault")

    def descriptor(self):
        """The ls_fault of this slip event (frame fields on the device)."""
        f = _lib.Fault()
        for k, feat in enumerate(self.features):
            if getattr(feat, "faults", None):
                raise NotImplementedError("frame features displaced by other faults are not supported")
            interp = _interpolator_of(feat)
            interp.update()
            fr = f.frame[k]
            fr.grid = interp.support.grid3()
            fr.d_c = _lib.ptr(interp._c_device())
            to_local, to_world = _affine_of(getattr(interp, "bounding_box", None))
            for a in range(3):
                for b in range(4):
                    fr.to_local[a][b] = float(to_local[a, b])
                for b in range(3):
                    fr.to_world[a][b] = float(to_world[a, b])
        f.displacement = float(self.displacement)
        f.steps = int(self.steps)
        fn = self._faultfunction
        f.has_function = 0 if fn is None else 1
        if fn is not None:
            f.scale = float(fn.scale)
            for k, prof in enumerate((fn.gx, fn.gy, fn.gz)):
                f.profile[k] = profile_spec(prof)
        return f

    def apply_to_points(self, points, reverse=False):
        """Restored positions of `points` (N x 3) through this fault (FS:315-423)."""
        return apply_faults([self], np.asarray(points, dtype=float))


def apply_faults(faults, pts):
    """Points restored through each fault in order (host arrays in and out;
    one upload, one kernel per fault, one download)."""
    import torch

    pts = np.ascontiguousarray(np.asarray(pts, dtype=float)[:, :3])
    if pts.shape[0] == 0:
        return pts.copy()
    dev = torch.from_numpy(pts.copy()).to(_lib.device())
    lib = _lib.load()
    keep = []  # descriptors (and the device arrays they point at) live until the kernels ran
    for fault in faults:
        if not getattr(fault, "faults_enabled", True):
            continue
        desc = fault.descriptor()
        keep.append(desc)
        _lib.check(lib.ls_fault_apply(C.byref(desc), _lib.ptr(dev), dev.shape[0], 3, _lib.stream_ptr()))
    return dev.cpu().numpy()


_REGULAR_TETRA = np.array([[np.sqrt(8 / 9), 0.0, -1 / 3], [-np.sqrt(2 / 9), np.sqrt(2 / 3), -1 / 3],
                           [-np.sqrt(2 / 9), -np.sqrt(2 / 3), -1 / 3], [0.0, 0.0, 1.0]])


def regular_tetrahedra(pos, scale):
    """A regular tetrahedron of edge ~1.63 scale centred on every point (N, 4, 3)."""
    return pos[:, None, :] + scale * _REGULAR_TETRA[None, :, :]


def tetrahedron_gradient(feature, pos, mask, scale, max_halvings=64):
    """GF:187-226: tetrahedra around the points, shrunk (all of them) while any
    one straddles a fault surface (its four gx values not all of one sign;
    NaN gx filled from the nearest evaluated vertex), then restored through
    the faults; the field at the restored vertices over the original
    tetrahedra gives the gradient.  The reference shrinks without end for a
    point exactly on a fault; here that raises after `max_halvings`."""
    import torch

    tet = regular_tetrahedra(pos, scale)
    for _ in range(max_halvings + 1):
        resolved = True
        for f in feature.faults:
            gx = GeologicalFeature("gx", _interpolator_of(f[0])).evaluate_value(tet.reshape(-1, 3), fillnan="nearest")
            gx = gx.reshape(-1, 4)
            same = np.all(gx > 0, axis=1) | np.all(gx < 0, axis=1)
            if not np.all(same):
                logger.warning("Points are too close to fault %s. Refining the tetrahedron", getattr(f, "name", ""))
                scale *= 0.5
                tet = regular_tetrahedra(pos, scale)
                resolved = False
        if resolved:
            break
    else:
        raise RuntimeError("tetrahedra still straddle a fault after %d halvings: a point lies on a fault surface"
                           % max_halvings)
    moved = feature._apply_faults(tet.reshape(-1, 3))
    values = feature.interpolator.evaluate_value(moved).reshape(-1, 4)
    out = np.full(pos.shape, np.nan)
    if np.any(mask):
        dev = _lib.device()
        t = torch.from_numpy(np.ascontiguousarray(tet[mask])).to(dev)
        vv = torch.from_numpy(np.ascontiguousarray(values[mask])).to(dev)
        g = torch.empty((t.shape[0], 3), dtype=torch.float64, device=dev)
        _lib.check(_lib.load().ls_tetra_gradient(_lib.ptr(t), _lib.ptr(vv), t.shape[0], _lib.ptr(g),
                                                  _lib.stream_ptr()))
        out[mask] = g.cpu().numpy()
    return out
