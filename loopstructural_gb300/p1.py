"""P1 (structured TetMesh) interpolator on the GPU.

Mirrors packages/loop_interpolation/src/loop_interpolation/_p1interpolator.py
(P1): constant-gradient face regularisation (P1:115-166), normal rows
(P1:73-96, w = npw, no /3), value rows (P1:98-113, per-point weight column
ignored), gradient constraints a no-op (P1:70-71), setup order P1:180-246.
"""
from __future__ import annotations

import ctypes as C
import logging

import numpy as np

from . import _lib, fd
from .interpolators import SetupReport, _DiscreteInterpolatorBase

logger = logging.getLogger(__name__)


def face_rows(mesh, weight: float, with_topology: bool = False):
    """All face rows of the mesh on the device (K3): (idc (F,8), a, b, w[, pairs, shared])."""
    import torch

    dev = _lib.device()
    lib = _lib.load()
    g = mesh.grid3()
    nf = C.c_int64(0)
    _lib.check(lib.ls_p1_face_count(C.byref(g), C.byref(nf)))
    F = nf.value
    idc = torch.empty((F, 8), dtype=torch.int64, device=dev)
    a = torch.empty((F, 8), dtype=torch.float64, device=dev)
    b = torch.empty(F, dtype=torch.float64, device=dev)
    w = torch.empty(F, dtype=torch.float64, device=dev)
    pairs = torch.empty((F, 2), dtype=torch.int64, device=dev) if with_topology else None
    shared = torch.empty((F, 3), dtype=torch.int64, device=dev) if with_topology else None
    _lib.check(lib.ls_p1_face_rows(C.byref(g), float(weight), _lib.ptr(pairs), _lib.ptr(shared), _lib.ptr(idc),
                                   _lib.ptr(a), _lib.ptr(b), _lib.ptr(w), _lib.stream_ptr()))
    if with_topology:
        return idc, a, b, w, pairs, shared
    return idc, a, b, w


def face_rows_directional(mesh, weight: float, vectors: np.ndarray):
    """Face rows with the normal replaced by one direction per face (F, 3)."""
    import torch

    dev = _lib.device()
    lib = _lib.load()
    g = mesh.grid3()
    nf = C.c_int64(0)
    _lib.check(lib.ls_p1_face_count(C.byref(g), C.byref(nf)))
    F = nf.value
    d_vec = torch.from_numpy(np.ascontiguousarray(vectors, dtype=np.float64)).to(dev)
    idc = torch.empty((F, 8), dtype=torch.int64, device=dev)
    a = torch.empty((F, 8), dtype=torch.float64, device=dev)
    b = torch.empty(F, dtype=torch.float64, device=dev)
    w = torch.empty(F, dtype=torch.float64, device=dev)
    _lib.check(lib.ls_p1_face_rows_directional(C.byref(g), float(weight), _lib.ptr(d_vec), _lib.ptr(idc), _lib.ptr(a),
                                               _lib.ptr(b), _lib.ptr(w), _lib.stream_ptr()))
    return idc, a, b, w


def face_centres(mesh):
    """Centroid of each face's three shared nodes, in face order (P1:169-170)."""
    shared = face_rows(mesh, 1.0, with_topology=True)[5].cpu().numpy()
    n = np.asarray(mesh.nsteps, dtype=np.int64)
    ijk = np.stack([shared % n[0], (shared // n[0]) % n[1], shared // (n[0] * n[1])], axis=-1)
    coords = np.asarray(mesh.origin, dtype=float) + ijk * np.asarray(mesh.step_vector, dtype=float)
    return coords.mean(axis=1)


def locate(mesh, pts: np.ndarray):
    import torch

    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n = pts.shape[0]
    d_pts = torch.from_numpy(pts).to(dev)
    tet = torch.empty(n, dtype=torch.int64, device=dev)
    bc = torch.empty((n, 4), dtype=torch.float64, device=dev)
    g = mesh.grid3()
    _lib.check(lib.ls_p1_locate(C.byref(g), _lib.ptr(d_pts), n, pts.shape[1], _lib.ptr(tet), _lib.ptr(bc),
                                _lib.stream_ptr()))
    return tet.cpu().numpy(), bc.cpu().numpy()


def point_rows(mesh, kind: int, pts: np.ndarray, weight: float):
    import torch

    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, ld = pts.shape
    per = 3 if kind == _lib.ROWS_NORM else 1
    d_pts = torch.from_numpy(pts).to(dev)
    idc = torch.empty((per * n, 4), dtype=torch.int64, device=dev)
    a = torch.empty((per * n, 4), dtype=torch.float64, device=dev)
    b = torch.empty(per * n, dtype=torch.float64, device=dev)
    w = torch.empty(per * n, dtype=torch.float64, device=dev)
    cnt = C.c_int64(0)
    g = mesh.grid3()
    _lib.check(lib.ls_p1_point_rows(C.byref(g), kind, _lib.ptr(d_pts), n, ld, float(weight), _lib.ptr(idc),
                                    _lib.ptr(a), _lib.ptr(b), _lib.ptr(w), C.byref(cnt), _lib.stream_ptr()))
    r = per * cnt.value
    return idc[:r], a[:r], b[:r], w[:r]


def eval_points(mesh, c, pts: np.ndarray, value=True, gradient=True):
    import torch

    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n = pts.shape[0]
    c_t = c if isinstance(c, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(c, dtype=np.float64))
    c_t = c_t.to(device=dev, dtype=torch.float64).contiguous()
    d_pts = torch.from_numpy(pts).to(dev)
    v = torch.empty(n, dtype=torch.float64, device=dev) if value else None
    gr = torch.empty((n, 3), dtype=torch.float64, device=dev) if gradient else None
    g = mesh.grid3()
    _lib.check(lib.ls_p1_eval_points(C.byref(g), _lib.ptr(c_t), _lib.ptr(d_pts), n, pts.shape[1], _lib.ptr(v),
                                     _lib.ptr(gr), _lib.stream_ptr()))
    return (fd.to_host(v) if value else None, fd.to_host(gr) if gradient else None)


class P1Interpolator(_DiscreteInterpolatorBase):
    """Piecewise-linear interpolator on a TetMesh (P1:23-299)."""

    def __init__(self, mesh):
        super().__init__(mesh)
        self.interpolation_weights = {"cgw": 0.1, "cpw": 1.0, "npw": 1.0, "gpw": 1.0, "tpw": 1.0, "ipw": 1.0}
        self.use_regularisation_weight_scale = False

    def setup_interpolator(self, **kwargs) -> SetupReport:
        self.reset()
        cfg = self.resolve_regularisation_config(regularisation=kwargs.get("regularisation", None),
                                                 directional_regularisation=kwargs.get("directional_regularisation",
                                                                                       None))
        if cfg.isotropic is not None:
            self.interpolation_weights["cgw"] = cfg.isotropic
        for k, v in kwargs.items():
            self.up_to_date = False
            if k in ("regularisation", "directional_regularisation"):
                continue
            self.interpolation_weights[k] = v
        self.use_regularisation_weight_scale = bool(kwargs.get("use_regularisation_weight_scale", False))
        self.regularisation_weight_sigma = kwargs.get("regularisation_weight_sigma", None)
        self._reg_scale = self._regularisation_scale() if self.use_regularisation_weight_scale else None  # P1:212-214
        w = self.interpolation_weights
        if w["cgw"] > 0.0:
            self.minimise_edge_jumps(w["cgw"])
        self.add_directional_regularisation(cfg.directional)  # P1:229
        # gradient constraints: no-op in the reference P1 (P1:70-71)
        normals = self.get_norm_constraints()
        if normals.shape[0] > 0:
            self._add_family("norm", *point_rows(self.support, _lib.ROWS_NORM, normals, w["npw"]))
        values = self.get_value_constraints()
        if values.shape[0] > 0:
            self._add_family("value", *point_rows(self.support, _lib.ROWS_VALUE, values, w["cpw"]))
        tangents = self.get_tangent_constraints()
        if tangents.shape[0] > 0:  # DI:668-682 add_tangent_constraints
            self.add_gradient_orthogonal_constraints(tangents[:, :3], tangents[:, 3:6], w["tpw"])
        self.add_value_inequality_constraints()  # P1:243-244 (the DI defaults: upper bound 1.0)
        self.add_inequality_pairs_constraints()
        self.up_to_date = False
        return SetupReport({name: f.n_rows for name, f in self.constraints.items()})

    # -- inequality rows (DI:509-593 on the TetMesh) ---------------------------
    def _barycentric_rows(self, points):
        """(idc, raw barycentric weights) of the points inside the mesh, in
        order (device), and the host mask of those points."""
        tet, _bc = locate(self.support, np.ascontiguousarray(points[:, :3]))
        inside = tet >= 0
        if not inside.any():
            return None, None, inside
        pts = np.ascontiguousarray(np.column_stack([points[:, :3], np.zeros(points.shape[0])]))
        idc, a, _b, _w = point_rows(self.support, _lib.ROWS_VALUE, pts, 1.0)
        # the rows come normalised (bc / |bc|); barycentric weights sum to 1
        return idc, a / a.sum(dim=1, keepdim=True), inside

    def add_value_inequality_constraints(self, w=1.0):
        """lower <= f(x) <= upper at the inequality points inside the mesh
        (DI:509-518); w is not used, as in the reference."""
        import torch

        points = self.get_inequality_value_constraints()
        if points.shape[0] == 0:
            return
        idc, a, inside = self._barycentric_rows(points)
        if idc is None:
            return
        bounds = torch.from_numpy(np.ascontiguousarray(points[inside, 3:5])).to(_lib.device())
        self._add_inequality_family("inequality_value", idc, a, bounds)

    def add_inequality_pairs_constraints(self, w=1.0, upper_bound=1.0, lower_bound=-np.inf, pairs=None):
        """lower_bound <= f(p) - f(q) <= upper_bound for every point p of the
        group pair[0] and q of pair[1] inside the mesh; without ``pairs``,
        every pair of distinct group ids (i < j) (DI:520-593)."""
        import torch

        points = self.get_inequality_pairs_constraints()
        if points.shape[0] == 0:
            return
        ids = points[:, 3]
        if not pairs:
            u = np.unique(ids)
            pairs = [(u[i], u[j]) for i in range(len(u)) for j in range(i + 1, len(u))]
        dev = _lib.device()
        for pair in pairs:
            upper, lower = points[ids == pair[0]], points[ids == pair[1]]
            iu_, au, in_u = self._barycentric_rows(upper)
            il_, al, in_l = self._barycentric_rows(lower)
            if (~in_u).sum() > 0:
                logger.warning(f"Upper points not in mesh {upper[~in_u]}")
            if (~in_l).sum() > 0:
                logger.warning(f"Lower points not in mesh {lower[~in_l]}")
            if iu_ is None or il_ is None:
                continue
            nu, nl = int(in_u.sum()), int(in_l.sum())
            gu, gl = np.meshgrid(np.arange(nu), np.arange(nl))  # upper index fastest
            su = torch.from_numpy(gu.ravel()).to(dev)
            sl = torch.from_numpy(gl.ravel()).to(dev)
            idc = torch.cat([iu_[su], il_[sl]], 1).contiguous()
            a = torch.cat([au[su], -al[sl]], 1).contiguous()
            bounds = torch.empty((idc.shape[0], 2), dtype=torch.float64, device=dev)
            bounds[:, 0] = float(lower_bound)
            bounds[:, 1] = float(upper_bound)
            self._add_inequality_family(f"inequality_pairs_{pair[0]}_{pair[1]}", idc, a, bounds)

    def add_gradient_orthogonal_constraints(self, points, vectors, w=1.0, b=0,
                                            name="undefined gradient orthogonal constraint"):
        """Rows grad(f) . v/|v| = b at the points inside the mesh, weight w
        times the containing tetrahedron's volume (P1:248-296).  The reference
        normalises the caller's ``vectors`` in place; here the caller's array
        is left unchanged."""
        points = np.asarray(points, dtype=float)
        if points.shape[0] == 0:
            return
        vectors = np.asarray(vectors, dtype=float)
        arr = np.empty((points.shape[0], 7))
        arr[:, :3] = points[:, :3]
        arr[:, 3:6] = vectors[:, :3]
        arr[:, 6] = b
        idc, a, bb, ww = point_rows(self.support, _lib.ROWS_ORTHOGONAL, arr, float(w))
        if idc.shape[0] == 0:
            logger.warning("%d gradient constraints not added: outside of model bounding box", points.shape[0])
        else:
            self._add_family(name, idc, a, bb, ww)
        self.up_to_date = False

    # -- directional regularisation (P1:169-178) -----------------------------
    def get_regularisation_sample_points(self) -> np.ndarray:
        return face_centres(self.support)

    def _regularisation_sample_shape(self):
        nf = C.c_int64(0)
        _lib.check(_lib.load().ls_p1_face_count(C.byref(self.support.grid3()), C.byref(nf)))
        return (int(nf.value), 3)

    def _add_directional_regularisation(self, weight, vectors, name="directional regularisation"):
        self.minimise_edge_jumps(w=weight, vector=vectors, name=name)

    def minimise_edge_jumps(self, w=0.1, vector_func=None, vector=None, name="edge jump"):
        """Constant-gradient face rows (P1:115-166); ``vector`` (one row per
        face) or ``vector_func`` (evaluated at the midpoint of each shared
        face's first two nodes, P1:126-127; ``vector`` wins when both are
        given) replaces the face normal.  The shared nodes are taken in
        ascending order; the reference's come from an unstable sort that keeps
        that order on the meshes the fixtures record.  With use_regularisation_weight_scale
        each row's weight is w times the mean of the two tetrahedra's mean
        node scales (P1:150-155)."""
        nfaces = self._regularisation_sample_shape()[0]
        if vector is None or np.shape(vector)[0] != nfaces:
            vector = None
            if vector_func is not None:
                shared = face_rows(self.support, 1.0, with_topology=True)[5].cpu().numpy()
                nodes = self.support.nodes
                vector = np.asarray(vector_func((nodes[shared[:, 0]] + nodes[shared[:, 1]]) / 2), dtype=float)
        if vector is not None:
            idc, a, b, ww = face_rows_directional(self.support, w, np.asarray(vector, dtype=float))
        else:
            idc, a, b, ww = face_rows(self.support, w)
        if self._reg_scale is not None:
            s = self._reg_scale[idc]
            m1 = (((s[:, 0] + s[:, 1]) + s[:, 2]) + s[:, 3]) / 4
            m2 = (((s[:, 4] + s[:, 5]) + s[:, 6]) + s[:, 7]) / 4
            ww = (0.5 * (m1 + m2) * float(w)).contiguous()
        self._add_family(name, idc, a, b, ww)
        self.up_to_date = False

    def _data_rows(self):
        return [(f.idc, f.a, f.b, f.w) for f in self.constraints.values()]

    def _make_system(self, rows):
        ridge = self.ridge_factor if self.add_ridge_regulatisation else 0.0
        zero = {k: 0.0 for k in ("dxx", "dyy", "dzz", "dxy", "dyz", "dxz", "dx", "dy", "dz")}
        return fd.FdSystem(self.support, zero, rows, ridge)

    def _build_system(self):
        return self._make_system(self._data_rows())

    def _solver_options(self, solver, tol, solver_kwargs):
        solver, opts = super()._solver_options(solver, tol, solver_kwargs)
        # the multigrid hierarchy is the FD stencil's: Jacobi-PCG for P1
        if solver == "admm":
            opts[1]["preconditioner"] = "jacobi"
        else:
            opts["preconditioner"] = "jacobi"
        return solver, opts

    def _matrix_rows(self):
        return sum(f.n_rows for f in self.constraints.values())

    def _matrix_nnz(self):
        return sum(f.n_rows * f.idc.shape[1] for f in self.constraints.values())

    def _eval_points(self, loc, value=True, gradient=True):
        return eval_points(self.support, self._c_device(), loc, value=value, gradient=gradient)

    def _evaluate_value_local(self, locations):
        self.update()
        loc = np.asarray(locations, dtype=float)
        if loc.shape[0] == 0:
            return np.zeros(0)
        return eval_points(self.support, self._c_device(), loc, value=True, gradient=False)[0]

    def _evaluate_gradient_local(self, locations):
        self.update()
        loc = np.asarray(locations, dtype=float)
        if loc.shape[0] == 0:
            return np.zeros((0, 3))
        return eval_points(self.support, self._c_device(), loc, value=False, gradient=True)[1]


PiecewiseLinearInterpolator = P1Interpolator
