"""Device-side FD engine: thin Python wrappers over the C ABI that own the
device buffers (torch tensors) handed to the kernels."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

REG_TAP_VALUES = {
    # normalised stencil values in the reference column order (OP:10-43 masks
    # divided by their L2 norm, DI:361-366)
    "dxx": np.array([1.0, -2.0, 1.0]) / np.sqrt(6.0),
    "dxy": np.array([-0.5, 0.5, 0.5, -0.5]),
}
for _n in ("dyy", "dzz", "dx_lower", "dx_upper", "dy_lower", "dy_upper", "dz_lower", "dz_upper"):
    REG_TAP_VALUES[_n] = REG_TAP_VALUES["dxx"]
for _n in ("dyz", "dxz"):
    REG_TAP_VALUES[_n] = REG_TAP_VALUES["dxy"]


def _torch():
    import torch

    return torch


def point_rows(support, kind: int, pts: np.ndarray, weight: float):
    """Constraint rows of ``kind`` for the point array (GPU, K1).

    Returns (count, [(idc, a, b, w) per family], nan_flag) with device
    tensors restricted to the inside points."""
    torch = _torch()
    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    npts, ld = pts.shape
    fam = {_lib.ROWS_VALUE: 1, _lib.ROWS_NORM: 3, _lib.ROWS_GRADIENT: 2, _lib.ROWS_TANGENT: 1,
           _lib.ROWS_ORTHOGONAL: 1}[kind]
    d_pts = torch.from_numpy(pts).to(dev)
    idc = torch.empty((fam * npts, 8), dtype=torch.int64, device=dev)
    a = torch.empty((fam * npts, 8), dtype=torch.float64, device=dev)
    b = torch.empty(fam * npts, dtype=torch.float64, device=dev)
    w = torch.empty(fam * npts, dtype=torch.float64, device=dev)
    count = C.c_int64(0)
    nan = C.c_int32(0)
    g = support.grid3()
    _lib.check(lib.ls_fd_point_rows(C.byref(g), kind, _lib.ptr(d_pts), npts, ld, float(weight), _lib.ptr(idc),
                                    _lib.ptr(a), _lib.ptr(b), _lib.ptr(w), C.byref(count), C.byref(nan),
                                    _lib.stream_ptr()))
    n = count.value
    out = [(idc[f * npts:f * npts + n], a[f * npts:f * npts + n], b[f * npts:f * npts + n], w[f * npts:f * npts + n])
           for f in range(fam)]
    return n, out, bool(nan.value)


def weight_scale(support, pts: np.ndarray, alpha: float, sigma: float, scale):
    """scale += 1 + alpha exp(-d^2 / 2 sigma^2), d = the distance from each node
    to the nearest of the points (GPU, ls_fd_weight_scale); `scale` is a device
    FP64 tensor of one entry per node, updated in place."""
    torch = _torch()
    pts = np.ascontiguousarray(pts[:, :3], dtype=np.float64)
    d_pts = torch.from_numpy(pts).to(_lib.device())
    g = support.grid3()
    _lib.check(_lib.load().ls_fd_weight_scale(C.byref(g), _lib.ptr(d_pts), pts.shape[0], 3, float(alpha), float(sigma),
                                              _lib.ptr(scale), _lib.stream_ptr()))
    return scale


def scaled_weights(support, scale, weights, omega):
    """The interior regularisation families with a per-node scale added to the
    directional weight planes `omega` (GPU, ls_fd_scaled_weights); `weights`
    = the six row weights in (dxx, dyy, dzz, dxy, dxz, dyz) order."""
    g = support.grid3()
    w6 = (C.c_double * 6)(*[float(v) for v in weights])
    _lib.check(_lib.load().ls_fd_scaled_weights(C.byref(g), _lib.ptr(scale), C.byref(w6), _lib.ptr(omega),
                                                _lib.stream_ptr()))
    return omega


def pair_rows(support, pts: np.ndarray, pairs: np.ndarray, weight: float):
    """Interface pair rows (GPU): 16 columns per row."""
    torch = _torch()
    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    pairs = np.ascontiguousarray(pairs, dtype=np.int64)
    n = pairs.shape[0]
    d_pts = torch.from_numpy(pts).to(dev)
    d_pairs = torch.from_numpy(pairs).to(dev)
    idc = torch.empty((n, 16), dtype=torch.int64, device=dev)
    a = torch.empty((n, 16), dtype=torch.float64, device=dev)
    b = torch.empty(n, dtype=torch.float64, device=dev)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    g = support.grid3()
    _lib.check(lib.ls_fd_pair_rows(C.byref(g), _lib.ptr(d_pts), pts.shape[1], _lib.ptr(d_pairs), n, float(weight),
                                   _lib.ptr(idc), _lib.ptr(a), _lib.ptr(b), _lib.ptr(w), _lib.stream_ptr()))
    return idc, a, b, w


def directional_weights(support, vector: np.ndarray, weight: float, omega):
    """Adds one directional term's weights to ``omega`` (6 x dof FP64 device
    tensor, family-major) on the GPU; returns the row count of each family
    (dxx, dyy, dzz, dxy, dxz, dyz) the reference would add."""
    torch = _torch()
    lib = _lib.load()
    vec = torch.from_numpy(np.ascontiguousarray(vector, dtype=np.float64)).to(omega.device)
    counts = (C.c_int64 * 6)()
    g = support.grid3()
    _lib.check(lib.ls_fd_directional_weights(C.byref(g), _lib.ptr(vec), 3, float(weight), _lib.ptr(omega), counts,
                                             _lib.stream_ptr()))
    return [int(c) for c in counts]


def reg_shape(support, family: str):
    lib = _lib.load()
    rows = C.c_int64(0)
    taps = C.c_int32(0)
    g = support.grid3()
    _lib.check(lib.ls_fd_reg_shape(C.byref(g), _lib.REG_FAMILIES.index(family), C.byref(rows), C.byref(taps)))
    return rows.value, taps.value


def reg_rows(support, family: str):
    """Explicit column indices of a regularisation family (GPU, K2)."""
    torch = _torch()
    dev = _lib.device()
    lib = _lib.load()
    rows, taps = reg_shape(support, family)
    idc = torch.empty((rows, taps), dtype=torch.int64, device=dev)
    g = support.grid3()
    _lib.check(lib.ls_fd_reg_rows(C.byref(g), _lib.REG_FAMILIES.index(family), _lib.ptr(idc), _lib.stream_ptr()))
    return idc


class FdSystem:
    """Owns an ``ls_fd_handle``: the matrix-free normal equations of one
    interpolator setup."""

    def __init__(self, support, reg_weights: dict, rows, ridge: float, directional=None):
        torch = _torch()
        self.dev = _lib.device()
        self.lib = _lib.load()
        self.support = support
        if rows:
            width = max(r[0].shape[1] for r in rows)
            idc, a, b, w = [], [], [], []
            for ri, ra, rb, rw in rows:
                k = ri.shape[1]
                if k < width:
                    pad_i = torch.full((ri.shape[0], width - k), -1, dtype=torch.int64, device=self.dev)
                    pad_a = torch.zeros((ri.shape[0], width - k), dtype=torch.float64, device=self.dev)
                    ri = torch.cat([ri, pad_i], 1)
                    ra = torch.cat([ra, pad_a], 1)
                idc.append(ri)
                a.append(ra)
                b.append(rb)
                w.append(rw)
            self._idc = torch.cat(idc).contiguous()
            self._a = torch.cat(a).contiguous()
            self._b = torch.cat(b).contiguous()
            self._w = torch.cat(w).contiguous()
            nrows = self._idc.shape[0]
        else:
            width, nrows = 8, 0
            self._idc = self._a = self._b = self._w = None
        s = _lib.FdSystem()
        s.grid = support.grid3()
        for k in ("dxx", "dyy", "dzz", "dxy", "dyz", "dxz", "dx", "dy", "dz"):
            setattr(s, "w_" + k, float(reg_weights.get(k, 0.0)))
        s.ridge = float(ridge)
        s.nrows = nrows
        s.width = width
        s.d_idc = _lib.ptr(self._idc)
        s.d_a = _lib.ptr(self._a)
        s.d_b = _lib.ptr(self._b)
        s.d_w = _lib.ptr(self._w)
        s.d_dir = _lib.ptr(directional) if directional is not None else None
        self.nrows = nrows
        self.handle = C.c_void_p()
        _lib.check(self.lib.ls_fd_create(C.byref(s), C.byref(self.handle), _lib.stream_ptr()))
        self.n = int(self.lib.ls_fd_dof(self.handle))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.ls_fd_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def staged_apply(self) -> bool:
        """True when the finest-level FP32 applies run the TMA-staged kernel."""
        return bool(self.lib.ls_fd_staged_apply(self.handle))

    def apply(self, x):
        torch = _torch()
        x = x.to(self.dev).contiguous()
        y = torch.empty_like(x)
        fn = self.lib.ls_fd_apply if x.dtype == torch.float64 else self.lib.ls_fd_apply_f32
        _lib.check(fn(self.handle, _lib.ptr(x), _lib.ptr(y), _lib.stream_ptr()))
        return y

    def rhs(self):
        torch = _torch()
        y = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        _lib.check(self.lib.ls_fd_rhs(self.handle, _lib.ptr(y), _lib.stream_ptr()))
        return y

    def diagonal(self):
        torch = _torch()
        y = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        _lib.check(self.lib.ls_fd_diagonal(self.handle, _lib.ptr(y), _lib.stream_ptr()))
        return y

    def admm_step(self, row0: int, lo, hi, z, u, x):
        """One ADMM projection over the data rows [row0, row0 + len(z)) (the
        inequality rows; ls_fd_admm_step): updates z, u and the rows'
        right-hand sides in place and returns the five sums
        (|qx - z|^2, |z - z_prev|^2, |qx|^2, |z|^2, |u|^2)."""
        out = (C.c_double * 5)()
        _lib.check(self.lib.ls_fd_admm_step(self.handle, int(row0), int(z.shape[0]), _lib.ptr(lo), _lib.ptr(hi),
                                            _lib.ptr(z), _lib.ptr(u), _lib.ptr(x), out, _lib.stream_ptr()))
        return np.array(out[:], dtype=float)

    def solve(self, x=None, atol=0.0, rtol=1e-5, maxiter=None, precision="mixed", reliable_delta=0.1,
              check_every=64, preconditioner="mg", mg_degree=0):
        """Returns (x device tensor, stats dict)."""
        x, o = self._prepare(x, atol, rtol, maxiter, precision, reliable_delta, check_every, preconditioner)
        o.mg_degree = int(mg_degree)
        st = _lib.SolveStats()
        status = self.lib.ls_fd_solve(self.handle, C.byref(o), _lib.ptr(x), C.byref(st), _lib.stream_ptr())
        _lib.check(status, allow_positive=True)
        return x, _stats_dict(st)

    def _prepare(self, x, atol, rtol, maxiter, precision, reliable_delta, check_every, preconditioner):
        torch = _torch()
        o = _lib.SolveOpts()
        o.precision = _lib.LS_MIXED if precision == "mixed" else _lib.LS_FP64
        if x is None:
            x = torch.zeros(self.n, dtype=torch.float64, device=self.dev)
            o.use_x0 = 0
        else:
            x = x.to(device=self.dev, dtype=torch.float64).contiguous().clone()
            o.use_x0 = 1
        o.atol = float(atol)
        o.rtol = float(rtol)
        o.maxiter = int(maxiter) if maxiter is not None else 0
        o.reliable_delta = float(reliable_delta)
        o.check_every = int(check_every)
        if preconditioner not in ("mg", "jacobi"):
            raise ValueError(f"preconditioner must be 'mg' or 'jacobi', not {preconditioner!r}")
        o.preconditioner = _lib.LS_PRECOND_MG if preconditioner == "mg" else _lib.LS_PRECOND_JACOBI
        return x, o


def _stats_dict(st):
    stats = {k: getattr(st, k) for k, _ in _lib.SolveStats._fields_}
    stats["preconditioner"] = "mg" if st.preconditioner == _lib.LS_PRECOND_MG else "jacobi"
    return stats


def solve_batched(systems, concurrency=8, atol=0.0, rtol=1e-5, maxiter=None, precision="mixed",
                  reliable_delta=0.1, check_every=64, preconditioner="mg"):
    """Solves independent systems (a model ensemble) with up to `concurrency`
    solves in flight on the GPU; returns [(x, stats), ...] in input order."""
    n = len(systems)
    if n == 0:
        return []
    prepared = [s._prepare(None, atol, rtol, maxiter, precision, reliable_delta, check_every, preconditioner)
                for s in systems]
    handles = (C.c_void_p * n)(*[s.handle for s in systems])
    opts = (_lib.SolveOpts * n)(*[o for _, o in prepared])
    xs = (C.c_void_p * n)(*[_lib.ptr(x) for x, _ in prepared])
    stats = (_lib.SolveStats * n)()
    statuses = (C.c_int * n)()
    _torch().cuda.current_stream().synchronize()
    _lib.check(systems[0].lib.ls_fd_solve_batched(handles, opts, xs, stats, n, int(concurrency), statuses))
    out = []
    for i, (x, _) in enumerate(prepared):
        _lib.check(statuses[i], allow_positive=True)
        out.append((x, _stats_dict(stats[i])))
    return out


MG_PROFILE_FIELDS = ("nodes", "apply_ms", "cheb_apply_ms", "resid_apply_ms", "restrict_ms", "prolong_ms",
                     "rows_ms", "coarse_solve_ms", "cheb_main_ms", "cheb_aux_ms")


def mg_vcycle(system: "FdSystem", r):
    """z = V(r): one application of the multigrid preconditioner (FP32
    device tensors)."""
    torch = _torch()
    r = r.to(device=system.dev, dtype=torch.float32).contiguous()
    z = torch.empty_like(r)
    _lib.check(system.lib.ls_fd_mg_vcycle(system.handle, _lib.ptr(r), _lib.ptr(z), _lib.stream_ptr()))
    return z


def profile_mg(system: "FdSystem", reps=20, max_levels=16):
    """Device time per launch of each part of the multigrid V-cycle, per level."""
    out = (C.c_double * (max_levels * len(MG_PROFILE_FIELDS)))()
    nl = C.c_int(0)
    _lib.check(system.lib.ls_fd_profile_mg(system.handle, int(reps), out, max_levels, C.byref(nl), _lib.stream_ptr()))
    k = len(MG_PROFILE_FIELDS)
    return [{f: out[l * k + i] for i, f in enumerate(MG_PROFILE_FIELDS)} for l in range(nl.value)]


MG_SETUP_PHASES = ("host_rows", "tables", "row_coarsening", "data_upload", "diagonals", "eigenvalues",
                   "coarse_inverse", "total")


def setup_profile(system: "FdSystem"):
    """Host wall time (ms) of the multigrid setup phases of the last build."""
    out = (C.c_double * 8)()
    k = _lib.check(system.lib.ls_fd_setup_profile(system.handle, out, 8), allow_positive=True)
    return {MG_SETUP_PHASES[i]: out[i] for i in range(k)}


def mg_apply_level(system: "FdSystem", level: int, x=None):
    """(nodes, A_level x): the FP32 operator of a multigrid level (diagnostic)."""
    torch = _torch()
    nodes = C.c_int64(0)
    _lib.check(system.lib.ls_fd_mg_apply_level(system.handle, int(level), None, None, C.byref(nodes),
                                               _lib.stream_ptr()))
    if x is None:
        return nodes.value, None
    x = x.to(device=system.dev, dtype=torch.float32).contiguous()
    y = torch.empty_like(x)
    _lib.check(system.lib.ls_fd_mg_apply_level(system.handle, int(level), _lib.ptr(x), _lib.ptr(y), C.byref(nodes),
                                               _lib.stream_ptr()))
    return nodes.value, y


def profile_iteration(system: "FdSystem", precision="mixed", reps=20):
    """Device time per launch of each kernel class of one CG iteration."""
    prof = _lib.FdProfile()
    prec = _lib.LS_MIXED if precision == "mixed" else _lib.LS_FP64
    _lib.check(system.lib.ls_fd_profile_iteration(system.handle, prec, int(reps), C.byref(prof), _lib.stream_ptr()))
    return {k: getattr(prof, k) for k, _ in _lib.FdProfile._fields_}


def eval_points(support, c, pts: np.ndarray, value=True, gradient=True):
    torch = _torch()
    dev = _lib.device()
    lib = _lib.load()
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    if pts.ndim == 1:
        pts = pts[None, :]
    n = pts.shape[0]
    c_t = c if isinstance(c, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(c, dtype=np.float64))
    c_t = c_t.to(device=dev, dtype=torch.float64).contiguous()
    if c_t.shape[0] != support.n_nodes:
        raise ValueError(f"cannot assign {c_t.shape[0]} vlaues to array of shape {support.n_nodes}")
    d_pts = torch.from_numpy(pts).to(dev)
    v = torch.empty(n, dtype=torch.float64, device=dev) if value else None
    gr = torch.empty((n, 3), dtype=torch.float64, device=dev) if gradient else None
    g = support.grid3()
    _lib.check(lib.ls_fd_eval_points(C.byref(g), _lib.ptr(c_t), _lib.ptr(d_pts), n, pts.shape[1], _lib.ptr(v),
                                     _lib.ptr(gr), _lib.stream_ptr()))
    return (to_host(v) if value else None, to_host(gr) if gradient else None)


def to_host(t):
    """Device tensor -> numpy array through page-locked host memory: the
    device-to-host copy runs at the interconnect's rate instead of a pageable
    copy's (the page-locked block comes from torch's caching host allocator,
    reused once the returned array is released)."""
    torch = _torch()
    h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    h.copy_(t)
    return h.numpy()


def eval_lattice(support, c_dev, origin, step, counts, value=True, gradient=True):
    """Device tensors of value (Q,) and gradient (Q, 3) on a regular lattice."""
    torch = _torch()
    dev = _lib.device()
    lib = _lib.load()
    q = int(np.prod(counts))
    v = torch.empty(q, dtype=torch.float64, device=dev) if value else None
    gr = torch.empty((q, 3), dtype=torch.float64, device=dev) if gradient else None
    g = support.grid3()
    o3 = (C.c_double * 3)(*[float(x) for x in origin])
    s3 = (C.c_double * 3)(*[float(x) for x in step])
    n3 = (C.c_int64 * 3)(*[int(x) for x in counts])
    _lib.check(lib.ls_fd_eval_lattice(C.byref(g), _lib.ptr(c_dev), C.byref(o3), C.byref(s3), C.byref(n3), _lib.ptr(v),
                                      _lib.ptr(gr), _lib.stream_ptr()))
    return v, gr


def isosurface(support, values, iso: float, normals: bool = True):
    """Level set {f = iso} of node values on a StructuredGrid (GPU): returns
    (vertices (V, 3), triangles (T, 3) int64, normals (V, 3) or None) as host
    arrays.  ``values`` is a device tensor of one value per node."""
    torch = _torch()
    lib = _lib.load()
    values = values.to(dtype=torch.float64).contiguous()
    g = support.grid3()
    h = C.c_void_p()
    nv, nt = C.c_int64(0), C.c_int64(0)
    _lib.check(lib.ls_iso_extract(C.byref(g), _lib.ptr(values), float(iso), C.byref(h), C.byref(nv), C.byref(nt),
                                  _lib.stream_ptr()))
    try:
        verts = torch.empty((nv.value, 3), dtype=torch.float64, device=values.device)
        nrm = torch.empty((nv.value, 3), dtype=torch.float64, device=values.device) if normals else None
        tris = torch.empty((nt.value, 3), dtype=torch.int64, device=values.device)
        _lib.check(lib.ls_iso_copy(h, _lib.ptr(verts), _lib.ptr(nrm), _lib.ptr(tris), _lib.stream_ptr()))
        out = (verts.cpu().numpy(), tris.cpu().numpy(), nrm.cpu().numpy() if normals else None)
    finally:
        lib.ls_iso_destroy(h)
    return out
