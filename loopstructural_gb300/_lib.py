"""ctypes binding of ``libls_gb300.so`` (C ABI in ``include/ls_gb300.h``).

The library is the only compute path: when it is missing or no CUDA device
is visible, every compute entry point raises ``ExtensionUnavailable`` -- there
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

LS_OK = 0
LS_NOT_CONVERGED = 1
LS_NAN = 2
LS_BREAKDOWN = 3
LS_FP64 = 0
ABI_VERSION = 2  # LS_ABI_VERSION of include/ls_gb300.h
LS_MIXED = 1
LS_PRECOND_JACOBI = 0
LS_PRECOND_MG = 1
NOALLOC_MAX_ROWS = 1048576

ROWS_VALUE, ROWS_NORM, ROWS_GRADIENT, ROWS_TANGENT, ROWS_ORTHOGONAL = 0, 1, 2, 3, 4
# directional regularisation weight planes (ls_fd_directional_weights)
DIRECTIONAL_FAMILIES = ("dxx", "dyy", "dzz", "dxy", "dxz", "dyz")
REG_FAMILIES = (
    "dxy", "dyz", "dxz", "dxx", "dyy", "dzz",
    "dx_lower", "dx_upper", "dy_lower", "dy_upper", "dz_lower", "dz_upper",
)

# every symbol include/ls_gb300.h declares
EXPORTS = (
    "ls_last_error", "ls_abi_version",
    "ls_fd_point_rows", "ls_fd_pair_rows", "ls_fd_reg_shape", "ls_fd_reg_rows", "ls_fd_directional_weights", "ls_fd_weight_scale", "ls_fd_scaled_weights",
    "ls_fd_create", "ls_fd_destroy", "ls_fd_dof", "ls_fd_apply", "ls_fd_apply_f32", "ls_fd_apply_noalloc", "ls_fd_rhs",
    "ls_fd_diagonal", "ls_fd_solve", "ls_fd_profile_iteration", "ls_fd_profile_mg", "ls_fd_eval_points", "ls_fd_eval_lattice",
    "ls_fd_eval_adjoint", "ls_fd_set_rhs", "ls_fd_data_rows_apply", "ls_fd_admm_step", "ls_fd_device", "ls_fd_prepare", "ls_fd_solve_batched",
    "ls_fd_mg_apply_level", "ls_fd_setup_profile", "ls_fd_staged_apply", "ls_fd_mg_vcycle", "ls_fd_eval_jets", "ls_fault_apply", "ls_tetra_gradient",
    "ls_p1_face_count", "ls_p1_face_rows", "ls_p1_face_rows_directional", "ls_p1_locate", "ls_p1_point_rows",
    "ls_p1_eval_points", "ls_iso_extract", "ls_iso_copy", "ls_iso_destroy",
)


class ExtensionUnavailable(RuntimeError):
    """The sm_103a library is not built or cannot run here."""


class LsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libls_gb300 status {status}: {msg}")
        self.status = status


class Grid3(C.Structure):
    _fields_ = [("nsteps", C.c_int64 * 3), ("origin", C.c_double * 3), ("step", C.c_double * 3)]

    @classmethod
    def make(cls, nsteps_nodes, origin, step):
        g = cls()
        for d in range(3):
            g.nsteps[d] = int(nsteps_nodes[d])
            g.origin[d] = float(origin[d])
            g.step[d] = float(step[d])
        return g


class FdSystem(C.Structure):
    _fields_ = [
        ("grid", Grid3),
        ("w_dxx", C.c_double), ("w_dyy", C.c_double), ("w_dzz", C.c_double),
        ("w_dxy", C.c_double), ("w_dyz", C.c_double), ("w_dxz", C.c_double),
        ("w_dx", C.c_double), ("w_dy", C.c_double), ("w_dz", C.c_double),
        ("ridge", C.c_double),
        ("nrows", C.c_int64), ("width", C.c_int32),
        ("d_idc", C.c_void_p), ("d_a", C.c_void_p), ("d_b", C.c_void_p), ("d_w", C.c_void_p),
        ("d_dir", C.c_void_p),
    ]


class SolveOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("use_x0", C.c_int32), ("atol", C.c_double), ("rtol", C.c_double),
        ("maxiter", C.c_int64), ("reliable_delta", C.c_double), ("check_every", C.c_int32),
        ("preconditioner", C.c_int32), ("mg_degree", C.c_int32),
    ]


class SolveStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int64), ("reliable_updates", C.c_int64), ("residual", C.c_double),
        ("rhs_norm", C.c_double), ("threshold", C.c_double), ("device_ms", C.c_double),
        ("status", C.c_int32), ("preconditioner", C.c_int32), ("kernel_launches", C.c_int64),
    ]


# fault displacement (ls_fault_*): profile kinds and structures
PROFILE_ONES, PROFILE_ZEROS, PROFILE_SMOOTH_PEAK, PROFILE_CUBIC, PROFILE_COMPOSITE = 0, 1, 2, 3, 4


class FaultProfile(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("w", (C.c_double * 4) * 2),
                ("lim", (C.c_double * 2) * 2), ("clamp", (C.c_double * 2) * 2)]


class FaultField(C.Structure):
    _fields_ = [("grid", Grid3), ("d_c", C.c_void_p), ("to_local", (C.c_double * 4) * 3),
                ("to_world", (C.c_double * 3) * 3)]


class Fault(C.Structure):
    _fields_ = [("frame", FaultField * 3), ("displacement", C.c_double), ("steps", C.c_int32),
                ("has_function", C.c_int32), ("scale", C.c_double), ("profile", FaultProfile * 3)]


class FdProfile(C.Structure):
    _fields_ = [("stencil_ms", C.c_double), ("data_ms", C.c_double), ("update_ms", C.c_double),
                ("iteration_ms", C.c_double), ("stencil_bytes", C.c_double), ("iteration_bytes", C.c_double)]


_lock = threading.Lock()
_lib = None

_P = C.c_void_p
_SIGS = {
    "ls_last_error": (C.c_char_p, []),
    "ls_abi_version": (C.c_int, []),
    "ls_fd_point_rows": (C.c_int, [C.POINTER(Grid3), C.c_int, _P, C.c_int64, C.c_int64, C.c_double, _P, _P, _P, _P,
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int32), _P]),
    "ls_fd_pair_rows": (C.c_int, [C.POINTER(Grid3), _P, C.c_int64, _P, C.c_int64, C.c_double, _P, _P, _P, _P, _P]),
    "ls_fd_reg_shape": (C.c_int, [C.POINTER(Grid3), C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "ls_fd_reg_rows": (C.c_int, [C.POINTER(Grid3), C.c_int, _P, _P]),
    "ls_fd_weight_scale": (C.c_int, [C.POINTER(Grid3), _P, C.c_int64, C.c_int64, C.c_double, C.c_double, _P, _P]),
    "ls_fd_scaled_weights": (C.c_int, [C.POINTER(Grid3), _P, C.POINTER(C.c_double * 6), _P, _P]),
    "ls_fd_directional_weights": (C.c_int, [C.POINTER(Grid3), _P, C.c_int64, C.c_double, _P,
                                            C.POINTER(C.c_int64), _P]),
    "ls_fd_create": (C.c_int, [C.POINTER(FdSystem), C.POINTER(_P), _P]),
    "ls_fd_destroy": (C.c_int, [_P]),
    "ls_fd_dof": (C.c_int64, [_P]),
    "ls_fd_apply": (C.c_int, [_P, _P, _P, _P]),
    "ls_fd_apply_f32": (C.c_int, [_P, _P, _P, _P]),
    "ls_fd_apply_noalloc": (C.c_int, [C.POINTER(FdSystem), _P, _P, C.POINTER(C.c_double), _P]),
    "ls_fd_rhs": (C.c_int, [_P, _P, _P]),
    "ls_fd_diagonal": (C.c_int, [_P, _P, _P]),
    "ls_fd_solve": (C.c_int, [_P, C.POINTER(SolveOpts), _P, C.POINTER(SolveStats), _P]),
    "ls_fd_profile_iteration": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(FdProfile), _P]),
    "ls_fd_profile_mg": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int), _P]),
    "ls_fd_eval_points": (C.c_int, [C.POINTER(Grid3), _P, _P, C.c_int64, C.c_int64, _P, _P, _P]),
    "ls_fd_eval_adjoint": (C.c_int, [C.POINTER(Grid3), _P, C.c_int64, C.c_int64, _P, _P, _P, _P]),
    "ls_fd_set_rhs": (C.c_int, [_P, _P, _P]),
    "ls_fd_device": (C.c_int, [_P]),
    "ls_fd_staged_apply": (C.c_int, [_P]),
    "ls_fd_mg_vcycle": (C.c_int, [_P, _P, _P, _P]),
    "ls_fd_eval_jets": (C.c_int, [C.POINTER(Grid3), _P, _P, C.c_int64, C.c_int64, _P, _P]),
    "ls_fault_apply": (C.c_int, [C.POINTER(Fault), _P, C.c_int64, C.c_int64, _P]),
    "ls_tetra_gradient": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "ls_fd_prepare": (C.c_int, [_P, C.POINTER(SolveOpts)]),
    "ls_fd_mg_apply_level": (C.c_int, [_P, C.c_int, _P, _P, C.POINTER(C.c_int64), _P]),
    "ls_fd_solve_batched": (C.c_int, [C.POINTER(_P), C.POINTER(SolveOpts), C.POINTER(_P), C.POINTER(SolveStats),
                                      C.c_int64, C.c_int, C.POINTER(C.c_int)]),
    "ls_fd_data_rows_apply": (C.c_int, [_P, _P, _P, _P]),
    "ls_fd_admm_step": (C.c_int, [_P, C.c_int64, C.c_int64, _P, _P, _P, _P, _P, C.POINTER(C.c_double), _P]),
    "ls_fd_eval_lattice": (C.c_int, [C.POINTER(Grid3), _P, C.POINTER(C.c_double * 3), C.POINTER(C.c_double * 3),
                                     C.POINTER(C.c_int64 * 3), _P, _P, _P]),
    "ls_p1_face_count": (C.c_int, [C.POINTER(Grid3), C.POINTER(C.c_int64)]),
    "ls_p1_face_rows": (C.c_int, [C.POINTER(Grid3), C.c_double, _P, _P, _P, _P, _P, _P, _P]),
    "ls_p1_face_rows_directional": (C.c_int, [C.POINTER(Grid3), C.c_double, _P, _P, _P, _P, _P, _P]),
    "ls_iso_extract": (C.c_int, [C.POINTER(Grid3), _P, C.c_double, C.POINTER(_P), C.POINTER(C.c_int64),
                                 C.POINTER(C.c_int64), _P]),
    "ls_iso_copy": (C.c_int, [_P, _P, _P, _P, _P]),
    "ls_iso_destroy": (C.c_int, [_P]),
    "ls_fd_setup_profile": (C.c_int, [_P, _P, C.c_int]),
    "ls_p1_locate": (C.c_int, [C.POINTER(Grid3), _P, C.c_int64, C.c_int64, _P, _P, _P]),
    "ls_p1_point_rows": (C.c_int, [C.POINTER(Grid3), C.c_int, _P, C.c_int64, C.c_int64, C.c_double, _P, _P, _P, _P,
                                   C.POINTER(C.c_int64), _P]),
    "ls_p1_eval_points": (C.c_int, [C.POINTER(Grid3), _P, _P, C.c_int64, C.c_int64, _P, _P, _P]),
}


def load(build_if_missing: bool = False):
    """Load the shared library (building it first when asked)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise ExtensionUnavailable(
                    f"{path} is not built; run `python -c 'import __graft_entry__ as g; g.build()'` "
                    "(needs nvcc from CUDA 13)")
            _build.build()
        lib = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.ls_abi_version() != ABI_VERSION:
            raise ExtensionUnavailable(f"{path} has ABI {lib.ls_abi_version()}, this binding needs {ABI_VERSION}; rebuild it")
        _lib = lib
        return lib


def check(status: int, allow_positive: bool = False) -> int:
    if status < 0 or (status > 0 and not allow_positive):
        msg = _lib.ls_last_error().decode() if _lib is not None else "?"
        raise LsError(status, msg)
    return status


def device():
    """The CUDA device the kernels run on; raises when none is visible."""
    import torch

    if not torch.cuda.is_available():
        raise ExtensionUnavailable("no CUDA device is visible: the GB300 kernels cannot run (no CPU fallback)")
    load(build_if_missing=True)
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None
