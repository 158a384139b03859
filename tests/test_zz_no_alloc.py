"""ls_fd_apply_noalloc: the normal-operator apply for callers that cannot
allocate device memory (a host framework that owns every device allocation
through its own pool, or a plugin under a fixed device-memory budget).  It
keeps its scratch in a static device array, so the caller passes only inputs
and outputs.

Checked through the C ABI against the allocating entry point ls_fd_apply on
two calls in a row (the static scratch keeps the previous call's contents),
at the operator tolerance the other GPU tests use (1e-12 relative to max |N x|;
the no-allocation scatter uses FP64 atomics, so only the last bits may differ).
This file is collected last so that a run stopping at its first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import loopstructural_gb300 as L  # noqa: E402
from loopstructural_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu


def _system():
    rng = np.random.default_rng(7)
    cells = np.array([11, 9, 13])
    grid = L.StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells)
    interp = L.FiniteDifferenceInterpolator(grid)
    vp = rng.uniform(0, 1, size=(80, 3))
    interp.set_value_constraints(np.column_stack([vp, vp[:, 2], rng.uniform(0.5, 2, 80)]))
    npnt = rng.uniform(0, 1, size=(20, 3))
    interp.set_normal_constraints(np.column_stack([npnt, rng.normal(size=(20, 3)), np.ones(20)]))
    ip = rng.uniform(0, 1, size=(6, 3))
    interp.set_interface_constraints(np.column_stack([ip, [0, 0, 0, 1, 1, 1], np.ones(6)]))
    interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0, ipw=1.0, dx=0.5)
    return interp, interp._build_system()


def _desc(system, interp):
    s = _lib.FdSystem()
    s.grid = interp.support.grid3()
    w = interp._reg_weights()
    for k in ("dxx", "dyy", "dzz", "dxy", "dyz", "dxz", "dx", "dy", "dz"):
        setattr(s, "w_" + k, float(w[k]))
    s.ridge = float(interp.ridge_factor)
    s.nrows = system.nrows
    s.width = system._idc.shape[1]
    s.d_idc = _lib.ptr(system._idc)
    s.d_a = _lib.ptr(system._a)
    s.d_b = _lib.ptr(system._b)
    s.d_w = _lib.ptr(system._w)
    return s


def test_noalloc_apply_matches_allocating_apply_twice():
    interp, system = _system()
    lib = _lib.load()
    desc = _desc(system, interp)
    assert desc.width == 16  # interface rows pad the block to 16 columns
    rng = np.random.default_rng(11)
    for call in range(2):
        x = torch.from_numpy(rng.normal(size=system.n)).cuda()
        ref = system.apply(x)
        y = torch.full_like(x, float("nan"))
        xnx = C.c_double(0.0)
        status = lib.ls_fd_apply_noalloc(C.byref(desc), _lib.ptr(x), _lib.ptr(y), C.byref(xnx), _lib.stream_ptr())
        assert status == 0, lib.ls_last_error()
        torch.cuda.synchronize()
        scale = float(ref.abs().max())
        assert float((y - ref).abs().max()) <= 1e-12 * scale, f"call {call}"
        dot = float(torch.dot(x, ref))
        assert abs(xnx.value - dot) <= 1e-12 * abs(dot), f"call {call}"
    system.close()


def test_noalloc_rejects_oversized_systems():
    lib = _lib.load()
    s = _lib.FdSystem()
    s.grid = _lib.Grid3.make((4, 4, 4), np.zeros(3), np.ones(3))
    s.nrows = _lib.NOALLOC_MAX_ROWS + 1
    s.width = 8
    s.d_idc = s.d_a = s.d_b = s.d_w = C.c_void_p(16)  # never dereferenced: rejected first
    x = C.c_void_p(16)
    assert lib.ls_fd_apply_noalloc(C.byref(s), x, x, None, None) == -1
    assert b"static scratch limit" in lib.ls_last_error()


def test_noalloc_without_dot_product_enqueues_only():
    """h_xNx = NULL: the call only enqueues the apply (no host copy, no sync)."""
    interp, system = _system()
    lib = _lib.load()
    desc = _desc(system, interp)
    rng = np.random.default_rng(12)
    for call in range(2):
        x = torch.from_numpy(rng.normal(size=system.n)).cuda()
        ref = system.apply(x)
        y = torch.full_like(x, float("nan"))
        status = lib.ls_fd_apply_noalloc(C.byref(desc), _lib.ptr(x), _lib.ptr(y), None, _lib.stream_ptr())
        assert status == 0, lib.ls_last_error()
        torch.cuda.synchronize()
        assert float((y - ref).abs().max()) <= 1e-12 * float(ref.abs().max()), f"call {call}"
    system.close()


def test_noalloc_skips_and_reports_out_of_range_columns():
    """A data-row column equal to dof (one past the grid) is skipped by the
    kernels, which check every column before using it, and the call reports
    LS_ERR_ARG when it reads x.Nx back; a following valid call succeeds."""
    interp, system = _system()
    lib = _lib.load()
    bad_idc = system._idc.clone()
    row = 3
    col = int(torch.nonzero(bad_idc[row] >= 0)[0, 0])
    bad_idc[row, col] = system.n
    desc = _desc(system, interp)
    desc.d_idc = _lib.ptr(bad_idc)
    x = torch.from_numpy(np.random.default_rng(13).normal(size=system.n)).cuda()
    y = torch.zeros_like(x)
    xnx = C.c_double(0.0)
    assert lib.ls_fd_apply_noalloc(C.byref(desc), _lib.ptr(x), _lib.ptr(y), C.byref(xnx), _lib.stream_ptr()) == -1
    assert b"outside [0, dof)" in lib.ls_last_error()
    assert bool(torch.isfinite(y).all())
    good = _desc(system, interp)
    assert lib.ls_fd_apply_noalloc(C.byref(good), _lib.ptr(x), _lib.ptr(y), C.byref(xnx), _lib.stream_ptr()) == 0
    ref = system.apply(x)
    torch.cuda.synchronize()
    assert float((y - ref).abs().max()) <= 1e-12 * float(ref.abs().max())
    system.close()
