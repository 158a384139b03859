"""C-ABI library: builds, loads and exports every declared symbol (no GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from loopstructural_gb300 import _build, _lib
from oracle import fd_oracle as fdo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    syms = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            syms |= set(re.findall(r"\b(ls_[a-z0-9_]+)\s*\(", text))
    return syms


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert declared, "no declarations found"
    for s in declared:
        assert hasattr(lib, s), f"{s} declared in include/ but not exported"
    assert set(_lib.EXPORTS) == declared


def test_abi_version(lib):
    assert lib.ls_abi_version() == 2


@pytest.mark.parametrize("cells", [(5, 5, 5), (3, 4, 2), (2, 5, 6), (1, 4, 4), (8, 6, 12)])
def test_regularisation_shapes_match_oracle(lib, cells):
    g = _lib.Grid3.make(np.array(cells) + 1, np.zeros(3), np.ones(3))
    grid = fdo.Grid(np.zeros(3), cells, np.ones(3))
    for fam_id, name in enumerate(_lib.REG_FAMILIES):
        rows, taps = C.c_int64(0), C.c_int32(0)
        assert lib.ls_fd_reg_shape(C.byref(g), fam_id, C.byref(rows), C.byref(taps)) == 0
        if name in fdo.INTERIOR_MASKS:
            idc, vals = fdo.family_rows(grid, fdo.INTERIOR_MASKS[name])
        else:
            axis = "xyz".index(name[1])
            mask = (fdo.DXX_MASK, fdo.DYY_MASK, fdo.DZZ_MASK)[axis]
            ind = fdo.boundary_indexes(grid, axis, name.endswith("upper"))
            idc = np.zeros((0, 3)) if ind is None else fdo.family_rows(grid, mask, ind)[0]
            vals = np.zeros(3)
        assert rows.value == idc.shape[0], name
        assert taps.value == len(vals), name


def test_invalid_arguments_report_errors(lib):
    g = _lib.Grid3.make((1, 5, 5), np.zeros(3), np.ones(3))
    rows = C.c_int64(0)
    assert lib.ls_fd_reg_shape(C.byref(g), 0, C.byref(rows), None) == -1
    assert b"at least 2 nodes" in lib.ls_last_error()
    g = _lib.Grid3.make((5, 5, 5), np.zeros(3), np.ones(3))
    assert lib.ls_fd_reg_shape(C.byref(g), 99, C.byref(rows), None) == -1
    assert b"unknown regularisation family" in lib.ls_last_error()
    g = _lib.Grid3.make((5, 5, 5), np.zeros(3), (1.0, 0.0, 1.0))
    assert lib.ls_fd_reg_shape(C.byref(g), 0, C.byref(rows), None) == -1
    assert lib.ls_fd_create(None, None, None) == -1


# Entry points whose first statement rejects a NULL handle, grid, mesh or
# buffer: called with every pointer NULL and every number 0 they must return
# LS_ERR_ARG with a message, before any CUDA call (so this runs without a GPU).
NULL_CHECKED = [
    "ls_fd_point_rows", "ls_fd_pair_rows", "ls_fd_reg_shape", "ls_fd_reg_rows", "ls_fd_weight_scale",
    "ls_fd_scaled_weights", "ls_fd_directional_weights", "ls_fault_apply", "ls_fd_eval_jets", "ls_fd_eval_adjoint",
    "ls_fd_eval_points", "ls_fd_eval_lattice", "ls_iso_extract", "ls_iso_copy", "ls_fd_apply_noalloc",
    "ls_fd_create", "ls_fd_device", "ls_fd_set_rhs", "ls_fd_data_rows_apply", "ls_fd_admm_step",
    "ls_fd_diagonal", "ls_fd_apply", "ls_fd_apply_f32", "ls_fd_setup_profile", "ls_fd_prepare", "ls_fd_solve",
    "ls_fd_mg_apply_level", "ls_fd_mg_vcycle", "ls_fd_profile_mg", "ls_fd_profile_iteration",
    "ls_p1_face_count", "ls_p1_face_rows", "ls_p1_face_rows_directional", "ls_p1_locate", "ls_p1_point_rows",
    "ls_p1_eval_points",
]


def _null_args(fn):
    out = []
    for t in fn.argtypes:
        if t in (C.c_double, C.c_float):
            out.append(0.0)
        elif t in (C.c_int, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_size_t):
            out.append(0)
        else:
            out.append(None)
    return out


@pytest.mark.parametrize("name", NULL_CHECKED)
def test_null_arguments_are_rejected_before_device_work(lib, name):
    fn = getattr(lib, name)
    assert fn(*_null_args(fn)) == -1, name
    assert lib.ls_last_error(), name


def test_tetra_gradient_and_destroy_accept_empty_input(lib):
    assert lib.ls_tetra_gradient(None, None, 0, None, None) == 0
    assert lib.ls_tetra_gradient(None, None, 1, None, None) == -1
    assert lib.ls_fd_destroy(None) == 0
    assert lib.ls_iso_destroy(None) == 0
