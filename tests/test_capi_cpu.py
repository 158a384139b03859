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
