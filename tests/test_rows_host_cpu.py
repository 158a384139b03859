"""The multigrid host row split (csrc/mg_rows_host.hpp, plain C++) on the CPU:
cell rows (lowest corner clamped on the upper faces, corner coefficients,
Morton order, stable) and the rows left in row form, against a numpy
restatement of the same rules."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("rows") / "rows_probe.so")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-o", out, os.path.join(HERE, "cpp", "rows_probe.cpp")],
                   check=True)
    lib = C.CDLL(out)
    P = C.c_void_p
    lib.split_rows_probe.restype = C.c_int64
    lib.split_rows_probe.argtypes = [C.c_int64, C.c_int, P, P, P, C.c_int, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P]
    return lib


def _morton(i, j, k):
    code = 0
    for b in range(21):
        code |= ((i >> b) & 1) << (3 * b) | ((j >> b) & 1) << (3 * b + 1) | ((k >> b) & 1) << (3 * b + 2)
    return code


def _expected(cols, a, w2, dims):
    nx, ny, nz = dims
    cells, rest = [], []
    for r in range(cols.shape[0]):
        sel = cols[r] >= 0
        cc = cols[r][sel]
        if cc.size == 0:
            rest.append(r)
            continue
        xyz = np.stack([cc % nx, (cc // nx) % ny, cc // (nx * ny)], axis=1)
        if np.any(xyz.max(0) - xyz.min(0) > 1):
            rest.append(r)
            continue
        base = np.minimum(xyz.min(0), np.array(dims) - 2)
        c8 = np.zeros(8)
        for (x, y, z), v in zip(xyz - base, a[r][sel]):
            c8[x | (y << 1) | (z << 2)] += v
        cells.append((_morton(*map(int, base)), r, base, c8, w2[r]))
    order = sorted(range(len(cells)), key=lambda t: (cells[t][0], cells[t][1]))
    return [cells[t] for t in order], rest


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_split_matches_restatement(probe, seed):
    rng = np.random.default_rng(seed)
    dims = (9, 7, 11)
    nx, ny, nz = dims
    R, width = 300, 16
    cols = np.full((R, width), -1, dtype=np.int64)
    a = np.zeros((R, width))
    for r in range(R):
        kind = rng.integers(0, 4)
        if kind < 2:  # a point row: the 8 corners of a cell, in corner order
            i, j, k = rng.integers(0, nx - 1), rng.integers(0, ny - 1), rng.integers(0, nz - 1)
            for b in range(8):
                cols[r, b] = (i + (b & 1)) + nx * ((j + ((b >> 1) & 1)) + ny * (k + ((b >> 2) & 1)))
            a[r, :8] = rng.normal(size=8)
        elif kind == 2:  # an interface pair: two cells, 16 columns
            for h in range(2):
                i, j, k = rng.integers(0, nx - 1), rng.integers(0, ny - 1), rng.integers(0, nz - 1)
                for b in range(8):
                    cols[r, 8 * h + b] = (i + (b & 1)) + nx * ((j + ((b >> 1) & 1)) + ny * (k + ((b >> 2) & 1)))
            a[r] = rng.normal(size=16)
        else:  # a few columns on the upper faces (extent 0: the box is clamped), one repeated
            g = (nx - 1) + nx * ((ny - 1) + ny * rng.integers(0, nz))
            cols[r, :3] = [g, g, g - nx]
            a[r, :3] = rng.normal(size=3)
    w2 = rng.uniform(0.5, 2.0, size=R)
    out_i = np.zeros(R, np.int32)
    out_j = np.zeros(R, np.int32)
    out_k = np.zeros(R, np.int32)
    out_c = np.zeros(8 * R)
    out_w = np.zeros(R)
    rn = C.c_int64(0)
    rc = np.zeros(R * width, np.int64)
    ra = np.zeros(R * width)
    rw = np.zeros(R)
    ptr = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
    n = probe.split_rows_probe(R, width, ptr(cols), ptr(a), ptr(w2), nx, ny, nz, ptr(out_i), ptr(out_j), ptr(out_k),
                               ptr(out_c), ptr(out_w), C.byref(rn), ptr(rc), ptr(ra), ptr(rw))
    cells, rest = _expected(cols, a, w2, dims)
    assert n == len(cells) and rn.value == len(rest)
    for t, (_code, _r, base, c8, w) in enumerate(cells):
        assert (out_i[t], out_j[t], out_k[t]) == tuple(base)
        np.testing.assert_array_equal(out_c[8 * t:8 * t + 8], c8)
        assert out_w[t] == w
    np.testing.assert_array_equal(rc[:len(rest) * width].reshape(-1, width), cols[rest])
    np.testing.assert_array_equal(rw[:len(rest)], w2[rest])
    # every coarser level keeps each cell's rows contiguous
    cell = np.stack([out_i[:n], out_j[:n], out_k[:n]], axis=1)
    for _lvl in range(4):
        keys = [tuple(x) for x in cell]
        runs = [keys[0]] + [keys[t] for t in range(1, n) if keys[t] != keys[t - 1]]
        assert len(runs) == len(set(runs))
        cell = cell >> 1
