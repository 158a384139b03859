"""Finite-difference (StructuredGrid) oracle: numpy/scipy restatement of the
reference FD interpolation path.  TEST INFRASTRUCTURE ONLY (see package doc).

Reference files (paths inside the LoopStructural 1.8.0 source tree):
  S  = packages/loop_common/src/loop_common/supports/_3d_base_structured.py
  G  = packages/loop_common/src/loop_common/supports/_3d_structured_grid.py
  FD = packages/loop_interpolation/src/loop_interpolation/_finite_difference_interpolator.py
  DI = packages/loop_interpolation/src/loop_interpolation/_discrete_interpolator.py
  SP = packages/loop_interpolation/src/loop_interpolation/_solver_pipeline.py
  SS = packages/loop_interpolation/src/loop_interpolation/_solver_strategy.py
  OP = packages/loop_interpolation/src/loop_interpolation/_operator.py
  M  = packages/loop_common/src/loop_common/math/_maths.py
"""
from __future__ import annotations

import numpy as np
from scipy import sparse
from scipy.sparse import linalg as spla

# --------------------------------------------------------------------------
# Stencil masks, (z, y, x) index order.  OP:10-43.
# --------------------------------------------------------------------------
_Z = np.zeros((3, 3))
DXX_MASK = np.array([_Z, [[0, 0, 0], [1, -2, 1], [0, 0, 0]], _Z], dtype=float)
DYY_MASK = DXX_MASK.swapaxes(1, 2)
DZZ_MASK = DXX_MASK.swapaxes(0, 2)
DXY_MASK = np.array([_Z, [[-0.25, 0, 0.25], [0, 0, 0], [0.25, 0, -0.25]], _Z]) / np.sqrt(2)
DXZ_MASK = DXY_MASK.swapaxes(0, 1)
DYZ_MASK = DXY_MASK.swapaxes(0, 2)

# 27 neighbour offsets, x fastest then y then z (FD:541-634); the same
# enumeration as ``mask.flatten()`` of a (z, y, x) mask.
FULL_NEIGHBOUR_MASK = np.array(
    [[(k % 3) - 1 for k in range(27)], [((k // 3) % 3) - 1 for k in range(27)], [(k // 9) - 1 for k in range(27)]]
)

INTERIOR_FAMILIES = ("dxy", "dyz", "dxz", "dxx", "dyy", "dzz")  # G:502-509 order
INTERIOR_MASKS = {
    "dxy": DXY_MASK,
    "dyz": DYZ_MASK,
    "dxz": DXZ_MASK,
    "dxx": DXX_MASK,
    "dyy": DYY_MASK,
    "dzz": DZZ_MASK,
}
BORDER_FAMILIES = ("dx_lower", "dx_upper", "dy_lower", "dy_upper", "dz_lower", "dz_upper")  # FD:1102-1139

DEFAULT_FD_WEIGHTS = {  # FD:102-119
    "dxy": 1.0, "dyz": 1.0, "dxz": 1.0, "dxx": 1.0, "dyy": 1.0, "dzz": 1.0,
    "dx": 1.0, "dy": 1.0, "dz": 1.0,
    "cpw": 1.0, "gpw": 1.0, "npw": 10.0, "tpw": 1.0, "ipw": 1.0,
}


class Grid:
    """StructuredGrid geometry.  ``nsteps_cells`` cells per axis, nodes =
    cells + 1, F-order node numbering gi = i + nx*j + nx*ny*k
    (S:328-351)."""

    def __init__(self, origin, nsteps_cells, step_vector):
        self.origin = np.array(origin, dtype=float)
        self.step_vector = np.array(step_vector, dtype=float)
        self.nsteps = np.array(nsteps_cells, dtype=int) + 1  # node counts
        self.nsteps_cells = self.nsteps - 1

    @property
    def n_nodes(self) -> int:
        return int(np.prod(self.nsteps))

    @property
    def maximum(self):
        return self.origin + self.nsteps_cells * self.step_vector

    @property
    def nodes(self):
        mx = self.origin + self.nsteps_cells * self.step_vector
        x = np.linspace(self.origin[0], mx[0], self.nsteps[0])
        y = np.linspace(self.origin[1], mx[1], self.nsteps[1])
        z = np.linspace(self.origin[2], mx[2], self.nsteps[2])
        xx, yy, zz = np.meshgrid(x, y, z, indexing="ij")
        return np.array([xx.flatten(order="F"), yy.flatten(order="F"), zz.flatten(order="F")]).T

    def inside(self, pos):
        extent = np.maximum(np.abs(self.maximum - self.origin), 1.0)
        tol = np.finfo(float).eps * 32.0 * extent
        return np.all((pos >= (self.origin - tol)) & (pos <= (self.maximum + tol)), axis=1)

    def position_to_cell_index(self, pos):
        inside = self.inside(pos)
        ci = np.zeros((pos.shape[0], 3), dtype=int)
        for d in range(3):
            x = pos[:, d] - self.origin[None, d]
            ci[inside, d] = np.floor(x[inside] / self.step_vector[None, d]).astype(int)
            ci[inside, d] = np.clip(ci[inside, d], 0, self.nsteps_cells[d] - 1)
        return ci, inside

    def position_to_cell_corners(self, pos):
        ci, inside = self.position_to_cell_index(pos)
        nx, ny = self.nsteps[0], self.nsteps[1]
        offsets = np.array([0, 1, nx, nx + 1, nx * ny, nx * ny + 1, nx * ny + nx, nx * ny + nx + 1], dtype=np.intp)
        g = ci[:, 0] + nx * ci[:, 1] + nx * ny * ci[:, 2]
        gidx = g[:, None] + offsets[None, :]
        gidx[~inside] = -1
        return gidx, inside

    def local_coordinates(self, pos):  # G:126-146
        ci, _ = self.position_to_cell_index(pos)
        cell_origin = self.origin[None, :] + self.step_vector[None, :] * ci
        local = (pos - cell_origin) / self.step_vector[None, :]
        return np.clip(local, 0.0, 1.0)

    @staticmethod
    def trilinear(lc):  # G:90-124 (same evaluation order)
        out = np.zeros((lc.shape[0], 8), dtype=np.float64)
        x, y, z = lc[:, 0], lc[:, 1], lc[:, 2]
        out[:, 0] = (1 - x) * (1 - y) * (1 - z)
        out[:, 1] = x * (1 - y) * (1 - z)
        out[:, 2] = (1 - x) * y * (1 - z)
        out[:, 4] = (1 - x) * (1 - y) * z
        out[:, 5] = x * (1 - y) * z
        out[:, 6] = (1 - x) * y * z
        out[:, 3] = x * y * (1 - z)
        out[:, 7] = x * y * z
        return out

    def dof_coefs(self, pos):  # G:148-162
        return self.trilinear(self.local_coordinates(pos))

    def element_gradient(self, pos):  # G:393-454, returns T (P,3,8)
        lc = self.local_coordinates(pos)
        x, y, z = lc[:, 0], lc[:, 1], lc[:, 2]
        T = np.zeros((pos.shape[0], 3, 8))
        T[:, 0, 0] = (1 - z) * (y - 1)
        T[:, 0, 1] = (1 - y) * (1 - z)
        T[:, 0, 2] = -y * (1 - z)
        T[:, 0, 4] = -(1 - y) * z
        T[:, 0, 5] = (1 - y) * z
        T[:, 0, 6] = -y * z
        T[:, 0, 3] = y * (1 - z)
        T[:, 0, 7] = y * z
        T[:, 1, 0] = (x - 1) * (1 - z)
        T[:, 1, 1] = -x * (1 - z)
        T[:, 1, 2] = (1 - x) * (1 - z)
        T[:, 1, 4] = -(1 - x) * z
        T[:, 1, 5] = -x * z
        T[:, 1, 6] = (1 - x) * z
        T[:, 1, 3] = x * (1 - z)
        T[:, 1, 7] = x * z
        T[:, 2, 0] = -(1 - x) * (1 - y)
        T[:, 2, 1] = -x * (1 - y)
        T[:, 2, 2] = -(1 - x) * y
        T[:, 2, 4] = (1 - x) * (1 - y)
        T[:, 2, 5] = x * (1 - y)
        T[:, 2, 6] = (1 - x) * y
        T[:, 2, 3] = -x * y
        T[:, 2, 7] = x * y
        T[:, 0, :] /= self.step_vector[None, 0]
        T[:, 1, :] /= self.step_vector[None, 1]
        T[:, 2, :] /= self.step_vector[None, 2]
        return T

    def node_index(self, gi):
        gi = np.asarray(gi)
        return np.stack([gi % self.nsteps[0], gi // self.nsteps[0] % self.nsteps[1], gi // self.nsteps[0] // self.nsteps[1]], axis=-1)

    def neighbour_global_indexes(self, mask, indexes=None):  # G:164-293
        if indexes is None:
            idx = self.node_index(np.arange(self.n_nodes))
            edge = np.ones(idx.shape[0], dtype=bool)
            for d in range(3):
                edge &= (idx[:, d] > 0) & (idx[:, d] < self.nsteps[d] - 1)
            indexes = idx[edge, :].T
        nb = indexes[:, None, :] + mask[:, :, None]
        return (nb[0] + self.nsteps[0] * nb[1] + self.nsteps[0] * self.nsteps[1] * nb[2]).astype(np.int64)

    # -- evaluation ----------------------------------------------------------
    def evaluate_value(self, pos, c):  # G:295-322
        idc, inside = self.position_to_cell_corners(pos)
        v = np.full(idc.shape, np.nan)
        v[inside, :] = self.dof_coefs(pos[inside, :])
        v[inside, :] *= c[idc[inside, :]]
        return np.sum(v, axis=1)

    def evaluate_gradient(self, pos, c):  # G:324-391
        idc, inside = self.position_to_cell_corners(pos)
        T = np.zeros((idc.shape[0], 3, 8))
        T[inside] = self.element_gradient(pos[inside, :])
        for d in range(3):
            T[inside, d, :] *= c[idc[inside, :]]
        return np.array([np.sum(T[:, 0, :], axis=1), np.sum(T[:, 1, :], axis=1), np.sum(T[:, 2, :], axis=1)]).T


def evaluate_value_local(grid: Grid, pos, c):
    """DI:1342-1362: NaN input rows give 0, outside points give NaN."""
    pos = np.asarray(pos, dtype=float)
    out = np.zeros(pos.shape[0])
    nanrow = np.any(np.isnan(pos), axis=1)
    if np.any(~nanrow):
        out[~nanrow] = grid.evaluate_value(pos[~nanrow], c)
    return out


def evaluate_gradient_local(grid: Grid, pos, c):
    """DI:1364-1379: outside (and NaN) points give a zero gradient."""
    pos = np.asarray(pos, dtype=float)
    if pos.shape[0] == 0:
        return np.zeros((0, 3))
    return grid.evaluate_gradient(pos, c)


# --------------------------------------------------------------------------
# strike / dip helpers (M:126-160, M:276-298, M:300-332)
# --------------------------------------------------------------------------
def get_vectors(normal):
    normal = np.array(normal, dtype=float)
    length = np.linalg.norm(normal, axis=1)[:, None]
    normal /= length
    nv = np.array(normal)
    nv /= np.linalg.norm(nv, axis=1)[:, None]
    strike = np.rad2deg(-np.arctan2(nv[:, 1], nv[:, 0]))
    s = np.deg2rad(strike)
    strike_vec = np.array([np.sin(-s), -np.cos(-s), np.zeros(s.shape[0])])
    strike_vec /= np.linalg.norm(strike_vec, axis=0)[None, :]
    dip_vec = np.cross(strike_vec, normal, axisa=0, axisb=1).T
    dip_vec /= np.linalg.norm(dip_vec, axis=0)[None, :]
    return strike_vec * length.T, dip_vec * length.T


# --------------------------------------------------------------------------
# least-squares container (DI:316-389)
# --------------------------------------------------------------------------
class ConstraintSet:
    """Ordered dict of constraint families {name: dict(idc, A, B, w)} with
    the reference's row normalisation and name de-duplication."""

    def __init__(self, dof: int):
        self.dof = dof
        self.families: dict[str, dict] = {}

    def add(self, A, B, idc, w=1.0, name="undefined"):
        A = np.array(A, dtype=float)
        B = np.array(B, dtype=float)
        idc = np.array(idc)
        if A.shape != idc.shape:
            return
        if A.ndim > 2:
            if isinstance(w, np.ndarray):
                w = np.tile(w, (A.shape[1]))
            A = A.reshape((A.shape[0] * A.shape[1], A.shape[2]))
            idc = idc.reshape((idc.shape[0] * idc.shape[1], idc.shape[2]))
            B = B.reshape(A.shape[0])
        if np.any(np.isnan(idc)) or np.any(np.isnan(A)) or np.any(np.isnan(B)):
            return
        length = np.linalg.norm(A, axis=1)
        B[length > 0] /= length[length > 0]
        A[length > 0, :] /= length[length > 0, None]
        if isinstance(w, (float, int)):
            w = np.ones(A.shape[0]) * w
        w = np.asarray(w, dtype=float)
        if w.shape[0] != A.shape[0]:
            raise ValueError("Weight array does not match number of constraints")
        base = name
        while name in self.families:
            count = 0
            if "_" in name:
                count = int(name.split("_")[1]) + 1
            name = base + f"_{count}"
        self.families[name] = {"idc": idc.astype(np.int64), "A": A, "B": B.flatten(), "w": w}

    def matrix(self):
        """DI:684-705: stack W-weighted rows in insertion order."""
        mats, bs = [], []
        for f in self.families.values():
            n = f["A"].shape[0]
            if n == 0:
                continue
            rows = np.tile(np.arange(n), (f["A"].shape[1], 1)).T
            m = sparse.coo_matrix((f["A"].flatten(), (rows.flatten(), f["idc"].flatten())), shape=(n, self.dof)).tocsr()
            mats.append(m.multiply(f["w"][:, None]).tocsr())
            bs.append(f["B"] * f["w"])
        if not mats:
            return sparse.csr_matrix((0, self.dof)), np.zeros(0)
        return sparse.vstack(mats).tocsr(), np.hstack(bs)


# --------------------------------------------------------------------------
# FD assembly (FD:132-224 and the add_* methods)
# --------------------------------------------------------------------------
def add_value_constraints(grid, cs, points, w):  # FD:236-269
    if points.shape[0] == 0:
        return
    idc, inside = grid.position_to_cell_corners(points[:, :3])
    a = grid.dof_coefs(points[inside, :3])
    cs.add(a, points[inside, 3], idc[inside, :], w=w * points[inside, 4], name="value")


def add_norm_constraints(grid, cs, points, w):  # FD:403-476
    if points.shape[0] == 0:
        return
    idc, inside = grid.position_to_cell_corners(points[:, :3])
    T = grid.element_gradient(points[inside, :3])
    pw = np.ones(int(np.sum(inside)))
    if points.shape[1] > 6:
        pw = points[inside, 6]
    cw = float(w / 3) * pw
    for d in range(3):
        cs.add(T[:, d, :], points[inside, 3 + d], idc[inside, :], w=cw, name=f"norm_{d}")


def add_gradient_constraints(grid, cs, points, w):  # FD:342-401
    if points.shape[0] == 0:
        return
    points = np.array(points, dtype=float)
    idc, inside = grid.position_to_cell_corners(points[:, :3])
    T = grid.element_gradient(points[inside, :3])
    norm = np.linalg.norm(points[:, 3:6], axis=1)
    points[:, 3:6] /= norm[:, None]
    T /= norm[inside, None, None]
    strike, dip = get_vectors(points[inside, 3:6])
    B = np.zeros(int(np.sum(inside)))
    cs.add(np.einsum("ij,ijk->ik", strike.T, T), B, idc[inside, :], w=w, name="gradient")
    cs.add(np.einsum("ij,ijk->ik", dip.T, T), B, idc[inside, :], w=w, name="gradient")


def add_gradient_orthogonal_constraints(grid, cs, points, vectors, w, b=0.0, name="gradient orthogonal"):  # FD:478-539
    if points.shape[0] == 0:
        return
    vectors = np.array(vectors, dtype=float)
    idc, inside = grid.position_to_cell_corners(points[:, :3])
    norm = np.linalg.norm(vectors, axis=1)
    vectors[norm > 0, :] /= norm[norm > 0, None]
    T = grid.element_gradient(points[inside, :3])
    ni = norm[inside]
    T[ni > 0, :, :] /= ni[ni > 0, None, None]
    A = np.einsum("ij,ijk->ik", vectors[inside, :3], T)
    cs.add(A, np.zeros(int(np.sum(inside))) + b, idc[inside, :], w=w, name=name)


def interface_pair_indices(n, mode="auto", threshold=200, fallback="star"):  # FD:271-295
    if n < 2:
        return np.zeros((0, 2), dtype=int)
    threshold = max(2, int(threshold))
    if mode == "auto":
        mode = fallback if n > threshold else "all"
    if mode == "all":
        ii, jj = np.triu_indices(n, k=1)
        return np.column_stack([ii, jj]).astype(int)
    if mode == "star":
        return np.column_stack([np.zeros(n - 1, dtype=int), np.arange(1, n, dtype=int)])
    if mode == "chain":
        return np.column_stack([np.arange(0, n - 1, dtype=int), np.arange(1, n, dtype=int)])
    raise ValueError(mode)


def add_interface_constraints(grid, cs, points, w, mode="auto", threshold=200, fallback="star"):  # FD:297-340
    if points.shape[0] <= 1:
        return
    idc_all, inside = grid.position_to_cell_corners(points[:, :3])
    idc = idc_all[inside, :]
    A = grid.dof_coefs(points[inside, :3])
    ids = points[np.logical_and(~np.isnan(points[:, 3]), inside), 3]
    for uid in np.unique(ids):
        mask = points[inside, 3] == uid
        pair = interface_pair_indices(int(np.sum(mask)), mode, threshold, fallback)
        if pair.shape[0] == 0:
            continue
        iA = np.hstack([A[mask, :][pair[:, 0], :], -A[mask, :][pair[:, 1], :]])
        iI = np.hstack([idc[mask, :][pair[:, 0], :], idc[mask, :][pair[:, 1], :]])
        cs.add(iA, np.zeros(iA.shape[0]), iI, w=w, name=f"interface_{uid}")


def family_rows(grid: Grid, mask, indexes=None):
    """FD:643-692 ``_assemble_operator`` without the weight: returns
    (idc (R,k) int64, raw operator values (k,)) in the reference's column
    order (active taps of ``mask.flatten()``)."""
    active = mask.flatten() != 0
    vals = mask.flatten()[active]
    gidx = grid.neighbour_global_indexes(FULL_NEIGHBOUR_MASK[:, active], indexes)
    return gidx.T, vals


def boundary_indexes(grid: Grid, axis, upper=False):  # FD:636-641
    if grid.nsteps[axis] < 3:
        return None
    idx = grid.node_index(np.arange(grid.n_nodes))
    bi = grid.nsteps[axis] - 2 if upper else 1
    return idx[idx[:, axis] == bi, :].T


def compute_weighting(nodes, points, alpha=10.0, sigma=1.0):  # FD:66-90
    """1 + alpha exp(-d^2 / 2 sigma^2), d = distance from each node to the
    nearest point (a KD-tree query, as the reference)."""
    from scipy.spatial import cKDTree

    d, _ = cKDTree(points).query(nodes, k=1)
    return 1 + alpha * np.exp(-(d**2) / (2 * sigma**2))


def regularisation_scale(grid, normals, sigma=None):  # DI:313, FD:416-444
    """The per-node scale ``use_regularisation_weight_scale`` puts on every
    regularisation row's centre: 1 (reset), plus compute_weighting over the
    normal constraints inside the grid (sigma defaults to 10 x the node count
    along x)."""
    scale = np.ones(grid.n_nodes)
    if normals.shape[0] == 0:
        return scale
    _idc, inside = grid.position_to_cell_corners(normals[:, :3])
    if inside.any():
        s = grid.nsteps[0] * 10 if sigma is None else sigma
        scale = scale + compute_weighting(grid.nodes, normals[inside, :3], sigma=s)
    return scale


def _row_centres(grid, indexes=None):
    """Centre node of every row of a family (FD:662-667)."""
    return grid.neighbour_global_indexes(np.zeros((3, 1), dtype=int), indexes)[0]


def add_regularisation(grid, cs, weights, directional=(), scale=None):
    """Interior operators (G:489-510 order and /4 cross weights), the
    directional terms ((w, vector, name) triples, FD:222), then borders
    (FD:1052-1144).  ``scale`` (per node): every interior and border row's
    weight times the scale at its centre (FD:668-672)."""
    ops = {
        "dxy": (DXY_MASK, weights["dxy"] / 4),
        "dyz": (DYZ_MASK, weights["dyz"] / 4),
        "dxz": (DXZ_MASK, weights["dxz"] / 4),
        "dxx": (DXX_MASK, weights["dxx"] / 1),
        "dyy": (DYY_MASK, weights["dyy"] / 1),
        "dzz": (DZZ_MASK, weights["dzz"] / 1),
    }
    for name, (mask, w) in ops.items():
        idc, vals = family_rows(grid, mask)
        if idc.size == 0:
            continue
        if scale is not None:
            w = scale[_row_centres(grid)] * w
        cs.add(np.tile(vals, (idc.shape[0], 1)), np.zeros(idc.shape[0]), idc, w=w, name=name)
    for dw, vector, dname in directional:
        if dw != 0:
            add_directional_regularisation(grid, cs, dw, vector, dname)
    borders = [
        (DXX_MASK, weights["dx"], "dx_lower", boundary_indexes(grid, 0, False)),
        (DXX_MASK, weights["dx"], "dx_upper", boundary_indexes(grid, 0, True)),
        (DYY_MASK, weights["dy"], "dy_lower", boundary_indexes(grid, 1, False)),
        (DYY_MASK, weights["dy"], "dy_upper", boundary_indexes(grid, 1, True)),
        (DZZ_MASK, weights["dz"], "dz_lower", boundary_indexes(grid, 2, False)),
        (DZZ_MASK, weights["dz"], "dz_upper", boundary_indexes(grid, 2, True)),
    ]
    for mask, w, name, indexes in borders:
        if w == 0 or indexes is None or indexes.shape[1] == 0:
            continue
        idc, vals = family_rows(grid, mask, indexes)
        if scale is not None:
            w = scale[_row_centres(grid, indexes)] * w
        cs.add(np.tile(vals, (idc.shape[0], 1)), np.zeros(idc.shape[0]), idc, w=w, name=name)


DIRECTIONAL_FAMILIES = ("dxx", "dyy", "dzz", "dxy", "dxz", "dyz")  # FD:1262-1269 order


def add_directional_regularisation(grid, cs, w, vector, name="directional regularisation"):  # FD:1207-1337
    """The six interior second-derivative families again, row weight
    w * c_f(v) at each interior node (c = vx², vy², vz², 2vxvy, 2vxvz, 2vyvz);
    rows whose weight is not > 0 in magnitude (zero or NaN) are dropped, and
    a family with no row left is not added."""
    vector = None if vector is None else np.asarray(vector, dtype=float)
    if vector is None or vector.ndim != 2 or vector.shape != (grid.n_nodes, 3):
        return
    masks = {"dxx": DXX_MASK, "dyy": DYY_MASK, "dzz": DZZ_MASK, "dxy": DXY_MASK, "dxz": DXZ_MASK, "dyz": DYZ_MASK}
    centre = grid.neighbour_global_indexes(np.zeros((3, 1), dtype=int))
    if centre is None or centre.size == 0:
        return
    rows = centre.T[:, 0].astype(int)
    vx, vy, vz = vector[rows, 0], vector[rows, 1], vector[rows, 2]
    comp = {"dxx": vx**2, "dyy": vy**2, "dzz": vz**2,
            "dxy": 2.0 * vx * vy, "dxz": 2.0 * vx * vz, "dyz": 2.0 * vy * vz}
    for op in DIRECTIONAL_FAMILIES:
        idc, vals = family_rows(grid, masks[op])
        if idc.size == 0:
            continue
        row_w = w * comp[op]
        keep = np.abs(row_w) > 0.0
        if not np.any(keep):
            continue
        A = np.tile(vals, (idc.shape[0], 1))
        cs.add(A[keep], np.zeros(int(np.sum(keep))), idc[keep], w=row_w[keep], name=f"{name}_{op}")


def fold_norm_target(fold, normals, fold_norm=-1.0, dgz_alignment="warn"):
    """_fold_norm_alignment.py:9-118: the grad . dgz target, sign-flipped under
    'correct' when the median unit dot(dgz, normal) at the normal points is
    below -0.2."""
    target = float(-1.0 if fold_norm is None else fold_norm)
    mode = "warn" if dgz_alignment is None else str(dgz_alignment).strip().lower()
    normals = np.asarray(normals, dtype=float)
    if mode == "none" or normals.ndim != 2 or normals.shape[0] == 0 or normals.shape[1] < 6:
        return target
    _, _, dgz = fold.get_deformed_orientation(normals[:, :3])
    dgz = np.asarray(dgz, dtype=float)
    vec = normals[:, 3:6]
    nn, dn = np.linalg.norm(vec, axis=1), np.linalg.norm(dgz, axis=1)
    ok = np.all(np.isfinite(vec), axis=1) & np.all(np.isfinite(dgz), axis=1) & (nn > 1e-12) & (dn > 1e-12)
    if not np.any(ok):
        return target
    med = float(np.median(np.einsum("ij,ij->i", dgz[ok] / dn[ok, None], vec[ok] / nn[ok, None])))
    if med < -0.2 and mode == "correct":
        target *= -1.0
    return target


def add_fold_constraints(grid, cs, fold, normals, fold_orientation=10.0, fold_axis_w=10.0,
                         fold_regularisation=(0.1, 0.01, 0.01), fold_normalisation=1.0, fold_norm=-1.0,
                         dgz_alignment="warn", mask_fn=None):
    """_fd_fold_interpolator.py:93-237 (FDFoldInterpolator.add_fold_constraints)."""
    nodes = grid.nodes
    deformed, axis, dgz = fold.get_deformed_orientation(nodes)
    weight = np.ones(grid.n_nodes)
    if mask_fn is not None:
        weight[mask_fn(nodes)] = 0.0
    active = weight > 0.0
    pos = nodes[active]
    if fold_orientation is not None:
        add_gradient_orthogonal_constraints(grid, cs, pos, np.array(deformed)[active], fold_orientation,
                                            name="fold orientation")
    if fold_axis_w is not None:
        add_gradient_orthogonal_constraints(grid, cs, pos, np.array(axis)[active], fold_axis_w, name="fold axis")
    if fold_normalisation is not None:
        target = fold_norm_target(fold, normals, fold_norm, dgz_alignment)
        add_gradient_orthogonal_constraints(grid, cs, pos, np.array(dgz)[active], fold_normalisation, b=target,
                                            name="fold normalisation")
    if fold_regularisation is not None:
        for w, v, name in zip(fold_regularisation, (dgz, deformed, axis),
                              ("fold regularisation 1", "fold regularisation 2", "fold regularisation 3")):
            v = np.asarray(v, dtype=float).copy()
            v[~active] = 0.0
            if w != 0:
                add_directional_regularisation(grid, cs, w, v, name)


def resolve_weights(regularisation=None, **kwargs):
    """FD:159-175: isotropic ``regularisation`` sets dxx..dyz; every other
    keyword overwrites ``interpolation_weights``."""
    w = dict(DEFAULT_FD_WEIGHTS)
    if regularisation is not None:
        for k in ("dxy", "dyz", "dxz", "dxx", "dyy", "dzz"):
            w[k] = float(regularisation)
    for k, v in kwargs.items():
        w[k] = v
    return w


def assemble(grid: Grid, data: dict, weights: dict, directional=(), weight_scale=False,
             weight_sigma=None) -> ConstraintSet:
    """FD:209-223 ``setup_interpolator`` family order; ``weight_scale`` =
    ``use_regularisation_weight_scale`` (with ``regularisation_weight_sigma``)."""
    cs = ConstraintSet(grid.n_nodes)
    add_norm_constraints(grid, cs, data.get("normal", np.zeros((0, 7))), weights["npw"])
    add_gradient_constraints(grid, cs, data.get("gradient", np.zeros((0, 7))), weights["gpw"])
    add_value_constraints(grid, cs, data.get("value", np.zeros((0, 5))), weights["cpw"])
    tangent = data.get("tangent", np.zeros((0, 7)))
    if tangent.shape[0] > 0:
        add_gradient_orthogonal_constraints(grid, cs, tangent[:, :3], tangent[:, 3:6], weights["tpw"])
    add_interface_constraints(grid, cs, data.get("interface", np.zeros((0, 5))), weights["ipw"])
    scale = regularisation_scale(grid, data.get("normal", np.zeros((0, 7))), weight_sigma) if weight_scale else None
    add_regularisation(grid, cs, weights, directional, scale=scale)
    return cs


# --------------------------------------------------------------------------
# normal equations and solves (SP:86-124, SS:48-72)
# --------------------------------------------------------------------------
RIDGE = 1e-8  # DI:76-78


def normal_equations(A, b, ridge=RIDGE):
    """(AᵀWA + ridge² I, AᵀWb) with A, b already W^{1/2}-weighted."""
    N = (A.T @ A).tocsr() + sparse.eye(A.shape[1], format="csr") * (ridge * ridge)
    return N.tocsr(), np.asarray(A.T @ b).reshape(-1)


def jacobi_diagonal(A, ridge=RIDGE):
    """Squared column norms of [A; ridge I] (DI:815-833 ``compute_column_scaling_matrix``)."""
    return np.asarray(A.multiply(A).sum(axis=0)).reshape(-1) + ridge * ridge


def solve_direct(A, b, ridge=RIDGE):
    N, rhs = normal_equations(A, b, ridge)
    return spla.spsolve(N.tocsc(), rhs)


def reference_cg_system(A, b, ridge=RIDGE):
    """Everything the reference's default solve does before scipy's CG
    iterations (SP:86-124, DI:815-833, SS:48-72): ridge rows, column scaling
    S = 1/|col|, the normal matrix (AS)ᵀ(AS) and its right-hand side.
    Returns (N, rhs, s) with s the diagonal of S."""
    Af = sparse.vstack([A, sparse.eye(A.shape[1]) * ridge]).tocsr()
    bf = np.hstack([b, np.zeros(A.shape[1])])
    cn = sparse.linalg.norm(Af, axis=0)
    s = np.ones(Af.shape[1])
    s[cn > 0] = 1.0 / cn[cn > 0]
    As = (Af @ sparse.diags(s)).tocsr()
    return (As.T @ As).tocsr(), As.T @ bf, s


def solve_reference_cg(A, b, tol=None, rtol=1e-5, maxiter=None, ridge=RIDGE, x0=None):
    """The reference default path verbatim in scipy: ridge rows, column
    scaling, cg on (AS)ᵀ(AS), scale back (SP:86-124, SS:48-72, DI:1312)."""
    N, rhs, s = reference_cg_system(A, b, ridge)
    S = sparse.diags(s)
    kw = {"rtol": rtol}
    if tol is not None:
        kw["atol"] = tol
    if maxiter is not None:
        kw["maxiter"] = maxiter
    if x0 is not None:
        kw["x0"] = x0 / s
    info = {}

    def cb(_):
        info["it"] = info.get("it", 0) + 1

    y, flag = spla.cg(N, rhs, callback=cb, **kw)
    return S @ y, flag, info.get("it", 0)


def pcg_scaled_residual(A, b, x, ridge=RIDGE):
    """‖S(rhs − N x)‖ -- the residual norm the reference's scaled CG tests."""
    N, rhs = normal_equations(A, b, ridge)
    d = jacobi_diagonal(A, ridge)
    r = rhs - N @ x
    return float(np.sqrt(np.dot(r, r / d))), float(np.sqrt(np.dot(rhs, rhs / d)))
