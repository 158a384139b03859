"""P1 (TetMesh, 5 tetrahedra per hexahedral cell) oracle: numpy/scipy
restatement of the reference P1 interpolation path.  TEST INFRASTRUCTURE ONLY.

Reference files (inside the LoopStructural 1.8.0 source tree):
  T  = packages/loop_common/src/loop_common/supports/_3d_structured_tetra.py
  S  = packages/loop_common/src/loop_common/supports/_3d_base_structured.py
  P1 = packages/loop_interpolation/src/loop_interpolation/_p1interpolator.py
"""
from __future__ import annotations

import numpy as np
from scipy.sparse import coo_matrix, tril

from .fd_oracle import ConstraintSet, Grid

# T:28-34 -- local corner numbers (corner k <-> (k&1, k>>1&1, k>>2)) of the
# five tetrahedra of an even ((i+j+k) % 2 == 0) and an odd cell.
TETRA_MASK_EVEN = np.array([[7, 1, 2, 4], [6, 2, 4, 7], [5, 1, 4, 7], [0, 1, 2, 4], [3, 1, 2, 7]])
TETRA_MASK_ODD = np.array([[0, 6, 5, 3], [7, 3, 5, 6], [4, 0, 5, 6], [2, 0, 3, 6], [1, 0, 3, 5]])
_GRAD_I = np.array([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]])

DEFAULT_P1_WEIGHTS = {"cgw": 0.1, "cpw": 1.0, "npw": 1.0, "gpw": 1.0, "tpw": 1.0, "ipw": 1.0}  # P1:40-47


class TetMesh(Grid):
    """Structured tetrahedral mesh geometry (T:16-765)."""

    def __init__(self, origin, nsteps_cells, step_vector):
        super().__init__(origin, nsteps_cells, step_vector)
        self._elements = None

    @property
    def n_cells(self):
        return int(np.prod(self.nsteps_cells))

    @property
    def ntetra(self):
        return self.n_cells * 5

    def inside(self, pos):  # T:264-272 (strict)
        inside = np.ones(pos.shape[0], dtype=bool)
        for i in range(3):
            inside &= pos[:, i] > self.origin[i]
            inside &= pos[:, i] < self.origin[i] + self.step_vector[i] * self.nsteps_cells[i]
        return inside

    def _base_inside(self, pos):
        return Grid.inside(self, pos)

    def position_to_cell_index(self, pos):  # S:251-282 with the tolerant inside
        inside = self._base_inside(pos)
        ci = np.zeros((pos.shape[0], 3), dtype=int)
        for d in range(3):
            x = pos[:, d] - self.origin[None, d]
            ci[inside, d] = np.floor(x[inside] / self.step_vector[None, d]).astype(int)
            ci[inside, d] = np.clip(ci[inside, d], 0, self.nsteps_cells[d] - 1)
        return ci, inside

    def _cell_corners(self, ci):
        xc = np.array([0, 1, 0, 1, 0, 1, 0, 1])
        yc = np.array([0, 0, 1, 1, 0, 0, 1, 1])
        zc = np.array([0, 0, 0, 0, 1, 1, 1, 1])
        out = np.zeros((ci.shape[0], 8, 3), dtype=int)
        out[:, :, 0] = ci[:, None, 0] + xc[None, :]
        out[:, :, 1] = ci[:, None, 1] + yc[None, :]
        out[:, :, 2] = ci[:, None, 2] + zc[None, :]
        return out

    def _gi(self, idx):
        return idx[..., 0] + self.nsteps[0] * idx[..., 1] + self.nsteps[0] * self.nsteps[1] * idx[..., 2]

    def _all_cells(self):
        x = np.arange(self.nsteps_cells[0])
        y = np.arange(self.nsteps_cells[1])
        z = np.arange(self.nsteps_cells[2])
        zz, yy, xx = np.meshgrid(z, y, x, indexing="ij")
        return np.array([xx.flatten(), yy.flatten(), zz.flatten()]).T

    @property
    def elements(self):  # T:376-399
        if self._elements is None:
            ci = self._all_cells()
            gi = self._gi(self._cell_corners(ci))
            even = np.sum(ci, axis=1) % 2 == 0
            tet = np.zeros((ci.shape[0], 5, 4), dtype=np.int64)
            tet[even] = gi[even][:, TETRA_MASK_EVEN]
            tet[~even] = gi[~even][:, TETRA_MASK_ODD]
            self._elements = tet.reshape(-1, 4)
        return self._elements

    @property
    def barycentre(self):  # T:105-118
        return np.sum(self.nodes[self.elements][:, :, :], axis=1) / 4.0

    def element_gradients(self, elements=None):  # T:421-486
        ci = self._all_cells()
        even = np.sum(ci, axis=1) % 2 == 0
        nodes = self.origin[None, None, :] + self.step_vector[None, None, :] * self._cell_corners(ci)
        pts = np.zeros((ci.shape[0], 5, 4, 3))
        pts[even] = nodes[even][:, TETRA_MASK_EVEN, :]
        pts[~even] = nodes[~even][:, TETRA_MASK_ODD, :]
        ps = pts.reshape(-1, 4, 3)
        m = np.array([[ps[:, k, d] - ps[:, 0, d] for d in range(3)] for k in (1, 2, 3)])
        m = np.swapaxes(m, 0, 2)
        g = np.linalg.inv(m).swapaxes(1, 2) @ _GRAD_I
        if elements is None:
            return g
        return g[elements]

    def neighbours(self):  # T:626-740
        tet = np.arange(self.ntetra)
        nb = np.full((self.ntetra, 4), -9999, dtype=np.int64)
        nb[tet % 5 == 0, :] = tet[tet % 5 == 0, None] + np.arange(1, 5)[None, :]
        nb[tet % 5 != 0, 0] = np.tile(tet[tet % 5 == 0], (4, 1)).flatten(order="F")
        cx, cy = self.nsteps_cells[0], self.nsteps_cells[1]
        cell = tet // 5
        cidx = np.array([cell % cx, cell // cx % cy, cell // cx // cy])
        odd = (np.sum(cidx, axis=0) % 2 == 1)
        tables = [
            (1, True, [[1, 0, 0, 1], [0, 1, 0, 2], [0, 0, 1, 4]]),
            (2, True, [[-1, 0, 0, 2], [0, -1, 0, 1], [0, 0, 1, 3]]),
            (3, True, [[-1, 0, 0, 4], [0, 1, 0, 3], [0, 0, -1, 1]]),
            (4, True, [[1, 0, 0, 3], [0, -1, 0, 4], [0, 0, -1, 2]]),
            (1, False, [[-1, 0, 0, 1], [0, 1, 0, 2], [0, 0, 1, 3]]),
            (2, False, [[1, 0, 0, 2], [0, -1, 0, 1], [0, 0, 1, 4]]),
            (3, False, [[-1, 0, 0, 4], [0, -1, 0, 3], [0, 0, -1, 2]]),
            (4, False, [[1, 0, 0, 3], [0, 1, 0, 4], [0, 0, -1, 1]]),
        ]
        for local, want_odd, mask in tables:
            mask = np.array(mask)
            logic = (tet % 5 == local) & (odd == want_odd)
            c = cidx[:, logic]
            ncell = np.zeros((c.shape[1], 3, 3), dtype=int)
            for d in range(3):
                ncell[:, :, d] = c[d][:, None] + mask[:, d]
            ok = np.ones(ncell.shape[:2], dtype=bool)
            for d in range(3):
                ok &= (ncell[:, :, d] >= 0) & (ncell[:, :, d] < self.nsteps_cells[d])
            g = (ncell[:, :, 0] + ncell[:, :, 1] * cx + ncell[:, :, 2] * cx * cy) * 5 + mask[:, 3]
            g[~ok] = -1
            nb[logic, 1:] = g
        return nb

    def face_table(self):
        """T:120-184: unique face-sharing tet pairs (i > j, CSR order) and the
        three shared node ids of each face."""
        elements = self.elements
        nb = self.neighbours()
        rows = np.tile(np.arange(self.ntetra)[:, None], (1, 4))
        en = coo_matrix((np.ones(elements.shape[0] * 4), (rows.ravel(), elements.ravel())),
                        shape=(self.ntetra, self.n_nodes), dtype=bool).tocsr()
        n1 = np.tile(np.arange(nb.shape[0], dtype=int)[:, None], (1, 4)).flatten()
        n2 = nb.flatten()
        n1, n2 = n1[n2 >= 0], n2[n2 >= 0]
        pairs = coo_matrix((np.ones(n1.shape[0]), (n1, n2))).tocsr()
        i, j = tril(pairs).nonzero()
        rel = np.stack([i, j], axis=1)
        faces = en[rel[:, 0], :].multiply(en[rel[:, 1], :])
        row, col = faces.nonzero()
        order = np.argsort(row, kind="stable")
        row, col = row[order], col[order]
        shared = np.full((rel.shape[0], 3), -1, dtype=int)
        shared[row.reshape(-1, 3)[:, 0], :] = col.reshape(-1, 3)
        return rel.astype(np.int64), shared.astype(np.int64)

    def face_normals(self, shared):  # T:186-194
        nodes = self.nodes
        v1 = nodes[shared[:, 1]] - nodes[shared[:, 0]]
        v2 = nodes[shared[:, 2]] - nodes[shared[:, 0]]
        return np.cross(v1, v2, axisa=1, axisb=1)

    def element_for_location(self, pos):  # T:274-365
        pos = np.array(pos)[:, :3]
        ci, inside = self.position_to_cell_index(pos)
        even = np.sum(ci, axis=1) % 2 == 0
        corners = self._cell_corners(ci)
        nodes = self.origin[None, None, :] + self.step_vector[None, None, :] * corners
        verts = np.full((pos.shape[0], 5, 4, 3), np.nan)
        verts[even] = nodes[even][:, TETRA_MASK_EVEN, :]
        verts[~even] = nodes[~even][:, TETRA_MASK_ODD, :]
        vap = pos[:, None, :] - verts[:, :, 0, :]
        vbp = pos[:, None, :] - verts[:, :, 1, :]
        vab = verts[:, :, 1, :] - verts[:, :, 0, :]
        vac = verts[:, :, 2, :] - verts[:, :, 0, :]
        vad = verts[:, :, 3, :] - verts[:, :, 0, :]
        vbc = verts[:, :, 2, :] - verts[:, :, 1, :]
        vbd = verts[:, :, 3, :] - verts[:, :, 1, :]
        va = np.einsum("ikj, ikj->ik", vbp, np.cross(vbd, vbc, axisa=2, axisb=2)) / 6.0
        vb = np.einsum("ikj, ikj->ik", vap, np.cross(vac, vad, axisa=2, axisb=2)) / 6.0
        vc = np.einsum("ikj, ikj->ik", vap, np.cross(vad, vab, axisa=2, axisb=2)) / 6.0
        vd = np.einsum("ikj, ikj->ik", vap, np.cross(vab, vac, axisa=2, axisb=2)) / 6.0
        v = np.einsum("ikj, ikj->ik", vab, np.cross(vac, vad, axisa=2, axisb=2)) / 6.0
        c = np.stack([va / v, vb / v, vc / v, vd / v], axis=2)
        mask = np.all(c >= 0, axis=2)
        i, j = np.where(mask)
        last = dict(zip(i, j))
        mask[:] = False
        mask[list(last.keys()), list(last.values())] = True
        inside = inside & np.any(mask, axis=1) & self.inside(pos)
        mask[~inside, :] = False
        c_ret = np.full((pos.shape[0], 4), np.nan)
        c_ret[inside] = c[mask]
        v_ret = np.full((pos.shape[0], 4, 3), np.nan)
        v_ret[inside] = verts[mask]
        local = np.tile(np.arange(5)[None, :], (mask.shape[0], 1))[mask]
        tet = np.full(pos.shape[0], -1, dtype=np.int64)
        cx, cy = self.nsteps_cells[0], self.nsteps_cells[1]
        cin = ci[inside]
        tet[inside] = local + cin[:, 0] * 5 + cx * cin[:, 1] * 5 + cx * cy * cin[:, 2] * 5
        return v_ret, c_ret, tet, inside

    def evaluate_value(self, pos, c):  # T:208-229
        vals = np.full(pos.shape[0], np.nan)
        _, bc, tet, inside = self.element_for_location(pos)
        vals[inside] = np.sum(bc[inside] * c[self.elements[tet[inside]]], axis=1)
        return vals

    def evaluate_gradient(self, pos, c):  # T:231-262, T:502-545
        vals = np.full(pos.shape, np.nan)
        verts, _, tet, inside = self.element_for_location(pos)
        ps = verts[inside]
        m = np.array([[ps[:, k, d] - ps[:, 0, d] for d in range(3)] for k in (1, 2, 3)])
        m = np.swapaxes(m, 0, 2)
        g = np.linalg.inv(m).swapaxes(1, 2) @ _GRAD_I
        vals[inside] = (g * c[self.elements[tet[inside]]][:, None, :]).sum(2)
        return vals


def minimise_edge_jumps(mesh: TetMesh, cs: ConstraintSet, w, vector=None, name="edge jump", scale=None):  # P1:115-166
    """``vector`` (one row per face, P1:129-130) replaces the face normal:
    the directional regularisation of P1:172-178.  ``scale`` (per node,
    ``use_regularisation_weight_scale``): each face row's weight times the
    mean of the two tetrahedra's mean node scales (P1:150-155)."""
    rel, shared = mesh.face_table()
    norm = mesh.face_normals(shared)
    if vector is not None and np.asarray(vector).shape[0] == rel.shape[0]:
        norm = np.asarray(vector, dtype=float)
    g = mesh.element_gradients()
    Dt = g[rel[:, 0]]
    Dn = g[rel[:, 1]]
    const = np.hstack([np.einsum("ij,ijk->ik", norm, Dt), -np.einsum("ij,ijk->ik", norm, Dn)])
    idc = np.hstack([mesh.elements[rel[:, 0]], mesh.elements[rel[:, 1]]])
    if scale is not None:
        w = 0.5 * (scale[mesh.elements[rel[:, 0]]].mean(axis=1) + scale[mesh.elements[rel[:, 1]]].mean(axis=1)) * w
    cs.add(const, np.zeros(const.shape[0]), idc, w=w, name=name)
    return rel, shared


def face_centres(mesh: TetMesh):
    """P1:169-170 regularisation sample points: mean of the 3 shared face nodes."""
    _rel, shared = mesh.face_table()
    return mesh.nodes[shared].mean(axis=1)


def add_norm_constraints(mesh: TetMesh, cs: ConstraintSet, points, w):  # P1:73-96
    if points.shape[0] == 0:
        return
    _, _, tet, inside = mesh.element_for_location(points[:, :3])
    grad = mesh.element_gradients(tet)
    wt = np.ones(int(np.sum(inside))) * w
    el = np.tile(mesh.elements[tet[inside]], (3, 1, 1)).swapaxes(0, 1)
    cs.add(grad[inside], points[inside, 3:6], el, w=wt, name="norm")


def add_value_constraints(mesh: TetMesh, cs: ConstraintSet, points, w):  # P1:98-113
    if points.shape[0] == 0:
        return
    _, bc, tet, inside = mesh.element_for_location(points[:, :3])
    wt = np.ones(int(np.sum(inside))) * w
    cs.add(bc[inside], points[inside, 3], mesh.elements[tet[inside], :], w=wt, name="value")


def element_size(mesh: TetMesh):  # T:81-95
    """Volume of every tetrahedron, |det(edges)| / 6."""
    nodes = mesh.nodes[mesh.elements]
    vecs = nodes[:, 1:, :] - nodes[:, 0, None, :]
    return np.abs(np.linalg.det(vecs)) / 6


def add_gradient_orthogonal_constraints(mesh: TetMesh, cs: ConstraintSet, points, vectors, w=1.0, b=0.0,
                                        name="undefined gradient orthogonal constraint"):  # P1:248-296
    """grad(f) . v/|v| = b at the points inside, weight w x the tetrahedron's
    volume (the tangent constraints of DI:668-682 with b = 0)."""
    if points.shape[0] == 0:
        return
    _, _, tet, inside = mesh.element_for_location(points[:, :3])
    grad = mesh.element_gradients(tet)
    size = element_size(mesh)[tet[inside]]
    wt = np.ones(size.shape[0])
    wt *= w * size
    v = np.array(vectors, dtype=float)
    nrm = np.linalg.norm(v, axis=1)
    v[nrm > 0, :] /= nrm[nrm > 0, None]
    A = np.einsum("ij,ijk->ik", v[inside, :3], grad[inside, :, :])
    B = np.zeros(int(inside.sum())) + b
    cs.add(A, B, mesh.elements[tet[inside], :], w=wt, name=name)


def resolve_weights(regularisation=None, **kwargs):  # P1:180-246
    w = dict(DEFAULT_P1_WEIGHTS)
    if regularisation is not None:
        w["cgw"] = float(regularisation)
    w.update(kwargs)
    return w


def regularisation_scale(mesh: TetMesh, normals, sigma=None):  # P1:52-69
    """1 + compute_weighting over the normal constraints inside the mesh."""
    from .fd_oracle import compute_weighting

    scale = np.ones(mesh.n_nodes)
    if normals.shape[0] == 0:
        return scale
    _, _, _tet, inside = mesh.element_for_location(normals[:, :3])
    if inside.any():
        s = mesh.nsteps[0] * 10 if sigma is None else sigma
        scale = scale + compute_weighting(mesh.nodes, normals[inside, :3], sigma=s)
    return scale


def assemble(mesh: TetMesh, data: dict, weights: dict, directional=(), weight_scale=False,
             weight_sigma=None) -> ConstraintSet:
    """P1:180-246 family order: edge jumps, directional terms ((w, vector,
    name) triples, P1:229), (gradient: no-op), norm, value;
    ``weight_scale`` = ``use_regularisation_weight_scale``."""
    cs = ConstraintSet(mesh.n_nodes)
    scale = regularisation_scale(mesh, data.get("normal", np.zeros((0, 7))), weight_sigma) if weight_scale else None
    if weights["cgw"] > 0.0:
        minimise_edge_jumps(mesh, cs, weights["cgw"], scale=scale)
    for dw, vector, dname in directional:
        if dw != 0:
            minimise_edge_jumps(mesh, cs, dw, vector=vector, name=dname, scale=scale)
    add_norm_constraints(mesh, cs, data.get("normal", np.zeros((0, 7))), weights["npw"])
    add_value_constraints(mesh, cs, data.get("value", np.zeros((0, 5))), weights["cpw"])
    tangent = data.get("tangent", np.zeros((0, 7)))
    if tangent.shape[0] > 0:  # DI:668-682
        add_gradient_orthogonal_constraints(mesh, cs, tangent[:, :3], tangent[:, 3:6], weights["tpw"])
    return cs
