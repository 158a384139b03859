"""Generate golden vectors from the reference LoopStructural implementation.

Run in a container where the reference source tree is available:

    python tests/golden/make_golden.py /path/to/LoopStructural
    python tests/golden/make_golden.py /path/to/LoopStructural --directional
    python tests/golden/make_golden.py /path/to/LoopStructural --configs
    python tests/golden/make_golden.py /path/to/LoopStructural --faults
    python tests/golden/make_golden.py /path/to/LoopStructural --admm
    python tests/golden/make_golden.py /path/to/LoopStructural --weight-scale

It imports the reference's ``loop_interpolation`` / ``loop_common`` packages
(``pyvista`` and ``yaml`` are stubbed: they are only used for VTK/YAML export)
and writes small ``.npz`` fixtures next to this script.  The fixtures are
committed; tests read them without the reference being present.

What is recorded per case:
  * every constraint family the reference adds (name, the raw column indices
    passed to ``add_constraints_to_least_squares`` and the stored CSC matrix,
    b and w after row normalisation),
  * the assembled weighted system's FP64 direct solution of
    (AᵀWA + 1e-16 I) x = AᵀWb,
  * the reference's own ``solve_system('cg')`` solution at a tight tolerance,
  * ``evaluate_value`` / ``evaluate_gradient`` of that solution at query
    points (inside, on faces/corners, outside, NaN rows).
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _import_reference(root):
    for name in ("pyvista", "yaml"):
        if name not in sys.modules:
            try:
                __import__(name)
            except Exception:
                sys.modules[name] = types.ModuleType(name)
    sys.path.insert(0, os.path.join(root, "packages", "loop_common", "src"))
    sys.path.insert(0, os.path.join(root, "packages", "loop_interpolation", "src"))
    import loop_interpolation as li  # noqa: F401
    from loop_common.supports import StructuredGrid, TetMesh

    return li, StructuredGrid, TetMesh


def _field(p, fault=False):
    f = p[:, 2] + 0.1 * np.sin(2 * np.pi * p[:, 0]) + 0.05 * np.cos(2 * np.pi * p[:, 1])
    if fault:
        f = f + 0.2 * (p[:, 0] > 0.5)
    return f


def _grad(p):
    g = np.zeros_like(p)
    g[:, 0] = 0.1 * 2 * np.pi * np.cos(2 * np.pi * p[:, 0])
    g[:, 1] = -0.05 * 2 * np.pi * np.sin(2 * np.pi * p[:, 1])
    g[:, 2] = 1.0
    return g


def _hook(li):
    """Record every add_constraints_to_least_squares call's raw idc."""
    from loop_interpolation._discrete_interpolator import DiscreteInterpolator

    calls = []
    orig = DiscreteInterpolator.add_constraints_to_least_squares

    def wrapped(self, A, B, idc, w=1.0, name="undefined"):
        before = set(self.constraints.keys())
        orig(self, A, B, idc, w=w, name=name)
        after = [k for k in self.constraints.keys() if k not in before]
        if after:
            idc_arr = np.array(idc)
            if idc_arr.ndim > 2:
                idc_arr = idc_arr.reshape(-1, idc_arr.shape[-1])
            calls.append((after[0], idc_arr.astype(np.int64)))

    DiscreteInterpolator.add_constraints_to_least_squares = wrapped
    return calls, (DiscreteInterpolator, orig)


def _families_to_arrays(interp, calls, prefix, out):
    names = []
    for name, idc in calls:
        c = interp.constraints[name]
        m = c["matrix"].tocsr()
        m.sort_indices()
        names.append(name)
        out[f"{prefix}fam_{name}_idc"] = idc
        out[f"{prefix}fam_{name}_indptr"] = m.indptr.astype(np.int64)
        out[f"{prefix}fam_{name}_indices"] = m.indices.astype(np.int64)
        out[f"{prefix}fam_{name}_data"] = m.data
        out[f"{prefix}fam_{name}_b"] = np.asarray(c["b"], dtype=float)
        out[f"{prefix}fam_{name}_w"] = np.asarray(c["w"], dtype=float)
    out[f"{prefix}family_names"] = np.array(names)


def _solve_direct(interp):
    from scipy import sparse
    from scipy.sparse.linalg import spsolve

    A, b = interp.build_matrix()
    A = A.tocsr()
    N = (A.T @ A).tocsc() + sparse.eye(A.shape[1], format="csc") * (interp.ridge_factor**2)
    return spsolve(N, A.T @ b)


def _queries(rng, lo, hi, n=64):
    q = rng.uniform(lo, hi, size=(n, 3))
    extra = np.array(
        [
            [lo, lo, lo], [hi, hi, hi], [hi, lo, lo], [lo, hi, hi],
            [hi, 0.5 * (lo + hi), 0.25 * (lo + hi)],
            [hi + 1e-3, 0.5, 0.5], [lo - 1e-3, 0.5, 0.5], [0.5, hi + 0.5, 0.5],
            [np.nan, 0.5, 0.5],
        ]
    )
    return np.vstack([q, extra])


def fd_case(li, StructuredGrid, name, cells, n_val, n_norm, n_grad, n_tan, n_iface, seed, setup_kwargs, out):
    calls, (cls, orig) = _hook(li)
    try:
        rng = np.random.default_rng(seed)
        grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.FiniteDifferenceInterpolator(grid)
        vp = rng.uniform(0, 1, size=(n_val, 3))
        vp[:4] = [[0, 0, 0], [1, 1, 1], [1, 0.5, 0.25], [0.5, 1.0, 0.0]]
        vp[4] = [1.05, 0.5, 0.5]  # outside
        vp[5] = [1.0 + 1e-17, 0.3, 0.3]  # inside by tolerance
        val = np.column_stack([vp, _field(vp), rng.uniform(0.5, 2.0, n_val)])
        val = np.vstack([val, [[0.3, np.nan, 0.2, 1.0, 1.0]]])  # dropped by validation
        interp.set_value_constraints(val)
        data = {"value_in": val}
        if n_norm:
            npnt = rng.uniform(0, 1, size=(n_norm, 3))
            g = _grad(npnt)
            g /= np.linalg.norm(g, axis=1)[:, None]
            g += rng.normal(0, 0.02, size=g.shape)
            nrm = np.column_stack([npnt, g, rng.uniform(0.5, 2.0, n_norm)])
            interp.set_normal_constraints(nrm)
            data["normal_in"] = nrm
        if n_grad:
            gp = rng.uniform(0, 1, size=(n_grad, 3))
            gv = _grad(gp)
            gv[0] = [0.0, 0.0, 2.0]  # vertical: strike from atan2(0, 0)
            grd = np.column_stack([gp, gv, np.ones(n_grad)])
            interp.set_gradient_constraints(grd)
            data["gradient_in"] = grd
        if n_tan:
            tp = rng.uniform(0, 1, size=(n_tan, 3))
            tv = rng.normal(size=(n_tan, 3))
            tan = np.column_stack([tp, tv, np.ones(n_tan)])
            interp.set_tangent_constraints(tan)
            data["tangent_in"] = tan
        if n_iface:
            ip = rng.uniform(0, 1, size=(n_iface, 3))
            ids = np.array([0.0, 1.0] * (n_iface // 2) + [0.0] * (n_iface % 2))
            ifc = np.column_stack([ip, ids, np.ones(n_iface)])
            interp.set_interface_constraints(ifc)
            data["interface_in"] = ifc
        for k in ("value", "normal", "gradient", "tangent", "interface"):
            out[f"{name}_data_{k}"] = np.asarray(interp.data[k], dtype=float)
        for k, v in data.items():
            out[f"{name}_{k}"] = v
        interp.setup_interpolator(**setup_kwargs)
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_weights_keys"] = np.array(list(interp.interpolation_weights.keys()))
        out[f"{name}_weights_vals"] = np.array([float(v) if np.isscalar(v) else np.nan for v in interp.interpolation_weights.values()])
        out[f"{name}_c_direct"] = _solve_direct(interp)
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "maxiter": 200000})
        out[f"{name}_c_cg_tight"] = np.array(interp.c)
        q = _queries(rng, 0.0, 1.0)
        out[f"{name}_query"] = q
        interp.c = out[f"{name}_c_direct"].copy()
        out[f"{name}_eval_value"] = interp.evaluate_value(q)
        out[f"{name}_eval_gradient"] = interp.evaluate_gradient(q)
    finally:
        cls.add_constraints_to_least_squares = orig


def reg_index_case(li, StructuredGrid, cells, out):
    """All twelve regularisation families' raw idc at a tiny grid."""
    calls, (cls, orig) = _hook(li)
    try:
        grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells), step_vector=np.ones(3))
        interp = li.FiniteDifferenceInterpolator(grid)
        kw = dict(dxy=1.0, dyz=0.8, dxz=1.3, dxx=0.5, dyy=0.4, dzz=0.6, dx=0.7, dy=0.9, dz=1.1,
                  cpw=0.0, gpw=0.0, npw=0.0, tpw=0.0, ipw=0.0)
        interp.setup_interpolator(**kw)
        tag = "reg_" + "x".join(str(c) for c in cells) + "_"
        _families_to_arrays(interp, calls, tag, out)
    finally:
        cls.add_constraints_to_least_squares = orig


def p1_case(li, TetMesh, name, cells, n_val, n_norm, seed, setup_kwargs, out):
    calls, (cls, orig) = _hook(li)
    try:
        rng = np.random.default_rng(seed)
        mesh = TetMesh(origin=np.zeros(3), nsteps_cells=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.P1Interpolator(mesh)
        vp = rng.uniform(0, 1, size=(n_val, 3))
        vp[0] = [0.0, 0.5, 0.5]  # on the boundary: outside for the strict TetMesh.inside
        val = np.column_stack([vp, _field(vp, fault=True) + rng.normal(0, 0.01, n_val), np.ones(n_val)])
        interp.set_value_constraints(val)
        npnt = rng.uniform(0, 1, size=(n_norm, 3))
        g = _grad(npnt)
        nrm = np.column_stack([npnt, g, np.ones(n_norm)])
        interp.set_normal_constraints(nrm)
        out[f"{name}_value_in"] = val
        out[f"{name}_normal_in"] = nrm
        interp.setup_interpolator(**setup_kwargs)
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_shared_rel"] = np.asarray(mesh.shared_element_relationships, dtype=np.int64)
        out[f"{name}_shared_nodes"] = np.asarray(mesh.shared_elements, dtype=np.int64)
        out[f"{name}_elements"] = np.asarray(mesh.elements, dtype=np.int64)
        out[f"{name}_neighbours"] = np.asarray(mesh.get_neighbours(), dtype=np.int64)
        out[f"{name}_c_direct"] = _solve_direct(interp)
        # solve once so that evaluate_* (which calls update()) does not re-solve
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "maxiter": 200000})
        out[f"{name}_c_cg_tight"] = np.array(interp.c)
        q = _queries(rng, 0.0, 1.0)
        out[f"{name}_query"] = q
        interp.c = out[f"{name}_c_direct"].copy()
        out[f"{name}_eval_value"] = interp.evaluate_value(q)
        out[f"{name}_eval_gradient"] = interp.evaluate_gradient(q)
        vtx, bc, tet, inside = mesh.get_element_for_location(q[:-1])
        out[f"{name}_loc_bc"] = bc
        out[f"{name}_loc_tet"] = tet.astype(np.int64)
        out[f"{name}_loc_inside"] = inside
    finally:
        cls.add_constraints_to_least_squares = orig


def _direction_field(p):
    """A smoothly varying unit direction with exact zero components on part of
    the grid (so that some directional rows have weight 0 and are skipped)."""
    v = np.column_stack([np.cos(2.0 * p[:, 2]), 0.4 * np.sin(3.0 * p[:, 0]), 0.3 + p[:, 1]])
    v[p[:, 0] < 0.25, 0] = 0.0
    v[p[:, 2] > 0.8, 1] = 0.0
    return v / np.linalg.norm(v, axis=1)[:, None]


def fd_directional_case(li, StructuredGrid, name, cells, seed, out):
    """Directional regularisation (FD:1207-1337) given as an array and as a
    callable, plus a gradient-orthogonal family with a non-zero target
    (FD:478-539) added after setup."""
    from loop_interpolation._regularisation import DirectionalRegularisation

    calls, (cls, orig) = _hook(li)
    try:
        rng = np.random.default_rng(seed)
        grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.FiniteDifferenceInterpolator(grid)
        vp = rng.uniform(0, 1, size=(30, 3))
        val = np.column_stack([vp, _field(vp, fault=True), np.ones(30)])
        interp.set_value_constraints(val)
        npnt = rng.uniform(0, 1, size=(8, 3))
        g = _grad(npnt)
        nrm = np.column_stack([npnt, g / np.linalg.norm(g, axis=1)[:, None], np.ones(8)])
        interp.set_normal_constraints(nrm)
        nodes = np.asarray(grid.nodes)
        v1 = _direction_field(nodes)

        def v2(p):
            return np.column_stack([np.zeros(len(p)), np.ones(len(p)), p[:, 2]])

        reg = {"isotropic": 0.1,
               "directional": [DirectionalRegularisation(weight=0.5, direction=v1, name="fold a"),
                               {"weight": 0.2, "direction": v2, "name": "fold b"}]}
        interp.setup_interpolator(regularisation=reg, cpw=1.0, npw=1.0)
        op = rng.uniform(0, 1, size=(12, 3))
        ov = rng.normal(size=(12, 3))
        interp.add_gradient_orthogonal_constraints(op, ov.copy(), w=2.0, b=0.3, name="fold normalisation")
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_value_in"] = val
        out[f"{name}_normal_in"] = nrm
        out[f"{name}_dir_a"] = v1
        out[f"{name}_dir_b"] = v2(nodes)
        out[f"{name}_orth_points"] = op
        out[f"{name}_orth_vectors"] = ov
        out[f"{name}_c_direct"] = _solve_direct(interp)
    finally:
        cls.add_constraints_to_least_squares = orig


def p1_directional_case(li, TetMesh, name, cells, seed, out):
    """P1 directional regularisation (P1:115-178): edge-jump rows whose
    normal is the given per-face vector."""
    calls, (cls, orig) = _hook(li)
    try:
        rng = np.random.default_rng(seed)
        mesh = TetMesh(origin=np.zeros(3), nsteps_cells=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.P1Interpolator(mesh)
        vp = rng.uniform(0.05, 0.95, size=(25, 3))
        val = np.column_stack([vp, _field(vp, fault=True), np.ones(25)])
        interp.set_value_constraints(val)
        centres = interp.get_regularisation_sample_points()
        vec = _direction_field(centres)
        interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0,
                                  directional_regularisation={"weight": 0.3, "direction": vec, "name": "fold p1"})
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_value_in"] = val
        out[f"{name}_dir"] = vec
        out[f"{name}_c_direct"] = _solve_direct(interp)
    finally:
        cls.add_constraints_to_least_squares = orig


class SyntheticFold:
    """A fold geometry provider with the reference FoldEvent's
    ``get_deformed_orientation(points) -> (deformed_orientation, fold_axis,
    dgz)`` contract: the fold axis plunges gently along y, the across-fold
    direction dgz rotates with x, the deformed orientation completes the
    frame.  Plain numpy, so both implementations see identical vectors."""

    def get_deformed_orientation(self, points):
        p = np.asarray(points, dtype=float)
        ang = 1.5 * np.pi * p[:, 0]
        dgz = np.column_stack([np.sin(ang), np.zeros(len(p)), -np.cos(ang)])
        axis = np.tile([0.0, 1.0, 0.15], (len(p), 1))
        axis /= np.linalg.norm(axis, axis=1)[:, None]
        deformed = np.cross(dgz, axis)
        return deformed, axis, dgz


def fold_case_weights():
    """The fold_weights of the fd_fold case (shared with the tests)."""
    return {"fold_orientation": 5.0, "fold_axis_w": 3.0, "fold_regularisation": [0.2, 0.05, 0.02],
            "fold_normalisation": 1.5, "fold_norm": -1.0, "dgz_alignment": "correct",
            "mask_fn": lambda p: p[:, 2] > 0.85}


def fd_fold_case(li, StructuredGrid, name, cells, seed, out):
    """FDFoldInterpolator (_fd_fold_interpolator.py) with a synthetic fold,
    a node mask and dgz alignment correction."""
    from loop_interpolation._fd_fold_interpolator import FDFoldInterpolator

    calls, (cls, orig) = _hook(li)
    try:
        rng = np.random.default_rng(seed)
        grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = FDFoldInterpolator(grid, fold=SyntheticFold())
        vp = rng.uniform(0, 1, size=(25, 3))
        val = np.column_stack([vp, _field(vp), np.ones(25)])
        interp.set_value_constraints(val)
        npnt = rng.uniform(0, 1, size=(10, 3))
        g = _grad(npnt)
        nrm = np.column_stack([npnt, g / np.linalg.norm(g, axis=1)[:, None], np.ones(10)])
        interp.set_normal_constraints(nrm)
        fold_weights = fold_case_weights()
        interp.setup_interpolator(regularisation=0.05, cpw=1.0, npw=1.0, fold_weights=fold_weights)
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_value_in"] = val
        out[f"{name}_normal_in"] = nrm
        out[f"{name}_c_direct"] = _solve_direct(interp)
    finally:
        cls.add_constraints_to_least_squares = orig


# ---------------------------------------------------------------------------
# cases at the benchmark configurations' sizes (--configs)
# ---------------------------------------------------------------------------
def _repo_bench():
    """The benchmark's seeded workload generator (same data for the fixtures,
    the GPU tests and bench.py)."""
    root = os.path.dirname(os.path.dirname(HERE))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench

    return bench


def _point_families(interp, calls, prefix, out, keep=("value", "norm")):
    """Full rows of the point families (value / norm_k): raw idc plus the
    stored coefficients; and the names and row counts of every family."""
    names = []
    for name, idc in calls:
        if not name.startswith(keep):
            continue
        c = interp.constraints[name]
        m = c["matrix"].tocsr()
        m.sort_indices()
        names.append(name)
        out[f"{prefix}fam_{name}_idc"] = idc
        out[f"{prefix}fam_{name}_indptr"] = m.indptr.astype(np.int64)
        out[f"{prefix}fam_{name}_indices"] = m.indices.astype(np.int64)
        out[f"{prefix}fam_{name}_data"] = m.data
        out[f"{prefix}fam_{name}_b"] = np.asarray(c["b"], dtype=float)
        out[f"{prefix}fam_{name}_w"] = np.asarray(c["w"], dtype=float)
    out[f"{prefix}point_family_names"] = np.array(names)
    out[f"{prefix}all_family_names"] = np.array(list(interp.constraints.keys()))
    out[f"{prefix}all_family_rows"] = np.array([interp.constraints[k]["matrix"].shape[0] for k in interp.constraints])


def cfg1_case(li, StructuredGrid, out):
    """Configuration 1 exactly: 50^3 nodes in the unit box, 200 value points,
    50 noisy normals (sigma 0.02) of the unfaulted layered field,
    regularisation 0.1.  The reference's own CG to rtol 1e-12 (atol 1e-10,
    its `tol`), and value / gradient of that solution on 4096 points of the
    100^3 evaluation lattice."""
    bench = _repo_bench()
    cells, val, nrm = bench.cfg1_workload()
    calls, (cls, orig) = _hook(li)
    try:
        grid = StructuredGrid(origin=np.zeros(3), nsteps=cells, step_vector=1.0 / cells.astype(float))
        interp = li.FiniteDifferenceInterpolator(grid)
        interp.set_value_constraints(val)
        interp.set_normal_constraints(nrm)
        interp.setup_interpolator(regularisation=bench.REGULARISATION, cpw=1.0, npw=1.0)
        _point_families(interp, calls, "cfg1_", out)
        interp.solve_system("cg", tol=1e-10, solver_kwargs={"rtol": 1e-12, "maxiter": 400000})
        out["cfg1_c_tight"] = np.array(interp.c)
        ax = np.linspace(0.0, 1.0, bench.CFG1_LATTICE)
        pick = np.random.default_rng(2).choice(bench.CFG1_LATTICE ** 3, 4096, replace=False)
        i, j, k = np.unravel_index(pick, (bench.CFG1_LATTICE,) * 3, order="F")
        q = np.column_stack([ax[i], ax[j], ax[k]])
        out["cfg1_lattice_pick"] = pick.astype(np.int64)
        out["cfg1_eval_value"] = interp.evaluate_value(q)
        out["cfg1_eval_gradient"] = interp.evaluate_gradient(q)
    finally:
        cls.add_constraints_to_least_squares = orig


def factory_case(li, out):
    """An FD interpolator built by the reference's own factory from a
    BoundingBox with a non-zero origin and an anisotropic extent
    (InterpolatorFactory.create_interpolator("FDI", boundingbox, nelements)):
    the support lives in the box's local frame with non-unit cells, the
    setters project world points, evaluation projects query points and
    reprojects gradients."""
    from loop_common.geometry import BoundingBox

    calls, (cls, orig) = _hook(li)
    try:
        origin = np.array([100.0, -50.0, 20.0])
        maximum = np.array([600.0, 250.0, 120.0])
        bb = BoundingBox(origin=origin, maximum=maximum)
        interp = li.InterpolatorFactory.create_interpolator("FDI", boundingbox=bb, nelements=3000)
        sup = interp.support
        rng = np.random.default_rng(9)
        ext = maximum - origin

        def f(p):
            u = (p - origin) / ext
            return u[:, 2] + 0.1 * np.sin(2 * np.pi * u[:, 0]) + 0.05 * np.cos(2 * np.pi * u[:, 1])

        def grad(p):
            u = (p - origin) / ext
            g = np.column_stack([0.2 * np.pi * np.cos(2 * np.pi * u[:, 0]),
                                 -0.1 * np.pi * np.sin(2 * np.pi * u[:, 1]), np.ones(len(u))])
            return g / ext

        vp = origin + ext * rng.uniform(0, 1, size=(300, 3))
        val = np.column_stack([vp, f(vp), np.ones(300)])
        npnt = origin + ext * rng.uniform(0, 1, size=(60, 3))
        g = grad(npnt)
        g /= np.linalg.norm(g, axis=1)[:, None]
        g += rng.normal(0, 0.02, size=g.shape)
        nrm = np.column_stack([npnt, g, np.ones(60)])
        interp.set_value_constraints(val)
        interp.set_normal_constraints(nrm)
        interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
        out["fac_value_in"] = val
        out["fac_normal_in"] = nrm
        out["fac_origin"] = np.asarray(sup.origin, dtype=float)
        out["fac_step"] = np.asarray(sup.step_vector, dtype=float)
        out["fac_nsteps"] = np.asarray(sup.nsteps, dtype=np.int64)  # nodes per axis
        out["fac_world_to_local"] = np.asarray(bb.world_to_local_matrix, dtype=float)
        out["fac_local_to_world"] = np.asarray(bb.local_to_world_matrix, dtype=float)
        out["fac_local_rotation"] = np.asarray(bb.local_rotation, dtype=float)
        out["fac_data_value"] = np.asarray(interp.data["value"], dtype=float)
        out["fac_data_normal"] = np.asarray(interp.data["normal"], dtype=float)
        _point_families(interp, calls, "fac_", out)
        interp.solve_system("cg", tol=1e-12, solver_kwargs={"rtol": 1e-13, "maxiter": 400000})
        out["fac_c_tight"] = np.array(interp.c)
        q = origin + ext * rng.uniform(-0.05, 1.05, size=(500, 3))
        out["fac_query"] = q
        out["fac_eval_value"] = interp.evaluate_value(q)
        out["fac_eval_gradient"] = interp.evaluate_gradient(q)
    finally:
        cls.add_constraints_to_least_squares = orig


def anisotropic_case(li, StructuredGrid, out):
    """A StructuredGrid with a shifted origin and a different cell size per
    axis (0.07 / 0.13 / 0.21): 250 values, 50 normals, regularisation 0.1."""
    calls, (cls, orig) = _hook(li)
    try:
        origin = np.array([-1.5, 2.0, 0.25])
        cells = np.array([22, 15, 11])
        step = np.array([0.07, 0.13, 0.21])
        ext = cells * step
        rng = np.random.default_rng(13)
        grid = StructuredGrid(origin=origin, nsteps=cells, step_vector=step)
        interp = li.FiniteDifferenceInterpolator(grid)
        vp = origin + ext * rng.uniform(0, 1, size=(250, 3))
        u = (vp - origin) / ext
        val = np.column_stack([vp, _field(u), np.ones(250)])
        npnt = origin + ext * rng.uniform(0, 1, size=(50, 3))
        g = _grad((npnt - origin) / ext) / ext
        g /= np.linalg.norm(g, axis=1)[:, None]
        nrm = np.column_stack([npnt, g + rng.normal(0, 0.02, size=g.shape), np.ones(50)])
        interp.set_value_constraints(val)
        interp.set_normal_constraints(nrm)
        interp.setup_interpolator(regularisation=0.1, cpw=1.0, npw=1.0)
        out["ani_origin"], out["ani_cells"], out["ani_step"] = origin, cells, step
        out["ani_value_in"], out["ani_normal_in"] = val, nrm
        _point_families(interp, calls, "ani_", out)
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "maxiter": 400000})
        out["ani_c_tight"] = np.array(interp.c)
        q = origin + ext * rng.uniform(-0.05, 1.05, size=(400, 3))
        out["ani_query"] = q
        out["ani_eval_value"] = interp.evaluate_value(q)
        out["ani_eval_gradient"] = interp.evaluate_gradient(q)
    finally:
        cls.add_constraints_to_least_squares = orig


def p1_config_case(li, TetMesh, out):
    """P1 at 16^3 cells (20,480 tetrahedra): 600 noisy values of the faulted
    field and 120 normals, cgw 0.1.  Face rows are recorded as their count, an
    order-sensitive checksum over all rows' indices and every 37th row in
    full (coefficients summed per column, as the stored matrix holds them)."""
    calls, (cls, orig) = _hook(li)
    try:
        cells = np.array([16, 16, 16])
        rng = np.random.default_rng(11)
        mesh = TetMesh(origin=np.zeros(3), nsteps_cells=cells, step_vector=1.0 / cells.astype(float))
        interp = li.P1Interpolator(mesh)
        vp = rng.uniform(0, 1, size=(600, 3))
        val = np.column_stack([vp, _field(vp, fault=True) + rng.normal(0, 0.01, 600), np.ones(600)])
        npnt = rng.uniform(0, 1, size=(120, 3))
        nrm = np.column_stack([npnt, _grad(npnt), np.ones(120)])
        interp.set_value_constraints(val)
        interp.set_normal_constraints(nrm)
        interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0)
        out["p1c_value_in"] = val
        out["p1c_normal_in"] = nrm
        out["p1c_cells"] = cells
        _point_families(interp, calls, "p1c_", out)
        for name, idc in calls:
            if name != "edge jump":
                continue
            m = interp.constraints[name]["matrix"].tocsr()
            m.sort_indices()
            nrow = idc.shape[0]
            rw = (np.arange(nrow, dtype=np.int64) % 1009) + 1
            out["p1c_face_rows"] = np.array(nrow)
            out["p1c_face_idc_checksum"] = np.array(np.sum(idc * (np.arange(idc.shape[1]) + 1)[None, :] * rw[:, None]))
            sub = np.arange(0, nrow, 37)
            dense = m[sub].toarray()
            out["p1c_face_sub_rows"] = sub
            out["p1c_face_sub_idc"] = idc[sub]
            out["p1c_face_sub_vals"] = np.take_along_axis(dense, idc[sub], axis=1)
            out["p1c_face_w"] = np.asarray(interp.constraints[name]["w"], dtype=float)[sub]
        interp.solve_system("cg", solver_kwargs={"rtol": 1e-13, "atol": 0.0, "maxiter": 400000})
        out["p1c_c_tight"] = np.array(interp.c)
        q = _queries(rng, 0.0, 1.0, n=400)
        out["p1c_query"] = q
        out["p1c_eval_value"] = interp.evaluate_value(q)
        out["p1c_eval_gradient"] = interp.evaluate_gradient(q)
    finally:
        cls.add_constraints_to_least_squares = orig


def main_configs(root):
    li, StructuredGrid, TetMesh = _import_reference(root)
    out = {}
    cfg1_case(li, StructuredGrid, out)
    factory_case(li, out)
    anisotropic_case(li, StructuredGrid, out)
    p1_config_case(li, TetMesh, out)
    path = os.path.join(HERE, "config_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


# ---------------------------------------------------------------------------
# faulted features (--faults)
# ---------------------------------------------------------------------------
def _import_reference_modelling(root):
    """The reference's modelling package (fault segments, geological
    features).  Its top-level import needs pandas, scikit-image and its own
    installed metadata, none of which the fault path uses: they are stubbed
    (only here, for recording fixtures)."""
    import importlib.metadata as md

    _version = md.version
    md.version = lambda name: "1.8.0" if name.lower() == "loopstructural" else _version(name)
    for name in ("pyvista", "yaml", "pandas", "skimage", "skimage.measure"):
        if name in sys.modules:
            continue
        try:
            __import__(name)
        except Exception:
            m = types.ModuleType(name)
            if name == "pandas":
                m.DataFrame = type("DataFrame", (), {})
                m.Series = type("Series", (), {})
            if name == "skimage.measure":
                m.marching_cubes = m.marching_cubes_lewiner = lambda *a, **k: None
            sys.modules[name] = m
    if "skimage.measure" in sys.modules and isinstance(sys.modules.get("skimage"), types.ModuleType):
        sys.modules["skimage"].measure = sys.modules["skimage.measure"]
    li, StructuredGrid, _ = _import_reference(root)
    sys.path.insert(0, root)
    from LoopStructural.modelling.features import GeologicalFeature
    from LoopStructural.modelling.features.fault._fault_function import CubicFunction, FaultDisplacement, Ones
    from LoopStructural.modelling.features.fault._fault_segment import FaultSegment

    return li, StructuredGrid, GeologicalFeature, FaultSegment, (CubicFunction, FaultDisplacement, Ones)


def _frame_fields(p, variant):
    """Analytic fault-frame coordinates: gx across a dipping fault surface,
    gy along slip (a curved direction), gz along the fault's extent."""
    if variant == 0:
        gx = (p[:, 0] - 0.5 - 0.1 * (p[:, 2] - 0.5)) / 0.4
        gy = (0.1 * p[:, 0] + p[:, 2] + 0.05 * np.sin(2 * np.pi * p[:, 1]) - 0.55) / 0.6
        gz = (p[:, 1] - 0.5) / 0.45
    else:
        gx = (p[:, 1] - 0.45 + 0.15 * (p[:, 0] - 0.5)) / 0.35
        gy = (p[:, 2] - 0.5 + 0.2 * p[:, 1] + 0.03 * np.cos(2 * np.pi * p[:, 0])) / 0.5
        gz = (p[:, 0] - 0.5) / 0.5
    return gx, gy, gz


def main_faults(root):
    li, StructuredGrid, GeologicalFeature, FaultSegment, (CubicFunction, FaultDisplacement, Ones) = \
        _import_reference_modelling(root)
    out = {}

    def fd_field(cells, origin, step, values_fn, name):
        grid = StructuredGrid(origin=np.asarray(origin, dtype=float), nsteps=np.asarray(cells),
                              step_vector=np.asarray(step, dtype=float))
        interp = li.FiniteDifferenceInterpolator(grid)
        interp.c = values_fn(grid.nodes)
        interp.up_to_date = True
        out[f"{name}_cells"] = np.asarray(cells)
        out[f"{name}_origin"] = np.asarray(origin, dtype=float)
        out[f"{name}_step"] = np.asarray(step, dtype=float)
        out[f"{name}_c"] = np.asarray(interp.c, dtype=float)
        return interp

    faults = []
    for k, (cells, disp) in enumerate((((14, 13, 12), 0.2), ((12, 14, 13), -0.15))):
        frame = []
        for j, nm in enumerate(("gx", "gy", "gz")):
            interp = fd_field(cells, (-0.05, -0.05, -0.05), 1.1 / np.asarray(cells, dtype=float),
                              lambda p, j=j, k=k: _frame_fields(p, k)[j], f"f{k}_{nm}")
            frame.append(GeologicalFeature(f"fault{k}_{nm}", builder=None, interpolator=interp))
        fault = FaultSegment(f"fault{k}", frame, displacement=disp)
        out[f"f{k}_displacement"] = np.array(disp)
        faults.append(fault)
    strat = fd_field((16, 15, 17), (0.0, 0.0, 0.0), 1.0 / np.array([16.0, 15.0, 17.0]),
                     lambda p: p[:, 2] + 0.1 * np.sin(2 * np.pi * p[:, 0]) + 0.05 * np.cos(2 * np.pi * p[:, 1]),
                     "strat")
    rng = np.random.default_rng(21)
    pts = rng.uniform(0.05, 0.95, size=(400, 3))
    out["points"] = pts
    # restoration through each fault with the default profile, BaseFault3D,
    # and a custom displacement with a cubic slip profile
    for k, f in enumerate(faults):
        out[f"restored_f{k}_base"] = f.apply_to_points(pts)
    faults[0].faultfunction = "BaseFault3D"
    out["restored_f0_base3d"] = faults[0].apply_to_points(pts)
    gyf = CubicFunction()
    gyf.add_cstr(-1, 0)
    gyf.add_cstr(1, 0)
    gyf.add_cstr(0, 1)
    gyf.add_grad(0, 0)
    gyf.add_min(-1)
    gyf.add_max(1)
    hw = CubicFunction()
    hw.add_cstr(0, 1)
    hw.add_grad(0, 0)
    hw.add_cstr(1, 0)
    hw.add_grad(1, 0)
    hw.set_lim(0, 1)
    fw = CubicFunction()
    fw.add_cstr(0, -1)
    fw.add_grad(0, 0)
    fw.add_cstr(-1, 0)
    fw.add_grad(-1, 0)
    fw.set_lim(-1, 0)
    faults[0].faultfunction = FaultDisplacement(hw=hw, fw=fw, gy=gyf, gz=Ones(), scale=0.7)
    out["restored_f0_custom"] = faults[0].apply_to_points(pts)
    faults[0].faultfunction = "BaseFault"
    feature = GeologicalFeature("strat", builder=None, interpolator=strat, faults=faults)
    out["faulted_value"] = feature.evaluate_value(pts)
    try:
        out["faulted_gradient"] = feature.evaluate_gradient(pts, element_scale_parameter=0.01)
        out["faulted_gradient_error"] = np.array("")
    except Exception as exc:  # recorded: the reference's faulted gradient path
        out["faulted_gradient_error"] = np.array(f"{type(exc).__name__}: {exc}")
    # the same steps with the reference's own functions and the result stored
    # in an (N, 3) array (GF:187-226 with the straddle-check values kept apart)
    from LoopStructural.utils.maths import gradient_from_tetrahedron, regular_tetraherdron_for_points

    esp = 0.01
    tet = regular_tetraherdron_for_points(pts, esp)
    resolved = False
    while not resolved:
        resolved = True
        for f in faults:
            gxv = f[0].evaluate_value(tet.reshape(-1, 3), fillnan="nearest").reshape(tet.shape[0], 4)
            if np.any(~(np.all(gxv > 0, axis=1) | np.all(gxv < 0, axis=1))):
                esp *= 0.5
                tet = regular_tetraherdron_for_points(pts, esp)
                resolved = False
    moved = feature._apply_faults(np.array(tet.reshape(-1, 3))).reshape(tet.shape)
    vals = strat.evaluate_value(moved.reshape(-1, 3)).reshape(-1, 4)
    out["faulted_gradient_reference_steps"] = gradient_from_tetrahedron(tet, vals)
    out["faulted_gradient_scale"] = np.array(esp)
    plain = GeologicalFeature("strat", builder=None, interpolator=strat)
    out["plain_gradient"] = plain.evaluate_gradient(pts)
    path = os.path.join(HERE, "fault_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes;", str(out["faulted_gradient_error"]))


def _exact_lsq(matrix, rhs, x0=None, **_kw):
    """Exact inner least-squares solve for the reference's ADMM (a callable
    ``linsys_solver``): the normal equations by sparse LU."""
    from scipy.sparse.linalg import splu

    m = matrix.tocsr()
    return splu((m.T @ m).tocsc()).solve(np.asarray(m.T @ rhs).reshape(-1))


ADMM_CASES = {
    # name: (cells, seed, solver kwargs besides linsys_solver, feature bound, bound spread)
    "admm_const": ((10, 9, 12), 11, dict(admm_weight=1.0, nmajor=80), None, 1.0),
    "admm_sched": ((9, 8, 10), 12, dict(admm_weight=0.05, admm_weight_final=2.0, nmajor=25,
                                         admm_weight_schedule="geometric"), None, 1.0),
    "admm_adapt": ((8, 9, 10), 13, dict(admm_weight=0.1, adaptive_rho=True, nmajor=60, min_iterations=3),
                   0.25, 1.0),
    # loose bounds and a start from x0: stops on the primal/dual test
    "admm_loose": ((9, 9, 9), 14, dict(admm_weight=0.5, nmajor=200, x0="nodes_z"), None, 20.0),
}

ADMM_X0 = {"nodes_z": lambda support: support.nodes[:, 2].copy()}


def admm_case(li, StructuredGrid, name, out):
    """Value + normal constraints with value inequalities and inequality pairs
    that the unconstrained field violates; ``solve_system('admm')`` with an
    exact inner solver; optionally a lower-bound inequality feature."""
    cells, seed, kwargs, feature, spread = ADMM_CASES[name]
    rng = np.random.default_rng(seed)
    grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
    interp = li.FiniteDifferenceInterpolator(grid)
    vp = rng.uniform(0.05, 0.95, size=(30, 3))
    val = np.column_stack([vp, _field(vp), np.ones(30)])
    npnt = rng.uniform(0.05, 0.95, size=(8, 3))
    g = _grad(npnt)
    g /= np.linalg.norm(g, axis=1)[:, None]
    nrm = np.column_stack([npnt, g, np.ones(8)])
    ip = rng.uniform(0.1, 0.9, size=(12, 3))
    f0 = _field(ip)
    lo = f0 + rng.uniform(0.02, 0.1, 12)  # above the unconstrained field: active
    hi = lo + rng.uniform(0.05, 0.2, 12)
    lo[8:] = -10.0  # upper-bound-only rows below the field: active from above
    hi[8:] = f0[8:] - 0.05
    if spread > 1.0:  # wide bounds around the field: inactive at the solution
        lo, hi = f0 - spread, f0 + spread
    ineq = np.column_stack([ip, lo, hi, np.ones(12)])
    ineq = np.vstack([ineq, [[1.2, 0.5, 0.5, 0.0, 1.0, 1.0]]])  # outside: dropped
    pp = np.vstack([rng.uniform(0.1, 0.9, size=(5, 3)), rng.uniform(0.1, 0.9, size=(4, 3))])
    pp[:5, 2] = rng.uniform(0.6, 0.9, 5)  # group 0 above group 1: f(0) <= f(1) is violated
    pp[5:, 2] = rng.uniform(0.1, 0.4, 4)
    if spread > 1.0:
        pp[:, 2] = pp[::-1, 2]  # group 0 below group 1: satisfied
    pairs = np.column_stack([pp, np.r_[np.zeros(5), np.ones(4)], np.ones(9)])
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.set_value_inequality_constraints(ineq)
    interp.set_inequality_pairs_constraints(pairs)
    setup = dict(regularisation=0.1, cpw=1.0, npw=1.0)
    interp.setup_interpolator(**setup)
    if feature is not None:
        interp.add_inequality_feature(lambda p: p[:, 2] - feature, lower=True,
                                      mask=grid.nodes[:, 0] > 0.5)
    Q, bounds = interp.build_inequality_matrix()
    Q = Q.tocoo()
    out[f"{name}_cells"] = np.array(cells)
    out[f"{name}_value"] = val
    out[f"{name}_normal"] = nrm
    out[f"{name}_ineq"] = ineq
    out[f"{name}_pairs"] = pairs
    out[f"{name}_feature"] = np.array([np.nan if feature is None else feature])
    out[f"{name}_Q_row"] = Q.row.astype(np.int64)
    out[f"{name}_Q_col"] = Q.col.astype(np.int64)
    out[f"{name}_Q_val"] = Q.data
    out[f"{name}_bounds"] = np.asarray(bounds, dtype=float)
    out[f"{name}_ineq_names"] = np.array(list(interp.ineq_constraints.keys()))
    out[f"{name}_kwargs_keys"] = np.array(list(kwargs.keys()))
    out[f"{name}_kwargs_vals"] = np.array([str(v) for v in kwargs.values()])
    run = dict(kwargs, linsys_solver=_exact_lsq, return_history=True)
    if "x0" in run:
        run["x0"] = ADMM_X0[run["x0"]]
    ok = interp.solve_system("admm", solver_kwargs=run)
    assert ok
    hist = interp.solver_history
    out[f"{name}_c"] = np.array(interp.c)
    out[f"{name}_iterations"] = np.array(len(hist))
    for k in ("primal_norm", "dual_norm", "eps_pri", "eps_dual", "rho"):
        out[f"{name}_hist_{k}"] = np.array([h[k] for h in hist], dtype=float)
    A, b = interp.build_matrix()
    A = A.tocsr()
    from scipy import sparse
    from scipy.sparse.linalg import spsolve

    N = (A.T @ A).tocsc() + sparse.eye(A.shape[1], format="csc") * (interp.ridge_factor ** 2)
    out[f"{name}_c_unconstrained"] = spsolve(N, A.T @ b)


def weight_scale_cases(li, StructuredGrid, TetMesh, out):
    """``use_regularisation_weight_scale``: the per-node scale 1 + sum over the
    normal-constraint calls of (1 + 10 exp(-d^2 / 2 sigma^2)), d the distance
    to the nearest inside normal point, on every regularisation row's centre
    (FD) or the mean over the face's two tetrahedra (P1).  The default sigma
    (10 x the node count along x) and a small one."""
    for name, cells, sigma in (("ws_fd_default", (9, 8, 10), None), ("ws_fd_sigma", (10, 9, 8), 0.15)):
        calls, (cls, orig) = _hook(li)
        try:
            rng = np.random.default_rng(21 if sigma is None else 22)
            grid = StructuredGrid(origin=np.zeros(3), nsteps=np.array(cells),
                                  step_vector=1.0 / np.array(cells, dtype=float))
            interp = li.FiniteDifferenceInterpolator(grid)
            vp = rng.uniform(0.02, 0.98, size=(40, 3))
            interp.set_value_constraints(np.column_stack([vp, _field(vp), np.ones(40)]))
            npnt = rng.uniform(0.05, 0.95, size=(12, 3))
            npnt[0] = [1.2, 0.5, 0.5]  # outside: not a distance target
            g = _grad(npnt)
            g /= np.linalg.norm(g, axis=1)[:, None]
            interp.set_normal_constraints(np.column_stack([npnt, g, np.ones(12)]))
            kw = dict(regularisation=0.1, cpw=1.0, npw=1.0, use_regularisation_weight_scale=True)
            if sigma is not None:
                kw["regularisation_weight_sigma"] = sigma
            interp.setup_interpolator(**kw)
            out[f"{name}_cells"] = np.array(cells)
            out[f"{name}_sigma"] = np.array([np.nan if sigma is None else sigma])
            out[f"{name}_value"] = np.asarray(interp.data["value"], dtype=float)
            out[f"{name}_normal"] = np.asarray(interp.data["normal"], dtype=float)
            out[f"{name}_scale"] = np.asarray(interp.regularisation_scale, dtype=float)
            _families_to_arrays(interp, calls, f"{name}_", out)
            out[f"{name}_c_direct"] = _solve_direct(interp)
        finally:
            cls.add_constraints_to_least_squares = orig
    calls, (cls, orig) = _hook(li)
    try:
        name = "ws_p1"
        cells = (3, 4, 3)
        rng = np.random.default_rng(23)
        mesh = TetMesh(origin=np.zeros(3), nsteps_cells=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.P1Interpolator(mesh)
        vp = rng.uniform(0.02, 0.98, size=(30, 3))
        interp.set_value_constraints(np.column_stack([vp, _field(vp), np.ones(30)]))
        npnt = rng.uniform(0.05, 0.95, size=(8, 3))
        interp.set_normal_constraints(np.column_stack([npnt, _grad(npnt), np.ones(8)]))
        interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0, use_regularisation_weight_scale=True,
                                  regularisation_weight_sigma=0.2)
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_value"] = np.asarray(interp.data["value"], dtype=float)
        out[f"{name}_normal"] = np.asarray(interp.data["normal"], dtype=float)
        out[f"{name}_scale"] = np.asarray(interp.regularisation_scale, dtype=float)
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_c_direct"] = _solve_direct(interp)
    finally:
        cls.add_constraints_to_least_squares = orig


def p1_orthogonal_case(li, TetMesh, out):
    """P1 tangent constraints (DI:668-682) and gradient-orthogonal rows with a
    target (P1:248-296) after setup: rows weighted by the tetrahedron volume,
    one point outside the mesh."""
    calls, (cls, orig) = _hook(li)
    try:
        name = "p1_orth"
        cells = (4, 3, 3)
        rng = np.random.default_rng(24)
        mesh = TetMesh(origin=np.zeros(3), nsteps_cells=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
        interp = li.P1Interpolator(mesh)
        vp = rng.uniform(0.02, 0.98, size=(25, 3))
        interp.set_value_constraints(np.column_stack([vp, _field(vp), np.ones(25)]))
        tp = rng.uniform(0.02, 0.98, size=(10, 3))
        tp[0] = [1.5, 0.5, 0.5]
        tv = rng.normal(size=(10, 3))
        interp.set_tangent_constraints(np.column_stack([tp, tv, np.ones(10)]))
        interp.setup_interpolator(cgw=0.1, cpw=1.0, tpw=2.0)
        op = rng.uniform(0.02, 0.98, size=(6, 3))
        ov = rng.normal(size=(6, 3))
        out[f"{name}_orth_points"] = op
        out[f"{name}_orth_vectors"] = ov.copy()
        interp.add_gradient_orthogonal_constraints(op, ov, w=0.7, b=0.3, name="orth")
        out[f"{name}_cells"] = np.array(cells)
        out[f"{name}_value"] = np.asarray(interp.data["value"], dtype=float)
        out[f"{name}_tangent"] = np.asarray(interp.data["tangent"], dtype=float)
        _families_to_arrays(interp, calls, f"{name}_", out)
        out[f"{name}_c_direct"] = _solve_direct(interp)
    finally:
        cls.add_constraints_to_least_squares = orig


def main_weight_scale(root):
    li, StructuredGrid, TetMesh = _import_reference(root)
    out = {}
    weight_scale_cases(li, StructuredGrid, TetMesh, out)
    p1_orthogonal_case(li, TetMesh, out)
    path = os.path.join(HERE, "weight_scale_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


def admm_p1_case(li, TetMesh, out):
    """P1 with value inequalities and inequality pairs (P1:243-244: the
    default pair bounds [-inf, 1.0]) under ``solve_system('admm')`` with an
    exact inner solver."""
    name = "admm_p1"
    cells = (4, 4, 3)
    rng = np.random.default_rng(31)
    mesh = TetMesh(origin=np.zeros(3), nsteps_cells=np.array(cells), step_vector=1.0 / np.array(cells, dtype=float))
    interp = li.P1Interpolator(mesh)
    vp = rng.uniform(0.05, 0.95, size=(30, 3))
    val = np.column_stack([vp, _field(vp), np.ones(30)])
    npnt = rng.uniform(0.05, 0.95, size=(8, 3))
    nrm = np.column_stack([npnt, _grad(npnt), np.ones(8)])
    ip = rng.uniform(0.1, 0.9, size=(10, 3))
    f0 = _field(ip)
    lo = f0 + rng.uniform(0.05, 0.15, 10)
    ineq = np.column_stack([ip, lo, lo + 0.1, np.ones(10)])
    pp = rng.uniform(0.1, 0.9, size=(8, 3))
    pp[:4, 2] = rng.uniform(0.6, 0.9, 4)
    pp[4:, 2] = rng.uniform(0.1, 0.4, 4)
    pairs = np.column_stack([pp, np.r_[np.zeros(4), np.ones(4)], np.ones(8)])
    interp.set_value_constraints(val)
    interp.set_normal_constraints(nrm)
    interp.set_value_inequality_constraints(ineq)
    interp.set_inequality_pairs_constraints(pairs)
    interp.setup_interpolator(cgw=0.1, cpw=1.0, npw=1.0)
    Q, bounds = interp.build_inequality_matrix()
    Q = Q.tocoo()
    out[f"{name}_cells"] = np.array(cells)
    out[f"{name}_value"] = val
    out[f"{name}_normal"] = nrm
    out[f"{name}_ineq"] = ineq
    out[f"{name}_pairs"] = pairs
    out[f"{name}_Q_row"] = Q.row.astype(np.int64)
    out[f"{name}_Q_col"] = Q.col.astype(np.int64)
    out[f"{name}_Q_val"] = Q.data
    out[f"{name}_bounds"] = np.asarray(bounds, dtype=float)
    out[f"{name}_ineq_names"] = np.array(list(interp.ineq_constraints.keys()))
    ok = interp.solve_system("admm", solver_kwargs=dict(admm_weight=1.0, nmajor=60, linsys_solver=_exact_lsq,
                                                        return_history=True))
    assert ok
    hist = interp.solver_history
    out[f"{name}_c"] = np.array(interp.c)
    out[f"{name}_iterations"] = np.array(len(hist))
    for k in ("primal_norm", "dual_norm", "eps_pri", "eps_dual", "rho"):
        out[f"{name}_hist_{k}"] = np.array([h[k] for h in hist], dtype=float)


def main_admm(root):
    li, StructuredGrid, TetMesh = _import_reference(root)
    out = {}
    for name in ADMM_CASES:
        admm_case(li, StructuredGrid, name, out)
    admm_p1_case(li, TetMesh, out)
    path = os.path.join(HERE, "admm_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


def main_directional(root):
    li, StructuredGrid, TetMesh = _import_reference(root)
    out = {}
    fd_directional_case(li, StructuredGrid, "fd_dir", (7, 6, 8), seed=3, out=out)
    p1_directional_case(li, TetMesh, "p1_dir", (3, 4, 3), seed=4, out=out)
    fd_fold_case(li, StructuredGrid, "fd_fold", (8, 7, 9), seed=5, out=out)
    path = os.path.join(HERE, "directional_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


def main(root):
    li, StructuredGrid, TetMesh = _import_reference(root)
    out = {}
    fd_case(li, StructuredGrid, "fd_small", (8, 6, 12), 40, 12, 6, 4, 6, seed=0,
            setup_kwargs=dict(regularisation=0.1, cpw=1.0, npw=1.0, gpw=1.0, tpw=1.0, ipw=1.0), out=out)
    fd_case(li, StructuredGrid, "fd_cfg1_20", (20, 20, 20), 200, 50, 0, 0, 0, seed=0,
            setup_kwargs=dict(regularisation=0.1, cpw=1.0, npw=1.0), out=out)
    for cells in ((5, 5, 5), (3, 4, 2), (2, 5, 6)):
        reg_index_case(li, StructuredGrid, cells, out)
    p1_case(li, TetMesh, "p1_small", (4, 3, 5), 30, 8, seed=1,
            setup_kwargs=dict(cgw=0.1, cpw=1.0, npw=1.0), out=out)
    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes")


if __name__ == "__main__":
    # usage: make_golden.py <reference source root> [--directional | --configs | --faults]
    # (or the root in the LOOPSTRUCTURAL_REFERENCE environment variable)
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else os.environ.get("LOOPSTRUCTURAL_REFERENCE")
    if not root:
        sys.exit("make_golden.py: pass the LoopStructural source root (or set LOOPSTRUCTURAL_REFERENCE)")
    if "--directional" in sys.argv:
        main_directional(root)
    elif "--configs" in sys.argv:
        main_configs(root)
    elif "--faults" in sys.argv:
        main_faults(root)
    elif "--admm" in sys.argv:
        main_admm(root)
    elif "--weight-scale" in sys.argv:
        main_weight_scale(root)
    else:
        main(root)
