"""Drop-in interpolators: the reference's discrete-interpolator API
(setters, setup_interpolator, solve_system, evaluate_value/gradient,
get_last_solve_timing) backed by the sm_103a kernels.

Reference: packages/loop_interpolation/src/loop_interpolation/
  _geological_interpolator.py (GI)  setters :303-460, evaluate :723-742, clean :864-885
  _discrete_interpolator.py   (DI)  add_constraints_to_least_squares :316-389,
                                    solve_system :1221-1319, evaluate :1342-1379
  _finite_difference_interpolator.py (FD) setup_interpolator :132-224
  _solver_strategy.py (SS) solve_with_cg :48-72
"""
from __future__ import annotations

import logging
from time import perf_counter

import numpy as np

from . import _lib, admm, constraints, fd
from . import regularisation as regcfg

logger = logging.getLogger(__name__)

RIDGE_FACTOR = 1e-8


class ConstraintFamily:
    """One constraint family as the reference stores it after
    add_constraints_to_least_squares: normalised rows on the device."""

    def __init__(self, name, idc, a, b, w):
        self.name, self.idc, self.a, self.b, self.w = name, idc, a, b, w

    @property
    def n_rows(self):
        return int(self.idc.shape[0])

    def numpy(self):
        return {"idc": self.idc.cpu().numpy(), "A": self.a.cpu().numpy(), "B": self.b.cpu().numpy(),
                "w": self.w.cpu().numpy()}


class InequalityFamily:
    """One inequality family as the reference stores it
    (DI:467-507 add_inequality_constraints_to_matrix): raw rows over columns
    idc (m x k, device) with per-row bounds (m x 2: lower, upper)."""

    def __init__(self, idc, a, bounds):
        self.idc, self.a, self.bounds = idc, a, bounds

    @property
    def rows(self):
        return int(self.idc.shape[0])


def _row_weights(w, nrows):
    """Per-row weights: a Python number is broadcast; anything else must be an
    array of one weight per row (TypeError / ValueError otherwise, the
    reference's exceptions)."""
    if isinstance(w, (float, int)):
        return np.full(nrows, float(w))
    if not isinstance(w, np.ndarray):
        raise TypeError("w must be a numpy array")
    if w.shape[0] != nrows:
        raise ValueError("Weight array does not match number of constraints")
    return np.asarray(w, dtype=float)


def normalise_rows(A, B, idc, w=1.0, name="undefined"):
    """The row preparation of DI:316-389 add_constraints_to_least_squares on
    host arrays; returns (A, B, idc, w) as 2-D rows, or None when the family is
    dropped.

    * A and idc must have the same shape (else an error is logged, None).
    * A 3-D block (points x rows-per-point x columns) becomes point-major rows;
      an array w is then repeated once per row of a point, as the reference
      does (``np.tile``), so callers pass per-row weights that way.
    * A NaN anywhere in A, B or idc drops the family with a warning.
    * Every row with a non-zero L2 norm is divided by it, B with it.
    * w: see ``_row_weights``."""
    coef = np.array(A, dtype=float)
    cols = np.array(idc)
    if coef.shape != cols.shape:
        logger.error("Cannot add constraints: A and indexes have different shape : %s", name)
        return None
    rhs = np.array(B, dtype=float)
    if coef.ndim > 2:
        per_point = coef.shape[1]
        coef = coef.reshape(-1, coef.shape[-1])
        cols = cols.reshape(coef.shape)
        rhs = rhs.reshape(len(coef))
        if isinstance(w, np.ndarray):
            w = np.tile(w, per_point)
    if any(np.isnan(arr).any() for arr in (cols, coef, rhs)):
        logger.warning("Constraints contain nan not adding constraints: %s", name)
        return None
    norms = np.linalg.norm(coef, axis=1)
    scaled = norms > 0
    coef[scaled] /= norms[scaled, None]
    rhs[scaled] /= norms[scaled]
    return coef, rhs.reshape(-1), cols.astype(np.int64), _row_weights(w, len(coef))


class SetupReport(dict):
    """Row counts per constraint family (the reference returns a
    ConstraintDiagnosticsReport with the same information)."""


class _DiscreteInterpolatorBase:
    def __init__(self, support, data=None):
        self.support = support
        self.dimensions = 3
        self.bounding_box = None
        self.solver = "cg"
        self.apply_scaling_matrix = True
        self.add_ridge_regulatisation = True
        self.ridge_factor = RIDGE_FACTOR
        self.interpolation_weights = {}
        self.latest_solve_timing = {}
        self.constraints: dict[str, ConstraintFamily] = {}
        self.ineq_constraints: dict[str, InequalityFamily] = {}
        self.solver_history = None
        self._reg_scale = None
        self.family_order: list[str] = []
        self.up_to_date = False
        self._c = np.zeros(self.support.n_nodes)
        self._c_dev = None
        self._system = None
        self.clean()
        if data:
            for k, v in data.items():
                self.data[k] = np.array(v)

    # -- data (GI:303-460, GI:864-885) -------------------------------------
    def clean(self):
        self.data = {
            "gradient": np.zeros((0, 7)), "value": np.zeros((0, 5)), "normal": np.zeros((0, 7)),
            "tangent": np.zeros((0, 7)), "interface": np.zeros((0, 5)), "inequality": np.zeros((0, 6)),
            "inequality_pairs": np.zeros((0, 4)),
        }
        self.up_to_date = False

    def _project(self, points, has_vector=False):
        if self.bounding_box is None or points.shape[0] == 0:
            return points
        points = points.copy()
        points[:, :3] = self.bounding_box.project(points[:, :3])
        if has_vector:
            points[:, 3:6] = self.bounding_box.project_vectors(points[:, 3:6])
        return points

    def set_value_constraints(self, points):
        try:
            self.data["value"] = self._project(constraints.value_array(points)).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set value constraints: {e}") from e
        self.up_to_date = False

    def set_gradient_constraints(self, points):
        try:
            self.data["gradient"] = self._project(constraints.gradient_array(points), True).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set gradient constraints: {e}") from e
        self.up_to_date = False

    def set_normal_constraints(self, points):
        try:
            self.data["normal"] = self._project(constraints.gradient_array(points, is_normal=True), True).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set normal constraints: {e}") from e
        self.up_to_date = False

    def set_tangent_constraints(self, points):
        try:
            self.data["tangent"] = self._project(constraints.gradient_array(points, name="Tangent"), True).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set tangent constraints: {e}") from e
        self.up_to_date = False

    def set_interface_constraints(self, points):
        try:
            self.data["interface"] = self._project(constraints.value_array(points, name="Interface constraint")).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set interface constraints: {e}") from e
        self.up_to_date = False

    def set_value_inequality_constraints(self, points):
        """[x, y, z, lower, upper, (w)] (GI:464-493); lower < upper on every row."""
        try:
            self.data["inequality"] = self._project(constraints.inequality_array(points)).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set inequality value constraints: {e}") from e
        self.up_to_date = False

    def set_inequality_pairs_constraints(self, points):
        """[x, y, z, pair_id, (w)] (GI:495-522)."""
        try:
            self.data["inequality_pairs"] = self._project(constraints.inequality_pair_array(points)).copy()
        except constraints.ValidationError as e:
            raise constraints.ValidationError(f"Failed to set inequality pairs constraints: {e}") from e
        self.up_to_date = False

    def get_inequality_value_constraints(self):
        return self.data["inequality"]

    def get_inequality_pairs_constraints(self):
        return self.data["inequality_pairs"]

    def get_value_constraints(self):
        return self.data["value"]

    def get_gradient_constraints(self):
        return self.data["gradient"]

    def get_norm_constraints(self):
        return self.data["normal"]

    def get_tangent_constraints(self):
        return self.data["tangent"]

    def get_interface_constraints(self):
        return self.data["interface"]

    def set_interpolation_weights(self, weights):
        for k, v in weights.items():
            self.up_to_date = False
            self.interpolation_weights[k] = v

    @property
    def dof(self):
        return int(self.support.n_nodes)

    @property
    def n_elements(self):
        return self.support.n_elements

    # -- solution vector ------------------------------------------------------
    @property
    def c(self):
        return self._c

    @c.setter
    def c(self, value):
        self._c = np.asarray(value, dtype=float)
        self._c_dev = None

    def _c_device(self):
        import torch

        if self._c_dev is None:
            self._c_dev = torch.from_numpy(np.ascontiguousarray(self._c)).to(_lib.device())
        return self._c_dev

    def get_last_solve_timing(self) -> dict:
        return dict(self.latest_solve_timing)

    # -- least squares container (DI:316-389 semantics on device rows) ------
    @staticmethod
    def _unique_name(name, taken):
        """DI:374-379 name de-duplication (``name_k``)."""
        base = name
        while name in taken:
            count = 0
            if "_" in name:
                count = int(name.split("_")[1]) + 1
            name = base + f"_{count}"
        return name

    def _add_family(self, name, idc, a, b, w):
        import torch

        if idc.shape[0] == 0:
            return
        if bool(torch.isnan(a).any()) or bool(torch.isnan(b).any()):
            logger.warning("Constraints contain nan not adding constraints: %s", name)
            return
        name = self._unique_name(name, self._taken_names())
        self.constraints[name] = ConstraintFamily(name, idc, a, b, w)
        self.family_order.append(name)

    def _taken_names(self):
        taken = set(self.constraints)
        taken |= set(getattr(self, "regularisation_families", {}))
        taken |= set(getattr(self, "directional_families", {}))
        return taken

    def add_constraints_to_least_squares(self, A, B, idc, w=1.0, name="undefined"):
        """Adds a constraint family from host arrays (DI:316-389): rows of
        coefficients A over columns idc with targets B and weights w, row
        normalised; the family joins the next solve."""
        import torch

        out = normalise_rows(A, B, idc, w, name)
        if out is None:
            return
        A, B, idc, w = out
        if idc.size and (idc.min() < 0 or idc.max() >= self.dof):
            raise ValueError("constraint column index out of range")
        dev = _lib.device()
        self._add_family(name, torch.from_numpy(idc).to(dev), torch.from_numpy(A).to(dev),
                         torch.from_numpy(B).to(dev), torch.from_numpy(w).to(dev))
        self.up_to_date = False

    def add_inequality_constraints_to_matrix(self, A, bounds, idc, name="undefined"):
        """Inequality rows lower <= A c <= upper over columns idc
        (DI:467-507); bounds is n x 2 (lower, upper) or n x 3 (the third
        column is not used).  Raises ValueError on the reference's shape and
        range checks; a family of the same name is replaced."""
        import torch

        A = np.asarray(A, dtype=float)
        idc = np.asarray(idc, dtype=int)
        bounds = np.asarray(bounds, dtype=float)
        if A.ndim != 2 or idc.ndim != 2:
            raise ValueError("A and idc must be 2D arrays")
        if A.shape != idc.shape:
            raise ValueError("A and idc must have the same shape")
        if bounds.ndim != 2 or bounds.shape[0] != A.shape[0] or bounds.shape[1] not in (2, 3):
            raise ValueError("bounds must have shape (n_rows, 2) or (n_rows, 3)")
        if np.any(idc < 0) or np.any(idc >= self.dof):
            raise ValueError("Inequality constraint indices are out of range")
        dev = _lib.device()
        self._add_inequality_family(name, torch.from_numpy(idc.astype(np.int64)).to(dev), torch.from_numpy(A).to(dev),
                                    torch.from_numpy(np.ascontiguousarray(bounds[:, :2])).to(dev))

    def _add_inequality_family(self, name, idc, a, bounds):
        self.ineq_constraints[name] = InequalityFamily(idc.contiguous(), a.contiguous(), bounds.contiguous())
        self.up_to_date = False

    def add_inequality_feature(self, feature, lower=True, mask=None):
        """f >= feature (lower) or f <= feature at the support's nodes where
        the feature is not NaN and the mask holds (DI:595-632)."""
        import torch

        value = np.asarray(feature(self.support.nodes), dtype=float)
        if mask is None:
            mask = np.ones(value.shape[0], dtype=bool)
        lo = np.full(value.shape[0], -np.inf)
        hi = np.full(value.shape[0], np.inf)
        mask = np.logical_and(mask, ~np.isnan(value))
        if lower:
            lo[mask] = value[mask]
        else:
            hi[mask] = value[mask]
        dev = _lib.device()
        n = self.dof
        self._add_inequality_family("inequality_feature", torch.arange(n, dtype=torch.int64, device=dev)[:, None],
                                    torch.ones((n, 1), dtype=torch.float64, device=dev),
                                    torch.from_numpy(np.column_stack([lo, hi])).to(dev))

    def build_inequality_matrix(self):
        """(Q, bounds) of every inequality family, stacked in insertion order
        (DI:874-884): Q a CSR matrix over the dof, bounds n x 2."""
        from scipy import sparse

        mats, bounds = [], []
        for f in self.ineq_constraints.values():
            idc, a = f.idc.cpu().numpy(), f.a.cpu().numpy()
            n, k = idc.shape
            keep = idc.reshape(-1) >= 0
            rows = np.repeat(np.arange(n), k)[keep]
            mats.append(sparse.coo_matrix((a.reshape(-1)[keep], (rows, idc.reshape(-1)[keep])),
                                          shape=(n, self.dof)).tocsr())
            bounds.append(f.bounds.cpu().numpy())
        if not mats:
            return sparse.csr_matrix((0, self.dof), dtype=float), np.zeros((0, 3))
        return sparse.vstack(mats).tocsr(), np.vstack(bounds)

    def clear_constraints(self):
        """Drops every constraint family (DI:297-304)."""
        self.constraints = {}
        self.ineq_constraints = {}
        if hasattr(self, "regularisation_families"):
            self.regularisation_families = {}
        if hasattr(self, "_reset_directional"):
            self._reset_directional()
        self.family_order = []
        self._release_system()

    def _family_rows(self, name):
        """(idc, A, B, w) host arrays of any family, in the reference's form."""
        if name in self.constraints:
            return self.constraints[name].numpy()
        if name in getattr(self, "directional_families", {}):
            return self.directional_rows(name)
        return self.regularisation_rows(name)

    def calculate_residual_for_constraints(self):
        """A c - B of every family (DI:453-465), by family name."""
        c = np.asarray(self.c, dtype=float)
        out = {}
        for name in self.family_order:
            f = self._family_rows(name)
            idc = f["idc"]
            vals = np.where(idc >= 0, c[np.clip(idc, 0, None)], 0.0)
            out[name] = np.einsum("ij,ij->i", f["A"], vals) - f["B"].reshape(-1)
        return out

    def build_matrix(self):
        """The explicit weighted system (DI:684-755): every family's rows times
        its weights, stacked in the order the families were added, as a CSR
        matrix and right-hand side (no ridge; the solve adds it)."""
        from scipy import sparse

        mats, bs = [], []
        for name in self.family_order:
            f = self._family_rows(name)
            n, k = f["A"].shape
            if n == 0:
                continue
            keep = f["idc"].reshape(-1) >= 0
            rows = np.repeat(np.arange(n), k)[keep]
            m = sparse.coo_matrix((f["A"].reshape(-1)[keep], (rows, f["idc"].reshape(-1)[keep])),
                                  shape=(n, self.dof)).tocsr()
            mats.append(m.multiply(f["w"][:, None]).tocsr())
            bs.append(f["B"].reshape(-1) * f["w"])
        if not mats:
            return sparse.csr_matrix((0, self.dof)), np.zeros(0)
        return sparse.vstack(mats).tocsr(), np.hstack(bs)

    # -- regularisation weight scale (FD:66-90, 416-444; P1:52-69) -------------
    def _regularisation_scale(self):
        """Per-node scale of use_regularisation_weight_scale: 1, plus
        1 + 10 exp(-d^2 / 2 sigma^2) with d the distance to the nearest normal
        constraint inside the support (GPU); sigma defaults to 10 x the node
        count along x."""
        import torch

        scale = torch.ones(int(self.support.n_nodes), dtype=torch.float64, device=_lib.device())
        points = self.get_norm_constraints()
        if points.shape[0] == 0:
            return scale
        inside = np.asarray(self.support.inside(points[:, :3]), dtype=bool)
        if inside.any():
            sigma = self.regularisation_weight_sigma
            if sigma is None:
                sigma = float(self.support.nsteps[0]) * 10
            fd.weight_scale(self.support, points[inside, :3], 10.0, float(sigma), scale)
        return scale

    def regularisation_scale_array(self):
        """The per-node regularisation weight scale as a host array (ones
        without use_regularisation_weight_scale), as the reference's
        ``regularisation_scale``."""
        if self._reg_scale is None:
            return np.ones(int(self.support.n_nodes))
        return self._reg_scale.cpu().numpy()

    # -- directional regularisation (DI:395-451) ----------------------------
    def resolve_regularisation_config(self, regularisation=None, directional_regularisation=None):
        return regcfg.coerce_regularisation_config(regularisation=regularisation,
                                                   directional_regularisation=directional_regularisation)

    def get_regularisation_sample_points(self) -> np.ndarray:
        raise NotImplementedError(f"{self.__class__.__name__} does not define regularisation sample points")

    def _regularisation_sample_shape(self):
        return tuple(np.asarray(self.get_regularisation_sample_points()).shape)

    def _add_directional_regularisation(self, weight, vectors, name="directional regularisation"):
        raise NotImplementedError(f"{self.__class__.__name__} does not implement directional regularisation")

    def add_directional_regularisation(self, directional_regularisation):
        """Evaluates each term's direction at the regularisation sample points
        (when it is a callable) and adds its rows; terms of weight 0 are
        skipped, wrongly shaped directions warn and are skipped (DI:422-451)."""
        terms = self.resolve_regularisation_config(directional_regularisation=directional_regularisation).directional
        if len(terms) == 0:
            return terms
        sample = None
        expected = self._regularisation_sample_shape()
        for term in terms:
            if term.weight == 0:
                continue
            if callable(term.direction):
                if sample is None:
                    sample = np.asarray(self.get_regularisation_sample_points(), dtype=float)
                vectors = term.direction(sample)
            else:
                vectors = term.direction
            vectors = np.asarray(vectors, dtype=float)
            if vectors.shape != expected:
                logger.warning("%s: directional regularisation vectors must have shape %s, got %s. Skipping.",
                               term.name, expected, vectors.shape)
                continue
            self._add_directional_regularisation(term.weight, vectors, name=term.name)
        return terms

    def reset(self):
        self.constraints = {}
        self.family_order = []
        self._release_system()

    def _release_system(self):
        if self._system is not None:
            self._system.close()
            self._system = None

    def update(self) -> bool:
        if not self.up_to_date:
            self.setup_interpolator()
            self.up_to_date = self.solve_system(self.solver)
        return bool(self.up_to_date)

    # -- solve (DI:1221-1319, SS:48-72) ---------------------------------------
    def _solve_with_callable(self, solver):
        """A custom solver on the explicit system (DI:1283-1313 with
        SS:32-45): build_matrix, the ridge rows and the column scaling S of
        the reference's preprocessing, c = S solver(A S, b)."""
        from scipy import sparse

        started = perf_counter()
        A, b = self.build_matrix()
        t0 = perf_counter()
        if self.add_ridge_regulatisation:
            A = sparse.vstack([A, sparse.eye(A.shape[1]) * self.ridge_factor]).tocsr()
            b = np.hstack([b, np.zeros(A.shape[1])])
        S = None
        if self.apply_scaling_matrix:
            norms = sparse.linalg.norm(A, axis=0)
            scale = np.ones(A.shape[1])
            scale[norms > 0] = 1.0 / norms[norms > 0]
            S = sparse.diags(scale)
            A = A @ S
        t1 = perf_counter()
        logger.warning("Using custom solver")
        c = np.asarray(solver(A.tocsr(), b))
        t2 = perf_counter()
        self._c = np.asarray(S @ c if S is not None else c, dtype=float)
        self._c_dev = None
        self.up_to_date = True
        self.latest_solve_timing = {"solver": "callable", "backend": "host", "assembly_seconds": t0 - started,
                                    "preprocess_seconds": t1 - t0, "solve_seconds": t2 - t1,
                                    "matrix_rows": int(A.shape[0]), "matrix_cols": int(A.shape[1]),
                                    "matrix_nnz": int(A.nnz), "total_seconds": perf_counter() - started,
                                    "up_to_date": True}
        return True

    def _solver_options(self, solver, tol, solver_kwargs):
        if solver not in ("cg", "lsmr", "admm", None):
            logger.warning("Unknown solver %s using cg. Available solvers are cg, lsmr, admm", solver)
            solver = "cg"
        solver = "cg" if solver is None else solver
        if solver == "admm":
            return solver, admm.admm_options(solver_kwargs)
        kw = dict(solver_kwargs or {})
        kw.pop("backend", None)
        if solver == "lsmr":  # same least-squares solution; lsmr's btol maps to the relative tolerance
            if "btol" in kw:
                kw["rtol"] = kw.pop("btol")
            elif tol is not None:
                kw["rtol"] = tol
            kw.pop("atol", None)
            kw.setdefault("atol", 0.0)
            tol = None
        elif ("atol" not in kw or "rtol" not in kw) and tol is not None:
            kw["atol"] = tol
        opts = {
            "atol": float(kw.pop("atol", 0.0)),
            "rtol": float(kw.pop("rtol", 1e-5)),
            "maxiter": kw.pop("maxiter", None),
            "precision": kw.pop("precision", "mixed"),
            "reliable_delta": float(kw.pop("reliable_delta", 0.1)),
            "check_every": int(kw.pop("check_every", 64)),
            "preconditioner": kw.pop("preconditioner", "mg"),
        }
        x0 = kw.pop("x0", None)
        if callable(x0):
            x0 = x0(self.support)
        opts["x0"] = x0
        for k in list(kw):
            logger.info("solver kwarg %s ignored by the GPU CG", k)
        return solver, opts

    def _build_system(self):
        raise NotImplementedError

    def solve_system(self, solver=None, tol=None, solver_kwargs=None) -> bool:
        import torch

        if callable(solver):
            return self._solve_with_callable(solver)
        solve_started = perf_counter()
        self._c = np.full(self.support.n_nodes, np.nan)
        self._c_dev = None
        solver, opts = self._solver_options(solver, tol, solver_kwargs)
        timing = {"solver": solver, "backend": "gb300"}
        self.solver_history = None
        if solver == "admm":
            return self._solve_admm(opts, timing, solve_started)
        t0 = perf_counter()
        self._release_system()
        self._system = self._build_system()
        torch.cuda.synchronize()
        timing["assembly_seconds"] = perf_counter() - t0
        timing["matrix_rows"] = int(self._matrix_rows())
        timing["matrix_cols"] = int(self.dof)
        timing["matrix_nnz"] = int(self._matrix_nnz())
        timing["preprocess_seconds"] = 0.0
        x0 = opts.pop("x0")
        if x0 is not None:
            x0 = torch.as_tensor(np.asarray(x0, dtype=float))
        t1 = perf_counter()
        x, stats = self._system.solve(x=x0, **opts)
        timing["solve_seconds"] = perf_counter() - t1
        status = stats["status"]
        if status == _lib.LS_NOT_CONVERGED:
            logger.warning("CG reached iteration limit (%s) and did not converge; using last iteration",
                           stats["iterations"])
        elif status in (_lib.LS_NAN, _lib.LS_BREAKDOWN):
            logger.warning("CG stopped early (status %d: %s)", status, "nan" if status == _lib.LS_NAN else "breakdown")
        self._c_dev = x
        self._c = fd.to_host(x)
        timing.update({"iterations": int(stats["iterations"]), "reliable_updates": int(stats["reliable_updates"]),
                       "residual": stats["residual"], "threshold": stats["threshold"],
                       "device_ms": stats["device_ms"], "precision": opts["precision"], "status": int(status),
                       "preconditioner": stats["preconditioner"]})
        self.up_to_date = True
        timing["total_seconds"] = perf_counter() - solve_started
        timing["up_to_date"] = True
        self.latest_solve_timing = timing
        return True

    def _solve_admm(self, opts, timing, solve_started):
        """solver='admm' (DI:1171-1219, loopsolver/admm_solver.py): see
        admm.solve_admm."""
        import torch

        o, inner = opts
        self._release_system()
        t0 = perf_counter()
        ok = admm.solve_admm(self, o, inner, timing)
        torch.cuda.synchronize()
        timing["solve_seconds"] = perf_counter() - t0
        timing["matrix_rows"] = int(self._matrix_rows())
        timing["matrix_cols"] = int(self.dof)
        self.up_to_date = bool(ok)
        timing["total_seconds"] = perf_counter() - solve_started
        timing["up_to_date"] = bool(ok)
        self.latest_solve_timing = timing
        return bool(ok)

    # -- evaluation (GI:723-742, DI:1342-1379) ---------------------------------
    def evaluate_value(self, locations):
        loc = np.asarray(locations, dtype=float)
        if self.bounding_box is not None:
            loc = self.bounding_box.project(loc)
        return self._evaluate_value_local(loc)

    def evaluate_gradient(self, locations):
        loc = np.asarray(locations, dtype=float)
        if self.bounding_box is not None:
            loc = self.bounding_box.project(loc)
        g = self._evaluate_gradient_local(loc)
        if self.bounding_box is not None:
            g = self.bounding_box.reproject_vectors(g)
        return g

    def evaluate_value_and_gradient(self, locations):
        """``(evaluate_value(locations), evaluate_gradient(locations))`` from
        one upload of the points and one kernel launch (no reference
        counterpart: the reference evaluates the two separately)."""
        loc = np.asarray(locations, dtype=float)
        if self.bounding_box is not None:
            loc = self.bounding_box.project(loc)
        self.update()
        if loc.shape[0] == 0:
            return np.zeros(0), np.zeros((0, 3))
        v, g = self._eval_points(loc)
        if self.bounding_box is not None:
            g = self.bounding_box.reproject_vectors(g)
        return v, g


class FiniteDifferenceInterpolator(_DiscreteInterpolatorBase):
    """FD interpolator on a StructuredGrid (FD:91-224)."""

    REG_WEIGHT_KEYS = ("dxy", "dyz", "dxz", "dxx", "dyy", "dzz")

    def __init__(self, grid, data=None):
        super().__init__(grid, data)
        self.set_interpolation_weights({  # FD:102-119
            "dxy": 1.0, "dyz": 1.0, "dxz": 1.0, "dxx": 1.0, "dyy": 1.0, "dzz": 1.0,
            "dx": 1.0, "dy": 1.0, "dz": 1.0,
            "cpw": 1.0, "gpw": 1.0, "npw": 10.0, "tpw": 1.0, "ipw": 1.0,
        })
        self.interface_pair_mode = "auto"
        self.interface_pair_threshold = 200
        self.interface_pair_fallback = "star"
        self.use_regularisation_weight_scale = False
        self.regularisation_weight_sigma = None
        self.regularisation_families = {}
        self._reset_directional()

    def _reset_directional(self):
        # directional families: name -> (rows, term index, family); the terms'
        # (weight, direction); the summed device weights (6 x dof) of the operator
        self.directional_families = {}
        self._dir_terms = []
        self._dir_omega = None
        # use_regularisation_weight_scale: the per-node scale (device), and
        # whether the interior families went to the weight planes
        self._reg_scale = None
        self._scaled_interior = False

    def _omega(self):
        import torch

        if self._dir_omega is None:
            self._dir_omega = torch.zeros((len(_lib.DIRECTIONAL_FAMILIES), int(self.support.n_nodes)),
                                          dtype=torch.float64, device=_lib.device())
        return self._dir_omega

    def reset(self):
        super().reset()
        self.regularisation_families = {}
        self._reset_directional()

    def setup_interpolator(self, **kwargs) -> SetupReport:
        self.reset()
        cfg = self.resolve_regularisation_config(regularisation=kwargs.get("regularisation", None),
                                                 directional_regularisation=kwargs.get("directional_regularisation",
                                                                                       None))
        if cfg.isotropic is not None:
            for k in self.REG_WEIGHT_KEYS:
                self.interpolation_weights[k] = cfg.isotropic
        for k, v in kwargs.items():
            self.up_to_date = False
            if k in ("regularisation", "directional_regularisation"):
                continue
            self.interpolation_weights[k] = v
        self.use_regularisation_weight_scale = bool(kwargs.get("use_regularisation_weight_scale", False))
        self.regularisation_weight_sigma = kwargs.get("regularisation_weight_sigma", None)
        self.interface_pair_mode = kwargs.get("interface_pair_mode", self.interface_pair_mode)
        self.interface_pair_threshold = int(kwargs.get("interface_pair_threshold", self.interface_pair_threshold))
        self.interface_pair_fallback = kwargs.get("interface_pair_fallback", self.interface_pair_fallback)
        w = self.interpolation_weights
        t0 = perf_counter()
        self._add_point_rows(_lib.ROWS_NORM, self.get_norm_constraints(), w["npw"], ["norm_0", "norm_1", "norm_2"])
        if self.use_regularisation_weight_scale:
            self._reg_scale = self._regularisation_scale()
        self._add_point_rows(_lib.ROWS_GRADIENT, self.get_gradient_constraints(), w["gpw"], ["gradient", "gradient"])
        self._add_point_rows(_lib.ROWS_VALUE, self.get_value_constraints(), w["cpw"], ["value"])
        self._add_point_rows(_lib.ROWS_TANGENT, self.get_tangent_constraints(), w["tpw"], ["gradient orthogonal"])
        self._add_interface_rows(w["ipw"])
        self.add_value_inequality_constraints()  # FD:214-219
        self.add_inequality_pairs_constraints(pairs=kwargs.get("inequality_pairs", None),
                                              upper_bound=kwargs.get("inequality_pair_upper_bound",
                                                                     np.finfo(float).eps),
                                              lower_bound=kwargs.get("inequality_pair_lower_bound", -np.inf))
        self._add_regularisation_families(interior=True, borders=False)
        self.add_directional_regularisation(cfg.directional)  # FD:222, between interior and border families
        self._add_regularisation_families(interior=False, borders=True)
        self.setup_seconds = perf_counter() - t0
        self.up_to_date = False
        report = SetupReport({name: f.n_rows for name, f in self.constraints.items()})
        for name, (rows, _w) in self.regularisation_families.items():
            report[name] = rows
        for name, (rows, _t, _f) in self.directional_families.items():
            report[name] = rows
        for name, f in self.ineq_constraints.items():
            report[name] = f.rows
        return report

    # -- directional regularisation (FD:1207-1348) ----------------------------
    def get_regularisation_sample_points(self) -> np.ndarray:
        return self.support.nodes

    def _regularisation_sample_shape(self):
        return (int(self.support.n_nodes), 3)

    def _add_directional_regularisation(self, weight, vectors, name="directional regularisation"):
        self.minimise_directional_gradient_change(weight, vectors, name=name)

    def minimise_directional_gradient_change(self, w, vector, name="directional regularisation"):
        """Directional second-derivative regularisation: the six interior
        families again with row weight w * c_f(v) (c = vx², vy², vz², 2vxvy,
        2vxvz, 2vyvz) at each interior node, rows of zero weight dropped.  The
        rows stay matrix-free: their weights are summed per node and family
        on the device (ls_fd_directional_weights) and the operator applies
        sum_f D_f^T W_f D_f."""
        import torch

        n = int(self.support.n_nodes)
        if vector is None or np.ndim(vector) != 2 or np.shape(vector) != (n, 3):
            logger.warning("%s: vector must have shape (%d, 3), got %s.  Skipping.", name, n,
                           None if vector is None else np.shape(vector))
            return
        vector = np.asarray(vector, dtype=float)
        counts = fd.directional_weights(self.support, vector, float(w), self._omega())
        self._dir_terms.append((float(w), vector))
        taken = set(self.constraints) | set(self.regularisation_families) | set(self.directional_families)
        for f, op in enumerate(_lib.DIRECTIONAL_FAMILIES):
            if counts[f] > 0:
                fam = self._unique_name(f"{name}_{op}", taken)
                taken.add(fam)
                self.directional_families[fam] = (int(counts[f]), len(self._dir_terms) - 1, op)
                self.family_order.append(fam)
        self.up_to_date = False

    def add_gradient_orthogonal_constraints(self, points, vectors, w=1.0, b=0, name="gradient orthogonal"):
        """Rows grad(f) . v / |v| = b at the points (FD:478-539), normalised;
        points outside the grid are dropped."""
        points = np.asarray(points, dtype=float)
        if points.shape[0] == 0:
            return
        vectors = np.asarray(vectors, dtype=float)
        arr = np.empty((points.shape[0], 7))
        arr[:, :3] = points[:, :3]
        arr[:, 3:6] = vectors[:, :3]
        arr[:, 6] = b
        n, fams, _nan = fd.point_rows(self.support, _lib.ROWS_ORTHOGONAL, arr, float(w))
        if n <= 0:
            logger.warning("%d gradient constraints not added: outside of model bounding box", points.shape[0])
            return
        idc, a, bb, ww = fams[0]
        self._add_family(name, idc, a, bb, ww)
        self.up_to_date = False

    def directional_rows(self, name):
        """Explicit (idc, A, B, w) of a directional family as the reference
        stores it (parity inspection): the interior family's rows with
        w * c_f(v) at the row centre, zero-weight rows dropped."""
        _rows, term, op = self.directional_families[name]
        w, vec = self._dir_terms[term]
        idc = fd.reg_rows(self.support, op).cpu().numpy()
        nx, ny, nz = (int(v) for v in self.support.nsteps)
        i, j, k = np.meshgrid(np.arange(1, nx - 1), np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
        centre = (i + nx * (j + ny * k)).transpose(2, 1, 0).ravel()  # ascending node index
        vx, vy, vz = vec[centre, 0], vec[centre, 1], vec[centre, 2]
        comp = {"dxx": vx**2, "dyy": vy**2, "dzz": vz**2, "dxy": 2.0 * vx * vy, "dxz": 2.0 * vx * vz,
                "dyz": 2.0 * vy * vz}[op]
        row_w = w * comp
        keep = np.abs(row_w) > 0.0
        vals = fd.REG_TAP_VALUES[op]
        return {"idc": idc[keep], "A": np.tile(vals, (int(keep.sum()), 1)), "B": np.zeros(int(keep.sum())),
                "w": row_w[keep]}

    def _add_point_rows(self, kind, points, weight, names):
        if points.shape[0] == 0:
            return
        n, fams, _nan = fd.point_rows(self.support, kind, points, weight)
        if n <= 0:
            logger.warning("%d constraints not added: outside of model bounding box", points.shape[0])
            return
        for name, (idc, a, b, w) in zip(names, fams):
            self._add_family(name, idc, a, b, w)

    def _interface_pairs(self, n):
        if n < 2:
            return np.zeros((0, 2), dtype=int)
        mode = str(self.interface_pair_mode).lower()
        threshold = max(2, int(self.interface_pair_threshold))
        fallback = str(self.interface_pair_fallback).lower()
        if fallback not in ("star", "chain"):
            fallback = "star"
        if mode == "auto":
            mode = fallback if n > threshold else "all"
        if mode == "all":
            ii, jj = np.triu_indices(n, k=1)
            return np.column_stack([ii, jj]).astype(int)
        if mode == "star":
            return np.column_stack([np.zeros(n - 1, dtype=int), np.arange(1, n, dtype=int)])
        if mode == "chain":
            return np.column_stack([np.arange(0, n - 1, dtype=int), np.arange(1, n, dtype=int)])
        raise ValueError(f"Unknown interface_pair_mode '{self.interface_pair_mode}'. Use one of: auto, all, star, chain")

    def _add_interface_rows(self, weight):  # FD:297-340
        points = self.get_interface_constraints()
        if points.shape[0] <= 1:
            return
        inside = self.support.inside(points[:, :3])
        pin = points[inside]
        ids = points[np.logical_and(~np.isnan(points[:, 3]), inside), 3]
        for uid in np.unique(ids):
            sel = np.nonzero(pin[:, 3] == uid)[0]
            pairs = self._interface_pairs(sel.shape[0])
            if pairs.shape[0] == 0:
                continue
            idc, a, b, w = fd.pair_rows(self.support, pin, sel[pairs], weight)
            self._add_family(f"interface_{uid}", idc, a, b, w)

    def _add_regularisation_families(self, interior=True, borders=True):
        """Matrix-free: record (rows, weight) per family in the reference order
        (G:489-510 interior families, FD:1052-1144 borders)."""
        w = self.interpolation_weights
        scale = self._reg_scale
        if interior:
            self.regularisation_families = {}
            rw = {"dxy": w["dxy"] / 4, "dyz": w["dyz"] / 4, "dxz": w["dxz"] / 4, "dxx": w["dxx"], "dyy": w["dyy"],
                  "dzz": w["dzz"]}
            for name, weight in rw.items():
                rows, _ = fd.reg_shape(self.support, name)
                if rows > 0:
                    self.regularisation_families[name] = (rows, float(weight))
                    self.family_order.append(name)
            if scale is not None and self.regularisation_families:
                # rows of weight scale(centre) * w: the directional weight planes
                fd.scaled_weights(self.support, scale,
                                  [rw[f] if f in self.regularisation_families else 0.0
                                   for f in _lib.DIRECTIONAL_FAMILIES], self._omega())
                self._scaled_interior = True
        if borders:
            for name, key in (("dx_lower", "dx"), ("dx_upper", "dx"), ("dy_lower", "dy"), ("dy_upper", "dy"),
                              ("dz_lower", "dz"), ("dz_upper", "dz")):
                rows, _ = fd.reg_shape(self.support, name)
                if w[key] != 0 and rows > 0:
                    if scale is None:
                        self.regularisation_families[name] = (rows, float(w[key]))
                        self.family_order.append(name)
                    else:
                        # per-row weights scale(centre) * w: explicit data rows
                        import torch

                        idc = fd.reg_rows(self.support, name)
                        dev = idc.device
                        a = torch.from_numpy(np.tile(fd.REG_TAP_VALUES[name], (rows, 1))).to(dev)
                        self._add_family(name, idc, a, torch.zeros(rows, dtype=torch.float64, device=dev),
                                         (scale[idc[:, 1]] * float(w[key])).contiguous())

    def regularisation_rows(self, name):
        """Explicit (idc, A, B, w) of a matrix-free family, as the reference's
        explicit path would store it (parity inspection)."""
        rows, weight = self.regularisation_families[name]
        idc = fd.reg_rows(self.support, name).cpu().numpy()
        vals = fd.REG_TAP_VALUES[name]
        w = np.full(rows, weight)
        if self._scaled_interior:  # interior rows are centred on the interior nodes, ascending
            nx, ny, nz = (int(v) for v in self.support.nsteps)
            i, j, k = np.meshgrid(np.arange(1, nx - 1), np.arange(1, ny - 1), np.arange(1, nz - 1), indexing="ij")
            centre = (i + nx * (j + ny * k)).transpose(2, 1, 0).ravel()
            w = self.regularisation_scale_array()[centre] * weight
        return {"idc": idc, "A": np.tile(vals, (rows, 1)), "B": np.zeros(rows), "w": w}

    def _reg_weights(self):
        fam = self.regularisation_families
        out = {}
        for k in ("dxx", "dyy", "dzz", "dxy", "dyz", "dxz"):
            # scaled interior families live in the weight planes instead
            out[k] = fam[k][1] if (k in fam and not self._scaled_interior) else 0.0
        for k in ("dx", "dy", "dz"):
            out[k] = fam[k + "_lower"][1] if (k + "_lower") in fam else 0.0
        return out

    def _data_rows(self):
        return [(f.idc, f.a, f.b, f.w) for f in self.constraints.values()]

    def _make_system(self, rows):
        ridge = self.ridge_factor if self.add_ridge_regulatisation else 0.0
        omega = self._dir_omega if (self.directional_families or self._scaled_interior) else None
        return fd.FdSystem(self.support, self._reg_weights(), rows, ridge, directional=omega)

    def _build_system(self):
        return self._make_system(self._data_rows())

    # -- inequality rows (DI:509-630) -----------------------------------------
    def _trilinear_rows(self, points):
        """(idc, raw trilinear weights) of the points inside the grid, in
        order (device), and the host mask of those points."""
        import torch

        inside = np.asarray(self.support.inside(points[:, :3]), dtype=bool)
        if not inside.any():
            return None, None, inside
        pts = np.ascontiguousarray(np.column_stack([points[:, :3], np.zeros(points.shape[0]),
                                                    np.ones(points.shape[0])]))
        n, fams, _nan = fd.point_rows(self.support, _lib.ROWS_VALUE, pts, 1.0)
        if n != int(inside.sum()):
            raise RuntimeError("inside test of the row kernel and the support disagree")
        idc, a = fams[0][0], fams[0][1]
        # the rows come normalised (a / |a|); the trilinear weights sum to 1
        a = a / a.sum(dim=1, keepdim=True)
        return idc, a, inside

    def add_value_inequality_constraints(self, w=1.0):
        """lower <= f(x) <= upper at the inequality points inside the grid
        (DI:509-518); w is not used, as in the reference."""
        import torch

        points = self.get_inequality_value_constraints()
        if points.shape[0] == 0:
            return
        idc, a, inside = self._trilinear_rows(points)
        if idc is None:
            return
        bounds = torch.from_numpy(np.ascontiguousarray(points[inside, 3:5])).to(_lib.device())
        self._add_inequality_family("inequality_value", idc, a, bounds)

    def add_inequality_pairs_constraints(self, w=1.0, upper_bound=1.0, lower_bound=-np.inf, pairs=None):
        """lower_bound <= f(p) - f(q) <= upper_bound for every point p of the
        group pair[0] and q of pair[1] (inside points only); without
        ``pairs``, every pair of distinct group ids (i < j) (DI:520-593)."""
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
            upper = points[ids == pair[0]]
            lower = points[ids == pair[1]]
            in_u = np.asarray(self.support.inside(upper[:, :3]), dtype=bool)
            in_l = np.asarray(self.support.inside(lower[:, :3]), dtype=bool)
            if (~in_u).sum() > 0:
                logger.warning(f"Upper points not in mesh {upper[~in_u]}")
            if (~in_l).sum() > 0:
                logger.warning(f"Lower points not in mesh {lower[~in_l]}")
            nu, nl = int(in_u.sum()), int(in_l.sum())
            if nu == 0 or nl == 0:
                continue
            both = np.ascontiguousarray(np.vstack([upper[in_u, :3], lower[in_l, :3]]))
            # rows ordered as the reference's meshgrid: upper index fastest
            iu, il = np.meshgrid(np.arange(nu), np.arange(nl))
            pr = np.ascontiguousarray(np.column_stack([iu.ravel(), nu + il.ravel()]).astype(np.int64))
            idc, a, _b, _w = fd.pair_rows(self.support, both, pr, 1.0)
            a = a / a[:, :8].sum(dim=1, keepdim=True)
            bounds = torch.empty((pr.shape[0], 2), dtype=torch.float64, device=dev)
            bounds[:, 0] = float(lower_bound)
            bounds[:, 1] = float(upper_bound)
            self._add_inequality_family(f"inequality_pairs_{pair[0]}_{pair[1]}", idc, a, bounds)

    def _matrix_rows(self):
        return (sum(f.n_rows for f in self.constraints.values()) + sum(r for r, _ in self.regularisation_families.values())
                + sum(r for r, _t, _f in self.directional_families.values()))

    def _matrix_nnz(self):
        nnz = sum(f.n_rows * f.idc.shape[1] for f in self.constraints.values())
        for name, (r, _) in self.regularisation_families.items():
            nnz += r * (4 if name in ("dxy", "dyz", "dxz") else 3)
        for r, _t, op in self.directional_families.values():
            nnz += r * (4 if op in ("dxy", "dyz", "dxz") else 3)
        return nnz

    def _eval_points(self, loc, value=True, gradient=True):
        return fd.eval_points(self.support, self._c_device(), loc, value=value, gradient=gradient)

    def _evaluate_value_local(self, locations):
        self.update()
        loc = np.asarray(locations, dtype=float)
        if loc.shape[0] == 0:
            return np.zeros(0)
        return fd.eval_points(self.support, self._c_device(), loc, value=True, gradient=False)[0]

    def _evaluate_gradient_local(self, locations):
        self.update()
        loc = np.asarray(locations, dtype=float)
        if loc.shape[0] == 0:
            return np.zeros((0, 3))
        return fd.eval_points(self.support, self._c_device(), loc, value=False, gradient=True)[1]

    def surfaces(self, value, name="surface", **kwargs):
        """Isosurface(s) of the solved field on the grid nodes (DI:1395-1405):
        a list with one Surface per isovalue that the field crosses (an empty
        list when it crosses none).  ``value`` is a number or a sequence."""
        from .surface import Surface

        self.update()
        values = np.atleast_1d(np.asarray(value, dtype=float))
        out = []
        for v in values:
            verts, tris, nrm = fd.isosurface(self.support, self._c_device(), float(v))
            if verts.shape[0] == 0:
                continue
            if self.bounding_box is not None and hasattr(self.bounding_box, "reproject"):
                verts = self.bounding_box.reproject(verts)
            out.append(Surface(vertices=verts, triangles=tris, normals=nrm, name=name,
                               values=np.full(verts.shape[0], float(v))))
        return out

    def evaluate_lattice(self, origin, step, counts, value=True, gradient=True):
        """Dense-lattice evaluation on the device (K7 lattice kernel); returns
        device tensors (value (Q,), gradient (Q, 3)), i fastest."""
        self.update()
        return fd.eval_lattice(self.support, self._c_device(), origin, step, counts, value, gradient)
