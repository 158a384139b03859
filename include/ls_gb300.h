/*
 * ls_gb300.h -- C ABI of the GB300 (sm_103a) discrete implicit interpolation
 * hot path: structured-grid finite-difference (FD) and structured-tetra P1
 * constraint assembly, matrix-free normal-equations CG solve and field /
 * gradient evaluation.
 *
 * Conventions
 *   - Every pointer argument named d_* is a DEVICE pointer; h_* is a host
 *     pointer; structs passed by pointer live in host memory.
 *   - Node vectors use the reference's F-order numbering
 *     gi = i + nx*j + nx*ny*k (x fastest), so a solution array is directly the
 *     reference interpolator's `c`.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *   - Every function returns an int status (ls_status); on a negative status
 *     ls_last_error() returns a message for the calling thread.
 *   - No function allocates on the caller's behalf except ls_*_create, which
 *     owns its device workspace until ls_*_destroy.
 *
 * Reference files are cited relative to the LoopStructural 1.8.0 source tree:
 *   S  packages/loop_common/src/loop_common/supports/_3d_base_structured.py
 *   G  packages/loop_common/src/loop_common/supports/_3d_structured_grid.py
 *   T  packages/loop_common/src/loop_common/supports/_3d_structured_tetra.py
 *   FD packages/loop_interpolation/src/loop_interpolation/_finite_difference_interpolator.py
 *   P1 packages/loop_interpolation/src/loop_interpolation/_p1interpolator.py
 *   DI packages/loop_interpolation/src/loop_interpolation/_discrete_interpolator.py
 *   SP packages/loop_interpolation/src/loop_interpolation/_solver_pipeline.py
 *   SS packages/loop_interpolation/src/loop_interpolation/_solver_strategy.py
 */
#ifndef LS_GB300_H
#define LS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LS_ABI_VERSION 2

typedef enum ls_status {
  LS_OK = 0,
  LS_NOT_CONVERGED = 1, /* maxiter reached: the last iterate is returned (SS:66-71 warns, still True) */
  LS_NAN = 2,           /* a NaN / Inf appeared in the CG recurrence */
  LS_BREAKDOWN = 3,     /* p·Ap <= 0 */
  LS_ERR_ARG = -1,
  LS_ERR_CUDA = -2,
  LS_ERR_ALLOC = -3,
  LS_ERR_STATE = -4
} ls_status;

/* Structured support geometry: node counts per axis (cells + 1),
 * origin and cell size.  The same struct describes a TetMesh. */
typedef struct ls_grid3 {
  int64_t nsteps[3];
  double origin[3];
  double step[3];
} ls_grid3;

/* Message describing the last negative status returned on this thread. */
const char *ls_last_error(void);
int ls_abi_version(void);

/* ------------------------------------------------------------------ */
/* FD constraint assembly (K1/K2)                                      */
/* ------------------------------------------------------------------ */

/* Row kinds of ls_fd_point_rows and the reference method each replaces. */
typedef enum ls_row_kind {
  LS_ROWS_VALUE = 0,    /* FD:236-269 add_value_constraints: 1 row/point, w = weight*point_w */
  LS_ROWS_NORM = 1,     /* FD:403-476 add_norm_constraints: 3 rows/point (norm_0..2), w = weight/3*point_w */
  LS_ROWS_GRADIENT = 2, /* FD:342-401 add_gradient_constraints: 2 rows/point (strike, dip), w = weight */
  LS_ROWS_TANGENT = 3,  /* FD:478-539 add_gradient_orthogonal_constraints: 1 row/point, w = weight */
  LS_ROWS_ORTHOGONAL = 4 /* FD:478-539 with a target: columns x y z vx vy vz b, 1 row/point, w = weight */
} ls_row_kind;

/* Point-constraint rows on a StructuredGrid.  Replaces the per-family
 * position_to_cell_corners + trilinear / element-gradient shape
 * functions (G:90-162, G:393-454) + row normalisation
 * (DI:361-366 add_constraints_to_least_squares).
 *   d_pts     : npts x ld row-major FP64 (x, y, z, ...columns of the kind...)
 *   outputs   : rows_per_point families, family f occupying rows
 *               [f*npts, f*npts + *h_count): d_idc (int64 x 8) bit-identical to
 *               the reference COO columns, d_a (x 8) normalised coefficients,
 *               d_b, d_w.  Points outside the support are dropped in order.
 *   h_count   : number of inside points (host int64, written after a sync).
 *   h_nan     : set to 1 when a computed row holds a NaN (the reference then
 *               skips the whole family, DI:355-359). */
int ls_fd_point_rows(const ls_grid3 *grid, int kind, const double *d_pts, int64_t npts, int64_t ld,
                     double weight, int64_t *d_idc, double *d_a, double *d_b, double *d_w,
                     int64_t *h_count, int32_t *h_nan, void *stream);

/* Directional regularisation weights of FD:1207-1337
 * minimise_directional_gradient_change(w, vector): for every interior node m
 * (1 <= i, j, k <= n - 2) and family f in (dxx, dyy, dzz, dxy, dxz, dyz),
 * rw = weight * c_f(v_m), c = (vx^2, vy^2, vz^2, 2 vx vy, 2 vx vz, 2 vy vz);
 * a row with |rw| > 0 adds s_f^2 rw^2 to d_omega[f * dof + m] (s_f^2 = 1/6 for
 * dxx..dzz, 1/4 for the cross families: the squared row normalisation of
 * DI:361-366).  d_vec: dof x ld FP64 (vx, vy, vz first), the direction at
 * every node in node order; d_omega (6 x dof) accumulates over calls (zero it
 * first).  h_counts (6 int64, may be NULL): the rows of each family the
 * reference would add (FD:1320-1335 drops the others). */
int ls_fd_directional_weights(const ls_grid3 *grid, const double *d_vec, int64_t ld, double weight,
                              double *d_omega, int64_t *h_counts, void *stream);

/* Regularisation weight scale of use_regularisation_weight_scale
 * (FD:66-90 compute_weighting, called from FD:416-444 add_norm_constraints;
 * P1:52-69): for every node m, d_scale[m] += 1 + alpha exp(-d^2 / (2 sigma^2)),
 * d = the distance from the node (numpy linspace coordinates) to
 * the nearest of the npts points (x y z = the first columns of d_pts, npts x
 * ld FP64; pass the normal constraints inside the support).  The nearest
 * point is exact (an FP32 screen, then FP64 distances).  The reference scale
 * starts at 1 (DI:313), so d_scale starts as ones. */
int ls_fd_weight_scale(const ls_grid3 *grid, const double *d_pts, int64_t npts, int64_t ld, double alpha,
                       double sigma, double *d_scale, void *stream);

/* The six interior regularisation families with the per-node scale
 * (FD:668-672): for every interior node m (1 <= i, j, k <= n - 2) and family
 * f in (dxx, dyy, dzz, dxy, dxz, dyz), d_omega[f * dof + m] += s_f^2
 * (d_scale[m] h_w[f])^2 (s_f^2 = 1/6, 1/4), h_w = the families' row weights
 * (cross families already divided by 4).  d_omega is the d_dir weight
 * array of the system struct; it accumulates with ls_fd_directional_weights,
 * and the system's isotropic interior weights are then 0. */
int ls_fd_scaled_weights(const ls_grid3 *grid, const double *d_scale, const double h_w[6], double *d_omega,
                         void *stream);

/* Interface pair rows (FD:297-340 add_interface_constraints): row p is
 * [trilinear(i), -trilinear(j)] over 16 columns for d_pairs[p] = (i, j), both
 * indices into d_pts (all points must be inside), b = 0, w = weight. */
int ls_fd_pair_rows(const ls_grid3 *grid, const double *d_pts, int64_t ld, const int64_t *d_pairs,
                    int64_t npairs, double weight, int64_t *d_idc, double *d_a, double *d_b, double *d_w,
                    void *stream);

/* Regularisation families, in the reference order: the six interior families
 * of G:489-510 and the six border families of FD:1052-1144. */
typedef enum ls_reg_family {
  LS_REG_DXY = 0, LS_REG_DYZ = 1, LS_REG_DXZ = 2, LS_REG_DXX = 3, LS_REG_DYY = 4, LS_REG_DZZ = 5,
  LS_REG_DX_LOWER = 6, LS_REG_DX_UPPER = 7, LS_REG_DY_LOWER = 8, LS_REG_DY_UPPER = 9,
  LS_REG_DZ_LOWER = 10, LS_REG_DZ_UPPER = 11
} ls_reg_family;

/* Number of rows and taps of a regularisation family (FD:636-692). */
int ls_fd_reg_shape(const ls_grid3 *grid, int family, int64_t *h_rows, int32_t *h_taps);

/* Explicit column indices of a regularisation family (parity mode of the
 * matrix-free operator): FD:643-692 _assemble_operator +
 * G:164-293 neighbour_global_indexes, row-major rows x taps int64. */
int ls_fd_reg_rows(const ls_grid3 *grid, int family, int64_t *d_idc, void *stream);

/* ------------------------------------------------------------------ */
/* FD normal-equations system and CG solve (K4/K5/K6)                  */
/* ------------------------------------------------------------------ */

/* Weighted least-squares system
 *    minimise  sum_rows w^2 (a.x - b)^2 + ridge^2 |x|^2
 * whose normal equations (A^T W A + ridge^2 I) x = A^T W b are what
 * DI:1221-1319 solve_system('cg') solves (SP:86-124, SS:48-72).  The
 * regularisation rows are implicit (matrix-free stencils); data rows are
 * given explicitly. */
typedef struct ls_fd_system {
  ls_grid3 grid;
  /* row weights of the interior families as used by the reference, i.e. the
   * cross-derivative weights already divided by 4 (G:502-509) */
  double w_dxx, w_dyy, w_dzz, w_dxy, w_dyz, w_dxz;
  /* border family weights (FD:1102-1139); 0 disables the pair of families */
  double w_dx, w_dy, w_dz;
  double ridge; /* ridge row weight (DI:78, 1e-8); 0 disables */
  /* data rows (device, row-major nrows x width; a negative column is padding) */
  int64_t nrows;
  int32_t width;
  const int64_t *d_idc;
  const double *d_a; /* normalised coefficients */
  const double *d_b; /* normalised right-hand side */
  const double *d_w; /* row weights (W = w^2) */
  /* directional regularisation (FD:1207-1337), or NULL: 6 x dof FP64 weights,
   * family-major (dxx, dyy, dzz, dxy, dxz, dyz), as accumulated by
   * ls_fd_directional_weights; the handle keeps its own copy */
  const double *d_dir;
} ls_fd_system;

typedef struct ls_fd_handle ls_fd_handle;

int ls_fd_create(const ls_fd_system *sys, ls_fd_handle **out, void *stream);
int ls_fd_destroy(ls_fd_handle *h);
/* number of degrees of freedom */
int64_t ls_fd_dof(const ls_fd_handle *h);

/* y = (A^T W A + ridge^2 I) x in FP64 (matrix-free). */
int ls_fd_apply(ls_fd_handle *h, const double *d_x, double *d_y, void *stream);
/* the same operator in FP32 (the inner-iteration kernel of the mixed solve) */
int ls_fd_apply_f32(ls_fd_handle *h, const float *d_x, float *d_y, void *stream);
/* No-allocation variant of ls_fd_apply (no counterpart in the reference, which
 * has no device code).  For callers that cannot call cudaMalloc -- a host
 * framework that owns all device memory through its own pool, or a plugin
 * running under a fixed device-memory budget -- it takes the system
 * description directly (no handle) and keeps its private scratch (one FP64
 * value per data row plus reduction partials) in a static device array of
 * LS_NOALLOC_SCRATCH_DOUBLES doubles (~8.4 MB per GPU that loads the library,
 * held until the process exits).  Limits: sys->nrows <= LS_NOALLOC_MAX_ROWS,
 * sys->d_dir == NULL and at most 524,280 nodes along y, else LS_ERR_ARG.
 * Computes d_y = N d_x (FP64).  When h_xNx is not NULL it also writes x.Nx to
 * host memory, which copies to the host and synchronises `stream` before
 * returning; pass NULL for a call that only enqueues work.  Data-row columns
 * must be < dof: out-of-range columns are skipped, and reported as LS_ERR_ARG
 * when h_xNx is not NULL.  The first call on a device resolves the array's
 * device address (cudaGetSymbolAddress), so make that first call before any
 * stream capture.  Every call shares the one array, which keeps the last
 * call's contents: calls that overlap on the GPU race and must be serialised
 * by the caller.  The data-row scatter uses FP64 atomics, so the result can
 * differ from ls_fd_apply in the last bits. */
#define LS_NOALLOC_MAX_ROWS 1048576
#define LS_NOALLOC_SCRATCH_DOUBLES (LS_NOALLOC_MAX_ROWS + 4096 + 8)
int ls_fd_apply_noalloc(const ls_fd_system *sys, const double *d_x, double *d_y, double *h_xNx, void *stream);

/* A^T W b (FP64) */
int ls_fd_rhs(ls_fd_handle *h, double *d_rhs, void *stream);
/* Replaces the right-hand side A^T W b by d_rhs (device, dof FP64) for the
 * following solves: the adjoint solve N lambda = E^T g of a loss on evaluated
 * values reuses the factor-free operator of the forward solve.  No
 * counterpart in the reference (which has no adjoint). */
int ls_fd_set_rhs(ls_fd_handle *h, const double *d_rhs, void *stream);
/* s_r = w_r^2 (a_r . x) over the data rows (FP64; d_s has nrows entries):
 * with x = lambda, the gradient of the loss with respect to the rows'
 * right-hand sides b_r.  No counterpart in the reference. */
int ls_fd_data_rows_apply(ls_fd_handle *h, const double *d_x, double *d_s, void *stream);
/* One ADMM projection step over the data rows [row0, row0 + m), which hold
 * the inequality rows q'_r with weight rho (replaces the update of
 * loopsolver/admm_solver.py:380-404 admm_solve with
 * admm_method.py:12-25 ADMM.admm_method_iterate_admm_array, for exact inner
 * solves of the normal equations): qx = q'_r . x (x = d_x, the current
 * solution), arg = qx + u, z = arg when lo <= arg <= hi, else the bound it
 * passed (unchanged when arg is NaN), u = u + qx - z, and the row's
 * right-hand side becomes z - u; the handle's A^T W b is then recomputed, so
 * that the next ls_fd_solve minimises |A x - b|^2 + rho^2 |Q' x - (z - u)|^2.
 * d_lo, d_hi, d_z, d_u: m FP64 each (z and u updated in place).  h_sums (5
 * host doubles): sum (qx - z)^2, sum (z - z_prev)^2, sum qx^2, sum z^2,
 * sum u^2 of this step.  Synchronises the handle's stream. */
int ls_fd_admm_step(ls_fd_handle *h, int64_t row0, int64_t m, const double *d_lo, const double *d_hi, double *d_z,
                    double *d_u, const double *d_x, double *h_sums, void *stream);
/* diag(A^T W A + ridge^2 I): the squared column norms of the reference's
 * column scaling (DI:815-833) */
int ls_fd_diagonal(ls_fd_handle *h, double *d_diag, void *stream);

typedef enum ls_precision { LS_FP64 = 0, LS_MIXED = 1 } ls_precision;

/* CG preconditioner.  JACOBI reproduces the reference's column-scaled CG
 * iteration; MG (mixed precision only) is a geometric-multigrid V-cycle that
 * changes only the iteration path -- the stopping test stays the reference's
 * ||S r|| < max(atol, rtol ||S rhs||).  MG falls back to JACOBI for grids it
 * cannot coarsen (an axis below 5 nodes while the coarsest level is still
 * above 1000 nodes); ls_solve_stats.preconditioner reports the one used. */
typedef enum ls_preconditioner { LS_PRECOND_JACOBI = 0, LS_PRECOND_MG = 1 } ls_preconditioner;

typedef struct ls_solve_opts {
  int32_t precision;      /* ls_precision */
  int32_t use_x0;         /* d_x holds the initial guess (else zeros) */
  double atol;            /* absolute tolerance on ||S r|| (scipy cg atol) */
  double rtol;            /* relative tolerance (scipy cg rtol, default 1e-5) */
  int64_t maxiter;        /* <= 0: 10 * dof (scipy default) */
  double reliable_delta;  /* mixed: refresh the FP64 residual once ||S r|| fell by this factor (<=0: 0.1) */
  int32_t check_every;    /* iterations per device batch between host checks (<=0: 64) */
  int32_t preconditioner; /* ls_preconditioner */
  int32_t mg_degree;      /* multigrid: Chebyshev smoothing steps before and after the coarse correction (<=0: 3) */
} ls_solve_opts;

typedef struct ls_solve_stats {
  int64_t iterations;       /* CG iterations (scipy counting) */
  int64_t reliable_updates; /* FP64 residual refreshes (mixed) */
  double residual;          /* final ||S (rhs - N x)|| in FP64, S = diag^(-1/2) */
  double rhs_norm;          /* ||S rhs|| */
  double threshold;         /* max(atol, rtol * ||S rhs||) */
  double device_ms;         /* device time of the solve (CUDA events) */
  int32_t status;
  int32_t preconditioner;   /* ls_preconditioner actually used */
  int64_t kernel_launches;  /* kernels launched by this call (graph launches count their kernel nodes) */
} ls_solve_stats;

/* Jacobi-preconditioned CG on the normal equations -- the iteration of the
 * reference's column-scaled scipy cg (SS:48-72 with DI:815-833 scaling),
 * stopping at the same criterion ||S r|| < max(atol, rtol ||S rhs||).
 * d_x (device, dof FP64) receives the solution. */
int ls_fd_solve(ls_fd_handle *h, const ls_solve_opts *opts, double *d_x, ls_solve_stats *stats, void *stream);

/* Does the allocations a solve with these options would do on first use
 * (the multigrid hierarchy of a mixed multigrid solve); optional before
 * ls_fd_solve, done by ls_fd_solve_batched for every model. */
/* Host wall time (ms) of the multigrid setup phases of the handle's last
 * build (no counterpart in the reference): host copy of the data rows,
 * regularisation tables, data-row coarsening, data-term upload, diagonals,
 * eigenvalue estimates, coarsest inverse, total.  Returns the number of
 * values written (<= n, at most 8); zeros before a multigrid build. */
int ls_fd_setup_profile(const ls_fd_handle *h, double *h_out, int n);
int ls_fd_prepare(ls_fd_handle *h, const ls_solve_opts *opts);

/* Device the handle was created on. */
int ls_fd_device(const ls_fd_handle *h);

/* 1 when the handle's finest-level FP32 applies run the TMA-staged kernel
 * (grids whose x extent is a multiple of 4 nodes and every axis >= 8 nodes,
 * unless the environment variable LS_GB300_STAGED_APPLY=tiles was set when
 * the handle was created), 0 when they run the cp.async tile kernels.  No
 * counterpart in the reference. */
int ls_fd_staged_apply(const ls_fd_handle *h);

/* Solves `count` independent systems (a model ensemble) with up to
 * `concurrency` (<= 0: 8) solves in flight, each on its handle's stream:
 * model i solves with opts[i] into d_x[i], filling stats[i] and statuses[i]
 * (the ls_fd_solve status).  Returns the first negative status (its message
 * names the model), else 0.  Each result equals that of ls_fd_solve on the
 * same handle; the reference solves its models one by one (no counterpart). */
int ls_fd_solve_batched(ls_fd_handle *const *handles, const ls_solve_opts *opts, double *const *d_x,
                        ls_solve_stats *stats, int64_t count, int concurrency, int *statuses);

/* Per-kernel device times of one CG iteration, measured with CUDA events on
 * the handle's stream over `reps` back-to-back launches of each kernel class
 * (no counterpart in the reference, which has no device code). */
typedef struct ls_fd_profile {
  double stencil_ms;    /* matrix-free stencil part of N p (+ p.Np) */
  double data_ms;       /* data-row part of N p */
  double update_ms;     /* x, r, z updates and r.z + the p update */
  double iteration_ms;  /* one whole iteration */
  double stencil_bytes; /* algorithmic bytes of one stencil launch: read p, write q */
  double iteration_bytes; /* algorithmic bytes of one iteration (9 N s + 16 nnz_data) */
} ls_fd_profile;

int ls_fd_profile_iteration(ls_fd_handle *h, int precision, int reps, ls_fd_profile *out, void *stream);

/* Device time per launch (ms, CUDA events over `reps` back-to-back launches on
 * the handle's stream) of the parts of the multigrid V-cycle on every level,
 * building the hierarchy if needed.  out[l * LS_MG_PROFILE_FIELDS + f] for
 * level l < *levels (at most max_levels): f = 0 nodes, 1 operator apply
 * (plain), 2 apply with the Chebyshev epilogue, 3 apply with the residual
 * epilogue, 4 restriction to level l+1, 5 prolongation from level l+1,
 * 6 data rows (row form), 7 the coarsest dense solve (last level only),
 * 8 / 9 the Chebyshev apply's kernels alone: on a finest level run by the
 * TMA-staged kernel, that kernel / the data term after it (rows + fix-up); on levels
 * split into a staged interior and a boundary kernel, those two (0 otherwise).
 * Returns 0 with *levels = 0 when the grid does not coarsen.  The solver
 * vectors are overwritten.  No counterpart in the reference. */
#define LS_MG_PROFILE_FIELDS 10

/* y = A_l x with the FP32 operator of multigrid level l (0 = the system's
 * own grid; l+1 has n_l/2+1 nodes per axis), building the hierarchy if
 * needed; *h_nodes receives the level's node count (pass NULL vectors to only
 * query it).  A diagnostic of the preconditioner; no reference counterpart. */
int ls_fd_mg_apply_level(ls_fd_handle *h, int level, const float *d_x, float *d_y, int64_t *h_nodes, void *stream);
int ls_fd_profile_mg(ls_fd_handle *h, int reps, double *out, int max_levels, int *levels, void *stream);

/* z = V(r): one application of the multigrid preconditioner of the mixed
 * solve (FP32, dof entries each), building the hierarchy if needed.  A
 * diagnostic of the preconditioner (symmetric positive definite by
 * construction); overwrites the solver's vectors.  No reference counterpart. */
int ls_fd_mg_vcycle(ls_fd_handle *h, const float *d_r, float *d_z, void *stream);

/* ------------------------------------------------------------------ */
/* FD evaluation (K7)                                                   */
/* ------------------------------------------------------------------ */

/* Value / gradient of the trilinear field c at points (npts x ld, x y z
 * first): G:295-391 with DI:1342-1379 semantics -- value NaN outside the
 * support, 0 for a NaN input row; gradient 0 outside.  Either output may be
 * NULL. */
int ls_fd_eval_points(const ls_grid3 *grid, const double *d_c, const double *d_pts, int64_t npts, int64_t ld,
                      double *d_value, double *d_grad, void *stream);

/* Transpose of ls_fd_eval_points: d_out[node] += sum_i (trilinear weight of
 * the node at point i) * d_gvalue[i] + (its shape-function gradient) .
 * d_ggrad[3i..3i+2]; either input may be NULL; points outside the support
 * contribute nothing.  FP64 atomics (sum order varies at the ulp level).  The
 * adjoint of the evaluation for gradients through the solve; no counterpart
 * in the reference. */
int ls_fd_eval_adjoint(const ls_grid3 *grid, const double *d_pts, int64_t npts, int64_t ld, const double *d_gvalue,
                       const double *d_ggrad, double *d_out, void *stream);

/* Jets of the trilinear field c at points (npts x ld, x y z first): d_out
 * (npts x 11 FP64) = u, du/dx, du/dy, du/dz, d2u/dxdy, d2u/dxdz, d2u/dydz,
 * the local coordinates lx, ly, lz in the cell (G:126-146, clipped to [0, 1])
 * and 1 for points inside the support; all 0 outside.  The quantities the
 * adjoint with respect to point positions and normal vectors needs; no
 * counterpart in the reference. */
int ls_fd_eval_jets(const ls_grid3 *grid, const double *d_c, const double *d_pts, int64_t npts, int64_t ld,
                    double *d_out, void *stream);

/* The same on a regular lattice of points origin + step * (i, j, k),
 * i < n[0] fastest; output index i + n0*j + n0*n1*k. */
int ls_fd_eval_lattice(const ls_grid3 *grid, const double *d_c, const double lat_origin[3],
                       const double lat_step[3], const int64_t lat_n[3], double *d_value, double *d_grad,
                       void *stream);

/* ------------------------------------------------------------------ */
/* Fault displacement: evaluation of a faulted feature (the caller of K7) */
/* ------------------------------------------------------------------ */

/* A fault profile function of one fault-frame coordinate (the reference's
 * LoopStructural/modelling/features/fault/_fault_function.py, FF below):
 * ONES / ZEROS (FF:252-307), SMOOTH_PEAK x^4 - 2 x^2 + 1 on [-1, 1] else 0
 * (FF:12-16), CUBIC w0 v^3 + w1 v^2 + w2 v + w3 held at its value at lim[0] /
 * lim[1] outside them, then clamped to [min_v, max_v] (FF:40-150, the
 * coefficients already fitted), COMPOSITE: the cubic [0] for v > 0, the cubic
 * [1] for v < 0, 0 at 0 (FF:197-230). */
typedef enum ls_profile_kind {
  LS_PROFILE_ONES = 0, LS_PROFILE_ZEROS = 1, LS_PROFILE_SMOOTH_PEAK = 2, LS_PROFILE_CUBIC = 3,
  LS_PROFILE_COMPOSITE = 4
} ls_profile_kind;

typedef struct ls_fault_profile {
  int32_t kind;
  int32_t pad;
  double w[2][4];     /* cubic coefficients ([1] only for COMPOSITE, its negative side) */
  double lim[2][2];   /* [lower, upper] x limits of each cubic */
  double clamp[2][2]; /* [min_v, max_v] of each cubic */
} ls_fault_profile;

/* One fault-frame coordinate field: a solved FD field (node values d_c on
 * `grid`, device) and the affine maps of its interpolator's bounding box:
 * local = to_local[0..2][0..2] world + to_local[.][3], gradients back to the
 * world frame by the 3x3 rotation to_world. */
typedef struct ls_fault_field {
  ls_grid3 grid;
  const double *d_c;
  double to_local[3][4];
  double to_world[3][3];
} ls_fault_field;

/* A fault slip event (the reference's FaultSegment, LoopStructural/modelling/
 * features/fault/_fault_segment.py FS:25-60): the three frame fields
 * (gx normal to the fault, gy along slip, gz along extent), the displacement
 * magnitude, the number of integration steps, and the displacement function
 * scale * gx(gx) * gy(gy) * gz(gz) (FF:310-361); has_function = 0 gives unit
 * displacement on the hanging wall (gx > 0) instead. */
typedef struct ls_fault {
  ls_fault_field frame[3];
  double displacement;
  int32_t steps;
  int32_t has_function;
  double scale;
  ls_fault_profile profile[3];
} ls_fault;

/* Restores points through one fault in place (FS:315-423 apply_to_points):
 * per point, the frame coordinates and the displacement d at the point; points
 * with d = 0 (or a frame coordinate NaN: outside a frame field) stay put; the
 * others move `steps` times by d / steps along the unit gradient of the gy
 * field, re-evaluating the frame at every step.  As in the reference, the
 * `reverse` sign of apply_to_points does not reach the integration (its
 * displacement is recomputed each step), so there is no reverse flag here.
 * d_pts: npts x ld FP64 (x y z first), device. */
int ls_fault_apply(const ls_fault *fault, double *d_pts, int64_t npts, int64_t ld, void *stream);

/* Gradient of a linear field over tetrahedra (LoopStructural/utils/maths.py
 * gradient_from_tetrahedron): d_tetra (n x 4 x 3 vertex coordinates),
 * d_values (n x 4 vertex values) -> d_grad (n x 3) solving
 * (v_k - v_0) . g = f_k - f_0, k = 1..3.  Degenerate tetrahedra give NaN. */
int ls_tetra_gradient(const double *d_tetra, const double *d_values, int64_t n, double *d_grad, void *stream);

/* ------------------------------------------------------------------ */
/* P1 on a structured TetMesh (5 tetrahedra per cell) (K3)              */
/* ------------------------------------------------------------------ */

/* Number of face-sharing tetrahedron pairs of the mesh (T:120-184). */
int ls_p1_face_count(const ls_grid3 *mesh, int64_t *h_faces);

/* Constant-gradient face rows of P1:115-166 minimise_edge_jumps, in the
 * reference's face order (pairs (i, j), i > j, sorted by i then j; T:120-184):
 * row f = [n.grad(phi_i), -n.grad(phi_j)] over the 8 nodes of the two tets,
 * normalised, b = 0, w = weight.  d_pairs (F x 2) and d_shared (F x 3, the
 * shared face nodes ascending) may be NULL.  The row sign follows the order of
 * the shared nodes (the normal's orientation); it does not change A^T W A. */
int ls_p1_face_rows(const ls_grid3 *mesh, double weight, int64_t *d_pairs, int64_t *d_shared, int64_t *d_idc,
                    double *d_a, double *d_b, double *d_w, void *stream);

/* Directional face rows (P1:172-178 -> P1:115-166 with `vector`): the rows of
 * ls_p1_face_rows with the face normal replaced by d_vec[f] (F x 3 FP64, one
 * direction per face in the same face order), normalised, b = 0, w = weight. */
int ls_p1_face_rows_directional(const ls_grid3 *mesh, double weight, const double *d_vec, int64_t *d_idc,
                                double *d_a, double *d_b, double *d_w, void *stream);

/* Containing tetrahedron (-1 outside) and barycentric coordinates of points
 * (T:274-365: last containing tet of the 5 candidates wins; strict inside). */
int ls_p1_locate(const ls_grid3 *mesh, const double *d_pts, int64_t npts, int64_t ld, int64_t *d_tet, double *d_bc,
                 void *stream);

/* Value rows (kind LS_ROWS_VALUE, P1:98-113: barycentric, per-point weight
 * column ignored, w = weight), normal rows (LS_ROWS_NORM, P1:73-96: 3
 * gradient rows per point, point-major, w = weight) or gradient-orthogonal
 * rows (P1:248-296: v/|v| . grad phi, w = weight x the tetrahedron's volume;
 * LS_ROWS_TANGENT: columns x y z vx vy vz, b = 0, the tangent rows of
 * DI:668-682; LS_ROWS_ORTHOGONAL: a target b in column 6) of the inside
 * points, compacted in input order; 4 columns per row. */
int ls_p1_point_rows(const ls_grid3 *mesh, int kind, const double *d_pts, int64_t npts, int64_t ld, double weight,
                     int64_t *d_idc, double *d_a, double *d_b, double *d_w, int64_t *h_count, void *stream);

/* Value / gradient of the P1 field (T:208-262): NaN outside; a NaN input row
 * gives value 0 (DI:1342-1362). */
int ls_p1_eval_points(const ls_grid3 *mesh, const double *d_c, const double *d_pts, int64_t npts, int64_t ld,
                      double *d_value, double *d_grad, void *stream);

/* ------------------------------------------------------------------ */
/* Isosurfaces of a solved FD field (DI:1395-1405 surfaces(value))      */
/* ------------------------------------------------------------------ */

/* The level set {f = iso} of the node values d_values (one per grid node,
 * node order i + nx (j + ny k)) under the piecewise-linear interpolant on the
 * Freudenthal triangulation of the cells (6 tetrahedra per cell along the
 * main diagonal): one vertex per crossing edge (shared by all its
 * triangles), triangles wound with their normal towards increasing f.  The
 * reference contours the same node values with VTK's marching cubes.
 * ls_iso_extract classifies the cells and returns the vertex and triangle
 * counts (host, after a stream sync); ls_iso_copy writes d_verts (V x 3
 * FP64 coordinates), d_normals (V x 3, unit gradient direction; may be NULL)
 * and d_tris (T x 3 int64 vertex indices); d_values must stay valid until
 * ls_iso_copy has run.  NaN node values exclude their edges and cells. */
typedef struct ls_iso ls_iso;
int ls_iso_extract(const ls_grid3 *grid, const double *d_values, double iso, ls_iso **out, int64_t *h_nverts,
                   int64_t *h_ntris, void *stream);
int ls_iso_copy(ls_iso *h, double *d_verts, double *d_normals, int64_t *d_tris, void *stream);
int ls_iso_destroy(ls_iso *h);

#ifdef __cplusplus
}
#endif
#endif /* LS_GB300_H */
