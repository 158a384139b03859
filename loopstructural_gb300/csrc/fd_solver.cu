// Matrix-free normal-equations operator and CG solvers for the FD
// (StructuredGrid) interpolator.
//
// The least-squares system of the reference (DI:684-755 build_matrix,
// SP:86-124 ridge + column scaling) is
//     N = sum_f w_f^2 R_f^T R_f  +  A_d^T W A_d  +  ridge^2 I
// where R_f are the twelve second-derivative stencil families (six interior,
// six border, FD:643-692 / FD:1052-1144) and A_d the explicit data rows.
// N is never assembled: the stencil part is applied from node coordinates,
// the data part from a row list and a node->row incidence list.
//
// The solver is Jacobi-preconditioned CG, which is the reference's
// column-scaled CG (SS:48-72 on A S, S = diag(N)^-1/2) written without the
// explicit scaling: identical iterates x_k = S y_k and identical stopping test
// ||S r|| < max(atol, rtol ||S rhs||).
#include <cooperative_groups.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "fd_apply.cuh"
#include "fd_apply_tma.cuh"
#include "fd_directional.cuh"
#include "fd_mg.cuh"
#include "fd_mg_cells.cuh"
#include "mg_rows_host.hpp"
#include "fd_stencil.cuh"
#include "ls_common.cuh"

namespace ls {
namespace {

constexpr int kBlock = 256;
constexpr int kAuxDoubles = 8;

// Device-resident CG scalars.  All reductions land here so that a whole batch
// of iterations runs without host round trips.
struct CgScalars {
  double rz;       // r . z of the current residual
  double pq_s;     // p . (stencil part of N p)
  double pq_d;     // p . (data part of N p)
  double pq_x;     // p . (directional part of N p; 0 without directional terms)
  double beta;
  double thresh2;  // stopping threshold squared (on r . z)
  double rrj;      // r . D^-1 r of the current FP32 residual (MG stopping test)
  double rz64;     // FP64 refresh: r64 . D^-1 r64
  double rz32;     // FP64 refresh: r32 . D^-1 r32 (after rounding)
  double scratch;
  double trig2;    // mixed precision: stop the FP32 batch for a reliable update below this (0 = never)
  long long iters;
  long long maxiter;
  int done;        // DONE_* stop code
  int pending;     // stop code raised mid-iteration; becomes `done` once p is updated
  int profile;     // timing mode: never stop, never flag a breakdown
  int fault;       // a staged (TMA) apply gave up waiting for a copy
};

struct DataTerm {
  int64_t nrows = 0;
  int32_t width = 0;
  int64_t ntouched = 0;
  int32_t *cols = nullptr;     // nrows * width (padding = -1)
  double *a64 = nullptr;       // nrows * width
  float *a32 = nullptr;
  double *w2_64 = nullptr;     // nrows
  float *w2_32 = nullptr;
  double *b = nullptr;         // nrows
  int64_t *touched = nullptr;  // ntouched node ids, ascending
  int64_t *inc_ptr = nullptr;  // ntouched + 1
  int32_t *inc_row = nullptr;  // incidences (row of each)
  double *inc_a64 = nullptr;   // coefficient of each incidence
  float *inc_a32 = nullptr;
  uint32_t *mask = nullptr;    // touched-node bit mask, ceil(n/32) words
  int32_t *word_rank = nullptr;
};

}  // namespace
}  // namespace ls

struct ls_fd_handle {
  ls_grid3 grid;
  ls::StencilCoef coef;
  int64_t n = 0;
  ls::DataTerm data;
  cudaStream_t stream = nullptr;
  int device = 0;  // device the handle's memory lives on
  // persistent vectors
  double *rhs = nullptr, *diag = nullptr, *dinv64 = nullptr;
  float *dinv32 = nullptr;
  double *x64 = nullptr, *r64 = nullptr, *p64 = nullptr, *q64 = nullptr, *s64 = nullptr;
  float *x32 = nullptr, *r32 = nullptr, *p32 = nullptr, *q32 = nullptr, *s32 = nullptr;
  double rhs_norm2 = 0.0;  // rhs . D^-1 rhs
  // reductions
  ls::CgScalars *sc = nullptr;     // iteration scalars (device)
  ls::CgScalars *sc_h = nullptr;   // pinned host mirror
  double *partials = nullptr;      // 2 * max_blocks
  unsigned int *tickets = nullptr; // one per reduction site
  int red_blocks = 0;
  int64_t partials_cap = 0;        // doubles in partials (one per block of a one-value grid reduction)
  // graphs of one batch of iterations
  cudaGraphExec_t g64 = nullptr, g32 = nullptr, gmg = nullptr;
  int g64_batch = 0, g32_batch = 0, gmg_batch = 0;
  // kernel launches issued on the handle's stream (a graph launch counts its
  // kernel nodes); g*_kernels = kernel nodes of each cached graph
  int64_t launches = 0;
  int64_t g64_kernels = 0, g32_kernels = 0, gmg_kernels = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // multigrid preconditioner (built on first use)
  ls::MgHierarchy mg;
  float *z32 = nullptr;                 // preconditioned residual
  // directional regularisation weights (6 x n, family-major; null without)
  double *dir64 = nullptr;
  float *dir32 = nullptr;
  // TMA-staged finest-level FP32 apply (fd_apply_tma.cuh): tensor maps of the
  // grid's vectors
  ls::TmCache tm;
  double *aux = nullptr;                // kAuxDoubles of scratch (ADMM step sums)
  std::vector<int64_t> h_idc;           // host copy of the data rows (Galerkin coarsening)
  std::vector<double> h_a, h_w2;
  int h_width = 0;
};

namespace ls {
namespace {

// device-side stop codes (CgScalars::done); mapped to ls_status on the host
enum : int {
  DONE_RUNNING = 0,
  DONE_CONVERGED = 1,
  DONE_MAXITER = 2,
  DONE_NAN = 3,
  DONE_BREAKDOWN = 4,
  DONE_REFRESH = 5  // FP32 residual fell below trig2: reliable update due
};

int done_to_status(int d) {
  switch (d) {
    case DONE_CONVERGED: return LS_OK;
    case DONE_MAXITER: return LS_NOT_CONVERGED;
    case DONE_NAN: return LS_NAN;
    case DONE_BREAKDOWN: return LS_BREAKDOWN;
    default: return LS_OK;
  }
}

enum Ticket {
  T_STENCIL = 0,
  T_DATA = 1,
  T_UPDATE = 2,
  T_REFRESH = 3,
  T_MISC = 4,
  T_PUPD = 5,
  T_SHELL = 6,
  T_DIR = 7,
  T_COUNT = 8
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// alpha = rz / pq ; x += alpha p ; r -= alpha q ; rz' = r . D^-1 r ;
// the last block publishes beta = rz'/rz and tests convergence.  Converged,
// maximum-iteration and refresh stops are raised as `pending` so that the
// iteration completes (p updated) before the batch stops; NaN and breakdown
// stop at once (x and r untouched).
template <typename T>
__global__ void __launch_bounds__(kBlock) update_xr_kernel(int64_t n, T *__restrict__ x, T *__restrict__ r,
                                                           const T *__restrict__ p, const T *__restrict__ q,
                                                           const T *__restrict__ dinv, CgScalars *sc,
                                                           double *partials, unsigned int *ticket) {
  if (sc->done) return;
  const double pq = sc->pq_s + sc->pq_d + sc->pq_x;
  const double rz = sc->rz;
  const double alpha_d = rz / pq;
  if (!sc->profile && (!(pq > 0.0) || !isfinite(alpha_d))) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = isfinite(pq) ? DONE_BREAKDOWN : DONE_NAN;
    return;
  }
  const T alpha = (T)alpha_d;
  T local = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    x[g] += alpha * p[g];
    const T rn = r[g] - alpha * q[g];
    r[g] = rn;
    local += rn * (dinv[g] * rn);
  }
  double rz_new;
  if (grid_sum<kBlock, T>(local, partials, ticket, &rz_new)) {
    sc->iters += 1;
    sc->beta = rz_new / rz;
    sc->rz = rz_new;
    if (sc->profile) {
      sc->rz = 1.0;  // keep alpha and beta finite while timing
      sc->beta = 0.5;
    } else if (!isfinite(rz_new)) sc->done = DONE_NAN;
    else if (rz_new < sc->thresh2) sc->pending = DONE_CONVERGED;
    else if (sc->iters >= sc->maxiter) sc->pending = DONE_MAXITER;
    else if (rz_new < sc->trig2) sc->pending = DONE_REFRESH;
  }
}

// p = D^-1 r + beta p ; the last block turns a pending stop into `done`
template <typename T>
__global__ void __launch_bounds__(kBlock) update_p_kernel(int64_t n, const T *__restrict__ r, const T *__restrict__ dinv,
                                                          T *__restrict__ p, CgScalars *sc, unsigned int *ticket) {
  if (sc->done) return;
  const T beta = (T)sc->beta;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    p[g] = dinv[g] * r[g] + beta * p[g];
  if (sc->pending && grid_last_block(ticket)) {
    sc->done = sc->pending;
    sc->pending = 0;
  }
}

// FP64 residual refresh: r64 = rhs - q64 ; rz64 = r64 . D^-1 r64.
// With r32 given: r32 = (float) r64, rz32 = r32 . D^-1 r32 (FP64 sum),
// x32 = 0, and p32 = D^-1 r32 when init_p.  With p64 given (FP64 solver
// start): p64 = D^-1 r64.
__global__ void __launch_bounds__(kBlock) refresh_kernel(int64_t n, const double *__restrict__ rhs,
                                                         const double *__restrict__ q64, const double *__restrict__ dinv64,
                                                         double *__restrict__ r64, double *__restrict__ p64,
                                                         const float *__restrict__ dinv32, float *__restrict__ r32,
                                                         float *__restrict__ p32, float *__restrict__ x32,
                                                         CgScalars *sc, double *partials, unsigned int *ticket) {
  double l64 = 0.0, l32 = 0.0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const double rv = rhs[g] - (q64 ? q64[g] : 0.0);
    r64[g] = rv;
    const double zv = dinv64[g] * rv;
    l64 += rv * zv;
    if (p64) p64[g] = zv;
    if (r32) {
      const float rf = (float)rv;
      r32[g] = rf;
      const float zf = dinv32[g] * rf;
      l32 += (double)rf * (double)zf;
      if (p32) p32[g] = zf;
      x32[g] = 0.0f;
    }
  }
  double t0, t1;
  if (grid_sum2<kBlock>(l64, l32, partials, ticket, &t0, &t1)) {
    sc->rz64 = t0;
    sc->rz32 = t1;
  }
}

template <typename T>
__global__ void fill_kernel(int64_t n, T *__restrict__ v, T value) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    v[g] = value;
}

// x64 += x32
__global__ void fold_kernel(int64_t n, double *__restrict__ x64, const float *__restrict__ x32) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    x64[g] += (double)x32[g];
}

template <typename T>
__global__ void convert_kernel(int64_t n, const double *__restrict__ src, T *__restrict__ dst) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    dst[g] = (T)src[g];
}

// diag = ridge^2 + stencil diagonal (+ data diagonal added by diag_data_kernel)
__global__ void diag_stencil_kernel(StencilCoef c, double *__restrict__ d) {
  const int64_t n = c.nx * c.ny * c.nz;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = g % c.nx, j = (g / c.nx) % c.ny, k = g / (c.nx * c.ny);
    d[g] = stencil_diag_node(c, i, j, k);
  }
}

// touched nodes: diag += sum over rows w2 (sum of the row's coefficients at
// the node)^2 -- a row may hold a node twice (P1 face rows, pair rows within
// one cell), and the node's incidences are sorted by row, so the entries of
// one row are adjacent; rhs = sum a w2 b
__global__ void data_node_setup_kernel(int64_t ntouched, const int64_t *__restrict__ touched,
                                       const int64_t *__restrict__ ptr, const int32_t *__restrict__ row,
                                       const double *__restrict__ ia, const double *__restrict__ w2,
                                       const double *__restrict__ b, double *__restrict__ diag,
                                       double *__restrict__ rhs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntouched;
       t += (int64_t)gridDim.x * blockDim.x) {
    double dd = 0.0, rr = 0.0, run = 0.0;
    int32_t prev = -1;
    for (int64_t e = ptr[t]; e < ptr[t + 1]; ++e) {
      const double a = ia[e];
      const int32_t r = row[e];
      if (r != prev) {
        if (prev >= 0) dd += w2[prev] * run * run;
        prev = r;
        run = a;
      } else {
        run += a;
      }
      rr += a * w2[r] * b[r];
    }
    if (prev >= 0) dd += w2[prev] * run * run;
    const int64_t g = touched[t];
    diag[g] += dd;
    rhs[g] = rr;
  }
}

// touched nodes: rhs = sum a w2 b (the right-hand side after the rows' b
// changed; same summation order as data_node_setup_kernel)
__global__ void data_node_rhs_kernel(int64_t ntouched, const int64_t *__restrict__ touched,
                                     const int64_t *__restrict__ ptr, const int32_t *__restrict__ row,
                                     const double *__restrict__ ia, const double *__restrict__ w2,
                                     const double *__restrict__ b, double *__restrict__ rhs) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntouched;
       t += (int64_t)gridDim.x * blockDim.x) {
    double rr = 0.0;
    for (int64_t e = ptr[t]; e < ptr[t + 1]; ++e) rr += ia[e] * w2[row[e]] * b[row[e]];
    rhs[touched[t]] = rr;
  }
}

// ADMM projection over inequality rows (loopsolver/admm_method.py:12-25 and
// the per-iteration update of loopsolver/admm_solver.py:380-404): for row r,
// qx = a_r . x, arg = qx + u, z = arg inside [lo, hi], else the bound it
// passed (z unchanged when arg is NaN), u += qx - z, and the row's new
// right-hand side b = z - u.  Five sums per block, in this order:
// (qx - z)^2, (z - z_prev)^2, qx^2, z^2, u^2.
constexpr int kAdmmSums = 5;

__global__ void __launch_bounds__(kBlock) admm_rows_kernel(int64_t m, int width, const int32_t *__restrict__ cols,
                                                           const double *__restrict__ a, const double *__restrict__ x,
                                                           const double *__restrict__ lo, const double *__restrict__ hi,
                                                           double *__restrict__ z, double *__restrict__ u,
                                                           double *__restrict__ b, double *__restrict__ partials) {
  __shared__ double red[kBlock / 32];
  double s[kAdmmSums] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    double qx = 0.0;
    for (int k = 0; k < width; ++k) {
      const int32_t c = cols[r * width + k];
      if (c >= 0) qx += a[r * width + k] * x[c];
    }
    const double zo = z[r], uo = u[r], l = lo[r], h = hi[r];
    const double arg = qx + uo;
    double zn = zo;
    if (arg >= l && arg <= h)
      zn = arg;
    else if (arg < l)
      zn = l;
    else if (arg > h)
      zn = h;
    const double un = (uo + qx) - zn;
    z[r] = zn;
    u[r] = un;
    b[r] = zn - un;
    s[0] += (qx - zn) * (qx - zn);
    s[1] += (zn - zo) * (zn - zo);
    s[2] += qx * qx;
    s[3] += zn * zn;
    s[4] += un * un;
  }
#pragma unroll
  for (int k = 0; k < kAdmmSums; ++k) {
    const double t = block_sum<kBlock, double>(s[k], red);
    if (threadIdx.x == 0) partials[kAdmmSums * blockIdx.x + k] = t;
  }
}

// fixed-order sum of the per-block partials of admm_rows_kernel (one block)
__global__ void __launch_bounds__(kBlock) admm_sum_kernel(int nblocks, const double *__restrict__ partials,
                                                          double *__restrict__ out) {
  __shared__ double red[kBlock / 32];
#pragma unroll
  for (int k = 0; k < kAdmmSums; ++k) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += kBlock) v += partials[kAdmmSums * i + k];
    v = block_sum<kBlock, double>(v, red);
    if (threadIdx.x == 0) out[k] = v;
  }
}

__global__ void dinv_kernel(int64_t n, const double *__restrict__ d, double *__restrict__ i64, float *__restrict__ i32) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const double v = d[g] > 0.0 ? 1.0 / d[g] : 1.0;
    i64[g] = v;
    i32[g] = (float)v;
  }
}

__global__ void norm2_kernel(int64_t n, const double *__restrict__ v, const double *__restrict__ w, CgScalars *sc,
                             double *partials, unsigned int *ticket) {
  double l = 0.0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    l += v[g] * (w[g] * v[g]);
  double tot;
  if (grid_sum<kBlock>(l, partials, ticket, &tot)) sc->scratch = tot;
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
template <typename P>
int dev_alloc(P **ptr, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void **)ptr, count * sizeof(P));
  if (e != cudaSuccess) {
    set_error("cudaMalloc(%zu bytes): %s", count * sizeof(P), cudaGetErrorString(e));
    return LS_ERR_ALLOC;
  }
  return LS_OK;
}

int grid_for(const ls_fd_handle *h, int64_t n) {
  int g = stream_grid(n, kBlock, 8);
  return std::min(g, h->red_blocks);
}

template <typename T>
const T *dir_weights(const ls_fd_handle *h) {
  if constexpr (sizeof(T) == 8)
    return h->dir64;
  else
    return h->dir32;
}

template <typename T>
DataView<T> data_view(const ls_fd_handle *h, const T *s_rows, const T *inc_a) {
  DataView<T> dv;
  dv.mask = h->data.mask;
  dv.word_rank = h->data.word_rank;
  dv.inc_ptr = h->data.inc_ptr;
  dv.inc_row = h->data.inc_row;
  dv.inc_a = inc_a;
  dv.s_rows = s_rows;
  dv.qd = nullptr;
  dv.enabled = h->data.ntouched > 0;
  dv.kmask = nullptr;
  dv.krank = nullptr;
  dv.k27 = nullptr;
  dv.knt = 0;
  return dv;
}

// the finest level's data rows for the TMA launcher (FP32; s = rows' w^2 a.p)
TmData tm_data(const ls_fd_handle *h, float *s) {
  const DataTerm &d = h->data;
  TmData t;
  t.nrows = d.nrows;
  t.ntouched = d.ntouched;
  t.width = d.width;
  t.cols = d.cols;
  t.a = d.a32;
  t.w2 = d.w2_32;
  t.touched = d.touched;
  t.inc_ptr = d.inc_ptr;
  t.inc_row = d.inc_row;
  t.inc_a = d.inc_a32;
  t.s = s;
  return t;
}

// q = N p (rows kernel + fused apply); p.q lands in sc->pq_s (deep box or full
// grid) and sc->pq_d (boundary shell of a split grid; stays 0 otherwise)
template <typename T>
void launch_apply(ls_fd_handle *h, const T *p, T *q, T *s, const T *a, const T *w2, const T *ia, bool check_done,
                  cudaStream_t st) {
  const DataTerm &d = h->data;
  const int *done = check_done ? &h->sc->done : nullptr;
  EpiArgs<T> e{};
  e.q = q;
  int staged = 0;
  if constexpr (sizeof(T) == 4) {
    staged = tm_launch<EPI_STORE>(h->tm, coef_as<float>(h->coef), p, tm_data(h, s), e, done, h->partials,
                                  h->tickets + T_STENCIL, &h->sc->pq_s, &h->sc->pq_d, &h->sc->fault,
                                  (int)std::min<int64_t>(h->partials_cap, 0x7fffffff), st);
  }
  if (staged > 0) {
    h->launches += staged;
  } else {
    if (d.nrows > 0) {
      rows_kernel<T><<<grid_for(h, d.nrows), kBlock, 0, st>>>(d.nrows, d.width, d.cols, a, w2, p, s, done);
      ++h->launches;
    }
    h->launches += launch_operator<T, EPI_STORE>(coef_as<T>(h->coef), p, data_view<T>(h, s, ia), e, done,
                                                 h->partials, h->tickets + T_STENCIL, &h->sc->pq_s,
                                                 h->tickets + T_SHELL, &h->sc->pq_d, h->red_blocks, st);
  }
  if (h->dir64) {  // q += D^T W D p in place; its share of p.q lands in pq_x
    const DirView<T> dv{(int)h->grid.nsteps[0], (int)h->grid.nsteps[1], (int)h->grid.nsteps[2], dir_weights<T>(h)};
    dir_apply_kernel<T, EPI_STORE><<<grid_for(h, h->n), 256, 0, st>>>(dv, p, q, e, done, h->partials,
                                                                     h->tickets + T_DIR, &h->sc->pq_x);
    ++h->launches;
  }
}

void launch_apply64(ls_fd_handle *h, const double *p, double *q, bool check_done, cudaStream_t st) {
  launch_apply<double>(h, p, q, h->s64, h->data.a64, h->data.w2_64, h->data.inc_a64, check_done, st);
}
void launch_apply32(ls_fd_handle *h, const float *p, float *q, bool check_done, cudaStream_t st) {
  launch_apply<float>(h, p, q, h->s32, h->data.a32, h->data.w2_32, h->data.inc_a32, check_done, st);
}

template <typename T>
void launch_iteration(ls_fd_handle *h, T *x, T *r, T *p, T *q, const T *dinv, cudaStream_t st) {
  if (sizeof(T) == 8)
    launch_apply64(h, (const double *)p, (double *)q, true, st);
  else
    launch_apply32(h, (const float *)p, (float *)q, true, st);
  const int g = grid_for(h, h->n);
  update_xr_kernel<T><<<g, kBlock, 0, st>>>(h->n, x, r, p, q, dinv, h->sc, h->partials, h->tickets + T_UPDATE);
  ++h->launches;
  update_p_kernel<T><<<g, kBlock, 0, st>>>(h->n, r, dinv, p, h->sc, h->tickets + T_PUPD);
  ++h->launches;
}

template <typename T>
int build_graph(ls_fd_handle *h, int batch, cudaGraphExec_t *out, int64_t *kernels, T *x, T *r, T *p, T *q,
                const T *dinv) {
  cudaStream_t st = h->stream;
  const int64_t before = h->launches;
  LS_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  for (int it = 0; it < batch; ++it) launch_iteration<T>(h, x, r, p, q, dinv, st);
  *kernels = h->launches - before;
  h->launches = before;
  cudaGraph_t graph;
  LS_CUDA_TRY(cudaStreamEndCapture(st, &graph));
  cudaError_t e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
    return LS_ERR_CUDA;
  }
  return LS_OK;
}

int read_scalars(ls_fd_handle *h) {
  LS_CUDA_TRY(cudaMemcpyAsync(h->sc_h, h->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, h->stream));
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (h->sc_h->fault) {  // sticky: the handle's results can no longer be trusted
    set_error("a TMA-staged operator apply gave up waiting for a tensor copy");
    return LS_ERR_CUDA;
  }
  return LS_OK;
}

int write_scalars(ls_fd_handle *h) {
  h->sc_h->pending = 0;
  LS_CUDA_TRY(cudaMemcpyAsync(h->sc, h->sc_h, sizeof(CgScalars), cudaMemcpyHostToDevice, h->stream));
  return LS_OK;
}

// true FP64 residual of x64: r64 = rhs - N x64 (and r32 / p32 / x32 when given)
int refresh(ls_fd_handle *h, bool have_x, float *r32, float *p32) {
  cudaStream_t st = h->stream;
  if (have_x) launch_apply64(h, h->x64, h->q64, false, st);
  refresh_kernel<<<grid_for(h, h->n), kBlock, 0, st>>>(h->n, h->rhs, have_x ? h->q64 : nullptr, h->dinv64, h->r64,
                                                       r32 ? nullptr : h->p64, h->dinv32, r32, p32, h->x32, h->sc,
                                                       h->partials, h->tickets + T_REFRESH);
  ++h->launches;
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}


// ---------------------------------------------------------------------------
// multigrid: hierarchy construction and the V-cycle launch sequence
// ---------------------------------------------------------------------------

template <typename P>
int mg_alloc(MgHierarchy &mg, P **ptr, size_t count) {
  LS_TRY(dev_alloc(ptr, count));
  mg.allocations.push_back((void *)*ptr);
  return LS_OK;
}

}  // namespace
int ensure_host_rows(ls_fd_handle *h);
namespace {

// Galerkin coarsening of data rows: row_c = row_f P (trilinear P, weights 1 / 1/2 per axis)
HostRows galerkin_rows(const HostRows &f, int nfx, int nfy, int ncx, int ncy) {
  HostRows c;
  c.nrows = f.nrows;
  c.width = 27;
  c.cols.assign((size_t)c.nrows * 27, -1);
  c.a.assign((size_t)c.nrows * 27, 0.0);
  c.w2 = f.w2;
  std::vector<std::pair<int64_t, double>> acc;
  for (int64_t r = 0; r < f.nrows; ++r) {
    acc.clear();
    for (int k = 0; k < f.width; ++k) {
      const int64_t col = f.cols[r * f.width + k];
      if (col < 0) continue;
      const double v = f.a[r * f.width + k];
      const int i = (int)(col % nfx), j = (int)((col / nfx) % nfy), kk = (int)(col / ((int64_t)nfx * nfy));
      int ci[2], cj[2], ck[2];
      double wi[2], wj[2], wk[2];
      const int ni = (i & 1) ? 2 : 1, nj = (j & 1) ? 2 : 1, nk = (kk & 1) ? 2 : 1;
      ci[0] = i >> 1; ci[1] = (i >> 1) + 1; wi[0] = wi[1] = (i & 1) ? 0.5 : 1.0;
      cj[0] = j >> 1; cj[1] = (j >> 1) + 1; wj[0] = wj[1] = (j & 1) ? 0.5 : 1.0;
      ck[0] = kk >> 1; ck[1] = (kk >> 1) + 1; wk[0] = wk[1] = (kk & 1) ? 0.5 : 1.0;
      for (int c3 = 0; c3 < nk; ++c3)
        for (int b = 0; b < nj; ++b)
          for (int a = 0; a < ni; ++a) {
            const int64_t cc = ci[a] + (int64_t)ncx * (cj[b] + (int64_t)ncy * ck[c3]);
            const double w = v * wi[a] * wj[b] * wk[c3];
            bool found = false;
            for (auto &e : acc)
              if (e.first == cc) {
                e.second += w;
                found = true;
                break;
              }
            if (!found) acc.emplace_back(cc, w);
          }
    }
    std::sort(acc.begin(), acc.end());
    for (size_t e = 0; e < acc.size() && e < 27; ++e) {
      c.cols[r * 27 + e] = acc[e].first;
      c.a[r * 27 + e] = acc[e].second;
    }
  }
  return c;
}

__global__ void mg_diag_finish_kernel(int64_t n, double *__restrict__ diag, int64_t ntouched,
                                      const int64_t *__restrict__ touched, const double *__restrict__ ddata) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntouched; t += (int64_t)gridDim.x * blockDim.x)
    diag[touched[t]] += ddata[t];
}

__global__ void mg_invert_kernel(int64_t n, const double *__restrict__ diag, float *__restrict__ dinv) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    dinv[g] = diag[g] > 0.0 ? (float)(1.0 / diag[g]) : 1.0f;
}

__global__ void mg_fill_hash_kernel(int64_t n, float *__restrict__ v) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)g * 2654435761u + 12345u;
    h ^= h >> 13;
    h *= 0x5bd1e995u;
    h ^= h >> 15;
    v[g] = 0.5f + (float)(h & 0xffffu) / 65536.0f;
  }
}

// device data of one level from host rows (incidence list, bit mask, FP32 copies)
// bit mask of the marked nodes (x-fastest words) and the rank of each word's first node
void node_mask(int64_t n, const std::vector<int64_t> &marked, std::vector<uint32_t> &mask, std::vector<int32_t> &wr) {
  const int64_t nwords = (n + 31) / 32;
  mask.assign(nwords, 0u);
  wr.assign(nwords, 0);
  for (int64_t t : marked) mask[t >> 5] |= 1u << (t & 31);
  int32_t run = 0;
  for (int64_t w = 0; w < nwords; ++w) {
    wr[w] = run;
    run += __builtin_popcount(mask[w]);
  }
}

// exclusive scan of int32 counts into int64 offsets (one block; setup time)
__global__ void __launch_bounds__(1024) setup_scan_kernel(const int32_t *__restrict__ cnt, int64_t n,
                                                          int64_t *__restrict__ off, int64_t *__restrict__ total) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = (i < n) ? cnt[i] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int64_t excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
    if (i < n) off[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// Splits the finest level's data rows into cell rows -- columns within one
// 2 x 2 x 2 box, every point row -- uploaded as (cell, 8 corner coefficients,
// w^2) for the device path of fd_mg_cells.cuh, and the other rows (interface
// pairs spanning two cells), kept in row form.
int mg_split_rows(ls_fd_handle *h, const HostRows &rows, int nx, int ny, int nz, CellRows &cr, HostRows &rest) {
  CellRowsHost hc;
  split_cell_rows(rows, nx, ny, nz, hc, rest);
  cr.nrows = hc.nrows();
  if (cr.nrows == 0) return LS_OK;
  LS_TRY(dev_alloc(&cr.ci, cr.nrows));
  LS_TRY(dev_alloc(&cr.cj, cr.nrows));
  LS_TRY(dev_alloc(&cr.ck, cr.nrows));
  LS_TRY(dev_alloc(&cr.c, 8 * cr.nrows));
  LS_TRY(dev_alloc(&cr.w2, cr.nrows));
  cudaStream_t st = h->stream;
  LS_CUDA_TRY(cudaMemcpyAsync(cr.ci, hc.ci.data(), cr.nrows * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaMemcpyAsync(cr.cj, hc.cj.data(), cr.nrows * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaMemcpyAsync(cr.ck, hc.ck.data(), cr.nrows * sizeof(int32_t), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaMemcpyAsync(cr.c, hc.c.data(), 8 * cr.nrows * sizeof(double), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaMemcpyAsync(cr.w2, hc.w2.data(), cr.nrows * sizeof(double), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  return LS_OK;
}

void free_cell_rows(CellRows &cr) {
  void *p[] = {cr.ci, cr.cj, cr.ck, cr.c, cr.w2};
  for (void *q : p)
    if (q) cudaFree(q);
  cr = CellRows{};
}

// The level's 27-point form of its (already coarsened) cell rows: the runs of
// rows per cell, the marked nodes, then one gather per marked node.
int mg_cells_k27(ls_fd_handle *h, MgLevel &lv, const CellRows &cr) {
  MgHierarchy &mg = h->mg;
  cudaStream_t st = h->stream;
  const int cx = lv.nx - 1, cy = lv.ny - 1, cz = lv.nz - 1;
  const int64_t ncells = (int64_t)cx * cy * cz, nwords = (lv.n + 31) / 32;
  int32_t *wcount = nullptr;
  int64_t *start = nullptr, *end = nullptr, *wrank = nullptr, *tot = nullptr;
  LS_CUDA_TRY(cudaMallocAsync((void **)&start, ncells * sizeof(int64_t), st));
  LS_CUDA_TRY(cudaMallocAsync((void **)&end, ncells * sizeof(int64_t), st));
  LS_CUDA_TRY(cudaMallocAsync((void **)&wcount, nwords * sizeof(int32_t), st));
  LS_CUDA_TRY(cudaMallocAsync((void **)&wrank, (nwords + 1) * sizeof(int64_t), st));
  LS_CUDA_TRY(cudaMallocAsync((void **)&tot, sizeof(int64_t), st));
  LS_CUDA_TRY(cudaMemsetAsync(start, 0, ncells * sizeof(int64_t), st));
  LS_CUDA_TRY(cudaMemsetAsync(end, 0, ncells * sizeof(int64_t), st));
  cell_segments_kernel<<<grid_for(h, cr.nrows), kBlock, 0, st>>>(cr.nrows, cr.ci, cr.cj, cr.ck, cx, cy, start, end);
  LS_TRY(mg_alloc(mg, &lv.kmask, nwords));
  LS_TRY(mg_alloc(mg, &lv.krank, nwords));
  cell_touch_kernel<<<grid_for(h, nwords * 32), kBlock, 0, st>>>(lv.nx, lv.ny, lv.nz, start, end, lv.kmask, wcount);
  setup_scan_kernel<<<1, 1024, 0, st>>>(wcount, nwords, wrank, tot);
  h->launches += 3;
  int64_t knt = 0;
  LS_CUDA_TRY(cudaMemcpyAsync(&knt, tot, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  lv.knt = knt;
  if (knt > 0) {
    LS_TRY(mg_alloc(mg, &lv.k27, (size_t)27 * knt));
    cell_k27_kernel<<<grid_for(h, lv.n), kBlock, 0, st>>>(lv.nx, lv.ny, lv.nz, lv.kmask, wrank, start, end, cr.c,
                                                          cr.w2, knt, lv.k27, lv.krank);
    ++h->launches;
  }
  LS_CUDA_TRY(cudaGetLastError());
  void *tmp[] = {start, end, wcount, wrank, tot};
  for (void *q : tmp) LS_CUDA_TRY(cudaFreeAsync(q, st));
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  return LS_OK;
}

// host copies of the coarsest level's 27-point form (dense coarsest matrix)
int mg_k27_to_host(MgLevel &lv, cudaStream_t st) {
  lv.k27host.clear();
  lv.k27nodes.clear();
  if (lv.knt == 0) return LS_OK;
  const int64_t nwords = (lv.n + 31) / 32;
  std::vector<uint32_t> mask(nwords);
  lv.k27host.resize((size_t)27 * lv.knt);
  LS_CUDA_TRY(cudaMemcpyAsync(mask.data(), lv.kmask, nwords * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  LS_CUDA_TRY(cudaMemcpyAsync(lv.k27host.data(), lv.k27, lv.k27host.size() * sizeof(float), cudaMemcpyDeviceToHost,
                              st));
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  for (int64_t g = 0; g < lv.n; ++g)
    if (mask[g >> 5] & (1u << (g & 31))) lv.k27nodes.push_back(g);
  return LS_OK;
}

int mg_upload_level(ls_fd_handle *h, MgLevel &lv, const HostRows &rows, std::vector<int64_t> &touched,
                    std::vector<double> &data_diag) {
  MgHierarchy &mg = h->mg;
  const int64_t ne = rows.nrows * rows.width;
  std::vector<int32_t> cols(ne);
  std::vector<float> a32(ne), w2(rows.nrows);
  std::vector<std::pair<int64_t, int64_t>> inc;
  inc.reserve(ne);
  for (int64_t e = 0; e < ne; ++e) {
    cols[e] = rows.cols[e] < 0 ? -1 : (int32_t)rows.cols[e];
    a32[e] = (float)rows.a[e];
    if (rows.cols[e] >= 0) inc.emplace_back(rows.cols[e], e);
  }
  for (int64_t r = 0; r < rows.nrows; ++r) w2[r] = (float)rows.w2[r];
  std::stable_sort(inc.begin(), inc.end(), [](const std::pair<int64_t, int64_t> &x, const std::pair<int64_t, int64_t> &y) {
    return x.first < y.first;
  });
  std::vector<int64_t> ptr;
  std::vector<int32_t> irow;
  std::vector<float> ia;
  touched.clear();
  data_diag.clear();
  for (size_t t = 0; t < inc.size(); ++t) {
    if (t == 0 || inc[t].first != inc[t - 1].first) {
      touched.push_back(inc[t].first);
      ptr.push_back((int64_t)t);
      data_diag.push_back(0.0);
    }
    const int64_t e = inc[t].second, r = e / rows.width;
    irow.push_back((int32_t)r);
    ia.push_back((float)rows.a[e]);
    data_diag.back() += rows.w2[r] * rows.a[e] * rows.a[e];
  }
  ptr.push_back((int64_t)inc.size());
  const int64_t nwords = (lv.n + 31) / 32;
  std::vector<uint32_t> mask;
  std::vector<int32_t> wr;
  node_mask(lv.n, touched, mask, wr);
  lv.nrows = rows.nrows;
  lv.width = rows.width;
  lv.ntouched = (int64_t)touched.size();
  const int64_t ni = (int64_t)inc.size();
  LS_TRY(mg_alloc(mg, &lv.cols, ne));
  LS_TRY(mg_alloc(mg, &lv.a, ne));
  LS_TRY(mg_alloc(mg, &lv.w2, rows.nrows));
  LS_TRY(mg_alloc(mg, &lv.s, rows.nrows));
  LS_TRY(mg_alloc(mg, &lv.mask, nwords));
  LS_TRY(mg_alloc(mg, &lv.word_rank, nwords));
  LS_TRY(mg_alloc(mg, &lv.inc_ptr, lv.ntouched + 1));
  LS_TRY(mg_alloc(mg, &lv.inc_row, ni));
  LS_TRY(mg_alloc(mg, &lv.inc_a, ni));
  if (lv.ntouched > 0 && ni > 16 * lv.ntouched) LS_TRY(mg_alloc(mg, &lv.qd, lv.ntouched));
  cudaStream_t st = h->stream;
#define UPL(dst, src, cnt) \
  if ((cnt) > 0) LS_CUDA_TRY(cudaMemcpyAsync(dst, (src).data(), (cnt) * sizeof((src)[0]), cudaMemcpyHostToDevice, st));
  UPL(lv.cols, cols, ne);
  UPL(lv.a, a32, ne);
  UPL(lv.w2, w2, rows.nrows);
  UPL(lv.mask, mask, nwords);
  UPL(lv.word_rank, wr, nwords);
  UPL(lv.inc_ptr, ptr, lv.ntouched + 1);
  UPL(lv.inc_row, irow, ni);
  UPL(lv.inc_a, ia, ni);
#undef UPL
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  return LS_OK;
}

DataView<float> mg_view(const MgLevel &lv) {
  DataView<float> dv;
  dv.mask = lv.mask;
  dv.word_rank = lv.word_rank;
  dv.inc_ptr = lv.inc_ptr;
  dv.inc_row = lv.inc_row;
  dv.inc_a = lv.inc_a;
  dv.s_rows = lv.s;
  dv.qd = lv.qd;
  dv.enabled = lv.ntouched > 0;
  dv.kmask = lv.kmask;
  dv.krank = lv.krank;
  dv.k27 = lv.knt > 0 ? lv.k27 : nullptr;
  dv.knt = lv.knt;
  return dv;
}

DirCoarse dir_coarse(const MgLevel &lv) {
  DirCoarse dc;
  dc.nx = lv.nx;
  dc.ny = lv.ny;
  dc.nz = lv.nz;
  for (int a = 0; a < 3; ++a) dc.t[a] = lv.g1op.t[a];
  dc.sw = lv.dsw;
  return dc;
}

// q = A_l p on level l (rows + fused apply with an epilogue)
template <int EPI>
void mg_apply(ls_fd_handle *h, const MgLevel &lv, const float *p, const EpiArgs<float> &e, const int *done,
              cudaStream_t st) {
  if (&lv == &h->mg.levels[0] && h->tm.enabled) {
    // finest level: the TMA-staged kernel (isotropic + data; with directional
    // terms it stores to dq and the directional kernel completes the epilogue)
    EpiArgs<float> es{};
    es.q = lv.dq;
    const TmData td = tm_data(h, lv.s);
    const int staged =
        lv.dir ? tm_launch<EPI_STORE>(h->tm, lv.coef, p, td, es, done, nullptr, nullptr, nullptr, nullptr,
                                      &h->sc->fault, h->red_blocks, st)
               : tm_launch<EPI>(h->tm, lv.coef, p, td, e, done, nullptr, nullptr, nullptr, nullptr, &h->sc->fault,
                                h->red_blocks, st);
    if (staged > 0) {
      h->launches += staged;
      if (lv.dir) {
        const DirView<float> dv{lv.nx, lv.ny, lv.nz, lv.dir};
        dir_apply_kernel<float, EPI><<<grid_for(h, lv.n), 256, 0, st>>>(dv, p, lv.dq, e, done, nullptr, nullptr,
                                                                       nullptr);
        ++h->launches;
      }
      return;
    }
  }
  if (lv.nrows > 0) {
    rows_kernel<float><<<grid_for(h, lv.nrows), kBlock, 0, st>>>(lv.nrows, lv.width, lv.cols, lv.a, lv.w2, p, lv.s, done);
    ++h->launches;
  }
  if (lv.qd) {
    data_nodes_warp_kernel<float><<<std::max<int64_t>(1, std::min<int64_t>((lv.ntouched * 32 + 255) / 256, 8 * sm_count())), 256, 0, st>>>(
        lv.ntouched, lv.inc_ptr, lv.inc_row, lv.inc_a, lv.s, lv.qd, done);
    ++h->launches;
  }
  if (lv.dir) {
    // isotropic part stored to dq, then the directional kernel adds its term
    // and runs the epilogue
    EpiArgs<float> es{};
    es.q = lv.dq;
    if (lv.g1)
      h->launches += launch_g1<EPI_STORE>(lv.g1op, p, mg_view(lv), es, done, h->red_blocks / 8, st);
    else
      h->launches += launch_operator<float, EPI_STORE>(lv.coef, p, mg_view(lv), es, done, nullptr, nullptr, nullptr,
                                                       nullptr, nullptr, h->red_blocks, st);
    if (lv.dsw) {  // coarse level: S G S in three passes
      const DirCoarse dc = dir_coarse(lv);
      const int g = grid_for(h, lv.n);
      dir_coarse_x_kernel<<<g, 256, 0, st>>>(dc, p, h->mg.dir_u, done);
      dir_coarse_y_kernel<<<g, 256, 0, st>>>(dc, h->mg.dir_u, h->mg.dir_v, done);
      dir_coarse_z_kernel<EPI><<<g, 256, 0, st>>>(dc, h->mg.dir_v, p, lv.dq, e, done);
      h->launches += 3;
    } else {  // finest level: the exact term
      const DirView<float> dv{lv.nx, lv.ny, lv.nz, lv.dir};
      dir_apply_kernel<float, EPI><<<grid_for(h, lv.n), 256, 0, st>>>(dv, p, lv.dq, e, done, nullptr, nullptr, nullptr);
      ++h->launches;
    }
    return;
  }
  if (lv.g1)
    h->launches += launch_g1<EPI>(lv.g1op, p, mg_view(lv), e, done, h->red_blocks / 8, st);
  else
    h->launches += launch_operator<float, EPI>(lv.coef, p, mg_view(lv), e, done, nullptr, nullptr, nullptr, nullptr,
                                               nullptr, h->red_blocks, st);
}

// one Gauss-Jordan step on the augmented nc x 2nc matrix: row c divided by
// the pivot, every other row r minus in[r][c] times the new row c
__global__ void mg_gj_step_kernel(int nc, int c, double tiny, const double *__restrict__ in, double *__restrict__ out) {
  const int w = 2 * nc;
  double piv = in[(size_t)c * w + c];
  if (fabs(piv) < tiny) piv = piv < 0.0 ? -tiny : tiny;
  const int64_t total = (int64_t)nc * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / w), k = (int)(t - (int64_t)r * w);
    const double rowc = in[(size_t)c * w + k] / piv;
    out[t] = (r == c) ? rowc : in[t] - in[(size_t)r * w + c] * rowc;
  }
}

// The whole Gauss-Jordan elimination in one cooperative launch on the same
// ping-pong buffers, one grid-wide sync per pivot.  At step c only the columns
// c .. nc+c change: the left columns before c are already unit vectors and the
// right columns after nc+c are still the identity's, and neither is read again
// before it enters that window, so both buffers start as [A | I] and the
// window alone is written.  The cooperative launch guarantees that every
// block is resident, so the sync cannot wait on a block that never runs.
__global__ void mg_gj_coop_kernel(int nc, double tiny, double *b0, double *b1) {
  cooperative_groups::grid_group grid = cooperative_groups::this_grid();
  const int w = 2 * nc, span = nc + 1;
  const int64_t total = (int64_t)nc * span;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  for (int c = 0; c < nc; ++c) {
    const double *in = (c & 1) ? b1 : b0;
    double *out = (c & 1) ? b0 : b1;
    double piv = in[(size_t)c * w + c];
    if (fabs(piv) < tiny) piv = piv < 0.0 ? -tiny : tiny;
    for (int64_t t = tid; t < total; t += stride) {
      const int r = (int)(t / span), k = c + (int)(t - (int64_t)r * span);
      const double rowc = in[(size_t)c * w + k] / piv;
      out[(size_t)r * w + k] = (r == c) ? rowc : in[(size_t)r * w + k] - in[(size_t)r * w + c] * rowc;
    }
    grid.sync();
  }
}

int mg_read_scalar(ls_fd_handle *h, double *dev, double *out) {
  LS_CUDA_TRY(cudaMemcpyAsync(out, dev, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return LS_OK;
}

int mg_lambda_max(ls_fd_handle *h, MgLevel &lv, float *lmax_out) {
  cudaStream_t st = h->stream;
  const int g = grid_for(h, lv.n);
  float *v = lv.d0, *q = lv.d1;
  mg_fill_hash_kernel<<<g, kBlock, 0, st>>>(lv.n, v);
  ++h->launches;
  double nv = 0.0, nq = 0.0;
  double *slot = &h->sc->scratch;
  mg_dot_kernel<<<g, 256, 0, st>>>(lv.n, v, v, nullptr, h->partials, h->tickets + T_MISC, slot);
  ++h->launches;
  LS_TRY(mg_read_scalar(h, slot, &nv));
  double lam = 0.0;
  for (int it = 0; it < 20; ++it) {
    mg_scale_kernel<<<g, kBlock, 0, st>>>(lv.n, v, nullptr, (float)(1.0 / sqrt(nv)), v);
    ++h->launches;
    EpiArgs<float> e{};
    e.q = q;
    mg_apply<EPI_STORE>(h, lv, v, e, nullptr, st);
    mg_scale_kernel<<<g, kBlock, 0, st>>>(lv.n, q, lv.dinv, 1.0f, v);
    ++h->launches;
    mg_dot_kernel<<<g, 256, 0, st>>>(lv.n, v, v, nullptr, h->partials, h->tickets + T_MISC, slot);
    ++h->launches;
    LS_TRY(mg_read_scalar(h, slot, &nq));
    lam = sqrt(nq);  // |D^-1 A v| with |v| = 1
    nv = nq;
    if (!(nv > 0.0) || !isfinite(nv)) break;
  }
  LS_CUDA_TRY(cudaGetLastError());
  *lmax_out = (float)(lam > 0.0 && isfinite(lam) ? lam : 1.0);
  return LS_OK;
}

// dense inverse of the coarsest operator (FP64): assembled on the host,
// inverted by Gauss-Jordan on the GPU
int mg_coarse_inverse(ls_fd_handle *h, MgLevel &lv) {
  MgHierarchy &mg = h->mg;
  cudaStream_t st = h->stream;
  const int nc = (int)lv.n;
  std::vector<double> A((size_t)nc * nc, 0.0);
  if (lv.g1 && lv.g1op.shell_coef && lv.nrows == 0) {
    // the level's explicit stencils (every node of a small Galerkin level) and
    // its 27-point data term: the matrix without a single operator apply
    std::vector<float> coef((size_t)125 * nc);
    LS_CUDA_TRY(cudaMemcpy(coef.data(), lv.g1op.shell_coef, coef.size() * sizeof(float), cudaMemcpyDeviceToHost));
    const int nx = lv.nx, ny = lv.ny, nz = lv.nz;
    auto put = [&](int i, int dx, int dy, int dz, double v) {
      const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
      if (x + dx < 0 || x + dx >= nx || y + dy < 0 || y + dy >= ny || z + dz < 0 || z + dz >= nz) return;
      A[(size_t)i * nc + (i + dz * nx * ny + dy * nx + dx)] += v;
    };
    for (int i = 0; i < nc; ++i)
      for (int o = 0; o < 125; ++o) put(i, o % 5 - 2, (o / 5) % 5 - 2, o / 25 - 2, coef[(size_t)o * nc + i]);
    const int64_t nt = (int64_t)lv.k27nodes.size();
    for (int64_t t = 0; t < nt; ++t)
      for (int o = 0; o < 27; ++o)
        put((int)lv.k27nodes[t], o % 3 - 1, (o / 3) % 3 - 1, o / 9 - 1, lv.k27host[(size_t)o * nt + t]);
    if (lv.dsw) {
      // sum_f S_f (Tx_f (x) Ty_f (x) Tz_f) S_f from the FP64 tables
      std::vector<float> sw((size_t)kDirFamilies * nc);
      LS_CUDA_TRY(cudaMemcpy(sw.data(), lv.dsw, sw.size() * sizeof(float), cudaMemcpyDeviceToHost));
      const int nn[3] = {nx, ny, nz};
      auto tab = [&](int a, int f, int idx, int o) { return lv.g1host[a][((size_t)g1_kind(f, a) * nn[a] + idx) * 5 + o + 2]; };
      for (int g = 0; g < nc; ++g) {
        const int x = g % nx, y = (g / nx) % ny, z = g / (nx * ny);
        for (int f = 0; f < kDirFamilies; ++f) {
          const double sg = sw[(size_t)f * nc + g];
          if (sg == 0.0) continue;
          for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
              for (int dx = -2; dx <= 2; ++dx) {
                if (x + dx < 0 || x + dx >= nx || y + dy < 0 || y + dy >= ny || z + dz < 0 || z + dz >= nz) continue;
                const int g2 = g + dz * nx * ny + dy * nx + dx;
                const double t = tab(0, f, x, dx) * tab(1, f, y, dy) * tab(2, f, z, dz);
                if (t != 0.0) A[(size_t)g * nc + g2] += sg * t * sw[(size_t)f * nc + g2];
              }
        }
      }
    }
  } else {
    std::vector<float> col(nc);
    const float one = 1.0f;
    for (int j = 0; j < nc; ++j) {
      LS_CUDA_TRY(cudaMemsetAsync(lv.d0, 0, nc * sizeof(float), st));
      LS_CUDA_TRY(cudaMemcpyAsync(lv.d0 + j, &one, sizeof(float), cudaMemcpyHostToDevice, st));
      EpiArgs<float> e{};
      e.q = lv.d1;
      mg_apply<EPI_STORE>(h, lv, lv.d0, e, nullptr, st);
      LS_CUDA_TRY(cudaMemcpyAsync(col.data(), lv.d1, nc * sizeof(float), cudaMemcpyDeviceToHost, st));
      LS_CUDA_TRY(cudaStreamSynchronize(st));
      for (int i = 0; i < nc; ++i) A[(size_t)i * nc + j] = col[i];
    }
  }
  // symmetrise (the FP32 apply is symmetric up to rounding)
  for (int i = 0; i < nc; ++i)
    for (int j = i + 1; j < nc; ++j) {
      const double m = 0.5 * (A[(size_t)i * nc + j] + A[(size_t)j * nc + i]);
      A[(size_t)i * nc + j] = A[(size_t)j * nc + i] = m;
    }
  // Gauss-Jordan on the GPU: [A | I] -> [I | A^-1] (every element of step c
  // reads row c and column c of the previous matrix).  No pivoting: the coarsest operator is symmetric
  // positive definite (Galerkin products of SPD operators plus the ridge); a
  // vanishing pivot is replaced by +-1e-14 max|diag| as a guard.
  double maxdiag = 0.0;
  for (int i = 0; i < nc; ++i) maxdiag = std::max(maxdiag, fabs(A[(size_t)i * nc + i]));
  const int w = 2 * nc;
  std::vector<double> aug((size_t)nc * w, 0.0);
  for (int i = 0; i < nc; ++i) {
    std::copy(A.begin() + (size_t)i * nc, A.begin() + (size_t)(i + 1) * nc, aug.begin() + (size_t)i * w);
    aug[(size_t)i * w + nc + i] = 1.0;
  }
  double *buf[2] = {nullptr, nullptr};
  LS_TRY(dev_alloc(&buf[0], (size_t)nc * w));
  LS_TRY(dev_alloc(&buf[1], (size_t)nc * w));
  LS_CUDA_TRY(cudaMemcpyAsync(buf[0], aug.data(), aug.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  LS_CUDA_TRY(cudaMemcpyAsync(buf[1], buf[0], aug.size() * sizeof(double), cudaMemcpyDeviceToDevice, st));
  // one cooperative launch sized to the resident capacity; if the device
  // refuses it, one launch per pivot on ping-pong buffers
  double tiny = 1e-14 * maxdiag;
  int per_sm = 0, dev = 0, coop = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mg_gj_coop_kernel, 256, 0);
  const int64_t want = ((int64_t)nc * w + 255) / 256;
  const int cgs = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)nc * (nc + 1) + 255) / 256,
                                                              (int64_t)per_sm * sm_count()));
  void *args[] = {(void *)&nc, (void *)&tiny, (void *)&buf[0], (void *)&buf[1]};
  if (coop && per_sm > 0 &&
      cudaLaunchCooperativeKernel((void *)mg_gj_coop_kernel, dim3(cgs), dim3(256), args, 0, st) == cudaSuccess) {
    ++h->launches;
  } else {
    cudaGetLastError();
    const int gs = (int)std::min<int64_t>(want, 8 * sm_count());
    for (int c = 0; c < nc; ++c) {
      mg_gj_step_kernel<<<gs, 256, 0, st>>>(nc, c, tiny, buf[c & 1], buf[(c + 1) & 1]);
      ++h->launches;
    }
  }
  LS_CUDA_TRY(cudaGetLastError());
  const int result = nc & 1;
  LS_TRY(mg_alloc(mg, &mg.coarse_inv64, (size_t)nc * nc));
  LS_CUDA_TRY(cudaMemcpy2DAsync(mg.coarse_inv64, nc * sizeof(double), buf[result] + nc, w * sizeof(double),
                                nc * sizeof(double), nc, cudaMemcpyDeviceToDevice, st));
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(buf[0]);
  cudaFree(buf[1]);
  return LS_OK;
}

int mg_level_dinv(ls_fd_handle *h, MgLevel &lv, const std::vector<int64_t> &touched,
                  const std::vector<double> &data_diag) {
  cudaStream_t st = h->stream;
  double *diag = nullptr;
  int64_t *dt = nullptr;
  double *dd = nullptr;
  LS_TRY(dev_alloc(&diag, lv.n));
  LS_TRY(dev_alloc(&dt, touched.size()));
  LS_TRY(dev_alloc(&dd, data_diag.size()));
  if (!touched.empty()) {
    LS_CUDA_TRY(cudaMemcpyAsync(dt, touched.data(), touched.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    LS_CUDA_TRY(cudaMemcpyAsync(dd, data_diag.data(), data_diag.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  const int g = grid_for(h, lv.n);
  if (lv.g1)
    g1_diag_kernel<<<g, kBlock, 0, st>>>(lv.g1op, diag);
  else
    diag_stencil_kernel<<<g, kBlock, 0, st>>>(lv.coef64, diag);
  ++h->launches;
  if (lv.dsw) {
    dir_coarse_diag_kernel<<<g, kBlock, 0, st>>>(dir_coarse(lv), lv.dir, diag);
    ++h->launches;
  }
  if (lv.knt > 0) {
    k27_diag_kernel<<<g, kBlock, 0, st>>>(lv.n, lv.kmask, lv.krank, lv.k27, lv.knt, diag);
    ++h->launches;
  }
  if (!touched.empty()) {
    mg_diag_finish_kernel<<<grid_for(h, (int64_t)touched.size()), kBlock, 0, st>>>(lv.n, diag, (int64_t)touched.size(), dt, dd);
    ++h->launches;
  }
  mg_invert_kernel<<<g, kBlock, 0, st>>>(lv.n, diag, lv.dinv);
  ++h->launches;
  LS_CUDA_TRY(cudaStreamSynchronize(st));
  cudaFree(diag);
  cudaFree(dt);
  cudaFree(dd);
  return LS_OK;
}

StencilCoef coarsen_coef(const StencilCoef &f, int nx, int ny, int nz) {
  StencilCoef c = f;
  c.nx = nx;
  c.ny = ny;
  c.nz = nz;
  c.xx_int *= 0.5;
  c.yy_int *= 0.5;
  c.zz_int *= 0.5;
  c.xy *= 0.5;
  c.xz *= 0.5;
  c.yz *= 0.5;
  c.xx_bdr = nx >= 3 ? f.xx_bdr * 0.25 : 0.0;
  c.yy_bdr = ny >= 3 ? f.yy_bdr * 0.25 : 0.0;
  c.zz_bdr = nz >= 3 ? f.zz_bdr * 0.25 : 0.0;
  c.ridge2 *= 8.0;
  return c;
}

// 1-D banded coarse matrices P^T X P of the Galerkin operator along one axis
// (nf fine nodes, nc = nf/2 + 1 coarse nodes): out[kind][J][d + 2] for
// offsets d = -2..2 (0 past the ends).
void g1_tables_1d(int nf, int nc, std::vector<double> &out) {
  out.assign((size_t)G1_KINDS * nc * 5, 0.0);
  auto pw = [&](int i, int J) -> double {  // trilinear prolongation weight P[i][J]
    const int d = i - 2 * J;
    return d == 0 ? 1.0 : (d == 1 || d == -1) ? 0.5 : 0.0;
  };
  auto interior = [&](int c) { return (c >= 1 && c <= nf - 2) ? 1.0 : 0.0; };
  auto border = [&](int c) { return (double)((c == 1) + (c == nf - 2)); };
  // X[i][j] for each kind: sum over row centres c of m(c) D[c][i] D[c][j]
  auto X = [&](int kind, int i, int j) -> double {
    if (kind == G1_MI) return i == j ? interior(i) : 0.0;
    if (kind == G1_M0) return i == j ? 1.0 : 0.0;
    double acc = 0.0;
    for (int c = std::max(i, j) - 1; c <= std::min(i, j) + 1; ++c) {
      if (c < 0 || c >= nf) continue;
      const double m = kind == G1_D2B ? border(c) : interior(c);
      if (m == 0.0) continue;
      auto tap = [&](int node) -> double {
        const int o = node - c;
        if (kind == G1_D1I) return o == -1 ? -1.0 : o == 1 ? 1.0 : 0.0;
        return o == 0 ? -2.0 : (o == 1 || o == -1) ? 1.0 : 0.0;
      };
      acc += m * tap(i) * tap(j);
    }
    return acc;
  };
  for (int kind = 0; kind < G1_KINDS; ++kind)
    for (int J = 0; J < nc; ++J)
      for (int d = -2; d <= 2; ++d) {
        const int K = J + d;
        if (K < 0 || K >= nc) continue;
        double v = 0.0;
        for (int i = 2 * J - 1; i <= 2 * J + 1; ++i) {
          if (i < 0 || i >= nf) continue;
          for (int j = 2 * K - 1; j <= 2 * K + 1; ++j) {
            if (j < 0 || j >= nf) continue;
            v += pw(i, J) * X(kind, i, j) * pw(j, K);
          }
        }
        out[((size_t)kind * nc + J) * 5 + d + 2] = v;
      }
}

// P^T T P of banded 1-D tables T (nf nodes) onto nc = nf/2 + 1 coarse nodes
void g1_tables_coarsen(const std::vector<double> &tf, int nf, int nc, std::vector<double> &out) {
  out.assign((size_t)G1_KINDS * nc * 5, 0.0);
  auto pw = [&](int i, int J) -> double {
    const int d = i - 2 * J;
    return d == 0 ? 1.0 : (d == 1 || d == -1) ? 0.5 : 0.0;
  };
  for (int kind = 0; kind < G1_KINDS; ++kind)
    for (int J = 0; J < nc; ++J)
      for (int d = -2; d <= 2; ++d) {
        const int K = J + d;
        if (K < 0 || K >= nc) continue;
        double v = 0.0;
        for (int i = 2 * J - 1; i <= 2 * J + 1; ++i) {
          if (i < 0 || i >= nf) continue;
          for (int j = 2 * K - 1; j <= 2 * K + 1; ++j) {
            if (j < 0 || j >= nf || j - i < -2 || j - i > 2) continue;
            v += pw(i, J) * tf[((size_t)kind * nf + i) * 5 + (j - i) + 2] * pw(j, K);
          }
        }
        out[((size_t)kind * nc + J) * 5 + d + 2] = v;
      }
}

// the Galerkin regularisation operator of coarse level c of fine level f
// (tables from the fine stencil for the first coarse level, else by
// coarsening the fine level's tables)
int mg_build_g1(ls_fd_handle *h, MgHierarchy &mg, const MgLevel &f, MgLevel &c) {
  G1Op &g = c.g1op;
  g.nx = c.nx;
  g.ny = c.ny;
  g.nz = c.nz;
  const StencilCoef &k = mg.levels[0].coef64;  // G_l = P^T G_{l-1} P keeps the fine weights
  const double w[kG1Families] = {k.xx_int, k.yy_int, k.zz_int, k.xy, k.xz, k.yz, k.xx_bdr, k.yy_bdr, k.zz_bdr,
                                 k.ridge2};
  for (int fm = 0; fm < kG1Families; ++fm) g.w[fm] = (float)w[fm];
  const int nf[3] = {f.nx, f.ny, f.nz}, nc[3] = {c.nx, c.ny, c.nz};
  double irow[3][G1_KINDS][5];
  for (int a = 0; a < 3; ++a) {
    std::vector<double> &t = c.g1host[a];
    if (f.g1)
      g1_tables_coarsen(f.g1host[a], nf[a], nc[a], t);
    else
      g1_tables_1d(nf[a], nc[a], t);
    const int mid = nc[a] / 2;
    auto same = [&](int J) {
      for (int kind = 0; kind < G1_KINDS; ++kind)
        for (int d = 0; d < 5; ++d) {
          const double x = t[((size_t)kind * nc[a] + J) * 5 + d], y = t[((size_t)kind * nc[a] + mid) * 5 + d];
          if (fabs(x - y) > 1e-12 * (fabs(y) + 1.0)) return false;
        }
      return true;
    };
    int lo = mid, hi = mid;
    while (lo - 1 >= 2 && same(lo - 1)) --lo;
    while (hi + 1 <= nc[a] - 3 && same(hi + 1)) ++hi;
    if (!same(mid) || nc[a] < 5) {
      lo = 1;
      hi = 0;  // no interior: every node through the tables
    }
    g.lo[a] = lo;
    g.hi[a] = hi;
    for (int kind = 0; kind < G1_KINDS; ++kind)
      for (int d = 0; d < 5; ++d) irow[a][kind][d] = t[((size_t)kind * nc[a] + mid) * 5 + d];
    std::vector<float> t32(t.begin(), t.end());
    float *dt = nullptr;
    LS_TRY(mg_alloc(mg, &dt, t32.size()));
    LS_CUDA_TRY(cudaMemcpyAsync(dt, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    g.t[a] = dt;
  }
  for (int m = 0; m < 3; ++m)
    for (int dy = 0; dy < 5; ++dy)
      for (int dx = 0; dx < 5; ++dx) {
        double acc = 0.0;
        for (int fm = 0; fm < kG1Families; ++fm)
          acc += w[fm] * irow[0][g1_kind(fm, 0)][dx] * irow[1][g1_kind(fm, 1)][dy] * irow[2][g1_kind(fm, 2)][m + 2];
        g.c[m][dy][dx] = (float)acc;
      }
  // face stencils: one axis in its band (rows differ), the other two interior
  {
    std::vector<float> fcv((size_t)3 * kG1MaxBand * 125, 0.f);
    for (int a = 0; a < 3; ++a)
      for (int row = 0; row < kG1MaxBand; ++row) {
        const int half = kG1MaxBand / 2;
        const int idx = row < half ? row : nc[a] - 1 - (row - half);
        const bool band = row < half ? (idx < g.lo[a] && g.lo[a] <= half) : (idx > g.hi[a] && nc[a] - 1 - g.hi[a] <= half);
        if (!band || idx < 0 || idx >= nc[a]) continue;
        const std::vector<double> &t = c.g1host[a];
        for (int o = 0; o < 125; ++o) {
          const int d[3] = {o % 5, (o / 5) % 5, o / 25};  // dx, dy, dz (+2)
          double acc = 0.0;
          for (int fm = 0; fm < kG1Families; ++fm) {
            double prod = w[fm];
            for (int b = 0; b < 3; ++b) {
              const int kind = g1_kind(fm, b);
              prod *= b == a ? t[((size_t)kind * nc[a] + idx) * 5 + d[b]] : irow[b][kind][d[b]];
            }
            acc += prod;
          }
          fcv[((size_t)a * kG1MaxBand + row) * 125 + o] = (float)acc;
        }
      }
    float *dfc = nullptr;
    LS_TRY(mg_alloc(mg, &dfc, fcv.size()));
    LS_CUDA_TRY(cudaMemcpyAsync(dfc, fcv.data(), fcv.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    g.face_coef = dfc;
  }
  // edge stencils: two axes in their bands, the third interior
  {
    const int half = kG1MaxBand / 2;
    std::vector<float> ecv((size_t)3 * kG1MaxBand * kG1MaxBand * 125, 0.f);
    auto band_idx = [&](int a, int row) -> int {  // node index of band row `row` on axis a, or -1
      const int idx = row < half ? row : nc[a] - 1 - (row - half);
      const bool band = row < half ? (idx < g.lo[a] && g.lo[a] <= half) : (idx > g.hi[a] && nc[a] - 1 - g.hi[a] <= half);
      return (band && idx >= 0 && idx < nc[a]) ? idx : -1;
    };
    for (int out = 0; out < 3; ++out) {
      const int pa = out == 0 ? 1 : 0, pb = out == 2 ? 1 : 2, pair = 2 - out;
      for (int ra = 0; ra < kG1MaxBand; ++ra)
        for (int rb = 0; rb < kG1MaxBand; ++rb) {
          const int ia = band_idx(pa, ra), ib = band_idx(pb, rb);
          if (ia < 0 || ib < 0) continue;
          for (int o = 0; o < 125; ++o) {
            const int d[3] = {o % 5, (o / 5) % 5, o / 25};  // dx, dy, dz (+2)
            double acc = 0.0;
            for (int fm = 0; fm < kG1Families; ++fm) {
              double prod = w[fm];
              for (int b = 0; b < 3; ++b) {
                const int kind = g1_kind(fm, b);
                const std::vector<double> &t = c.g1host[b];
                prod *= b == pa   ? t[((size_t)kind * nc[b] + ia) * 5 + d[b]]
                        : b == pb ? t[((size_t)kind * nc[b] + ib) * 5 + d[b]]
                                  : irow[b][kind][d[b]];
              }
              acc += prod;
            }
            ecv[(((size_t)pair * kG1MaxBand + ra) * kG1MaxBand + rb) * 125 + o] = (float)acc;
          }
        }
    }
    float *dec = nullptr;
    LS_TRY(mg_alloc(mg, &dec, ecv.size()));
    LS_CUDA_TRY(cudaMemcpyAsync(dec, ecv.data(), ecv.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    g.edge_coef = dec;
  }
  // small levels: every node's explicit stencil, one node-per-thread kernel
  g.shell_coef = nullptr;
  g.full_coef = nullptr;
  if (c.n <= kG1ExplicitMax) {
    for (int a = 0; a < 3; ++a) {
      g.lo[a] = 1;
      g.hi[a] = 0;
    }
    float *coef = nullptr;
    LS_TRY(mg_alloc(mg, &coef, (size_t)125 * c.n));
    g1_coef_kernel<<<grid_for(h, c.n), kBlock, 0, h->stream>>>(g, coef);
    ++h->launches;
    g.shell_coef = coef;
  }
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  LS_CUDA_TRY(cudaGetLastError());
  c.g1 = true;
  return LS_OK;
}

constexpr int kMgDefaultDegree = 3;

// Chebyshev step coefficients of degree `deg` on [lmax/20, 1.05 lmax] (every level but the coarsest)
void mg_set_degree(MgHierarchy &mg, int deg) {
  mg.deg = deg;
  for (size_t l = 0; l + 1 < mg.levels.size(); ++l) {
    MgLevel &lv = mg.levels[l];
    const double lmax = 1.05 * lv.lmax, lmin = lv.lmax / 20.0;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
    double rho = 1.0 / sigma;
    lv.inv_theta = (float)(1.0 / theta);
    lv.c1.assign(deg, 0.f);
    lv.c2.assign(deg, 0.f);
    for (int k = 0; k < deg; ++k) {
      const double rn = 1.0 / (2.0 * sigma - rho);
      lv.c1[k] = (float)(rn * rho);
      lv.c2[k] = (float)(2.0 * rn / delta);
      rho = rn;
    }
  }
}

constexpr int64_t kMgMaxCoarse = 1000;       // largest dense coarsest level
constexpr int64_t kMgMaxCoarseSmall = 200;   // ... for grids below kMgSmallGrid nodes
constexpr int64_t kMgSmallGrid = 2000000;

// Builds the hierarchy; returns LS_OK with mg.built == false when the grid
// cannot be coarsened to a dense-solvable size (the solve then uses Jacobi).
int mg_build(ls_fd_handle *h, int deg) {
  MgHierarchy &mg = h->mg;
  if (mg.built || !mg.levels.empty()) return LS_OK;  // built, or tried and not applicable
  mg.deg = deg;
  using clock = std::chrono::steady_clock;
  const auto t_start = clock::now();
  auto t_phase = t_start;
  // adds the time since the last mark (after a stream sync) to setup phase `ph`
  auto mark = [&](int ph) -> int {
    LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    const auto now = clock::now();
    mg.setup_ms[ph] += std::chrono::duration<double, std::milli>(now - t_phase).count();
    t_phase = now;
    return LS_OK;
  };
  MgLevel L0;
  L0.nx = (int)h->grid.nsteps[0];
  L0.ny = (int)h->grid.nsteps[1];
  L0.nz = (int)h->grid.nsteps[2];
  L0.n = h->n;
  L0.coef64 = h->coef;
  L0.coef = coef_as<float>(h->coef);
  L0.nrows = h->data.nrows;
  L0.width = h->data.width;
  L0.cols = h->data.cols;
  L0.a = h->data.a32;
  L0.w2 = h->data.w2_32;
  L0.s = h->s32;
  L0.ntouched = h->data.ntouched;
  L0.mask = h->data.mask;
  L0.word_rank = h->data.word_rank;
  L0.inc_ptr = h->data.inc_ptr;
  L0.inc_row = h->data.inc_row;
  L0.inc_a = h->data.inc_a32;
  L0.dinv = h->dinv32;
  L0.dir = h->dir32;
  if (L0.dir) LS_TRY(mg_alloc(mg, &L0.dq, L0.n));
  L0.owns_bx = false;
  L0.b = h->r32;
  if (!h->z32) LS_TRY(dev_alloc(&h->z32, h->n));
  L0.x = h->z32;
  LS_TRY(mg_alloc(mg, &L0.r, L0.n));
  LS_TRY(mg_alloc(mg, &L0.d0, L0.n));
  LS_TRY(mg_alloc(mg, &L0.d1, L0.n));
  mg.levels.push_back(L0);
  LS_TRY(ensure_host_rows(h));
  HostRows rows;
  CellRows cells;
  {
    HostRows all;
    all.nrows = h->data.nrows;
    all.width = h->h_width;
    all.cols = h->h_idc;
    all.a = h->h_a;
    all.w2 = h->h_w2;
    const int st_split = mg_split_rows(h, all, L0.nx, L0.ny, L0.nz, cells, rows);
    if (st_split < 0) {
      free_cell_rows(cells);
      return st_split;
    }
  }
  struct CellRowsGuard {
    CellRows &c;
    ~CellRowsGuard() { free_cell_rows(c); }
  } cells_guard{cells};
  LS_TRY(mark(0));
  for (;;) {
    const MgLevel &f = mg.levels.back();
    // the dense coarsest solve costs O(n^3) to set up: grids too small for an
    // extra level's per-iteration cost to matter coarsen further
    const int64_t coarsest = h->n < kMgSmallGrid ? kMgMaxCoarseSmall : kMgMaxCoarse;
    if (f.n <= coarsest) break;
    if (f.nx < 5 || f.ny < 5 || f.nz < 5) break;
    MgLevel c;
    c.nx = f.nx / 2 + 1;
    c.ny = f.ny / 2 + 1;
    c.nz = f.nz / 2 + 1;
    c.n = (int64_t)c.nx * c.ny * c.nz;
    c.coef64 = coarsen_coef(f.coef64, c.nx, c.ny, c.nz);
    c.coef = coef_as<float>(c.coef64);
    LS_TRY(mg_build_g1(h, mg, f, c));
    LS_TRY(mark(1));
    if (rows.nrows > 0) rows = galerkin_rows(rows, f.nx, f.ny, c.nx, c.ny);
    if (cells.nrows > 0) {
      cell_coarsen_kernel<<<grid_for(h, cells.nrows), kBlock, 0, h->stream>>>(cells.nrows, cells.ci, cells.cj, cells.ck,
                                                                             cells.c);
      ++h->launches;
    }
    LS_TRY(mark(2));
    std::vector<int64_t> touched;
    std::vector<double> ddiag;
    LS_TRY(mg_alloc(mg, &c.b, c.n));
    LS_TRY(mg_alloc(mg, &c.x, c.n));
    LS_TRY(mg_alloc(mg, &c.r, c.n));
    LS_TRY(mg_alloc(mg, &c.d0, c.n));
    LS_TRY(mg_alloc(mg, &c.d1, c.n));
    LS_TRY(mg_alloc(mg, &c.dinv, c.n));
    if (f.dir) {
      LS_TRY(mg_alloc(mg, &c.dir, (size_t)kDirFamilies * c.n));
      LS_TRY(mg_alloc(mg, &c.dsw, (size_t)kDirFamilies * c.n));
      LS_TRY(mg_alloc(mg, &c.dmass, c.n));
      LS_TRY(mg_alloc(mg, &c.dq, c.n));
      if (!mg.dir_u) {  // the first coarse level is the largest
        LS_TRY(mg_alloc(mg, &mg.dir_u, (size_t)kDirFamilies * c.n));
        LS_TRY(mg_alloc(mg, &mg.dir_v, (size_t)kDirFamilies * c.n));
      }
      dir_average_kernel<<<grid_for(h, c.n), kBlock, 0, h->stream>>>(f.nx, f.ny, f.nz, f.dir, f.dmass, c.nx, c.ny,
                                                                      c.nz, c.dir, c.dmass, c.dsw);
      ++h->launches;
    }
    c.knt = 0;
    if (cells.nrows > 0) LS_TRY(mg_cells_k27(h, c, cells));
    if (c.g1op.shell_coef) {
      // explicit level: stencil and 27-point data term in one coefficient set
      float *full = nullptr;
      LS_TRY(mg_alloc(mg, &full, (size_t)kG1Row * c.n));
      g1_fold_k27_kernel<<<grid_for(h, c.n), kBlock, 0, h->stream>>>(c.g1op, c.kmask, c.krank,
                                                                     c.knt > 0 ? c.k27 : nullptr, c.knt, full);
      ++h->launches;
      c.g1op.full_coef = full;
    }
    LS_TRY(mg_upload_level(h, c, rows, touched, ddiag));
    LS_TRY(mark(3));
    // diagonal: regularisation, the row-form data term (touched / ddiag) and
    // the 27-point centre entries (added on the device)
    LS_TRY(mg_level_dinv(h, c, touched, ddiag));
    LS_TRY(mark(4));
    mg.levels.push_back(c);
  }
  if (mg.levels.back().n > kMgMaxCoarse) return LS_OK;  // not built: Jacobi fallback
  for (size_t l = 0; l + 1 < mg.levels.size(); ++l) {
    MgLevel &lv = mg.levels[l];
    float est = 1.0f;
    LS_TRY(mg_lambda_max(h, lv, &est));
    lv.lmax = est;
  }
  LS_TRY(mark(5));
  mg_set_degree(mg, deg);
  LS_TRY(mg_k27_to_host(mg.levels.back(), h->stream));
  LS_TRY(mg_coarse_inverse(h, mg.levels.back()));
  LS_TRY(mark(6));
  mg.setup_ms[7] = std::chrono::duration<double, std::milli>(clock::now() - t_start).count();
  mg.built = true;
  return LS_OK;
}

// z = V(r): levels[0].b must alias the residual, levels[0].x the output
void mg_vcycle(ls_fd_handle *h, const int *done, cudaStream_t st) {
  MgHierarchy &mg = h->mg;
  const int L = (int)mg.levels.size();
  for (int l = 0; l + 1 < L; ++l) {
    MgLevel &lv = mg.levels[l];
    mg_cheb_init_kernel<<<grid_for(h, lv.n), kBlock, 0, st>>>(lv.n, lv.b, lv.dinv, lv.inv_theta, lv.r, lv.d0, lv.x, done);
    ++h->launches;
    float *dc = lv.d0, *dn = lv.d1;
    for (int k = 0; k < mg.deg; ++k) {
      EpiArgs<float> e{};
      e.x = lv.x;
      e.r = lv.r;
      e.dinv = lv.dinv;
      e.d_out = dn;
      e.c1 = lv.c1[k];
      e.c2 = lv.c2[k];
      mg_apply<EPI_CHEB>(h, lv, dc, e, done, st);
      std::swap(dc, dn);
    }
    const MgLevel &cl = mg.levels[l + 1];
    mg_restrict_kernel<<<dim3((cl.nx + 31) / 32, (cl.ny + 7) / 8, cl.nz), dim3(32, 8), 0, st>>>(
        lv.nx, lv.ny, lv.nz, cl.nx, cl.ny, cl.nz, lv.r, cl.b, done);
    ++h->launches;
  }
  {
    MgLevel &cl = mg.levels[L - 1];
    mg_dense_kernel<<<(int)((cl.n * 32 + 255) / 256), 256, 0, st>>>((int)cl.n, mg.coarse_inv64, cl.b, cl.x, done);
    ++h->launches;
  }
  for (int l = L - 2; l >= 0; --l) {
    MgLevel &lv = mg.levels[l];
    const MgLevel &cl = mg.levels[l + 1];
    mg_prolong_kernel<<<dim3((lv.nx + 31) / 32, (lv.ny + 7) / 8, lv.nz), dim3(32, 8), 0, st>>>(
        lv.nx, lv.ny, lv.nz, cl.nx, cl.ny, cl.x, lv.x, done);
    ++h->launches;
    EpiArgs<float> e{};
    e.r = lv.r;
    e.b = lv.b;
    e.dinv = lv.dinv;
    e.d_out = lv.d0;
    e.c2 = lv.inv_theta;
    mg_apply<EPI_RESID>(h, lv, lv.x, e, done, st);
    float *dc = lv.d0, *dn = lv.d1;
    for (int k = 0; k < mg.deg; ++k) {
      EpiArgs<float> e2{};
      e2.x = lv.x;
      e2.r = lv.r;
      e2.dinv = lv.dinv;
      e2.d_out = dn;
      e2.c1 = lv.c1[k];
      e2.c2 = lv.c2[k];
      mg_apply<EPI_CHEB>(h, lv, dc, e2, done, st);
      std::swap(dc, dn);
    }
  }
}

// MG-CG kernels -------------------------------------------------------------
// x += alpha p, r -= alpha q, rrj = r . D^-1 r (stopping test only)
__global__ void __launch_bounds__(kBlock) mg_update_xr_kernel(int64_t n, float *__restrict__ x, float *__restrict__ r,
                                                              const float *__restrict__ p, const float *__restrict__ q,
                                                              const float *__restrict__ dinv, CgScalars *sc,
                                                              double *partials, unsigned int *ticket) {
  if (sc->done) return;
  const double pq = sc->pq_s + sc->pq_d + sc->pq_x;
  const double alpha_d = sc->rz / pq;
  if (!(pq > 0.0) || !isfinite(alpha_d)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) sc->done = isfinite(pq) ? DONE_BREAKDOWN : DONE_NAN;
    return;
  }
  const float alpha = (float)alpha_d;
  float local = 0.f;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    x[g] += alpha * p[g];
    const float rn = r[g] - alpha * q[g];
    r[g] = rn;
    local += rn * (dinv[g] * rn);
  }
  double rrj;
  if (grid_sum<kBlock, float>(local, partials, ticket, &rrj)) {
    sc->iters += 1;
    sc->rrj = rrj;
    if (!isfinite(rrj)) sc->done = DONE_NAN;
    else if (rrj < sc->thresh2) sc->pending = DONE_CONVERGED;
    else if (sc->iters >= sc->maxiter) sc->pending = DONE_MAXITER;
    else if (rrj < sc->trig2) sc->pending = DONE_REFRESH;
  }
}

// rz' = r . z ; beta = rz'/rz (set_only: just rz = rz')
__global__ void __launch_bounds__(kBlock) mg_rz_kernel(int64_t n, const float *__restrict__ r,
                                                       const float *__restrict__ z, CgScalars *sc, double *partials,
                                                       unsigned int *ticket, int set_only) {
  if (!set_only && sc->done) return;
  float local = 0.f;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    local += r[g] * z[g];
  double rz;
  if (grid_sum<kBlock, float>(local, partials, ticket, &rz)) {
    if (!set_only) sc->beta = rz / sc->rz;
    sc->rz = rz;
    if (!isfinite(rz)) sc->done = DONE_NAN;
  }
}

// p = z + beta p  (or p = z); the last block turns a pending stop into `done`
__global__ void mg_update_p_kernel(int64_t n, const float *__restrict__ z, float *__restrict__ p, CgScalars *sc,
                                   unsigned int *ticket, int reset) {
  if (!reset && sc->done) return;
  const float beta = reset ? 0.f : (float)sc->beta;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    p[g] = z[g] + beta * (reset ? 0.f : p[g]);
  if (!reset && sc->pending && grid_last_block(ticket)) {
    sc->done = sc->pending;
    sc->pending = 0;
  }
}

void mg_iteration(ls_fd_handle *h, cudaStream_t st) {
  launch_apply32(h, h->p32, h->q32, true, st);
  const int g = grid_for(h, h->n);
  mg_update_xr_kernel<<<g, kBlock, 0, st>>>(h->n, h->x32, h->r32, h->p32, h->q32, h->dinv32, h->sc, h->partials,
                                            h->tickets + T_UPDATE);
  ++h->launches;
  mg_vcycle(h, &h->sc->done, st);
  mg_rz_kernel<<<g, kBlock, 0, st>>>(h->n, h->r32, h->z32, h->sc, h->partials, h->tickets + T_UPDATE, 0);
  ++h->launches;
  mg_update_p_kernel<<<g, kBlock, 0, st>>>(h->n, h->z32, h->p32, h->sc, h->tickets + T_PUPD, 0);
  ++h->launches;
}

// after a residual refresh: z = V(r), rz = r.z, optionally p = z
int mg_restart(ls_fd_handle *h, bool reset_p) {
  cudaStream_t st = h->stream;
  const int g = grid_for(h, h->n);
  mg_vcycle(h, nullptr, st);
  mg_rz_kernel<<<g, kBlock, 0, st>>>(h->n, h->r32, h->z32, h->sc, h->partials, h->tickets + T_UPDATE, 1);
  ++h->launches;
  if (reset_p) {
    mg_update_p_kernel<<<g, kBlock, 0, st>>>(h->n, h->z32, h->p32, h->sc, h->tickets + T_PUPD, 1);
    ++h->launches;
  }
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

}  // namespace
}  // namespace ls

using namespace ls;

namespace ls {
namespace {

// ---- data-term setup on the device -----------------------------------------
// Per data entry: column check, int32 column, FP32 coefficient, node count.
__global__ void data_entries_kernel(int64_t ne, int64_t n, const int64_t *__restrict__ idc, const double *__restrict__ a,
                                    int32_t *__restrict__ cols, float *__restrict__ a32, int32_t *__restrict__ count,
                                    int *__restrict__ bad) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idc[e];
    const bool ok = c < n;
    if (!ok) atomicExch(bad, 1);
    cols[e] = (c < 0 || !ok) ? -1 : (int32_t)c;
    a32[e] = (float)a[e];
    if (c >= 0 && ok) atomicAdd(count + c, 1);
  }
}

__global__ void data_rows_setup_kernel(int64_t nrows, const double *__restrict__ w, const double *__restrict__ b,
                                       double *__restrict__ w2_64, float *__restrict__ w2_32, double *__restrict__ bc) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const double w2 = w[r] * w[r];
    w2_64[r] = w2;
    w2_32[r] = (float)w2;
    bc[r] = b[r];
  }
}


// entry e goes to the next free slot of its node's segment (any order)
__global__ void data_fill_kernel(int64_t ne, const int32_t *__restrict__ cols, const int64_t *__restrict__ start,
                                 int32_t *__restrict__ fill, int64_t *__restrict__ ent) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c = cols[e];
    if (c >= 0) ent[start[c] + atomicAdd(fill + c, 1)] = e;
  }
}

// each node's segment sorted by entry index (= row order), then the row
// index and coefficients of every incidence
__global__ void data_sort_kernel(int64_t n, const int64_t *__restrict__ start, int64_t *__restrict__ ent, int width,
                                 const double *__restrict__ a, int32_t *__restrict__ inc_row,
                                 double *__restrict__ inc_a64, float *__restrict__ inc_a32) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = start[g], s1 = start[g + 1];
    for (int64_t i = s0 + 1; i < s1; ++i) {
      const int64_t v = ent[i];
      int64_t k = i - 1;
      while (k >= s0 && ent[k] > v) {
        ent[k + 1] = ent[k];
        --k;
      }
      ent[k + 1] = v;
    }
    for (int64_t i = s0; i < s1; ++i) {
      const int64_t e = ent[i];
      inc_row[i] = (int32_t)(e / width);
      inc_a64[i] = a[e];
      inc_a32[i] = (float)a[e];
    }
  }
}

// mask word w = nodes 32w .. 32w+31 with incidences; popcount per word
__global__ void data_mask_kernel(int64_t n, int64_t nwords, const int32_t *__restrict__ count,
                                 uint32_t *__restrict__ mask, int32_t *__restrict__ wcount) {
  const int lane = threadIdx.x & 31;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g - lane < nwords * 32;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t word = __ballot_sync(0xffffffffu, g < n && count[g] > 0);
    if (lane == 0) {
      mask[g >> 5] = word;
      wcount[g >> 5] = __popc(word);
    }
  }
}

__global__ void data_touched_kernel(int64_t n, const uint32_t *__restrict__ mask, const int64_t *__restrict__ wrank64,
                                    const int64_t *__restrict__ start, int32_t *__restrict__ word_rank,
                                    int64_t *__restrict__ touched, int64_t *__restrict__ inc_ptr) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = g >> 5;
    const uint32_t word = mask[w], bit = 1u << (g & 31);
    if ((g & 31) == 0) word_rank[w] = (int32_t)wrank64[w];
    if (!(word & bit)) continue;
    const int64_t rank = wrank64[w] + __popc(word & (bit - 1u));
    touched[rank] = g;
    inc_ptr[rank] = start[g];
  }
}

}  // namespace

// Device copies of the data rows and the node -> row incidence list (CSR over
// the touched nodes in node order, each node's entries in row order), built
// on the device: counts, scan, fill, per-node sort, mask and ranks.
int setup_data_term(ls_fd_handle *h, const ls_fd_system *sys, int64_t ne) {
  DataTerm &d = h->data;
  const int64_t n = h->n;
  const int64_t nwords = (n + 31) / 32;
  cudaStream_t hs = h->stream;
  LS_TRY(dev_alloc(&d.cols, ne));
  LS_TRY(dev_alloc(&d.a64, ne));
  LS_TRY(dev_alloc(&d.a32, ne));
  LS_TRY(dev_alloc(&d.w2_64, d.nrows));
  LS_TRY(dev_alloc(&d.w2_32, d.nrows));
  LS_TRY(dev_alloc(&d.b, d.nrows));
  LS_TRY(dev_alloc(&h->s64, d.nrows));
  LS_TRY(dev_alloc(&h->s32, d.nrows));
  LS_TRY(dev_alloc(&d.mask, nwords));
  LS_TRY(dev_alloc(&d.word_rank, nwords));
  int32_t *count = nullptr, *fill = nullptr, *wcount = nullptr;
  int64_t *start = nullptr, *ent = nullptr, *wrank = nullptr, *totals = nullptr;
  int *bad = nullptr;
  auto release = [&]() {
    cudaFree(count);
    cudaFree(fill);
    cudaFree(wcount);
    cudaFree(start);
    cudaFree(ent);
    cudaFree(wrank);
    cudaFree(totals);
    cudaFree(bad);
  };
  int st = LS_OK;
  if ((st = dev_alloc(&count, n)) < 0 || (st = dev_alloc(&fill, n)) < 0 || (st = dev_alloc(&wcount, nwords)) < 0 ||
      (st = dev_alloc(&start, n + 1)) < 0 || (st = dev_alloc(&wrank, nwords + 1)) < 0 ||
      (st = dev_alloc(&totals, 2)) < 0 || (st = dev_alloc(&bad, 1)) < 0) {
    release();
    return st;
  }
  cudaMemsetAsync(count, 0, n * sizeof(int32_t), hs);
  cudaMemsetAsync(fill, 0, n * sizeof(int32_t), hs);
  cudaMemsetAsync(bad, 0, sizeof(int), hs);
  if (ne > 0) {
    data_entries_kernel<<<grid_for(h, ne), kBlock, 0, hs>>>(ne, n, sys->d_idc, sys->d_a, d.cols, d.a32, count, bad);
    ++h->launches;
    cudaMemcpyAsync(d.a64, sys->d_a, ne * sizeof(double), cudaMemcpyDeviceToDevice, hs);
    data_rows_setup_kernel<<<grid_for(h, d.nrows), kBlock, 0, hs>>>(d.nrows, sys->d_w, sys->d_b, d.w2_64, d.w2_32, d.b);
    ++h->launches;
  }
  setup_scan_kernel<<<1, 1024, 0, hs>>>(count, n, start, totals);
  ++h->launches;
  int64_t ni = 0;
  int hbad = 0;
  if (cudaMemcpyAsync(&ni, totals, sizeof(int64_t), cudaMemcpyDeviceToHost, hs) != cudaSuccess ||
      cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, hs) != cudaSuccess ||
      cudaStreamSynchronize(hs) != cudaSuccess) {
    release();
    set_error("data-row setup failed: %s", cudaGetErrorString(cudaGetLastError()));
    return LS_ERR_CUDA;
  }
  if (hbad) {
    release();
    set_error("a data-row column is out of range (dof %lld)", (long long)n);
    return LS_ERR_ARG;
  }
  cudaMemcpyAsync(start + n, &ni, sizeof(int64_t), cudaMemcpyHostToDevice, hs);
  if ((st = dev_alloc(&ent, ni)) < 0 || (st = dev_alloc(&d.inc_row, ni)) < 0 || (st = dev_alloc(&d.inc_a64, ni)) < 0 ||
      (st = dev_alloc(&d.inc_a32, ni)) < 0) {
    release();
    return st;
  }
  if (ne > 0) {
    data_fill_kernel<<<grid_for(h, ne), kBlock, 0, hs>>>(ne, d.cols, start, fill, ent);
    ++h->launches;
  }
  data_sort_kernel<<<grid_for(h, n), kBlock, 0, hs>>>(n, start, ent, d.width > 0 ? d.width : 1, d.a64, d.inc_row,
                                                       d.inc_a64, d.inc_a32);
  data_mask_kernel<<<grid_for(h, nwords * 32), kBlock, 0, hs>>>(n, nwords, count, d.mask, wcount);
  setup_scan_kernel<<<1, 1024, 0, hs>>>(wcount, nwords, wrank, totals + 1);
  h->launches += 3;
  int64_t nt = 0;
  if (cudaMemcpyAsync(&nt, totals + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, hs) != cudaSuccess ||
      cudaStreamSynchronize(hs) != cudaSuccess) {
    release();
    set_error("data-row setup failed: %s", cudaGetErrorString(cudaGetLastError()));
    return LS_ERR_CUDA;
  }
  d.ntouched = nt;
  if ((st = dev_alloc(&d.touched, nt)) < 0 || (st = dev_alloc(&d.inc_ptr, nt + 1)) < 0) {
    release();
    return st;
  }
  data_touched_kernel<<<grid_for(h, n), kBlock, 0, hs>>>(n, d.mask, wrank, start, d.word_rank, d.touched, d.inc_ptr);
  ++h->launches;
  cudaMemcpyAsync(d.inc_ptr + nt, &ni, sizeof(int64_t), cudaMemcpyHostToDevice, hs);
  const cudaError_t e = cudaStreamSynchronize(hs);
  release();
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    set_error("data-row setup kernels failed: %s", cudaGetErrorString(e));
    return LS_ERR_CUDA;
  }
  h->h_width = d.width;
  return LS_OK;
}

// host copy of the data rows, for the Galerkin coarsening of the multigrid
int ensure_host_rows(ls_fd_handle *h) {
  const DataTerm &d = h->data;
  const int64_t ne = d.nrows * d.width;
  if ((int64_t)h->h_idc.size() == ne && (int64_t)h->h_w2.size() == d.nrows) return LS_OK;
  std::vector<int32_t> cols(ne);
  h->h_idc.resize(ne);
  h->h_a.resize(ne);
  h->h_w2.resize(d.nrows);
  if (ne > 0) {
    LS_CUDA_TRY(cudaMemcpy(cols.data(), d.cols, ne * sizeof(int32_t), cudaMemcpyDeviceToHost));
    LS_CUDA_TRY(cudaMemcpy(h->h_a.data(), d.a64, ne * sizeof(double), cudaMemcpyDeviceToHost));
    LS_CUDA_TRY(cudaMemcpy(h->h_w2.data(), d.w2_64, d.nrows * sizeof(double), cudaMemcpyDeviceToHost));
  }
  for (int64_t e = 0; e < ne; ++e) h->h_idc[e] = cols[e];
  return LS_OK;
}

}  // namespace ls

extern "C" int ls_fd_create(const ls_fd_system *sys, ls_fd_handle **out, void *stream) {
  LS_ARG_CHECK(sys != nullptr && out != nullptr, "NULL argument");
  *out = nullptr;
  const ls_grid3 &g = sys->grid;
  for (int d = 0; d < 3; ++d) {
    LS_ARG_CHECK(g.nsteps[d] >= 2, "every axis needs at least 2 nodes");
    LS_ARG_CHECK(g.step[d] > 0.0, "step must be positive");
  }
  const int64_t n = g.nsteps[0] * g.nsteps[1] * g.nsteps[2];
  LS_ARG_CHECK(n < (int64_t)2000000000, "grid too large for 32-bit data-row columns");
  LS_ARG_CHECK(sys->nrows >= 0, "nrows < 0");
  LS_ARG_CHECK(sys->nrows == 0 || (sys->width >= 1 && sys->width <= 64), "width must be in [1, 64]");
  LS_ARG_CHECK(sys->nrows == 0 || (sys->d_idc && sys->d_a && sys->d_b && sys->d_w), "NULL data-row buffer");
  cudaStream_t cs = as_stream(stream);
  LS_CUDA_TRY(cudaStreamSynchronize(cs));

  ls_fd_handle *h = new ls_fd_handle();
  h->grid = g;
  h->n = n;
  h->coef = make_stencil_coef(g, sys->w_dxx, sys->w_dyy, sys->w_dzz, sys->w_dxy, sys->w_dyz, sys->w_dxz, sys->w_dx,
                              sys->w_dy, sys->w_dz, sys->ridge);
  int st = LS_OK;
  auto fail = [&](int s) {
    ls_fd_destroy(h);
    return s;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    return fail(LS_ERR_CUDA);
  }
  cudaGetDevice(&h->device);
  h->red_blocks = sm_count() * 8;
  {
    const dim3 a4 = apply_grid<float, 4>((int)g.nsteps[0], (int)g.nsteps[1], (int)g.nsteps[2], MODE_FULL);
    const dim3 a8 = apply_grid<double, 8>((int)g.nsteps[0], (int)g.nsteps[1], (int)g.nsteps[2], MODE_FULL);
    const size_t nb = std::max<size_t>({(size_t)h->red_blocks, (size_t)a4.x * a4.y * a4.z, (size_t)a8.x * a8.y * a8.z});
    if ((st = dev_alloc(&h->partials, 4 * nb)) < 0) return fail(st);
    h->partials_cap = (int64_t)(4 * nb);
  }
  if ((st = dev_alloc(&h->tickets, T_COUNT)) < 0) return fail(st);
  if ((st = dev_alloc(&h->aux, kAuxDoubles)) < 0) return fail(st);
  if ((st = dev_alloc(&h->sc, 1)) < 0) return fail(st);
  if (cudaMallocHost((void **)&h->sc_h, sizeof(CgScalars)) != cudaSuccess) {
    set_error("cudaMallocHost failed");
    return fail(LS_ERR_ALLOC);
  }
  cudaMemsetAsync(h->tickets, 0, T_COUNT * sizeof(unsigned int), h->stream);
  cudaMemsetAsync(h->sc, 0, sizeof(CgScalars), h->stream);
  // vectors
  double **v64[] = {&h->rhs, &h->diag, &h->dinv64, &h->x64, &h->r64, &h->p64, &h->q64};
  for (auto pp : v64)
    if ((st = dev_alloc(pp, n)) < 0) return fail(st);
  float **v32[] = {&h->dinv32, &h->x32, &h->r32, &h->p32, &h->q32};
  for (auto pp : v32)
    if ((st = dev_alloc(pp, n)) < 0) return fail(st);

  // ---- data rows: device copies and the node -> row incidence list ----
  DataTerm &d = h->data;
  d.nrows = sys->nrows;
  d.width = sys->nrows > 0 ? sys->width : 0;
  const int64_t ne = d.nrows * d.width;
  if ((st = setup_data_term(h, sys, ne)) < 0) return fail(st);
  cudaStream_t hs = h->stream;
  // ---- directional regularisation weights: FP64 copy and FP32 copy ----
  if (sys->d_dir) {
    const int64_t nd = (int64_t)kDirFamilies * n;
    if ((st = dev_alloc(&h->dir64, nd)) < 0) return fail(st);
    if ((st = dev_alloc(&h->dir32, nd)) < 0) return fail(st);
    if (cudaMemcpyAsync(h->dir64, sys->d_dir, nd * sizeof(double), cudaMemcpyDeviceToDevice, hs) != cudaSuccess) {
      set_error("copy of the directional weights failed");
      return fail(LS_ERR_CUDA);
    }
    dir_to_f32_kernel<<<grid_for(h, nd), kBlock, 0, hs>>>(nd, h->dir64, h->dir32);
    ++h->launches;
  }
  // ---- rhs, diagonal, inverse diagonal ----
  const int gn = grid_for(h, n);
  cudaMemsetAsync(h->rhs, 0, n * sizeof(double), hs);
  diag_stencil_kernel<<<gn, kBlock, 0, hs>>>(h->coef, h->diag);
  ++h->launches;
  if (h->dir64) {
    const DirView<double> dv{(int)g.nsteps[0], (int)g.nsteps[1], (int)g.nsteps[2], h->dir64};
    dir_diag_kernel<double><<<gn, kBlock, 0, hs>>>(dv, h->diag);
    ++h->launches;
  }
  if (d.ntouched > 0) {
    data_node_setup_kernel<<<grid_for(h, d.ntouched), kBlock, 0, hs>>>(d.ntouched, d.touched, d.inc_ptr, d.inc_row,
                                                                       d.inc_a64, d.w2_64, d.b, h->diag, h->rhs);
    ++h->launches;
  }
  dinv_kernel<<<gn, kBlock, 0, hs>>>(n, h->diag, h->dinv64, h->dinv32);
  ++h->launches;
  norm2_kernel<<<gn, kBlock, 0, hs>>>(n, h->rhs, h->dinv64, h->sc, h->partials, h->tickets + T_MISC);
  ++h->launches;
  if (cudaGetLastError() != cudaSuccess || read_scalars(h) < 0) {
    set_error("setup kernels failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(LS_ERR_CUDA);
  }
  h->rhs_norm2 = h->sc_h->scratch;
  {
    // the TMA-staged FP32 apply unless LS_GB300_STAGED_APPLY=tiles asks for
    // the cp.async tile kernels (same operator, for comparison)
    const char *mode = getenv("LS_GB300_STAGED_APPLY");
    const bool allow = !(mode && strcmp(mode, "tiles") == 0);
    tm_setup(h->tm, (int)g.nsteps[0], (int)g.nsteps[1], (int)g.nsteps[2], allow);
    if ((st = tm_autotune(h->tm, coef_as<float>(h->coef), h->p32, h->q32, &h->sc->fault, h->stream)) < 0) return fail(st);
  }
  cudaEventCreate(&h->ev0);
  cudaEventCreate(&h->ev1);
  *out = h;
  return LS_OK;
}

extern "C" int ls_fd_destroy(ls_fd_handle *h) {
  if (!h) return LS_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->g64) cudaGraphExecDestroy(h->g64);
  if (h->g32) cudaGraphExecDestroy(h->g32);
  if (h->gmg) cudaGraphExecDestroy(h->gmg);
  for (void *p : h->mg.allocations) cudaFree(p);
  if (h->z32) cudaFree(h->z32);
  void *ptrs[] = {h->rhs, h->diag, h->dinv64, h->dinv32, h->x64, h->r64, h->p64, h->q64, h->s64, h->x32, h->r32,
                  h->p32, h->q32, h->s32, h->sc, h->partials, h->tickets, h->data.cols, h->data.a64, h->data.a32,
                  h->data.w2_64, h->data.w2_32, h->data.b, h->data.touched, h->data.inc_ptr, h->data.inc_row,
                  h->data.inc_a64, h->data.inc_a32, h->data.mask, h->data.word_rank, h->dir64, h->dir32, h->aux};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h->sc_h) cudaFreeHost(h->sc_h);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return LS_OK;
}

extern "C" int64_t ls_fd_dof(const ls_fd_handle *h) { return h ? h->n : -1; }
extern "C" int ls_fd_device(const ls_fd_handle *h) { return h ? h->device : -1; }
extern "C" int ls_fd_staged_apply(const ls_fd_handle *h) { return h && h->tm.enabled ? 1 : 0; }

extern "C" int ls_fd_rhs(ls_fd_handle *h, double *d_rhs, void *stream) {
  LS_ARG_CHECK(h && d_rhs, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  LS_CUDA_TRY(cudaMemcpyAsync(d_rhs, h->rhs, h->n * sizeof(double), cudaMemcpyDeviceToDevice, as_stream(stream)));
  return LS_OK;
}

extern "C" int ls_fd_set_rhs(ls_fd_handle *h, const double *d_rhs, void *stream) {
  LS_ARG_CHECK(h && d_rhs, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  cudaStream_t hs = h->stream;
  LS_CUDA_TRY(cudaMemcpyAsync(h->rhs, d_rhs, h->n * sizeof(double), cudaMemcpyDeviceToDevice, hs));
  norm2_kernel<<<grid_for(h, h->n), kBlock, 0, hs>>>(h->n, h->rhs, h->dinv64, h->sc, h->partials, h->tickets + T_MISC);
  ++h->launches;
  LS_CUDA_TRY(cudaMemcpyAsync(h->sc_h, h->sc, sizeof(CgScalars), cudaMemcpyDeviceToHost, hs));
  LS_CUDA_TRY(cudaStreamSynchronize(hs));
  h->rhs_norm2 = h->sc_h->scratch;
  return LS_OK;
}

extern "C" int ls_fd_data_rows_apply(ls_fd_handle *h, const double *d_x, double *d_s, void *stream) {
  LS_ARG_CHECK(h && d_x && d_s, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  const DataTerm &d = h->data;
  if (d.nrows > 0) {
    rows_kernel<double><<<grid_for(h, d.nrows), kBlock, 0, h->stream>>>(d.nrows, d.width, d.cols, d.a64, d.w2_64, d_x,
                                                                        d_s, nullptr);
    ++h->launches;
  }
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return LS_OK;
}

extern "C" int ls_fd_admm_step(ls_fd_handle *h, int64_t row0, int64_t m, const double *d_lo, const double *d_hi,
                               double *d_z, double *d_u, const double *d_x, double *h_sums, void *stream) {
  LS_ARG_CHECK(h && d_lo && d_hi && d_z && d_u && d_x && h_sums, "NULL argument");
  const DataTerm &d = h->data;
  LS_ARG_CHECK(row0 >= 0 && m >= 1 && row0 + m <= d.nrows, "rows [row0, row0 + m) outside the data rows");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  cudaStream_t hs = h->stream;
  // partials hold 4 * max(red_blocks, ...) doubles: kAdmmSums per block fit
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((m + kBlock - 1) / kBlock, h->red_blocks / 2));
  admm_rows_kernel<<<nb, kBlock, 0, hs>>>(m, d.width, d.cols + row0 * d.width, d.a64 + row0 * d.width, d_x, d_lo,
                                          d_hi, d_z, d_u, d.b + row0, h->partials);
  admm_sum_kernel<<<1, kBlock, 0, hs>>>(nb, h->partials, h->aux);
  h->launches += 2;
  if (d.ntouched > 0) {
    data_node_rhs_kernel<<<grid_for(h, d.ntouched), kBlock, 0, hs>>>(d.ntouched, d.touched, d.inc_ptr, d.inc_row,
                                                                     d.inc_a64, d.w2_64, d.b, h->rhs);
    ++h->launches;
  }
  norm2_kernel<<<grid_for(h, h->n), kBlock, 0, hs>>>(h->n, h->rhs, h->dinv64, h->sc, h->partials, h->tickets + T_MISC);
  ++h->launches;
  LS_CUDA_TRY(cudaGetLastError());
  LS_CUDA_TRY(cudaMemcpyAsync(h_sums, h->aux, kAdmmSums * sizeof(double), cudaMemcpyDeviceToHost, hs));
  LS_TRY(read_scalars(h));  // synchronises
  h->rhs_norm2 = h->sc_h->scratch;
  return LS_OK;
}

extern "C" int ls_fd_diagonal(ls_fd_handle *h, double *d_diag, void *stream) {
  LS_ARG_CHECK(h && d_diag, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  LS_CUDA_TRY(cudaMemcpyAsync(d_diag, h->diag, h->n * sizeof(double), cudaMemcpyDeviceToDevice, as_stream(stream)));
  return LS_OK;
}

extern "C" int ls_fd_apply(ls_fd_handle *h, const double *d_x, double *d_y, void *stream) {
  LS_ARG_CHECK(h && d_x && d_y, "NULL argument");
  cudaStream_t cs = as_stream(stream);
  LS_CUDA_TRY(cudaStreamSynchronize(cs));
  launch_apply64(h, d_x, d_y, false, h->stream);
  LS_CUDA_TRY(cudaGetLastError());
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return LS_OK;
}

extern "C" int ls_fd_apply_f32(ls_fd_handle *h, const float *d_x, float *d_y, void *stream) {
  LS_ARG_CHECK(h && d_x && d_y, "NULL argument");
  cudaStream_t cs = as_stream(stream);
  LS_CUDA_TRY(cudaStreamSynchronize(cs));
  launch_apply32(h, d_x, d_y, false, h->stream);
  LS_CUDA_TRY(cudaGetLastError());
  return read_scalars(h);  // synchronises; reports a staged-apply fault
}

extern "C" int ls_fd_setup_profile(const ls_fd_handle *h, double *h_out, int n) {
  LS_ARG_CHECK(h && h_out, "NULL argument");
  const int k = std::min(n, 8);
  for (int i = 0; i < k; ++i) h_out[i] = h->mg.setup_ms[i];
  return k;
}

extern "C" int ls_fd_prepare(ls_fd_handle *h, const ls_solve_opts *opts) {
  LS_ARG_CHECK(h && opts, "NULL argument");
  if (opts->precision == LS_MIXED && opts->preconditioner == LS_PRECOND_MG && h->rhs_norm2 > 0.0)
    LS_TRY(mg_build(h, opts->mg_degree > 0 ? opts->mg_degree : kMgDefaultDegree));
  return LS_OK;
}

extern "C" int ls_fd_solve(ls_fd_handle *h, const ls_solve_opts *opts, double *d_x, ls_solve_stats *stats,
                           void *stream) {
  LS_ARG_CHECK(h && opts && d_x && stats, "NULL argument");
  LS_ARG_CHECK(opts->precision == LS_FP64 || opts->precision == LS_MIXED, "unknown precision");
  LS_ARG_CHECK(opts->atol >= 0.0 && opts->rtol >= 0.0, "tolerances must be >= 0");
  cudaStream_t cs = as_stream(stream);
  cudaStream_t st = h->stream;
  LS_CUDA_TRY(cudaStreamSynchronize(cs));
  const int64_t n = h->n;
  const int batch = opts->check_every > 0 ? opts->check_every : 64;
  const int64_t maxiter = opts->maxiter > 0 ? opts->maxiter : 10 * n;
  const double delta = opts->reliable_delta > 0.0 ? opts->reliable_delta : 0.1;
  *stats = ls_solve_stats{};
  const int64_t launches0 = h->launches;
  const double bnorm = sqrt(h->rhs_norm2);
  const double thresh = std::max(opts->atol, opts->rtol * bnorm);
  stats->rhs_norm = bnorm;
  stats->threshold = thresh;

  bool use_mg = false;
  if (opts->precision == LS_MIXED && opts->preconditioner == LS_PRECOND_MG && bnorm > 0.0) {
    const int deg = opts->mg_degree > 0 ? opts->mg_degree : kMgDefaultDegree;
    LS_TRY(mg_build(h, deg));
    use_mg = h->mg.built;
    if (use_mg && h->mg.deg != deg) {  // another smoother degree: new coefficients, new graph
      mg_set_degree(h->mg, deg);
      if (h->gmg) cudaGraphExecDestroy(h->gmg);
      h->gmg = nullptr;
    }
  }
  LS_CUDA_TRY(cudaEventRecord(h->ev0, st));
  if (opts->use_x0)
    LS_CUDA_TRY(cudaMemcpyAsync(h->x64, d_x, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  else
    LS_CUDA_TRY(cudaMemsetAsync(h->x64, 0, n * sizeof(double), st));
  CgScalars &s = *h->sc_h;
  int status = LS_OK;
  long long iters = 0, updates = 0;

  // FP32 Jacobi-CG on the correction, FP64 residual refreshed whenever the
  // recurrence residual fell by `delta` (reliable updates).  Also the
  // fallback after a multigrid breakdown (then started from x64).
  auto run_mixed_jacobi = [&](bool have_x) -> int {
    LS_TRY(refresh(h, have_x, h->r32, h->p32));  // r64, r32, p32, x32 = 0
    LS_TRY(read_scalars(h));
    double true_r = sqrt(std::max(s.rz64, 0.0));
    if (true_r < thresh) {
      status = LS_OK;
      return LS_OK;
    }
    const long long iters0 = iters;
    s.rz = s.rz32;
    s.pq_s = s.pq_d = s.pq_x = 0.0;
    s.thresh2 = thresh * thresh;
    s.iters = iters0;
    s.maxiter = maxiter;
    s.done = 0;
    s.trig2 = delta * delta * s.rz32;
    LS_TRY(write_scalars(h));
    if (!h->g32 || h->g32_batch != batch) {
      if (h->g32) cudaGraphExecDestroy(h->g32);
      h->g32 = nullptr;
      LS_TRY(build_graph<float>(h, batch, &h->g32, &h->g32_kernels, h->x32, h->r32, h->p32, h->q32, h->dinv32));
      h->g32_batch = batch;
    }
    double last_true_r = true_r;
    for (;;) {
      LS_CUDA_TRY(cudaGraphLaunch(h->g32, st));
      h->launches += h->g32_kernels;
      LS_TRY(read_scalars(h));
      if (s.done == DONE_RUNNING) continue;
      if (s.done == DONE_NAN) {
        status = LS_NAN;
        break;
      }
      // reliable update.  An FP32 breakdown (the recurrence residual reached
      // zero, or p.Np lost its sign in rounding) restarts the direction from
      // the refreshed residual; x32 still holds the last finite iterate.
      const bool broke = s.done == DONE_BREAKDOWN;
      fold_kernel<<<grid_for(h, n), kBlock, 0, st>>>(n, h->x64, h->x32);
      ++h->launches;
      LS_TRY(refresh(h, true, h->r32, broke ? h->p32 : nullptr));
      const long long it_now = s.iters;
      LS_TRY(read_scalars(h));
      ++updates;
      true_r = sqrt(std::max(s.rz64, 0.0));
      if (true_r < thresh) {
        status = LS_OK;
        break;
      }
      if (broke && !(true_r < 0.5 * last_true_r)) {  // no progress since the last refresh
        status = LS_BREAKDOWN;
        break;
      }
      last_true_r = true_r;
      if (it_now >= maxiter) {
        status = LS_NOT_CONVERGED;
        break;
      }
      if (!isfinite(true_r)) {
        status = LS_NAN;
        break;
      }
      s.rz = s.rz32;
      s.done = 0;
      s.trig2 = delta * delta * s.rz32;
      LS_TRY(write_scalars(h));
    }
    iters = s.iters;
    return LS_OK;
  };

  if (bnorm == 0.0) {  // scipy returns b (= 0) immediately
    LS_CUDA_TRY(cudaMemsetAsync(h->x64, 0, n * sizeof(double), st));
  } else if (opts->precision == LS_FP64) {
    LS_TRY(refresh(h, opts->use_x0 != 0, nullptr, nullptr));  // r64, p64 = D^-1 r64, rz64
    LS_TRY(read_scalars(h));
    s.rz = s.rz64;
    s.pq_s = s.pq_d = s.pq_x = 0.0;
    s.thresh2 = thresh * thresh;
    s.iters = 0;
    s.maxiter = maxiter;
    s.done = (s.rz < s.thresh2) ? DONE_CONVERGED : DONE_RUNNING;
    s.trig2 = 0.0;
    LS_TRY(write_scalars(h));
    if (!h->g64 || h->g64_batch != batch) {
      if (h->g64) cudaGraphExecDestroy(h->g64);
      h->g64 = nullptr;
      LS_TRY(build_graph<double>(h, batch, &h->g64, &h->g64_kernels, h->x64, h->r64, h->p64, h->q64, h->dinv64));
      h->g64_batch = batch;
    }
    while (!s.done) {
      LS_CUDA_TRY(cudaGraphLaunch(h->g64, st));
      h->launches += h->g64_kernels;
      LS_TRY(read_scalars(h));
    }
    iters = s.iters;
    status = done_to_status(s.done);
  } else if (use_mg) {
    // FP32 CG with the multigrid V-cycle as preconditioner; FP64 reliable
    // updates as below.  Stopping test on the Jacobi-scaled residual.
    LS_TRY(refresh(h, opts->use_x0 != 0, h->r32, nullptr));  // r64, r32, x32 = 0
    LS_TRY(read_scalars(h));
    double true_r = sqrt(std::max(s.rz64, 0.0));
    if (!(true_r < thresh)) {
      s.done = 0;
      s.iters = 0;
      LS_TRY(write_scalars(h));
      LS_TRY(mg_restart(h, true));
      LS_TRY(read_scalars(h));
      s.pq_s = s.pq_d = s.pq_x = 0.0;
      s.thresh2 = thresh * thresh;
      s.iters = 0;
      s.maxiter = maxiter;
      s.done = 0;
      s.rrj = s.rz32;
      s.trig2 = delta * delta * s.rz32;
      LS_TRY(write_scalars(h));
      const int mbatch = std::max(1, std::min(batch, 8));
      if (!h->gmg || h->gmg_batch != mbatch) {
        if (h->gmg) cudaGraphExecDestroy(h->gmg);
        h->gmg = nullptr;
        const int64_t before = h->launches;
        LS_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < mbatch; ++it) mg_iteration(h, st);
        h->gmg_kernels = h->launches - before;
        h->launches = before;
        cudaGraph_t graph;
        LS_CUDA_TRY(cudaStreamEndCapture(st, &graph));
        cudaError_t e = cudaGraphInstantiate(&h->gmg, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
          set_error("cudaGraphInstantiate: %s", cudaGetErrorString(e));
          return LS_ERR_CUDA;
        }
        h->gmg_batch = mbatch;
      }
      for (;;) {
        LS_CUDA_TRY(cudaGraphLaunch(h->gmg, st));
        h->launches += h->gmg_kernels;
        LS_TRY(read_scalars(h));
        if (s.done == DONE_RUNNING) continue;
        if (s.done == DONE_NAN || s.done == DONE_BREAKDOWN) {
          status = done_to_status(s.done);
          break;
        }
        fold_kernel<<<grid_for(h, n), kBlock, 0, st>>>(n, h->x64, h->x32);
        ++h->launches;
        LS_TRY(refresh(h, true, h->r32, nullptr));
        const long long it_now = s.iters;
        LS_TRY(read_scalars(h));
        ++updates;
        true_r = sqrt(std::max(s.rz64, 0.0));
        if (true_r < thresh) {
          status = LS_OK;
          break;
        }
        if (it_now >= maxiter) {
          status = LS_NOT_CONVERGED;
          break;
        }
        if (!isfinite(true_r)) {
          status = LS_NAN;
          break;
        }
        s.done = 0;
        LS_TRY(write_scalars(h));
        LS_TRY(mg_restart(h, false));
        LS_TRY(read_scalars(h));
        s.done = 0;
        s.rrj = s.rz32;
        s.trig2 = delta * delta * s.rz32;
        LS_TRY(write_scalars(h));
      }
      iters = s.iters;
    }
    if (status == LS_NAN || status == LS_BREAKDOWN) {
      // the V-cycle lost definiteness in FP32: finish with Jacobi from x64
      use_mg = false;
      status = LS_OK;
      LS_TRY(run_mixed_jacobi(true));
    }
  } else {
    LS_TRY(run_mixed_jacobi(opts->use_x0 != 0));
  }
  // final FP64 residual of the returned iterate
  LS_TRY(refresh(h, true, nullptr, nullptr));
  LS_CUDA_TRY(cudaMemcpyAsync(d_x, h->x64, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
  LS_CUDA_TRY(cudaEventRecord(h->ev1, st));
  LS_TRY(read_scalars(h));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  stats->iterations = iters;
  stats->reliable_updates = updates;
  stats->residual = sqrt(std::max(s.rz64, 0.0));
  stats->device_ms = ms;
  stats->status = status;
  stats->preconditioner = use_mg ? LS_PRECOND_MG : LS_PRECOND_JACOBI;
  stats->kernel_launches = h->launches - launches0;
  LS_CUDA_TRY(cudaGetLastError());
  return status;
}

extern "C" int ls_fd_mg_apply_level(ls_fd_handle *h, int level, const float *d_x, float *d_y, int64_t *h_nodes,
                                    void *stream) {
  LS_ARG_CHECK(h && h_nodes, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  LS_TRY(mg_build(h, kMgDefaultDegree));
  MgHierarchy &mg = h->mg;
  LS_ARG_CHECK(mg.built, "the grid does not coarsen");
  LS_ARG_CHECK(level >= 0 && level < (int)mg.levels.size(), "no such level");
  MgLevel &lv = mg.levels[level];
  *h_nodes = lv.n;
  if (!d_x || !d_y) return LS_OK;
  LS_ARG_CHECK(level + 1 < (int)mg.levels.size(), "the coarsest level has no apply");
  EpiArgs<float> e{};
  e.q = d_y;
  mg_apply<EPI_STORE>(h, lv, d_x, e, nullptr, h->stream);
  LS_CUDA_TRY(cudaStreamSynchronize(h->stream));
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_mg_vcycle(ls_fd_handle *h, const float *d_r, float *d_z, void *stream) {
  LS_ARG_CHECK(h && d_r && d_z, "NULL argument");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  LS_TRY(mg_build(h, kMgDefaultDegree));
  LS_ARG_CHECK(h->mg.built, "the grid does not coarsen");
  cudaStream_t st = h->stream;
  // levels[0].b aliases r32 and levels[0].x aliases z32
  LS_CUDA_TRY(cudaMemcpyAsync(h->r32, d_r, h->n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  mg_vcycle(h, nullptr, st);
  LS_CUDA_TRY(cudaMemcpyAsync(d_z, h->z32, h->n * sizeof(float), cudaMemcpyDeviceToDevice, st));
  LS_CUDA_TRY(cudaGetLastError());
  return read_scalars(h);  // synchronises; reports a staged-apply fault
}

extern "C" int ls_fd_profile_mg(ls_fd_handle *h, int reps, double *out, int max_levels, int *levels, void *stream) {
  LS_ARG_CHECK(h && out && levels && reps > 0 && max_levels > 0, "bad argument");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  *levels = 0;
  LS_TRY(mg_build(h, kMgDefaultDegree));
  MgHierarchy &mg = h->mg;
  if (!mg.built) return LS_OK;
  cudaStream_t st = h->stream;
  const int L = std::min((int)mg.levels.size(), max_levels);
  auto timed = [&](auto &&launch, double *ms_out) -> int {
    launch();
    LS_CUDA_TRY(cudaEventRecord(h->ev0, st));
    for (int r = 0; r < reps; ++r) launch();
    LS_CUDA_TRY(cudaEventRecord(h->ev1, st));
    LS_CUDA_TRY(cudaEventSynchronize(h->ev1));
    float ms = 0.0f;
    LS_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    *ms_out = ms / reps;
    return LS_OK;
  };
  for (int l = 0; l < L; ++l) {
    MgLevel &lv = mg.levels[l];
    double *o = out + (size_t)l * LS_MG_PROFILE_FIELDS;
    for (int f = 0; f < LS_MG_PROFILE_FIELDS; ++f) o[f] = 0.0;
    o[0] = (double)lv.n;
    const int g = grid_for(h, lv.n);
    fill_kernel<float><<<g, kBlock, 0, st>>>(lv.n, lv.b, 1.0f);
    fill_kernel<float><<<g, kBlock, 0, st>>>(lv.n, lv.x, 0.0f);
    fill_kernel<float><<<g, kBlock, 0, st>>>(lv.n, lv.r, 1.0f);
    fill_kernel<float><<<g, kBlock, 0, st>>>(lv.n, lv.d0, 1e-3f);
    fill_kernel<float><<<g, kBlock, 0, st>>>(lv.n, lv.d1, 1e-3f);
    h->launches += 5;
    if (l + 1 == (int)mg.levels.size()) {
      LS_TRY(timed([&] {
        mg_dense_kernel<<<(int)((lv.n * 32 + 255) / 256), 256, 0, st>>>((int)lv.n, mg.coarse_inv64, lv.b, lv.x, nullptr);
        ++h->launches;
      }, &o[7]));
      continue;
    }
    EpiArgs<float> es{};
    es.q = lv.d1;
    LS_TRY(timed([&] { mg_apply<EPI_STORE>(h, lv, lv.d0, es, nullptr, st); }, &o[1]));
    EpiArgs<float> ec{};
    ec.x = lv.x;
    ec.r = lv.r;
    ec.dinv = lv.dinv;
    ec.d_out = lv.d1;
    ec.c1 = 0.5f;
    ec.c2 = 1e-3f;
    LS_TRY(timed([&] { mg_apply<EPI_CHEB>(h, lv, lv.d0, ec, nullptr, st); }, &o[2]));
    if (l == 0 && h->tm.enabled && !lv.dir) {
      // the TMA-staged kernel alone, then the data term (rows + fix-up) alone
      const TmData td = tm_data(h, lv.s);
      auto part = [&](int parts) {
        return tm_launch<EPI_CHEB>(h->tm, lv.coef, lv.d0, td, ec, nullptr, nullptr, nullptr, nullptr, nullptr,
                                   &h->sc->fault, h->red_blocks, st, parts);
      };
      LS_TRY(timed([&] { h->launches += part(TM_APPLY); }, &o[8]));
      if (td.ntouched > 0) LS_TRY(timed([&] { h->launches += part(TM_DATA); }, &o[9]));
    } else if (lv.g1) {
      const DataView<float> dv = mg_view(lv);
      LS_TRY(timed([&] { h->launches += launch_g1<EPI_CHEB>(lv.g1op, lv.d0, dv, ec, nullptr, h->red_blocks / 8, st, 1); },
                   &o[8]));
      LS_TRY(timed([&] { h->launches += launch_g1<EPI_CHEB>(lv.g1op, lv.d0, dv, ec, nullptr, h->red_blocks / 8, st, 2); },
                   &o[9]));
    } else if (lv.n > kPointMaxNodes && apply_split(lv.nx, lv.ny, lv.nz)) {
      const DataView<float> dv = mg_view(lv);
      LS_TRY(timed([&] {
        launch_tiles<float, EPI_CHEB, MODE_DEEP>(lv.coef, lv.d0, dv, ec, nullptr, nullptr, nullptr, nullptr,
                                                 h->red_blocks / 8, st);
        ++h->launches;
      }, &o[8]));
      const int64_t ns = shell_count(lv.nx, lv.ny, lv.nz);
      const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((ns + 255) / 256, h->red_blocks));
      LS_TRY(timed([&] {
        fd_point_kernel<float, EPI_CHEB, false><<<gs, 256, 0, st>>>(lv.coef, lv.d0, dv, ec, nullptr, nullptr, nullptr,
                                                                    nullptr);
        ++h->launches;
      }, &o[9]));
    }
    EpiArgs<float> er{};
    er.r = lv.r;
    er.b = lv.b;
    er.dinv = lv.dinv;
    er.d_out = lv.d1;
    er.c2 = 1e-3f;
    LS_TRY(timed([&] { mg_apply<EPI_RESID>(h, lv, lv.x, er, nullptr, st); }, &o[3]));
    const MgLevel &cl = mg.levels[l + 1];
    LS_TRY(timed([&] {
      mg_restrict_kernel<<<dim3((cl.nx + 31) / 32, (cl.ny + 7) / 8, cl.nz), dim3(32, 8), 0, st>>>(
          lv.nx, lv.ny, lv.nz, cl.nx, cl.ny, cl.nz, lv.r, cl.b, nullptr);
      ++h->launches;
    }, &o[4]));
    LS_TRY(timed([&] {
      mg_prolong_kernel<<<dim3((lv.nx + 31) / 32, (lv.ny + 7) / 8, lv.nz), dim3(32, 8), 0, st>>>(
          lv.nx, lv.ny, lv.nz, cl.nx, cl.ny, cl.x, lv.x, nullptr);
      ++h->launches;
    }, &o[5]));
    if (lv.nrows > 0) {
      LS_TRY(timed([&] {
        rows_kernel<float><<<grid_for(h, lv.nrows), kBlock, 0, st>>>(lv.nrows, lv.width, lv.cols, lv.a, lv.w2, lv.d0,
                                                                     lv.s, nullptr);
        ++h->launches;
      }, &o[6]));
    }
  }
  *levels = L;
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_profile_iteration(ls_fd_handle *h, int precision, int reps, ls_fd_profile *out, void *stream) {
  LS_ARG_CHECK(h && out && reps > 0, "bad argument");
  LS_ARG_CHECK(precision == LS_FP64 || precision == LS_MIXED, "unknown precision");
  LS_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
  cudaStream_t st = h->stream;
  const bool f32 = precision == LS_MIXED;
  const size_t s = f32 ? 4 : 8;
  const int64_t n = h->n;
  // keep every kernel running: done = 0, far-away threshold and iteration cap
  CgScalars &sc = *h->sc_h;
  sc = CgScalars{};
  sc.rz = 1.0;
  sc.pq_s = 1.0;
  sc.thresh2 = -1.0;
  sc.maxiter = (long long)1 << 60;
  sc.profile = 1;
  LS_TRY(write_scalars(h));
  // p = r = 1: p.Np > 0, so every launch does its full work
  const int gf = grid_for(h, n);
  if (f32) {
    fill_kernel<float><<<gf, kBlock, 0, st>>>(n, h->p32, 1.0f);
    ++h->launches;
    fill_kernel<float><<<gf, kBlock, 0, st>>>(n, h->r32, 1.0f);
    ++h->launches;
    fill_kernel<float><<<gf, kBlock, 0, st>>>(n, h->x32, 0.0f);
    ++h->launches;
  } else {
    fill_kernel<double><<<gf, kBlock, 0, st>>>(n, h->p64, 1.0);
    ++h->launches;
    fill_kernel<double><<<gf, kBlock, 0, st>>>(n, h->r64, 1.0);
    ++h->launches;
    fill_kernel<double><<<gf, kBlock, 0, st>>>(n, h->x64, 0.0);
    ++h->launches;
  }
  auto timed = [&](auto &&fn, double *ms_out) -> int {
    fn();  // warm-up
    LS_CUDA_TRY(cudaEventRecord(h->ev0, st));
    for (int i = 0; i < reps; ++i) fn();
    LS_CUDA_TRY(cudaEventRecord(h->ev1, st));
    LS_CUDA_TRY(cudaEventSynchronize(h->ev1));
    float ms = 0.0f;
    LS_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    *ms_out = ms / reps;
    return LS_OK;
  };
  const int g = grid_for(h, n);
  const DataTerm &d = h->data;
  LS_TRY(timed([&] {
    if (f32) {
      EpiArgs<float> e{};
      e.q = h->q32;
      h->launches += launch_operator<float, EPI_STORE>(coef_as<float>(h->coef), h->p32,
                                                       data_view<float>(h, h->s32, d.inc_a32), e, nullptr, h->partials,
                                                       h->tickets + T_STENCIL, &h->sc->pq_s, h->tickets + T_SHELL,
                                                       &h->sc->pq_d, h->red_blocks, st);
    } else {
      EpiArgs<double> e{};
      e.q = h->q64;
      h->launches += launch_operator<double, EPI_STORE>(coef_as<double>(h->coef), h->p64,
                                                        data_view<double>(h, h->s64, d.inc_a64), e, nullptr, h->partials,
                                                        h->tickets + T_STENCIL, &h->sc->pq_s, h->tickets + T_SHELL,
                                                        &h->sc->pq_d, h->red_blocks, st);
    }
  }, &out->stencil_ms));
  out->data_ms = 0.0;
  if (d.nrows > 0) {
    LS_TRY(timed([&] {
      if (f32) {
        rows_kernel<float><<<grid_for(h, d.nrows), kBlock, 0, st>>>(d.nrows, d.width, d.cols, d.a32, d.w2_32, h->p32, h->s32, nullptr);
        ++h->launches;
      } else {
        rows_kernel<double><<<grid_for(h, d.nrows), kBlock, 0, st>>>(d.nrows, d.width, d.cols, d.a64, d.w2_64, h->p64, h->s64, nullptr);
        ++h->launches;
      }
    }, &out->data_ms));
  }
  LS_TRY(timed([&] {
    if (f32) {
      update_xr_kernel<float><<<g, kBlock, 0, st>>>(n, h->x32, h->r32, h->p32, h->q32, h->dinv32, h->sc, h->partials, h->tickets + T_UPDATE);
      ++h->launches;
      update_p_kernel<float><<<g, kBlock, 0, st>>>(n, h->r32, h->dinv32, h->p32, h->sc, h->tickets + T_PUPD);
      ++h->launches;
    } else {
      update_xr_kernel<double><<<g, kBlock, 0, st>>>(n, h->x64, h->r64, h->p64, h->q64, h->dinv64, h->sc, h->partials, h->tickets + T_UPDATE);
      ++h->launches;
      update_p_kernel<double><<<g, kBlock, 0, st>>>(n, h->r64, h->dinv64, h->p64, h->sc, h->tickets + T_PUPD);
      ++h->launches;
    }
  }, &out->update_ms));
  LS_TRY(timed([&] {
    if (f32) launch_iteration<float>(h, h->x32, h->r32, h->p32, h->q32, h->dinv32, st);
    else launch_iteration<double>(h, h->x64, h->r64, h->p64, h->q64, h->dinv64, st);
  }, &out->iteration_ms));
  sc = CgScalars{};
  LS_TRY(write_scalars(h));
  out->stencil_bytes = 2.0 * (double)n * (double)s;
  out->iteration_bytes = 9.0 * (double)n * (double)s + 16.0 * (double)(d.nrows * d.width);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}
