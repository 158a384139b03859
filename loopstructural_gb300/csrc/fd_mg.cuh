// Geometric multigrid V-cycle (FP32) used as the CG preconditioner of the
// mixed-precision FD solve.  Not a reference algorithm: it changes only the
// iteration path; the solution is still the one of the reference's normal
// equations (the outer CG stops on the reference's scaled-residual test).
//
// Hierarchy: level l+1 has n_{l+1} = n_l / 2 + 1 nodes per axis, coarse node J
// sitting on fine node 2J (the coarse grid may reach one fine cell past an
// even-sized fine grid).  Prolongation P is trilinear (weights 1 and 1/2 per
// axis), restriction is P^T.
//   * regularisation: Galerkin, P^T A_l P, on every coarse level -- a sum of
//     tensor products of 1-D banded matrices (fd_galerkin.cuh), coarsened
//     axis by axis;
//   * data rows: Galerkin, row_{l+1} = row_l P (at most 27 coarse columns).
//     P is exact on trilinear functions, so a row confined to one fine cell
//     stays confined to one coarse cell; on levels >= 1 the rows confined to
//     one cell are summed into a per-node 27-point stencil (sum of
//     w^2 a_i a_j over the rows), evaluated inside the apply kernel from the
//     staged neighbourhood; other rows keep the row form;
//   * ridge^2 scaled by 8 per level;
//   * smoother: Chebyshev polynomial of D^-1 A on [lmax/20, 1.05 lmax]
//     (lmax by power iteration), `deg` steps pre and post -- symmetric, so the
//     V-cycle is an SPD preconditioner;
//   * coarsest level (<= 512 nodes): dense inverse.
#pragma once

#include <vector>

#include "fd_apply.cuh"
#include "fd_galerkin.cuh"
#include "ls_common.cuh"

namespace ls {

struct MgLevel {
  int nx = 0, ny = 0, nz = 0;
  int64_t n = 0;
  StencilCoef coef64{};
  CoefT<float> coef{};
  // data rows (FP32)
  int64_t nrows = 0;
  int width = 0;
  int32_t *cols = nullptr;
  float *a = nullptr, *w2 = nullptr, *s = nullptr;
  int64_t ntouched = 0;
  uint32_t *mask = nullptr;
  int32_t *word_rank = nullptr;
  int64_t *inc_ptr = nullptr;
  int32_t *inc_row = nullptr;
  float *inc_a = nullptr;
  float *qd = nullptr;  // per-touched-node data totals (levels with long incidence lists)
  // 27-point form of the data rows confined to one cell (levels >= 1)
  int64_t knt = 0;
  uint32_t *kmask = nullptr;
  int32_t *krank = nullptr;
  float *k27 = nullptr;
  std::vector<float> k27host;      // host copy ([27][knt]) and the nodes, for the coarsest dense matrix
  std::vector<int64_t> k27nodes;
  float *dinv = nullptr;
  // directional regularisation weights (6 x n, family-major; level 0: the
  // handle's, coarse levels: restricted) and the scratch for the isotropic
  // part of an apply that the directional kernel completes
  float *dir = nullptr;
  float *dq = nullptr;
  // coarse levels: row mass of the averaged weights and their square roots
  float *dmass = nullptr, *dsw = nullptr;
  // Galerkin regularisation operator (first coarse level)
  bool g1 = false;
  G1Op g1op{};
  std::vector<double> g1host[3];  // the 1-D tables (FP64), for coarsening to the next level
  // vectors: b (rhs), x (solution), r (residual), d[2] (Chebyshev directions)
  float *b = nullptr, *x = nullptr, *r = nullptr, *d0 = nullptr, *d1 = nullptr;
  bool owns_bx = true;
  // Chebyshev
  float lmax = 0.f;
  std::vector<float> c1, c2;  // per step
  float inv_theta = 0.f;
};

struct MgHierarchy {
  std::vector<MgLevel> levels;
  double *coarse_inv64 = nullptr;  // dense inverse of the coarsest operator (FP64), row-major
  float *dir_u = nullptr, *dir_v = nullptr;  // 6 x n(level 1) scratch of the coarse directional passes
  int deg = 3;
  bool built = false;
  std::vector<void *> allocations;
  // host wall time (ms) of the setup phases, each ended by a stream sync:
  // host rows, regularisation tables, data-row coarsening, data-term upload,
  // diagonals, eigenvalue estimates, coarsest inverse, total
  double setup_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void mg_cheb_init_kernel(int64_t n, const float *__restrict__ b, const float *__restrict__ dinv,
                                    float inv_theta, float *__restrict__ r, float *__restrict__ d,
                                    float *__restrict__ x, const int *done) {
  if (done && *done) return;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const float bv = b[g];
    r[g] = bv;
    d[g] = inv_theta * dinv[g] * bv;
    x[g] = 0.f;
  }
}

// b_c = P^T r_f (3-D launch: block 32 x 8 over coarse x-y, blockIdx.z = coarse z)
__global__ void mg_restrict_kernel(int nfx, int nfy, int nfz, int ncx, int ncy, int ncz, const float *__restrict__ rf,
                                   float *__restrict__ bc, const int *done) {
  if (done && *done) return;
  const int I = blockIdx.x * blockDim.x + threadIdx.x, J = blockIdx.y * blockDim.y + threadIdx.y, K = blockIdx.z;
  if (I >= ncx || J >= ncy || K >= ncz) return;
  float acc = 0.f;
#pragma unroll
  for (int dz = -1; dz <= 1; ++dz) {
    const int k = 2 * K + dz;
    if (k < 0 || k >= nfz) continue;
    const float wz = dz == 0 ? 1.f : 0.5f;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const int j = 2 * J + dy;
      if (j < 0 || j >= nfy) continue;
      const float wyz = wz * (dy == 0 ? 1.f : 0.5f);
      const float *row = rf + ((size_t)k * nfy + j) * nfx;
#pragma unroll
      for (int dx = -1; dx <= 1; ++dx) {
        const int i = 2 * I + dx;
        if (i < 0 || i >= nfx) continue;
        acc += wyz * (dx == 0 ? 1.f : 0.5f) * __ldg(row + i);
      }
    }
  }
  bc[((size_t)K * ncy + J) * ncx + I] = acc;
}

// x_f += P x_c (3-D launch over fine x-y, blockIdx.z = fine z).  Branch-free:
// the 8 coarse corners of the fine node's coarse cell are always read (an
// index past the coarse grid is clamped and weighted 0); per axis the weights
// are (1, 0) on even fine indices and (1/2, 1/2) on odd ones.
__global__ void mg_prolong_kernel(int nfx, int nfy, int nfz, int ncx, int ncy, const float *__restrict__ xc,
                                  float *__restrict__ xf, const int *done) {
  if (done && *done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
  if (i >= nfx || j >= nfy || k >= nfz) return;
  const int i0 = i >> 1, j0 = j >> 1, k0 = k >> 1;
  const int oi = i & 1, oj = j & 1, ok = k & 1;
  const int i1 = i0 + oi, j1 = j0 + oj;  // = i0 on even fine indices (weight 0 there)
  const float wi1 = oi ? 0.5f : 0.f, wj1 = oj ? 0.5f : 0.f, wk1 = ok ? 0.5f : 0.f;
  const float wi0 = 1.f - wi1, wj0 = 1.f - wj1, wk0 = 1.f - wk1;
  const float *r00 = xc + ((size_t)k0 * ncy + j0) * ncx, *r01 = xc + ((size_t)k0 * ncy + j1) * ncx;
  const float *r10 = xc + ((size_t)(k0 + ok) * ncy + j0) * ncx, *r11 = xc + ((size_t)(k0 + ok) * ncy + j1) * ncx;
  const float v0 = wj0 * (wi0 * __ldg(r00 + i0) + wi1 * __ldg(r00 + i1)) + wj1 * (wi0 * __ldg(r01 + i0) + wi1 * __ldg(r01 + i1));
  const float v1 = wj0 * (wi0 * __ldg(r10 + i0) + wi1 * __ldg(r10 + i1)) + wj1 * (wi0 * __ldg(r11 + i0) + wi1 * __ldg(r11 + i1));
  xf[((size_t)k * nfy + j) * nfx + i] += wk0 * v0 + wk1 * v1;
}

// x = Minv b in FP64 (the coarsest operator can be ill-conditioned), one warp per row
__global__ void mg_dense_kernel(int nc, const double *__restrict__ minv, const float *__restrict__ b,
                                float *__restrict__ x, const int *done) {
  if (done && *done) return;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nc) return;
  double acc = 0.0;
  for (int j = lane; j < nc; j += 32) acc += minv[(int64_t)warp * nc + j] * (double)__ldg(b + j);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) x[warp] = (float)acc;
}

// sum of a.(w b) with an optional weight vector (FP32 in, FP64 out)
__global__ void __launch_bounds__(256) mg_dot_kernel(int64_t n, const float *__restrict__ a, const float *__restrict__ b,
                                                     const float *__restrict__ w, double *partials,
                                                     unsigned int *ticket, double *out) {
  float l = 0.f;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    l += a[g] * (w ? w[g] * b[g] : b[g]);
  double tot;
  if (grid_sum<256, float>(l, partials, ticket, &tot)) *out = tot;
}

__global__ void mg_scale_kernel(int64_t n, const float *__restrict__ src, const float *__restrict__ w, float scale,
                                float *__restrict__ dst) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    dst[g] = scale * (w ? w[g] : 1.f) * src[g];
}

}  // namespace ls
