// Data rows confined to one cell, on the coarse multigrid levels (device).
//
// A row whose columns lie in one cell (every point row: trilinear or
// element-gradient coefficients on the 8 corners of the point's cell) keeps
// that property under the trilinear prolongation: row_c = row_f P lies in the
// cell (i >> 1, j >> 1, k >> 1), and per axis the fine corners map to the
// coarse ones by the parity of i -- even: corner 0 -> 0, corner 1 -> (1/2, 1/2);
// odd: corner 0 -> (1/2, 1/2), corner 1 -> 1.  So a level's cell rows are
// (cell, 8 corner coefficients, w^2), coarsened in place, one thread per row.
//
// Their normal-equations block is w^2 c c^T on the cell's corners.  A node's
// 27-point stencil (offset o = 9 (dz + 1) + 3 (dy + 1) + (dx + 1)) sums it over
// the node's 8 cells in a fixed order and, within a cell, over the cell's rows
// in array order, so the result does not depend on thread scheduling -- no
// float atomics.  The rows are sorted once, on the finest level, by the Morton
// code of their cell; coarsening a cell drops the last 3 bits of its code, so
// on every level the rows of a cell stay one contiguous run of the array
// (cell_segments_kernel finds the runs; nothing is sorted per level).
#pragma once

#include "ls_common.cuh"

namespace ls {

struct CellRows {
  int64_t nrows = 0;
  int32_t *ci = nullptr, *cj = nullptr, *ck = nullptr;  // cell (lowest corner)
  double *c = nullptr;                                 // 8 per row, corner bits x | y << 1 | z << 2
  double *w2 = nullptr;
};

__device__ __forceinline__ int64_t cell_index(int i, int j, int k, int cx, int cy) {
  return i + (int64_t)cx * (j + (int64_t)cy * k);
}

__global__ void cell_coarsen_kernel(int64_t nrows, int32_t *__restrict__ ci, int32_t *__restrict__ cj,
                                    int32_t *__restrict__ ck, double *__restrict__ c) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int b[3] = {ci[r], cj[r], ck[r]};
    // m[a][fine corner][coarse corner]
    double m[3][2][2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const bool odd = b[a] & 1;
      m[a][0][0] = odd ? 0.5 : 1.0;
      m[a][0][1] = odd ? 0.5 : 0.0;
      m[a][1][0] = odd ? 0.0 : 0.5;
      m[a][1][1] = odd ? 1.0 : 0.5;
    }
    double in[8], out[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      in[q] = c[8 * r + q];
      out[q] = 0.0;
    }
#pragma unroll
    for (int f = 0; f < 8; ++f)
#pragma unroll
      for (int q = 0; q < 8; ++q)
        out[q] += in[f] * (m[0][f & 1][q & 1] * m[1][(f >> 1) & 1][(q >> 1) & 1] * m[2][(f >> 2) & 1][(q >> 2) & 1]);
#pragma unroll
    for (int q = 0; q < 8; ++q) c[8 * r + q] = out[q];
    ci[r] = b[0] >> 1;
    cj[r] = b[1] >> 1;
    ck[r] = b[2] >> 1;
  }
}

// [start, end) of each cell's run of rows (cells without rows keep 0, 0)
__global__ void cell_segments_kernel(int64_t nrows, const int32_t *__restrict__ ci, const int32_t *__restrict__ cj,
                                     const int32_t *__restrict__ ck, int cx, int cy, int64_t *__restrict__ start,
                                     int64_t *__restrict__ end) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = cell_index(ci[r], cj[r], ck[r], cx, cy);
    if (r == 0 || cell_index(ci[r - 1], cj[r - 1], ck[r - 1], cx, cy) != cell) start[cell] = r;
    if (r == nrows - 1 || cell_index(ci[r + 1], cj[r + 1], ck[r + 1], cx, cy) != cell) end[cell] = r + 1;
  }
}

// bit per node: does any of its (up to 8) cells hold rows?  Word counts for the ranks.
__global__ void cell_touch_kernel(int nx, int ny, int nz, const int64_t *__restrict__ start,
                                  const int64_t *__restrict__ end, uint32_t *__restrict__ mask,
                                  int32_t *__restrict__ wcount) {
  const int64_t n = (int64_t)nx * ny * nz, nwords = (n + 31) / 32;
  const int lane = threadIdx.x & 31;
  const int cx = nx - 1, cy = ny - 1, cz = nz - 1;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g - lane < nwords * 32;
       g += (int64_t)gridDim.x * blockDim.x) {
    bool t = false;
    if (g < n) {
      const int k = (int)(g / ((int64_t)nx * ny));
      const int rem = (int)(g - (int64_t)k * nx * ny);
      const int j = rem / nx, i = rem - j * nx;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        const int ii = i - (b & 1), jj = j - ((b >> 1) & 1), kk = k - ((b >> 2) & 1);
        if (ii >= 0 && jj >= 0 && kk >= 0 && ii < cx && jj < cy && kk < cz) {
          const int64_t cell = cell_index(ii, jj, kk, cx, cy);
          t |= end[cell] > start[cell];
        }
      }
    }
    const uint32_t word = __ballot_sync(0xffffffffu, t);
    if (lane == 0) {
      mask[g >> 5] = word;
      wcount[g >> 5] = __popc(word);
    }
  }
}

// the 27-point stencils of the marked nodes ([27][knt], rank order) and the
// per-word ranks
__global__ void cell_k27_kernel(int nx, int ny, int nz, const uint32_t *__restrict__ mask,
                                const int64_t *__restrict__ wrank64, const int64_t *__restrict__ start,
                                const int64_t *__restrict__ end, const double *__restrict__ c,
                                const double *__restrict__ w2, int64_t knt, float *__restrict__ k27,
                                int32_t *__restrict__ krank) {
  const int64_t n = (int64_t)nx * ny * nz;
  const int cx = nx - 1, cy = ny - 1, cz = nz - 1;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w = g >> 5;
    const uint32_t word = mask[w], bit = 1u << (g & 31);
    if ((g & 31) == 0) krank[w] = (int32_t)wrank64[w];
    if (!(word & bit)) continue;
    const int64_t rank = wrank64[w] + __popc(word & (bit - 1u));
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    double acc[27];
#pragma unroll
    for (int o = 0; o < 27; ++o) acc[o] = 0.0;
#pragma unroll
    for (int b = 0; b < 8; ++b) {  // the node is corner b of cell (i, j, k) - b
      const int ii = i - (b & 1), jj = j - ((b >> 1) & 1), kk = k - ((b >> 2) & 1);
      if (ii < 0 || jj < 0 || kk < 0 || ii >= cx || jj >= cy || kk >= cz) continue;
      const int64_t cell = cell_index(ii, jj, kk, cx, cy);
      for (int64_t r = start[cell]; r < end[cell]; ++r) {
        const double wb = w2[r] * c[8 * (int64_t)r + b];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const int o = 9 * (((q >> 2) & 1) - ((b >> 2) & 1) + 1) + 3 * (((q >> 1) & 1) - ((b >> 1) & 1) + 1) +
                        ((q & 1) - (b & 1) + 1);
          acc[o] += wb * c[8 * (int64_t)r + q];
        }
      }
    }
#pragma unroll
    for (int o = 0; o < 27; ++o) k27[o * knt + rank] = (float)acc[o];
  }
}

// diag[node] += centre entry of the node's 27-point stencil
__global__ void k27_diag_kernel(int64_t n, const uint32_t *__restrict__ mask, const int32_t *__restrict__ krank,
                                const float *__restrict__ k27, int64_t knt, double *__restrict__ diag) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t word = mask[g >> 5], bit = 1u << (g & 31);
    if (!(word & bit)) continue;
    const int64_t rank = krank[g >> 5] + __popc(word & (bit - 1u));
    diag[g] += (double)k27[13 * knt + rank];
  }
}

}  // namespace ls
