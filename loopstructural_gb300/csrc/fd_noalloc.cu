// ls_fd_apply_noalloc: the FP64 normal-operator apply for callers that cannot
// allocate device memory.
//
// Who needs it: code running where cudaMalloc is off limits -- a host
// framework that owns all device memory through its own pool and forbids side
// allocations, a plugin loaded into a process with a fixed device-memory
// budget, or a latency-critical loop that must not enter the driver's
// allocator.  Those callers still own every input and output buffer; what they
// cannot provide is the operator's private scratch (one FP64 value per data
// row, plus the reduction partials of the optional x.Nx dot product).
//
// The scratch is a file-scope static __device__ array of LS_NOALLOC_SCRATCH_DOUBLES
// doubles (8.4 MB) that every GPU which loads this library holds until the
// process exits.  It caps the data rows at LS_NOALLOC_MAX_ROWS; larger systems
// are rejected with LS_ERR_ARG.  All calls share the one array and it keeps
// the last call's contents: calls that overlap on the GPU (different streams,
// or different host threads) race on it and must be serialised by the caller.
// The data-row scatter uses FP64 atomics, so results may differ from
// ls_fd_apply in the last bits.  Data-row columns must be < dof: a column
// outside the grid is skipped by the kernels and raises a flag word in the
// scratch, which the call reports as LS_ERR_ARG when it reads x.Nx back.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>

#include "fd_stencil.cuh"
#include "ls_common.cuh"

namespace {

constexpr int kNoallocTX = 32, kNoallocTY = 8;
constexpr int kNoallocBlock = kNoallocTX * kNoallocTY;
constexpr int64_t kMaxRows = LS_NOALLOC_MAX_ROWS;
constexpr int kMaxBlocks = 4096;
// layout: [0, kMaxRows) per-row products | [kMaxRows, +kMaxBlocks) partials |
//         ticket word | dot result | bad-column flag
constexpr int64_t kScratchDoubles = kMaxRows + kMaxBlocks + 8;
static_assert(kScratchDoubles == LS_NOALLOC_SCRATCH_DOUBLES, "scratch size mismatch");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// device address of g_noalloc_scratch per device, resolved once per device
// (every thread that resolves it stores the same address)
std::atomic<double *> g_scratch_ptr[64];

__global__ void __launch_bounds__(kNoallocBlock) noalloc_stencil_kernel(ls::CoefT<double> c,
                                                                        const double *__restrict__ x,
                                                                        double *__restrict__ y) {
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int i = blockIdx.x * kNoallocTX + threadIdx.x, j = blockIdx.y * kNoallocTY + threadIdx.y;
  if (i >= nx || j >= ny) return;
  for (int k = blockIdx.z; k < nz; k += gridDim.z) {
    const int g = i + nx * (j + ny * k);
    y[g] = ls::stencil_node32<double>(c, x, g, i, j, k);
  }
}

// s_r = w_r^2 (a_r . x) into the scratch
// (a column >= n is skipped and raises *bad)
__global__ void noalloc_rows_kernel(int64_t nrows, int width, int64_t n, const int64_t *__restrict__ idc,
                                    const double *__restrict__ a, const double *__restrict__ w,
                                    const double *__restrict__ x, double *__restrict__ s, unsigned int *bad) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int k = 0; k < width; ++k) {
      const int64_t col = idc[r * width + k];
      if (col >= n) {
        *bad = 1u;
      } else if (col >= 0) {
        acc += a[r * width + k] * x[col];
      }
    }
    s[r] = w[r] * w[r] * acc;
  }
}

// y[col] += a_rk s_r
// (columns outside [0, n) are skipped; the rows kernel has flagged them)
__global__ void noalloc_scatter_kernel(int64_t nrows, int width, int64_t n, const int64_t *__restrict__ idc,
                                       const double *__restrict__ a, const double *__restrict__ s,
                                       double *__restrict__ y) {
  const int64_t ne = nrows * width;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t col = idc[e];
    if (col >= 0 && col < n) atomicAdd(y + col, a[e] * s[e / width]);
  }
}

// x . y with the fixed-order last-block reduction; partials and ticket live in
// the scratch
__global__ void __launch_bounds__(256) noalloc_dot_kernel(int64_t n, const double *__restrict__ x,
                                                          const double *__restrict__ y, double *partials,
                                                          unsigned int *ticket, double *out) {
  double l = 0.0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
    l += x[g] * y[g];
  double tot;
  if (ls::grid_sum<256>(l, partials, ticket, &tot)) *out = tot;
}

int scratch_for_current_device(double **out) {
  int dev = 0;
  LS_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    ls::set_error("device ordinal %d out of range", dev);
    return LS_ERR_ARG;
  }
  double *cached = g_scratch_ptr[dev].load(std::memory_order_relaxed);
  if (cached == nullptr) {
    void *p = nullptr;
    LS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    cached = static_cast<double *>(p);
    g_scratch_ptr[dev].store(cached, std::memory_order_relaxed);
  }
  *out = cached;
  return LS_OK;
}

}  // namespace

extern "C" int ls_fd_apply_noalloc(const ls_fd_system *sys, const double *d_x, double *d_y, double *h_xNx,
                                   void *stream) {
  LS_ARG_CHECK(sys != nullptr && d_x != nullptr && d_y != nullptr, "NULL argument");
  const ls_grid3 &g = sys->grid;
  for (int d = 0; d < 3; ++d) {
    LS_ARG_CHECK(g.nsteps[d] >= 2, "every axis needs at least 2 nodes");
    LS_ARG_CHECK(g.step[d] > 0.0, "step must be positive");
  }
  const int64_t n = g.nsteps[0] * g.nsteps[1] * g.nsteps[2];
  LS_ARG_CHECK(n < (int64_t)2000000000, "grid too large");
  LS_ARG_CHECK(sys->nrows >= 0, "nrows < 0");
  LS_ARG_CHECK(sys->d_dir == nullptr, "directional regularisation needs a handle; use ls_fd_create + ls_fd_apply");
  if (sys->nrows > kMaxRows) {
    ls::set_error("ls_fd_apply_noalloc: %lld data rows exceed the static scratch limit of %lld rows "
                  "(LS_NOALLOC_MAX_ROWS); use ls_fd_create + ls_fd_apply", (long long)sys->nrows,
                  (long long)kMaxRows);
    return LS_ERR_ARG;
  }
  LS_ARG_CHECK(sys->nrows == 0 || (sys->width >= 1 && sys->width <= 64), "width must be in [1, 64]");
  LS_ARG_CHECK(sys->nrows == 0 || (sys->d_idc && sys->d_a && sys->d_w), "NULL data-row buffer");
  double *scratch = nullptr;
  LS_TRY(scratch_for_current_device(&scratch));
  cudaStream_t s = ls::as_stream(stream);
  const ls::StencilCoef c64 = ls::make_stencil_coef(g, sys->w_dxx, sys->w_dyy, sys->w_dzz, sys->w_dxy, sys->w_dyz,
                                                  sys->w_dxz, sys->w_dx, sys->w_dy, sys->w_dz, sys->ridge);
  const int gx = (int)((g.nsteps[0] + kNoallocTX - 1) / kNoallocTX);
  const int64_t gy = (g.nsteps[1] + kNoallocTY - 1) / kNoallocTY;
  LS_ARG_CHECK(gy <= 65535, "ls_fd_apply_noalloc: the y axis is limited to 524,280 nodes");
  const int gz = (int)std::min<int64_t>(g.nsteps[2], 64);
  double *partials = scratch + kMaxRows;
  unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + kMaxRows + kMaxBlocks);
  double *out = scratch + kMaxRows + kMaxBlocks + 1;  // out[0] = x.Nx, out[1] = bad-column flag word
  unsigned int *bad = reinterpret_cast<unsigned int *>(out + 1);
  // the ticket and the flag must start at zero; the scratch keeps whatever the last call left
  LS_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(double), s));
  LS_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(double), s));
  noalloc_stencil_kernel<<<dim3(gx, (int)gy, gz), dim3(kNoallocTX, kNoallocTY), 0, s>>>(ls::coef_as<double>(c64), d_x,
                                                                                         d_y);
  if (sys->nrows > 0) {
    noalloc_rows_kernel<<<ls::stream_grid(sys->nrows, 256), 256, 0, s>>>(sys->nrows, sys->width, n, sys->d_idc,
                                                                         sys->d_a, sys->d_w, d_x, scratch, bad);
    noalloc_scatter_kernel<<<ls::stream_grid(sys->nrows * sys->width, 256), 256, 0, s>>>(
        sys->nrows, sys->width, n, sys->d_idc, sys->d_a, scratch, d_y);
  }
  if (h_xNx != nullptr) {
    const int nb = std::min(ls::stream_grid(n, 256), kMaxBlocks);
    noalloc_dot_kernel<<<nb, 256, 0, s>>>(n, d_x, d_y, partials, ticket, out);
    double back[2] = {0.0, 0.0};
    LS_CUDA_TRY(cudaMemcpyAsync(back, out, sizeof(back), cudaMemcpyDeviceToHost, s));
    LS_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned int flag = 0;
    memcpy(&flag, &back[1], sizeof(flag));
    if (flag != 0) {
      ls::set_error("ls_fd_apply_noalloc: a data-row column is outside [0, dof); those entries were skipped");
      return LS_ERR_ARG;
    }
    *h_xNx = back[0];
  }
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}
