// Shared helpers of the sm_103a kernels: error reporting, deterministic
// block/grid reductions and structured-grid index arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/ls_gb300.h"

namespace ls {

// Thread-local error text for ls_last_error().
void set_error(const char *fmt, ...);

#define LS_CUDA_TRY(expr)                                                                   \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) {                                                                \
      ::ls::set_error("%s:%d %s -> %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return LS_ERR_CUDA;                                                                   \
    }                                                                                       \
  } while (0)

#define LS_ARG_CHECK(cond, msg)                   \
  do {                                            \
    if (!(cond)) {                                \
      ::ls::set_error("invalid argument: %s", msg); \
      return LS_ERR_ARG;                          \
    }                                             \
  } while (0)

#define LS_TRY(expr)          \
  do {                        \
    int _s = (expr);          \
    if (_s < 0) return _s;    \
  } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per process, device 0..63).
int sm_count();

// Grid size for a grid-stride streaming kernel: a multiple of the SM count.
inline int stream_grid(int64_t n, int block, int per_sm = 8) {
  int64_t want = (n + block - 1) / block;
  int64_t cap = (int64_t)sm_count() * per_sm;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (int)want;
}

// ---------------------------------------------------------------------------
// Deterministic grid reduction: every block writes its partial (FP64) to
// partials[blockIdx.x]; the last block to arrive (ticket) sums the partials in
// index order and hands the total to `finish` -- no float atomics, so the
// result is bit-reproducible run to run.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int linear_tid() {
  return threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
}

template <int BLOCK, typename V>
__device__ __forceinline__ V block_sum(V v, V *smem) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int t = linear_tid();
  const int lane = t & 31, warp = t >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  v = (V)0;
  if (warp == 0) {
    v = (lane < BLOCK / 32) ? smem[lane] : (V)0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;  // valid in thread 0
}

// Returns true in thread 0 of the last block; *total then holds the sum.
// `tid` is the thread's linear index in its block, `bid` / `nblocks` the
// block's linear index and the grid size (3-D grids pass their own).
// The block partial is formed in the value type V (FP32 block sums keep the
// slow FP64 pipe out of FP32 kernels); partials and the final sum are FP64.
template <int BLOCK, typename V>
__device__ __forceinline__ bool grid_sum_ex(V v, double *partials, unsigned int *ticket, double *total,
                                            int tid, unsigned int bid, unsigned int nblocks) {
  __shared__ V redv[BLOCK / 32];
  __shared__ double red[BLOCK / 32];
  __shared__ bool last;
  const V bv = block_sum<BLOCK, V>(v, redv);
  if (tid == 0) {
    partials[bid] = (double)bv;
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == nblocks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // last block: fixed-order sum of the partials
  double s = 0.0;
  for (int i = tid; i < (int)nblocks; i += BLOCK) s += ((volatile double *)partials)[i];
  s = block_sum<BLOCK, double>(s, red);
  if (tid == 0) {
    *total = s;
    *ticket = 0u;  // re-arm for the next launch
  }
  return tid == 0;
}

// True in thread 0 of the last block of a 1-D grid to arrive here (all other
// blocks' writes fenced before); re-arms the ticket.  Every block must call it.
__device__ __forceinline__ bool grid_last_block(unsigned int *ticket) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
    if (last) *ticket = 0u;
  }
  __syncthreads();
  return last && threadIdx.x == 0;
}

template <int BLOCK, typename V = double>
__device__ __forceinline__ bool grid_sum(V v, double *partials, unsigned int *ticket, double *total) {
  return grid_sum_ex<BLOCK, V>(v, partials, ticket, total, threadIdx.x, blockIdx.x, gridDim.x);
}

// Two sums in one pass.
template <int BLOCK>
__device__ __forceinline__ bool grid_sum2(double v0, double v1, double *partials, unsigned int *ticket,
                                          double *t0, double *t1) {
  __shared__ double red[BLOCK / 32];
  __shared__ bool last;
  double b0 = block_sum<BLOCK, double>(v0, red);
  double b1 = block_sum<BLOCK, double>(v1, red);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = b0;
    partials[2 * blockIdx.x + 1] = b1;
    __threadfence();
    unsigned int t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s0 = 0.0, s1 = 0.0;
  for (int i = threadIdx.x; i < (int)gridDim.x; i += BLOCK) {
    s0 += ((volatile double *)partials)[2 * i];
    s1 += ((volatile double *)partials)[2 * i + 1];
  }
  s0 = block_sum<BLOCK>(s0, red);
  s1 = block_sum<BLOCK>(s1, red);
  if (threadIdx.x == 0) {
    *t0 = s0;
    *t1 = s1;
    *ticket = 0u;
  }
  return threadIdx.x == 0;
}

}  // namespace ls
