// Finest-level FP32 normal-operator apply with TMA-staged planes.
//
//     q = (sum_f w_f^2 R_f^T R_f + A_d^T W A_d + ridge^2 I) p,  then an epilogue
//
// One kernel covers every node of the grid (deep interior and the 3-node
// boundary shell).  A block owns a 32 x 8 column tile and marches along z
// through a segment of planes.  The planes of p it needs (the tile plus a
// 2-node halo, 40 x 12 nodes: x starts 4 nodes left of the tile so that the
// copy starts on a 16-byte boundary) arrive by cp.async.bulk.tensor into a
// ring of kTmSlots shared-memory slots, each tracked by one mbarrier; the
// same slot also receives, by TMA, the epilogue operands (x, r, D^-1 or b,
// D^-1) of the output plane two behind, so one wait per step covers both.
// Outside the grid the tensor copy fills zeros, which is exactly the zero
// halo the boundary formula needs.  Five planes (z-2 .. z+2) are live while
// plane z is emitted; the remaining kTmSlots - 5 slots are in flight.
//
// Deep nodes ([3, n-4]^3) use the constant composite stencil with register
// windows over z (as fd_apply.cuh); shell nodes use the exact branch-free sum
// shell_node() on the staged neighbourhood.  The data term at touched nodes
// is a per-node total qd[rank] produced just before by data_node_totals_kernel,
// prefetched one plane ahead.
//
// Every mbarrier wait is bounded (kTmSpin polls with a 1 us suspend hint); a
// timeout raises *fault, ends the block's march (after a bounded wait for its
// copies in flight) and the host reports it as an error.
#pragma once

#include <cuda.h>

#include <vector>

#include "fd_apply.cuh"

namespace ls {

constexpr int kTmX = 32, kTmY = 8, kTmThreads = kTmX * kTmY;
constexpr int kTmPX = kTmX + 8;             // staged plane: x0 - 4 .. x0 + 35
constexpr int kTmPY = kTmY + 4;             // y0 - 2 .. y0 + 9
constexpr int kTmPlane = kTmPX * kTmPY;     // 480 floats (1920 B)
constexpr int kTmOp = kTmX * kTmY;          // 256 floats (1 KB)
constexpr int kTmSlots = 8;
constexpr int kTmBlocksPerSm = 4;
constexpr int kTmSpin = 1 << 20;            // polls of one mbarrier before giving up
constexpr int kTmSuspendNs = 1000;          // suspend-time hint of one poll (~1 s in all)

template <int EPI>
struct TmOps {
  static constexpr int n = EPI == EPI_CHEB ? 3 : (EPI == EPI_RESID ? 2 : 0);
};

template <int EPI>
constexpr int tm_slot_floats() {
  return kTmPlane + TmOps<EPI>::n * kTmOp;
}

// dynamic shared memory of one block: the slots plus room to round the base
// up to a 128-byte boundary (tensor-copy destinations)
template <int EPI>
constexpr int tm_smem_bytes() {
  return kTmSlots * tm_slot_floats<EPI>() * (int)sizeof(float) + 128;
}

// Tensor maps of one launch (kernel parameter, __grid_constant__): the applied
// vector with the halo box, and the epilogue operands with the tile box.
struct TmMaps {
  CUtensorMap p;
  CUtensorMap op[3];
};

__device__ __forceinline__ uint32_t smem_u32(const void *ptr) {
  return (uint32_t)__cvta_generic_to_shared(ptr);
}

__device__ __forceinline__ void tm_bar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void tm_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void tm_expect(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tm_load3(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// true once the barrier's phase with this parity has completed; false after
// kTmSpin polls
__device__ __forceinline__ bool tm_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (int it = 0; it < kTmSpin; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2, %3;\n selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(kTmSuspendNs)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// qd[t] = sum over the incidences e of touched node t of a_e w_r^2 (a_r . p),
// r = row(e): the data term of every touched node, each row's dot product
// recomputed per incidence in the order of rows_kernel + data_term.
template <typename T>
__global__ void data_node_totals_kernel(int64_t ntouched, const int64_t *__restrict__ inc_ptr,
                                        const int32_t *__restrict__ inc_row, const T *__restrict__ inc_a, int width,
                                        const int32_t *__restrict__ cols, const T *__restrict__ a,
                                        const T *__restrict__ w2, const T *__restrict__ p, T *__restrict__ qd,
                                        const int *done) {
  if (done && *done) return;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntouched;
       t += (int64_t)gridDim.x * blockDim.x) {
    T acc = 0;
    const int64_t e1 = inc_ptr[t + 1];
    for (int64_t e = inc_ptr[t]; e < e1; ++e) {
      const int64_t r = inc_row[e];
      T dot = 0;
      for (int k = 0; k < width; ++k) {
        const int32_t col = cols[r * width + k];
        if (col >= 0) dot += a[r * width + k] * p[col];
      }
      acc += inc_a[e] * (w2[r] * dot);
    }
    qd[t] = acc;
  }
}

template <int EPI>
__global__ void __launch_bounds__(kTmThreads, kTmBlocksPerSm)
    fd_tma_apply_kernel(const __grid_constant__ TmMaps maps, CoefT<float> c, DataView<float> dv, EpiArgs<float> e,
                        const int *done, int ntx, int zlen, double *partials, unsigned int *ticket, double *dot_out,
                        double *dot_clear, int *fault) {
  if (done && *done) return;
  constexpr int NOP = TmOps<EPI>::n;
  constexpr int SLOT = tm_slot_floats<EPI>();
  extern __shared__ __align__(128) unsigned char tm_raw[];
  float *const tm_smem = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(tm_raw) + 127) & ~(uintptr_t)127);
  __shared__ __align__(8) uint64_t bars[kTmSlots];
  const int tid = threadIdx.x, tx = tid & (kTmX - 1), ty = tid / kTmX;
  const int x0 = (int)(blockIdx.x % ntx) * kTmX, y0 = (int)(blockIdx.x / ntx) * kTmY;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int z0 = blockIdx.y * zlen, z1 = min(nz, z0 + zlen);
  const int i = x0 + tx, j = y0 + ty;
  const bool col_in = (i < nx) & (j < ny);
  const int sxy = nx * ny;
  const int gcol = j * nx + i;
  const int tfirst = z0 - 2, tlast = z1 + 1;  // staged planes of p
  const int hx = tx + 4, hy = ty + 2;         // the column's position in a staged plane
  const int own = hy * kTmPX + hx;

  auto slot_of = [&](int t) -> float * { return tm_smem + ((t - tfirst) % kTmSlots) * SLOT; };
  auto bar_of = [&](int t) -> uint64_t * { return &bars[(t - tfirst) % kTmSlots]; };
  auto parity_of = [&](int t) -> uint32_t { return (uint32_t)(((t - tfirst) / kTmSlots) & 1); };
  // one elected thread: plane t of p and, when t - 2 is an output plane, the
  // epilogue operands of plane t - 2, all on the slot's barrier
  auto issue = [&](int t) {
    float *s = slot_of(t);
    uint64_t *b = bar_of(t);
    const bool ops = NOP > 0 && t - 2 >= z0;
    tm_expect(b, (uint32_t)((kTmPlane + (ops ? NOP * kTmOp : 0)) * sizeof(float)));
    tm_load3(s, &maps.p, x0 - 4, y0 - 2, t, b);
    if (ops) {
#pragma unroll
      for (int k = 0; k < NOP; ++k) tm_load3(s + kTmPlane + k * kTmOp, &maps.op[k], x0, y0, t - 2, b);
    }
  };

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < kTmSlots; ++s) tm_bar_init(&bars[s], 1);
    tm_fence_init();
  }
  __syncthreads();
  if (tid == 0)
    for (int t = tfirst; t <= min(tlast, tfirst + kTmSlots - 1); ++t) issue(t);

  // register windows over planes z-2 .. z+2: p, C_x p, C_y p at the column
  float P0 = 0.f, P1 = 0.f, P2 = 0.f, P3 = 0.f, P4 = 0.f;
  float X0 = 0.f, X1 = 0.f, X2 = 0.f, X3 = 0.f, X4 = 0.f;
  float Y0 = 0.f, Y1 = 0.f, Y2 = 0.f, Y3 = 0.f, Y4 = 0.f;
  auto inplane = [&](const float *pl, float &P, float &X, float &Y) {
    const float p0 = pl[own];
    P = p0;
    X = (pl[own - 2] + pl[own + 2]) - 2.f * p0;
    Y = (pl[own - 2 * kTmPX] + pl[own + 2 * kTmPX]) - 2.f * p0;
  };
  bool ok = true;
  {
    float *pls[4];
    for (int t = z0 - 2; t <= z0 + 1; ++t) {
      ok &= tm_wait(bar_of(t), parity_of(t));
      pls[t - z0 + 2] = slot_of(t);
    }
    inplane(pls[0], P0, X0, Y0);
    inplane(pls[1], P1, X1, Y1);
    inplane(pls[2], P2, X2, Y2);
    inplane(pls[3], P3, X3, Y3);
  }
  ok = __syncthreads_and(ok);

  // data term pipeline: mask word + word rank of plane z+1 / z+2, total of plane z / z+1
  const bool data_on = dv.enabled && col_in;
  auto word_of = [&](int z, uint32_t &w, int32_t &r) {
    w = 0u;
    r = 0;
    if (data_on && z < z1) {
      const int g = z * sxy + gcol;
      w = __ldg(dv.mask + (g >> 5));
      r = __ldg(dv.word_rank + (g >> 5));
    }
  };
  auto total_of = [&](int z, uint32_t w, int32_t r) -> float {
    if (!data_on || z >= z1) return 0.f;
    const int g = z * sxy + gcol;
    const uint32_t bit = 1u << (g & 31);
    return (w & bit) ? __ldg(dv.qd + r + __popc(w & (bit - 1u))) : 0.f;
  };
  uint32_t mw1 = 0u, mw2 = 0u;
  int32_t wr1 = 0, wr2 = 0;
  float qd0 = 0.f, qd1 = 0.f;
  {
    uint32_t mw0;
    int32_t wr0;
    word_of(z0, mw0, wr0);
    word_of(z0 + 1, mw1, wr1);
    qd0 = total_of(z0, mw0, wr0);
  }

  float local = 0.f;
  int z = z0;
  int zfail = z0 - 3;  // the step whose wait gave up (prologue: z0 - 3)
  for (; ok && z < z1; ++z) {
    ok = tm_wait(bar_of(z + 2), parity_of(z + 2));
    const float *pl2 = slot_of(z + 2);
    inplane(pl2, P4, X4, Y4);
    // data pipeline: total of plane z+1 requested, words of plane z+2 requested
    qd1 = total_of(z + 1, mw1, wr1);
    word_of(z + 2, mw2, wr2);
    if (col_in) {
      const float *po = slot_of(z);
      float q;
      const bool deep = (i >= 3) & (i <= nx - 4) & (j >= 3) & (j <= ny - 4) & (z >= 3) & (z <= nz - 4);
      if (deep) {
        const float q0 = P2;
        const float ex = po[own - 2] + po[own + 2], ey = po[own - 2 * kTmPX] + po[own + 2 * kTmPX];
        const float d4x = ex - 4.f * (po[own - 1] + po[own + 1]) + 6.f * q0;
        const float d4y = ey - 4.f * (po[own - kTmPX] + po[own + kTmPX]) + 6.f * q0;
        const float corners = (po[own - 2 * kTmPX - 2] + po[own - 2 * kTmPX + 2]) +
                              (po[own + 2 * kTmPX - 2] + po[own + 2 * kTmPX + 2]);
        const float d4z = (P0 + P4) - 4.f * (P1 + P3) + 6.f * q0;
        q = c.ridge2 * q0 + c.xx_int * d4x + c.yy_int * d4y + c.zz_int * d4z +
            c.xy * (corners - 2.f * (ex + ey) + 4.f * q0) + c.xz * ((X0 + X4) - 2.f * X2) +
            c.yz * ((Y0 + Y4) - 2.f * Y2);
      } else {
        const float *pm2 = slot_of(z - 2), *pm1 = slot_of(z - 1), *pp1 = slot_of(z + 1);
        auto pr = [&](int dz, int dy, int dx) -> float {
          const float *pl = dz == -2 ? pm2 : dz == -1 ? pm1 : dz == 0 ? po : dz == 1 ? pp1 : pl2;
          return pl[own + dy * kTmPX + dx];
        };
        q = shell_node<float>(c, pr, i, j, z);
      }
      q += qd0;
      const int g = z * sxy + gcol;
      const float *ops = pl2 + kTmPlane + ty * kTmX + tx;
      if (EPI == EPI_STORE) {
        e.q[g] = q;
        local += P2 * q;
      } else if (EPI == EPI_CHEB) {
        const float xv = ops[0], rv = ops[kTmOp], dinv = ops[2 * kTmOp];
        e.x[g] = xv + P2;
        const float rn = rv - q;
        e.r[g] = rn;
        e.d_out[g] = e.c1 * P2 + e.c2 * dinv * rn;
      } else {
        const float bv = ops[0], dinv = ops[kTmOp];
        const float rn = bv - q;
        e.r[g] = rn;
        e.d_out[g] = e.c2 * dinv * rn;
      }
    }
    P0 = P1; P1 = P2; P2 = P3; P3 = P4;
    X0 = X1; X1 = X2; X2 = X3; X3 = X4;
    Y0 = Y1; Y1 = Y2; Y2 = Y3; Y3 = Y4;
    qd0 = qd1;
    mw1 = mw2;
    wr1 = wr2;
    ok = __syncthreads_and(ok);  // plane z - 2 is free in every thread
    if (!ok) zfail = z;
    if (ok && tid == 0 && z + kTmSlots - 2 <= tlast) issue(z + kTmSlots - 2);
  }
  if (!ok) {
    // a copy never arrived: record it, give every copy this block issued a
    // bounded wait, and leave through the reduction so that tickets stay
    // consistent
    if (tid == 0) {
      atomicExch(fault, 1);
      const int issued_last = min(tlast, zfail + kTmSlots - 3);
      for (int t = max(tfirst, zfail - 2); t <= issued_last; ++t) (void)tm_wait(bar_of(t), parity_of(t));
    }
    local = 0.f;
  }
  if (dot_out) {
    double tot;
    const unsigned int bid = blockIdx.x + gridDim.x * blockIdx.y;
    if (grid_sum_ex<kTmThreads, float>(local, partials, ticket, &tot, tid, bid, gridDim.x * gridDim.y)) {
      *dot_out = tot;
      // the whole grid's share is in dot_out: a second partial that split
      // kernels would fill (the boundary shell's) must not keep a stale value
      if (dot_clear) *dot_clear = 0.0;
    }
  }
}

// Host side ------------------------------------------------------------------
// Encoded tensor maps of one grid, keyed by buffer and box kind (0: the halo'd
// plane box of an applied vector, 1: the tile box of an epilogue operand).
// Encoding is host-only work (no stream operation), so it may happen while a
// stream is being captured.
struct TmCache {
  struct Entry {
    const float *ptr;
    int kind;
    CUtensorMap map;
  };
  std::vector<Entry> entries;
  int nx = 0, ny = 0, nz = 0;
  bool enabled = false;  // the grid qualifies and the encoder is available
};

// Sets up the cache for an nx x ny x nz FP32 grid: TMA staging needs rows of a
// multiple of 16 bytes (nx % 4 == 0) and the driver's tensor-map encoder; the
// kernel attributes are set here (outside any capture).  `allow` = false
// keeps the staged-tile kernels of fd_apply.cuh.
void tm_setup(TmCache &cache, int nx, int ny, int nz, bool allow);

// q = N p with the epilogue through fd_tma_apply_kernel (plus the data-node
// totals kernel when the grid has touched nodes; `qd` receives them).  With
// `dot`, sum p.q lands there and `dot_clear` (may be NULL) is zeroed.
// `parts` selects what is launched: TM_TOTALS | TM_APPLY (both by default;
// the profiler times them one at a time).  Returns the number of kernels
// launched, 0 when the cache is not enabled or a map could not be encoded
// (the caller then uses launch_operator), or a negative status.
enum { TM_TOTALS = 1, TM_APPLY = 2 };
template <int EPI>
int tm_launch(TmCache &cache, const CoefT<float> &c, const float *p, DataView<float> dv, const EpiArgs<float> &e,
              const int *done, int64_t ntouched, const int64_t *inc_ptr, const int32_t *inc_row, const float *inc_a,
              int width, const int32_t *cols, const float *a, const float *w2, float *qd, double *partials,
              unsigned int *ticket, double *dot, double *dot_clear, int *fault, int max_blocks, cudaStream_t st,
              int parts = TM_TOTALS | TM_APPLY);

}  // namespace ls
