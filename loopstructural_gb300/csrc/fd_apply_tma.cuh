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
// shell_node() on the staged neighbourhood, specialised per warp to the axes
// along which the warp's nodes are near a face.
//
// The data term does not enter this kernel: the kernel leaves p unchanged, so
// the term A_d^T W A_d p of the few touched nodes is added afterwards, with its
// share of the epilogue, by rows_kernel + data_fixup_kernel (q += qd, or
// r -= qd and d -= c2 D^-1 qd).
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

// The data term of the finest level, after fd_tma_apply_kernel: for touched
// node t (rank order, node touched[t]) qd = sum_e a_e s[row(e)] over its
// incidences, s = w^2 (a_row . p) from rows_kernel, and the epilogue the main
// kernel ran without it corrected: STORE q += qd (p . qd added to *dot);
// CHEB / RESID r -= qd, d -= c2 D^-1 qd (both epilogues are linear in q).
template <int EPI>
__global__ void __launch_bounds__(256) data_fixup_kernel(int64_t ntouched, const int64_t *__restrict__ touched,
                                                         const int64_t *__restrict__ inc_ptr,
                                                         const int32_t *__restrict__ inc_row,
                                                         const float *__restrict__ inc_a, const float *__restrict__ s,
                                                         const float *__restrict__ p, EpiArgs<float> e,
                                                         const int *done, double *partials, unsigned int *ticket,
                                                         double *dot) {
  if (done && *done) return;
  float local = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntouched;
       t += (int64_t)gridDim.x * blockDim.x) {
    float qd = 0.f;
    const int64_t e1 = inc_ptr[t + 1];
    for (int64_t k = inc_ptr[t]; k < e1; ++k) qd += inc_a[k] * s[inc_row[k]];
    const int64_t g = touched[t];
    if (EPI == EPI_STORE) {
      e.q[g] += qd;
      local += p[g] * qd;
    } else {
      e.r[g] -= qd;
      e.d_out[g] -= e.c2 * e.dinv[g] * qd;
    }
  }
  if (dot) {
    double tot;
    if (grid_sum<256, float>(local, partials, ticket, &tot)) *dot += tot;
  }
}

// Data rows of the finest level as the TMA launcher needs them (FP32).
struct TmData {
  int64_t nrows = 0, ntouched = 0;
  int width = 0;
  const int32_t *cols = nullptr;
  const float *a = nullptr, *w2 = nullptr;  // nrows x width, nrows
  const int64_t *touched = nullptr, *inc_ptr = nullptr;
  const int32_t *inc_row = nullptr;
  const float *inc_a = nullptr;
  float *s = nullptr;  // nrows: w^2 (a_row . p) of the current p
};

// ZU: output planes per barrier step (1 or 2; the launcher picks the faster
// for the grid at first use).
template <int EPI, int ZU = 1>
__global__ void __launch_bounds__(kTmThreads, kTmBlocksPerSm)
    fd_tma_apply_kernel(const __grid_constant__ TmMaps maps, CoefT<float> c, EpiArgs<float> e, const int *done,
                        int ntx, int zlen, double *partials, unsigned int *ticket, double *dot_out, double *dot_clear,
                        int *fault) {
  if (done && *done) return;
  constexpr int NOP = TmOps<EPI>::n;
  constexpr int SLOT = tm_slot_floats<EPI>();
  // staged planes: float offsets into the shared array itself (so every read
  // stays a shared-memory access), the base rounded up to 128 bytes
  extern __shared__ __align__(128) float tm_smem[];
  const int sbase = (int)(((128u - (smem_u32(tm_smem) & 127u)) & 127u) >> 2);
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

  auto slot_of = [&](int t) -> int { return sbase + ((t - tfirst) & (kTmSlots - 1)) * SLOT; };
  auto bar_of = [&](int t) -> uint64_t * { return &bars[(t - tfirst) & (kTmSlots - 1)]; };
  auto parity_of = [&](int t) -> uint32_t { return (uint32_t)(((t - tfirst) >> 3) & 1); };
  static_assert(kTmSlots == 8, "slot arithmetic assumes 8 slots");
  // one elected thread: plane t of p and, when t - 2 is an output plane, the
  // epilogue operands of plane t - 2, all on the slot's barrier
  auto issue = [&](int t) {
    float *s = tm_smem + slot_of(t);
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

  // which formula a warp uses is decided for the whole warp (no divergence):
  // the deep composite stencil, or the exact sum specialised to the axes along
  // which the warp is near a face (x: the warp holds a column within 3 of an
  // x face; y: its row is; z: the plane is).  A warp is one tile row.
  const bool ydeep = (j >= 3) & (j <= ny - 4);
  const bool xshell_warp = __any_sync(0xffffffffu, col_in & !((i >= 3) & (i <= nx - 4))) != 0;

  // register windows over planes z-2 .. z+2: p, C_x p, C_y p at the column
  float P0 = 0.f, P1 = 0.f, P2 = 0.f, P3 = 0.f, P4 = 0.f;
  float X0 = 0.f, X1 = 0.f, X2 = 0.f, X3 = 0.f, X4 = 0.f;
  float Y0 = 0.f, Y1 = 0.f, Y2 = 0.f, Y3 = 0.f, Y4 = 0.f;
  auto inplane = [&](int pl, float &P, float &X, float &Y) {
    const float *q = tm_smem + pl + own;
    const float p0 = q[0];
    P = p0;
    X = (q[-2] + q[2]) - 2.f * p0;
    Y = (q[-2 * kTmPX] + q[2 * kTmPX]) - 2.f * p0;
  };
  bool ok = true;
  {
    int pls[4];
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

  float local = 0.f;
  int z = z0;
  int zfail = z0 - 3;  // the step whose wait gave up (prologue: z0 - 3)
  int pm2 = slot_of(z0 - 2), pm1 = slot_of(z0 - 1), po = slot_of(z0), pp1 = slot_of(z0 + 1);
  for (; ok && z < z1; z += ZU) {
#pragma unroll
   for (int u = 0; u < ZU; ++u) {
    const int zz = z + u;
    if (ZU > 1 && zz >= z1) break;  // uniform across the block
    ok = tm_wait(bar_of(zz + 2), parity_of(zz + 2)) && ok;
    const int pl2 = slot_of(zz + 2);
    inplane(pl2, P4, X4, Y4);
    float q;
    const bool zdeep = (zz >= 3) & (zz <= nz - 4);
    auto pr = [&](int dz, int dy, int dx) -> float {
      const int pl = dz == -2 ? pm2 : dz == -1 ? pm1 : dz == 0 ? po : dz == 1 ? pp1 : pl2;
      return tm_smem[pl + own + dy * kTmPX + dx];
    };
    if (ydeep & zdeep) {
      if (!xshell_warp) {
        const float q0 = P2;
        const float *o = tm_smem + po + own;
        const float ex = o[-2] + o[2], ey = o[-2 * kTmPX] + o[2 * kTmPX];
        const float d4x = ex - 4.f * (o[-1] + o[1]) + 6.f * q0;
        const float d4y = ey - 4.f * (o[-kTmPX] + o[kTmPX]) + 6.f * q0;
        const float corners = (o[-2 * kTmPX - 2] + o[-2 * kTmPX + 2]) + (o[2 * kTmPX - 2] + o[2 * kTmPX + 2]);
        const float d4z = (P0 + P4) - 4.f * (P1 + P3) + 6.f * q0;
        q = c.ridge2 * q0 + c.xx_int * d4x + c.yy_int * d4y + c.zz_int * d4z +
            c.xy * (corners - 2.f * (ex + ey) + 4.f * q0) + c.xz * ((X0 + X4) - 2.f * X2) +
            c.yz * ((Y0 + Y4) - 2.f * Y2);
      } else {
        q = shell_node<float, decltype(pr), false, false, true>(c, pr, i, j, zz);
      }
    } else if (!xshell_warp & ydeep) {  // a plane near a z face
      q = shell_node<float, decltype(pr), false, true, false>(c, pr, i, j, zz);
    } else if (!xshell_warp) {  // a row near a y face
      q = shell_node<float, decltype(pr), true, true, false>(c, pr, i, j, zz);
    } else {
      q = shell_node<float>(c, pr, i, j, zz);
    }
    // epilogue of one node: q (data term added), its p, operands in the slot
    auto emit = [&](int g, int opi, float qn, float pn) {
      const float *ops = tm_smem + pl2 + kTmPlane + opi;
      if (EPI == EPI_STORE) {
        e.q[g] = qn;
        local += pn * qn;
      } else if (EPI == EPI_CHEB) {
        const float xv = ops[0], rv = ops[kTmOp], dinv = ops[2 * kTmOp];
        e.x[g] = xv + pn;
        const float rn = rv - qn;
        e.r[g] = rn;
        e.d_out[g] = e.c1 * pn + e.c2 * dinv * rn;
      } else {
        const float bv = ops[0], dinv = ops[kTmOp];
        const float rn = bv - qn;
        e.r[g] = rn;
        e.d_out[g] = e.c2 * dinv * rn;
      }
    };
    if (col_in) emit(zz * sxy + gcol, ty * kTmX + tx, q, P2);
    P0 = P1; P1 = P2; P2 = P3; P3 = P4;
    X0 = X1; X1 = X2; X2 = X3; X3 = X4;
    Y0 = Y1; Y1 = Y2; Y2 = Y3; Y3 = Y4;
    pm2 = pm1; pm1 = po; po = pp1; pp1 = pl2;
   }
    ok = __syncthreads_and(ok);  // planes z - 2 .. z + ZU - 3 are free in every thread
    if (!ok) zfail = z;
    if (ok && tid == 0) {
#pragma unroll
      for (int u = 0; u < ZU; ++u)
        if (z + u < z1 && z + u + kTmSlots - 2 <= tlast) issue(z + u + kTmSlots - 2);
    }
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
  int segments = 0;      // z segments per column tile (0: ~16 planes each)
  int zu = 0;            // output planes per barrier step (0: not chosen yet)
};

// Sets up the cache for an nx x ny x nz FP32 grid: TMA staging needs rows of a
// multiple of 16 bytes (nx % 4 == 0) and the driver's tensor-map encoder; the
// kernel attributes are set here (outside any capture).  `allow` = false
// keeps the staged-tile kernels of fd_apply.cuh.
void tm_setup(TmCache &cache, int nx, int ny, int nz, bool allow);

// Picks the planes-per-step variant of the kernel for this grid by timing
// both on the handle's own vectors (p -> q, STORE epilogue, no data term);
// LS_GB300_TMA_STEP=1|2 forces one.  Outside any stream capture.
int tm_autotune(TmCache &cache, const CoefT<float> &c, const float *p, float *q, int *fault, cudaStream_t st);

// q = N p with the epilogue: fd_tma_apply_kernel, then, when the grid has
// touched nodes, rows_kernel + data_fixup_kernel for the data term.  With
// `dot`, sum p.q lands there and `dot_clear` (may be NULL) is zeroed.
// `parts` selects what is launched: TM_APPLY | TM_DATA (both by default; the
// profiler times them one at a time).  Returns the number of kernels
// launched, 0 when the cache is not enabled or a map could not be encoded
// (the caller then uses launch_operator), or a negative status.
enum { TM_DATA = 1, TM_APPLY = 2 };
template <int EPI>
int tm_launch(TmCache &cache, const CoefT<float> &c, const float *p, const TmData &d, const EpiArgs<float> &e,
              const int *done, double *partials, unsigned int *ticket, double *dot, double *dot_clear, int *fault,
              int max_blocks, cudaStream_t st, int parts = TM_DATA | TM_APPLY);

}  // namespace ls
