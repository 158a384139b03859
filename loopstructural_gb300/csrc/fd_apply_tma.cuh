// Finest-level FP32 normal-operator apply with TMA-staged planes.
//
//     q = (sum_f w_f^2 R_f^T R_f + A_d^T W A_d + ridge^2 I) p,  then an epilogue
//
// One kernel covers every node of the grid (deep interior and the 3-node
// boundary shell).  A block of 128 threads owns a 32 x 8 column tile (two
// x-adjacent columns per thread) and marches along z through a segment of
// planes.  The planes of p it needs (the tile plus a
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

constexpr int kTmX = 32, kTmY = 8;
constexpr int kTmThreads = kTmX * kTmY / 2;  // 16 x 8 threads, two x-adjacent nodes each
constexpr int kTmPX = kTmX + 8;             // staged plane: x0 - 4 .. x0 + 35
constexpr int kTmPY = kTmY + 4;             // y0 - 2 .. y0 + 9
constexpr int kTmPlane = kTmPX * kTmPY;     // 480 floats (1920 B)
constexpr int kTmOp = kTmX * kTmY;          // 256 floats (1 KB)
constexpr int kTmSlots = 8;
constexpr int kTmBlocksPerSm = 5;
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

// The exact sum at a node deep in y and z (index in [3, n-4]) but near an x
// face: shell_node() with iy = iz = 1 and by = bz = 0 written out, from the
// values the deep formula stages plus p at x -/+ 2 on planes z -/+ 2.  fi[0..2]
// = I(i-1), I(i), I(i+1) and fb[0..2] = B(i-1), B(i), B(i+1) are the node's
// x row-existence factors (interior row centre; border-layer rows).  Row and
// plane values: r* row y (x-2 .. x+2), u* / d* rows y-2 / y+2 at x-2, x, x+2,
// u1 / d1 rows y-1 / y+1 at x, m* / p* planes z-2 / z+2 at x-2, x, x+2, z1m /
// z1p planes z-1 / z+1 at x, ycross = (C_y p)(z-2) + (C_y p)(z+2) -
// 2 (C_y p)(z).  Cross terms use the one-sided differences
// R(v) = v(x+2) - v(x), L(v) = v(x) - v(x-2):
//   a_xy = I(i+1) (R(y+2) - 2 R(y) + R(y-2)) - I(i-1) (L(y+2) - 2 L(y) + L(y-2))
// (and a_xz alike over planes), which at I = 1 is the deep corner sum.
__device__ __forceinline__ float xshell_node(const CoefT<float> &c, const float fi[3], const float fb[3], float rm2,
                                             float rm1, float r0, float rp1, float rp2, float um, float u0, float up,
                                             float dm, float d0, float dp, float u1, float d1, float mm, float m0,
                                             float mp, float pm, float p0, float pp, float z1m, float z1p,
                                             float ycross) {
  const float sxm = rm2 - 2.f * rm1 + r0, sx0 = rm1 - 2.f * r0 + rp1, sxp = r0 - 2.f * rp1 + rp2;
  const float xpart = (c.xx_int * fi[0] + c.xx_bdr * fb[0]) * sxm - 2.f * (c.xx_int * fi[1] + c.xx_bdr * fb[1]) * sx0 +
                      (c.xx_int * fi[2] + c.xx_bdr * fb[2]) * sxp;
  const float R0 = rp2 - r0, L0 = r0 - rm2;
  const float axy = fi[2] * ((dp - d0) - 2.f * R0 + (up - u0)) - fi[0] * ((d0 - dm) - 2.f * L0 + (u0 - um));
  const float axz = fi[2] * ((pp - p0) - 2.f * R0 + (mp - m0)) - fi[0] * ((p0 - pm) - 2.f * L0 + (m0 - mm));
  const float d4y = (u0 + d0) - 4.f * (u1 + d1) + 6.f * r0;
  const float d4z = (m0 + p0) - 4.f * (z1m + z1p) + 6.f * r0;
  return c.ridge2 * r0 + xpart + c.xy * axy + c.xz * axz + fi[1] * (c.yy_int * d4y + c.zz_int * d4z + c.yz * ycross);
}

// The exact sum at a node deep in x and z but near a y face: shell_node()
// with ix = iz = 1, bx = bz = 0 written out.  fi / fb = I, B of rows j-1, j,
// j+1.  Values: r* row y (x-2 .. x+2) of plane z; u* / d* rows y-2 / y+2 at
// x-2, x, x+2; u1 / d1 rows y-1 / y+1 at x; p0..p4 planes z-2 .. z+2 at the
// node; zmu / zmd (zpu / zpd) plane z-2 (z+2) at rows y-2 / y+2; xcross =
// (C_x p)(z-2) + (C_x p)(z+2) - 2 (C_x p)(z).  With the z second difference
// G(r) of row y+r and the x second difference C(r) of row y+r:
//   a_yz = I(j+1) (G(2) - G(0)) - I(j-1) (G(0) - G(-2)),
//   a_xy = I(j+1) (C(2) - C(0)) - I(j-1) (C(0) - C(-2)).
__device__ __forceinline__ float yshell_node(const CoefT<float> &c, const float fi[3], const float fb[3], float rm2,
                                             float rm1, float r0, float rp1, float rp2, float um, float u0, float up,
                                             float dm, float d0, float dp, float u1, float d1, float p0, float p1,
                                             float p3, float p4, float zmu, float zmd, float zpu, float zpd,
                                             float xcross) {
  const float sym = u0 - 2.f * u1 + r0, sy0 = u1 - 2.f * r0 + d1, syp = r0 - 2.f * d1 + d0;
  const float ypart = (c.yy_int * fi[0] + c.yy_bdr * fb[0]) * sym - 2.f * (c.yy_int * fi[1] + c.yy_bdr * fb[1]) * sy0 +
                      (c.yy_int * fi[2] + c.yy_bdr * fb[2]) * syp;
  const float Cm = (um + up) - 2.f * u0, C0 = (rm2 + rp2) - 2.f * r0, Cp = (dm + dp) - 2.f * d0;
  const float axy = fi[2] * (Cp - C0) - fi[0] * (C0 - Cm);
  const float Gm = (zpu + zmu) - 2.f * u0, G0 = (p4 + p0) - 2.f * r0, Gp = (zpd + zmd) - 2.f * d0;
  const float ayz = fi[2] * (Gp - G0) - fi[0] * (G0 - Gm);
  const float d4x = (rm2 + rp2) - 4.f * (rm1 + rp1) + 6.f * r0;
  const float d4z = (p0 + p4) - 4.f * (p1 + p3) + 6.f * r0;
  return c.ridge2 * r0 + fi[1] * (c.xx_int * d4x + c.zz_int * d4z + c.xz * xcross) + ypart + c.xy * axy +
         c.yz * ayz;
}

// The exact sum at any node from the three axis planes through it: shell_node()
// with all factors general, written out over the values the pair loads give
// (for warps near two or three faces).  f* = {I(n-1), I(n), I(n+1), B(n-1),
// B(n), B(n+1)} of the node's x, y, z indices.  Values: r* the x line (x-2 ..
// x+2), u2 u1 d1 d2 the y line, p0 p1 p3 p4 the z line; corners of the xy
// plane um up dm dp (y-2 / y+2 at x-2 / x+2), of the xz plane mm mp pm pp
// (z-2 / z+2 at x-2 / x+2), of the yz plane zmu zmd zpu zpd (z-2 / z+2 at
// y-2 / y+2).  Each cross family sums its four row centres (a, b) = (+-1,
// +-1), e_ab = the difference of one-sided differences in the quadrant.
__device__ __forceinline__ float general_node(const CoefT<float> &c, const float fx[6], const float fy[6],
                                              const float fz[6], float rm2, float rm1, float r0, float rp1, float rp2,
                                              float u2, float u1, float d1, float d2, float p0, float p1, float p3,
                                              float p4, float um, float up, float dm, float dp, float mm, float mp,
                                              float pm, float pp, float zmu, float zmd, float zpu, float zpd) {
  auto axis = [&](float i_int, const float f[6], float wint, float wbdr, float a, float b, float cc, float d,
                  float e) {  // a..e: the line at -2 .. +2
    return (wint * f[0] * i_int + wbdr * f[3]) * ((a - 2.f * b) + cc) -
           2.f * (wint * f[1] * i_int + wbdr * f[4]) * ((b - 2.f * cc) + d) +
           (wint * f[2] * i_int + wbdr * f[5]) * ((cc - 2.f * d) + e);
  };
  float q = c.ridge2 * r0;
  q += axis(fy[1] * fz[1], fx, c.xx_int, c.xx_bdr, rm2, rm1, r0, rp1, rp2);
  q += axis(fx[1] * fz[1], fy, c.yy_int, c.yy_bdr, u2, u1, r0, d1, d2);
  q += axis(fx[1] * fy[1], fz, c.zz_int, c.zz_bdr, p0, p1, r0, p3, p4);
  // quadrant sums: (+,+), (-,+), (+,-), (-,-) of (first axis, second axis)
  auto cross = [&](const float fa[6], const float fb[6], float lm, float lp, float bm, float bp, float cmm,
                   float cmp, float cpm, float cpp) {
    // lm / lp: the first axis at -2 / +2 on the second axis' 0 line; bm / bp:
    // the second axis at -2 / +2 on the first axis' 0 line; c__: corners
    const float epp = (cpp - bp) - (lp - r0), emp = (bp - cpm) - (r0 - lm);
    const float epm = (lp - r0) - (cmp - bm), emm = (r0 - lm) - (bm - cmm);
    return fa[2] * fb[2] * epp - fa[0] * fb[2] * emp - fa[2] * fb[0] * epm + fa[0] * fb[0] * emm;
  };
  q += c.xy * fz[1] * cross(fx, fy, rm2, rp2, u2, d2, um, up, dm, dp);
  q += c.xz * fy[1] * cross(fx, fz, rm2, rp2, p0, p4, mm, mp, pm, pp);
  q += c.yz * fx[1] * cross(fy, fz, u2, d2, p0, p4, zmu, zmd, zpu, zpd);
  return q;
}

// ZU: output planes per barrier step (1 or 2; the launcher picks the faster
// for the grid at first use).
//
// Thread (tx, ty) of the 16 x 8 block owns the node pair (x0 + 2 tx, y0 + ty)
// and its right neighbour: every staged row is read as aligned float pairs
// (ld.shared.v2), so one load serves both nodes, and the epilogue moves pairs
// (nx is a multiple of 4, so a pair never straddles a row end).  A warp holds
// two tile rows.
template <int EPI, int ZU = 1>
__global__ void __launch_bounds__(kTmThreads, kTmBlocksPerSm)
    fd_tma_apply_kernel(const __grid_constant__ TmMaps maps, CoefT<float> c, EpiArgs<float> e, const int *done,
                        int ntx, int zlen, double *partials, unsigned int *ticket, double *dot_out, double *dot_clear,
                        int *fault) {
  if (done && *done) return;
  constexpr int NOP = TmOps<EPI>::n;
  constexpr int SLOT = tm_slot_floats<EPI>();
  // staged planes: float offsets into the shared array, the base rounded up
  // to 128 bytes; pairs are read through the array's shared-window address
  extern __shared__ __align__(128) float tm_smem[];
  const uint32_t sm0 = smem_u32(tm_smem);
  const int sbase = (int)(((128u - (sm0 & 127u)) & 127u) >> 2);
  __shared__ __align__(8) uint64_t bars[kTmSlots];
  const int tid = threadIdx.x, tx = tid & (kTmX / 2 - 1), ty = tid / (kTmX / 2);
  const int x0 = (int)(blockIdx.x % ntx) * kTmX, y0 = (int)(blockIdx.x / ntx) * kTmY;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int z0 = blockIdx.y * zlen, z1 = min(nz, z0 + zlen);
  const int i = x0 + 2 * tx, j = y0 + ty;     // the pair: (i, j) and (i + 1, j)
  const bool col_in = (i < nx) & (j < ny);  // nx even: i < nx implies i + 1 < nx
  const int sxy = nx * ny;
  const int gcol = j * nx + i;
  const int tfirst = z0 - 2, tlast = z1 + 1;  // staged planes of p
  const int hx = 2 * tx + 4, hy = ty + 2;     // the pair's position in a staged plane (hx even)
  const int own = hy * kTmPX + hx;

  auto slot_of = [&](int t) -> int { return sbase + ((t - tfirst) & (kTmSlots - 1)) * SLOT; };
  auto bar_of = [&](int t) -> uint64_t * { return &bars[(t - tfirst) & (kTmSlots - 1)]; };
  auto parity_of = [&](int t) -> uint32_t { return (uint32_t)(((t - tfirst) >> 3) & 1); };
  static_assert(kTmSlots == 8, "slot arithmetic assumes 8 slots");
  // a float pair at an even float offset of the shared array
  auto ld2 = [&](int off) -> float2 {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];\n" : "=f"(v.x), "=f"(v.y) : "r"(sm0 + 4u * (uint32_t)off));
    return v;
  };
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
  // which the warp is near a face (x: it holds a column within 3 of an x face;
  // y: one of its two rows is; z: the plane is)
  const bool xshell_warp = __any_sync(0xffffffffu, col_in & !((i >= 3) & (i + 1 <= nx - 4))) != 0;
  const bool ydeep_warp = __all_sync(0xffffffffu, !col_in | ((j >= 3) & (j <= ny - 4))) != 0;


  // register windows over planes z-2 .. z+2 for both nodes: p, C_x p, C_y p
  float2 P0 = {0.f, 0.f}, P1 = P0, P2 = P0, P3 = P0, P4 = P0;
  float2 X0 = P0, X1 = P0, X2 = P0, X3 = P0, X4 = P0;
  float2 Y0 = P0, Y1 = P0, Y2 = P0, Y3 = P0, Y4 = P0;
  auto inplane = [&](int pl, float2 &P, float2 &X, float2 &Y) {
    const int q = pl + own;
    const float2 cc = ld2(q), l = ld2(q - 2), r = ld2(q + 2);
    const float2 u = ld2(q - 2 * kTmPX), d = ld2(q + 2 * kTmPX);
    P = cc;
    X = make_float2((l.x + r.x) - 2.f * cc.x, (l.y + r.y) - 2.f * cc.y);
    Y = make_float2((u.x + d.x) - 2.f * cc.x, (u.y + d.y) - 2.f * cc.y);
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
    float qa, qb;
    const bool zdeep = (zz >= 3) & (zz <= nz - 4);
    auto pr = [&](int dz, int dy, int dx) -> float {
      const int pl = dz == -2 ? pm2 : dz == -1 ? pm1 : dz == 0 ? po : dz == 1 ? pp1 : pl2;
      return tm_smem[pl + own + dy * kTmPX + dx];
    };
    auto prb = [&](int dz, int dy, int dx) -> float { return pr(dz, dy, dx + 1); };
    // the general sum for warps near two faces (edges, corners); every other
    // case from the pair loads below
    const bool general = (xshell_warp & !(ydeep_warp & zdeep)) | (!ydeep_warp & !zdeep);
    if (!general) {
      const int o = po + own;
      // row y: columns hx-2 .. hx+3; rows y-/+1, y-/+2 at the pair; the
      // corner columns of rows y-/+2
      const float2 L = ld2(o - 2), R = ld2(o + 2);
      const float2 U1 = ld2(o - kTmPX), D1 = ld2(o + kTmPX), U2 = ld2(o - 2 * kTmPX), D2 = ld2(o + 2 * kTmPX);
      const float2 UL = ld2(o - 2 * kTmPX - 2), UR = ld2(o - 2 * kTmPX + 2);
      const float2 DL = ld2(o + 2 * kTmPX - 2), DR = ld2(o + 2 * kTmPX + 2);
      if (!(ydeep_warp & zdeep)) {
        if (ydeep_warp) {  // a plane near a z face: per-plane z factors, no further loads
          auto fI = [&](int a) -> float { return (a >= 1 && a <= nz - 2) ? 1.f : 0.f; };
          auto fB = [&](int a) -> float {
            return (float)((a == 1) + (a == nz - 2)) * ((a >= 0 && a < nz) ? 1.f : 0.f);
          };
          const float iz0 = fI(zz - 1), iz1 = fI(zz), iz2 = fI(zz + 1);
          const float w0 = c.zz_int * iz0 + c.zz_bdr * fB(zz - 1), w1 = c.zz_int * iz1 + c.zz_bdr * fB(zz),
                      w2 = c.zz_int * iz2 + c.zz_bdr * fB(zz + 1);
          {
            const float q0 = P2.x;
            const float ex = L.x + R.x, ey = U2.x + D2.x;
            const float d4x = ex - 4.f * (L.y + P2.y) + 6.f * q0;
            const float d4y = ey - 4.f * (U1.x + D1.x) + 6.f * q0;
            const float corners = (UL.x + UR.x) + (DL.x + DR.x);
            const float zpart = w0 * ((P0.x - 2.f * P1.x) + P2.x) - 2.f * w1 * ((P1.x - 2.f * P2.x) + P3.x) +
                                w2 * ((P2.x - 2.f * P3.x) + P4.x);
            qa = c.ridge2 * q0 + iz1 * (c.xx_int * d4x + c.yy_int * d4y + c.xy * (corners - 2.f * (ex + ey) + 4.f * q0)) +
                 zpart + c.xz * (iz2 * (X4.x - X2.x) - iz0 * (X2.x - X0.x)) +
                 c.yz * (iz2 * (Y4.x - Y2.x) - iz0 * (Y2.x - Y0.x));
          }
          {
            const float q0 = P2.y;
            const float ex = L.y + R.y, ey = U2.y + D2.y;
            const float d4x = ex - 4.f * (P2.x + R.x) + 6.f * q0;
            const float d4y = ey - 4.f * (U1.y + D1.y) + 6.f * q0;
            const float corners = (UL.y + UR.y) + (DL.y + DR.y);
            const float zpart = w0 * ((P0.y - 2.f * P1.y) + P2.y) - 2.f * w1 * ((P1.y - 2.f * P2.y) + P3.y) +
                                w2 * ((P2.y - 2.f * P3.y) + P4.y);
            qb = c.ridge2 * q0 + iz1 * (c.xx_int * d4x + c.yy_int * d4y + c.xy * (corners - 2.f * (ex + ey) + 4.f * q0)) +
                 zpart + c.xz * (iz2 * (X4.y - X2.y) - iz0 * (X2.y - X0.y)) +
                 c.yz * (iz2 * (Y4.y - Y2.y) - iz0 * (Y2.y - Y0.y));
          }
        } else {  // rows near a y face (deep in z): per-row y factors, p at rows y-/+2 of planes z-/+2
          const float2 MU = ld2(pm2 + own - 2 * kTmPX), MD = ld2(pm2 + own + 2 * kTmPX);
          const float2 QU = ld2(pl2 + own - 2 * kTmPX), QD = ld2(pl2 + own + 2 * kTmPX);
          auto fI = [&](int a) -> float { return (a >= 1 && a <= ny - 2) ? 1.f : 0.f; };
          auto fB = [&](int a) -> float {
            return (float)((a == 1) + (a == ny - 2)) * ((a >= 0 && a < ny) ? 1.f : 0.f);
          };
          const float fi[3] = {fI(j - 1), fI(j), fI(j + 1)}, fb[3] = {fB(j - 1), fB(j), fB(j + 1)};
          qa = yshell_node(c, fi, fb, L.x, L.y, P2.x, P2.y, R.x, UL.x, U2.x, UR.x, DL.x, D2.x, DR.x, U1.x, D1.x, P0.x,
                           P1.x, P3.x, P4.x, MU.x, MD.x, QU.x, QD.x, (X0.x + X4.x) - 2.f * X2.x);
          qb = yshell_node(c, fi, fb, L.y, P2.x, P2.y, R.x, R.y, UL.y, U2.y, UR.y, DL.y, D2.y, DR.y, U1.y, D1.y, P0.y,
                           P1.y, P3.y, P4.y, MU.y, MD.y, QU.y, QD.y, (X0.y + X4.y) - 2.f * X2.y);
        }
      } else if (xshell_warp) {  // columns near an x face: per-node x factors
        const float2 ML = ld2(pm2 + own - 2), MR = ld2(pm2 + own + 2);
        const float2 QL = ld2(pl2 + own - 2), QR = ld2(pl2 + own + 2);
        auto fI = [&](int a) -> float { return (a >= 1 && a <= nx - 2) ? 1.f : 0.f; };
        auto fB = [&](int a) -> float { return (float)((a == 1) + (a == nx - 2)) * ((a >= 0 && a < nx) ? 1.f : 0.f); };
        const float fia[3] = {fI(i - 1), fI(i), fI(i + 1)}, fba[3] = {fB(i - 1), fB(i), fB(i + 1)};
        const float fib[3] = {fI(i), fI(i + 1), fI(i + 2)}, fbb[3] = {fB(i), fB(i + 1), fB(i + 2)};
        qa = xshell_node(c, fia, fba, L.x, L.y, P2.x, P2.y, R.x, UL.x, U2.x, UR.x, DL.x, D2.x, DR.x, U1.x, D1.x, ML.x,
                         P0.x, MR.x, QL.x, P4.x, QR.x, P1.x, P3.x, (Y0.x + Y4.x) - 2.f * Y2.x);
        qb = xshell_node(c, fib, fbb, L.y, P2.x, P2.y, R.x, R.y, UL.y, U2.y, UR.y, DL.y, D2.y, DR.y, U1.y, D1.y, ML.y,
                         P0.y, MR.y, QL.y, P4.y, QR.y, P1.y, P3.y, (Y0.y + Y4.y) - 2.f * Y2.y);
      } else {
      {
        const float q0 = P2.x;
        const float ex = L.x + R.x, ey = U2.x + D2.x;
        const float d4x = ex - 4.f * (L.y + P2.y) + 6.f * q0;
        const float d4y = ey - 4.f * (U1.x + D1.x) + 6.f * q0;
        const float corners = (UL.x + UR.x) + (DL.x + DR.x);
        const float d4z = (P0.x + P4.x) - 4.f * (P1.x + P3.x) + 6.f * q0;
        qa = c.ridge2 * q0 + c.xx_int * d4x + c.yy_int * d4y + c.zz_int * d4z +
             c.xy * (corners - 2.f * (ex + ey) + 4.f * q0) + c.xz * ((X0.x + X4.x) - 2.f * X2.x) +
             c.yz * ((Y0.x + Y4.x) - 2.f * Y2.x);
      }
      {
        const float q0 = P2.y;
        const float ex = L.y + R.y, ey = U2.y + D2.y;
        const float d4x = ex - 4.f * (P2.x + R.x) + 6.f * q0;
        const float d4y = ey - 4.f * (U1.y + D1.y) + 6.f * q0;
        const float corners = (UL.y + UR.y) + (DL.y + DR.y);
        const float d4z = (P0.y + P4.y) - 4.f * (P1.y + P3.y) + 6.f * q0;
        qb = c.ridge2 * q0 + c.xx_int * d4x + c.yy_int * d4y + c.zz_int * d4z +
             c.xy * (corners - 2.f * (ex + ey) + 4.f * q0) + c.xz * ((X0.y + X4.y) - 2.f * X2.y) +
             c.yz * ((Y0.y + Y4.y) - 2.f * Y2.y);
      }
      }
    } else {  // near two or three faces: the general sum from the three axis planes
      const int o = po + own;
      const float2 L = ld2(o - 2), R = ld2(o + 2);
      const float2 U1 = ld2(o - kTmPX), D1 = ld2(o + kTmPX), U2 = ld2(o - 2 * kTmPX), D2 = ld2(o + 2 * kTmPX);
      const float2 UL = ld2(o - 2 * kTmPX - 2), UR = ld2(o - 2 * kTmPX + 2);
      const float2 DL = ld2(o + 2 * kTmPX - 2), DR = ld2(o + 2 * kTmPX + 2);
      const float2 ML = ld2(pm2 + own - 2), MR = ld2(pm2 + own + 2), QL = ld2(pl2 + own - 2), QR = ld2(pl2 + own + 2);
      const float2 MU = ld2(pm2 + own - 2 * kTmPX), MD = ld2(pm2 + own + 2 * kTmPX);
      const float2 QU = ld2(pl2 + own - 2 * kTmPX), QD = ld2(pl2 + own + 2 * kTmPX);
      auto fac = [](int a, int n, float f[6]) {
        for (int d = 0; d < 3; ++d) {
          const int v = a + d - 1;
          f[d] = (v >= 1 && v <= n - 2) ? 1.f : 0.f;
          f[3 + d] = (float)((v == 1) + (v == n - 2)) * ((v >= 0 && v < n) ? 1.f : 0.f);
        }
      };
      float fxa[6], fxb[6], fy[6], fz[6];
      fac(i, nx, fxa);
      fac(i + 1, nx, fxb);
      fac(j, ny, fy);
      fac(zz, nz, fz);
      qa = general_node(c, fxa, fy, fz, L.x, L.y, P2.x, P2.y, R.x, U2.x, U1.x, D1.x, D2.x, P0.x, P1.x, P3.x, P4.x,
                        UL.x, UR.x, DL.x, DR.x, ML.x, MR.x, QL.x, QR.x, MU.x, MD.x, QU.x, QD.x);
      qb = general_node(c, fxb, fy, fz, L.y, P2.x, P2.y, R.x, R.y, U2.y, U1.y, D1.y, D2.y, P0.y, P1.y, P3.y, P4.y,
                        UL.y, UR.y, DL.y, DR.y, ML.y, MR.y, QL.y, QR.y, MU.y, MD.y, QU.y, QD.y);
    }
    // epilogue of the pair: q, its p, operands in the slot (pairs throughout)
    if (col_in) {
      const int g = zz * sxy + gcol;  // even
      const int opo = pl2 + kTmPlane + ty * kTmX + 2 * tx;
      if (EPI == EPI_STORE) {
        *reinterpret_cast<float2 *>(e.q + g) = make_float2(qa, qb);
        local += P2.x * qa + P2.y * qb;
      } else if (EPI == EPI_CHEB) {
        const float2 xv = ld2(opo), rv = ld2(opo + kTmOp), dv = ld2(opo + 2 * kTmOp);
        *reinterpret_cast<float2 *>(e.x + g) = make_float2(xv.x + P2.x, xv.y + P2.y);
        const float ra = rv.x - qa, rb = rv.y - qb;
        *reinterpret_cast<float2 *>(e.r + g) = make_float2(ra, rb);
        *reinterpret_cast<float2 *>(e.d_out + g) =
            make_float2(e.c1 * P2.x + e.c2 * dv.x * ra, e.c1 * P2.y + e.c2 * dv.y * rb);
      } else {
        const float2 bv = ld2(opo), dv = ld2(opo + kTmOp);
        const float ra = bv.x - qa, rb = bv.y - qb;
        *reinterpret_cast<float2 *>(e.r + g) = make_float2(ra, rb);
        *reinterpret_cast<float2 *>(e.d_out + g) = make_float2(e.c2 * dv.x * ra, e.c2 * dv.y * rb);
      }
    }
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
