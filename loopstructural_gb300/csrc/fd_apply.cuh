// Fused matrix-free application of the FD normal operator
//     q = (sum_f w_f^2 R_f^T R_f + A_d^T W A_d + ridge^2 I) p
// with a per-use epilogue, as one z-marching kernel.
//
// Tiling: a block of 32 x 8 threads owns a 32 x 8 column tile of (x, y) and
// marches over a chunk of z planes.  Plane s is staged in shared memory with a
// 2-node halo in x and y (double-buffered: one __syncthreads per plane).  From
// it every thread forms, for its own column, the in-plane quantities of the
// composite deep-interior stencil
//     S(s)  = a_x d4_x p + a_y d4_y p + b_xy C_x C_y p      (12 shared reads)
//     Cx(s) = C_x p,  Cy(s) = C_y p,  P(s) = p
// and keeps them in register windows over z, so that at plane z = s - 2
//     q = ridge^2 P + S(z) + a_z d4_z P + b_xz C_z Cx + b_yz C_z Cy
// needs no further memory traffic (d4 = (1,-4,6,-4,1), C = (1,0,-2,0,1) at
// stride 2; a = w^2/6, b = w^2/4).  Nodes within 3 of a face take the exact
// two-pass path (fd_stencil.cuh stencil_node_general) straight from L1/L2.
//
// Data rows: the touched nodes are marked in a bit mask (x-fastest words); a
// touched node adds sum_e a_e s_row(e) over its incidence list, where
// s_row = w^2 (a_row . p) was produced by the rows kernel launched just before.
#pragma once

#include "fd_stencil.cuh"
#include "ls_common.cuh"

namespace ls {

constexpr int kAX = 32, kAY = 8;  // x-y tile of one block
constexpr int kHX = kAX + 4, kHY = kAY + 4;  // staged plane with a 2-node halo

template <typename T>
struct DataView {
  const uint32_t *mask;      // bit per node, x fastest; word w covers nodes 32w .. 32w+31
  const int32_t *word_rank;  // touched nodes before word w
  const int64_t *inc_ptr;    // per touched node (rank order)
  const int32_t *inc_row;
  const T *inc_a;
  const T *s_rows;           // w^2 (a_row . p) of the current p
  int enabled;
};

// Epilogues -----------------------------------------------------------------
enum EpiKind { EPI_STORE = 0, EPI_CHEB = 1, EPI_RESID = 2 };

template <typename T>
struct EpiArgs {
  T *q;            // STORE: q out
  T *x;            // CHEB: x += p
  T *r;            // CHEB: r -= q ; RESID: r = b - q
  const T *b;      // RESID
  const T *dinv;   // CHEB / RESID
  T *d_out;        // CHEB: c1 p + c2 D^-1 r ; RESID: c2 D^-1 r
  T c1, c2;
};

template <typename T, int EPI>
__device__ __forceinline__ T epilogue(const EpiArgs<T> &e, int g, T p_own, T q) {
  if (EPI == EPI_STORE) {
    e.q[g] = q;
    return p_own * q;
  } else if (EPI == EPI_CHEB) {
    e.x[g] += p_own;
    const T rn = e.r[g] - q;
    e.r[g] = rn;
    e.d_out[g] = e.c1 * p_own + e.c2 * e.dinv[g] * rn;
    return (T)0;
  } else {
    const T rn = e.b[g] - q;
    e.r[g] = rn;
    e.d_out[g] = e.c2 * e.dinv[g] * rn;
    return (T)0;
  }
}

template <typename T>
__device__ __forceinline__ T data_term(const DataView<T> &dv, int g) {
  const uint32_t word = __ldg(dv.mask + (g >> 5));
  const uint32_t bit = 1u << (g & 31);
  if (!(word & bit)) return (T)0;
  const int rank = __ldg(dv.word_rank + (g >> 5)) + __popc(word & (bit - 1u));
  T acc = 0;
  const int64_t e1 = __ldg(dv.inc_ptr + rank + 1);
  for (int64_t e = __ldg(dv.inc_ptr + rank); e < e1; ++e) acc += __ldg(dv.inc_a + e) * __ldg(dv.s_rows + __ldg(dv.inc_row + e));
  return acc;
}

// Per-axis row-existence factors of a node coordinate a on an axis of n nodes:
// I(a) interior row centre (1 <= a <= n-2), B(a) number of border-layer rows
// centred there (a == 1, a == n-2), both 0 outside the grid.
template <typename T>
__device__ __forceinline__ T ind_i(int a, int n) { return (a >= 1 && a <= n - 2) ? (T)1 : (T)0; }
template <typename T>
__device__ __forceinline__ T ind_b(int a, int n) { return (T)((a == 1) + (a == n - 2)) * ((a >= 0 && a < n) ? (T)1 : (T)0); }

// Exact N_reg p at any node from the staged 5 x 5 x 5 neighbourhood (ring
// planes z-2 .. z+2, in-plane halo 2).  Branch-free: every row centre's weight
// is a product of per-axis factors, so the boundary shell costs the same as
// the interior and needs no global loads.
template <typename T, typename PR>
__device__ __forceinline__ T shell_node(const CoefT<T> &c, const PR &pr, int i, int j, int k) {
  T ix[3], bx[3], iy[3], by[3], iz[3], bz[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ix[d] = ind_i<T>(i + d - 1, c.nx);
    bx[d] = ind_b<T>(i + d - 1, c.nx);
    iy[d] = ind_i<T>(j + d - 1, c.ny);
    by[d] = ind_b<T>(j + d - 1, c.ny);
    iz[d] = ind_i<T>(k + d - 1, c.nz);
    bz[d] = ind_b<T>(k + d - 1, c.nz);
  }
  const T p0 = pr(0, 0, 0);
  T q = c.ridge2 * p0;
  // (1,-2,1) families: rows at delta in {-1,0,1} along the axis, kappa = (1,-2,1)
#pragma unroll
  for (int d = -1; d <= 1; ++d) {
    const T kap = d == 0 ? (T)-2 : (T)1;
    const T sx = pr(0, 0, d - 1) - (T)2 * pr(0, 0, d) + pr(0, 0, d + 1);
    const T sy = pr(0, d - 1, 0) - (T)2 * pr(0, d, 0) + pr(0, d + 1, 0);
    const T sz = pr(d - 1, 0, 0) - (T)2 * pr(d, 0, 0) + pr(d + 1, 0, 0);
    q += kap * (c.xx_int * ix[d + 1] * iy[1] * iz[1] + c.xx_bdr * bx[d + 1]) * sx;
    q += kap * (c.yy_int * ix[1] * iy[d + 1] * iz[1] + c.yy_bdr * by[d + 1]) * sy;
    q += kap * (c.zz_int * ix[1] * iy[1] * iz[d + 1] + c.zz_bdr * bz[d + 1]) * sz;
  }
  // diagonal families: rows at (da, db) in {-1,1}^2, weight da*db*I*I, row value
  // sum_{u,v} u v p(da+u, db+v)
  T axy = 0, axz = 0, ayz = 0;
#pragma unroll
  for (int da = -1; da <= 1; da += 2) {
#pragma unroll
    for (int db = -1; db <= 1; db += 2) {
      const T sgn = (T)(da * db);
      const T exy = (pr(0, db + 1, da + 1) - pr(0, db + 1, da - 1)) - (pr(0, db - 1, da + 1) - pr(0, db - 1, da - 1));
      const T exz = (pr(db + 1, 0, da + 1) - pr(db + 1, 0, da - 1)) - (pr(db - 1, 0, da + 1) - pr(db - 1, 0, da - 1));
      const T eyz = (pr(db + 1, da + 1, 0) - pr(db + 1, da - 1, 0)) - (pr(db - 1, da + 1, 0) - pr(db - 1, da - 1, 0));
      axy += sgn * ix[da + 1] * iy[db + 1] * exy;
      axz += sgn * ix[da + 1] * iz[db + 1] * exz;
      ayz += sgn * iy[da + 1] * iz[db + 1] * eyz;
    }
  }
  q += c.xy * iz[1] * axy + c.xz * iy[1] * axz + c.yz * ix[1] * ayz;
  return q;
}

constexpr int kRing = 8;  // staged planes: window s-4 .. s plus two in flight
constexpr int kPrefetch = 2;

template <typename T>
struct ApplySmem {
  T ring[kRing][kHY][kHX];
};

// Asynchronous global -> shared copy of one element (cp.async, Ampere+); a
// zero src size fills zeros (outside the grid).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src, bool valid) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
  const int n = valid ? (int)sizeof(T) : 0;
  if (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(saddr), "l"(src), "r"(n));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(saddr), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// issue the copy of plane s (2-node halo) into ring slot `slot`; planes outside
// the grid are zero-filled synchronously
template <typename T>
__device__ __forceinline__ void stage_plane(const CoefT<T> &c, const T *__restrict__ p, T (&dst)[kHY][kHX], int s,
                                            int x0, int y0, int tid) {
  const int nx = c.nx, ny = c.ny;
  if (s >= 0 && s < c.nz) {
    const T *ps = p + (size_t)s * nx * ny;
    for (int e2 = tid; e2 < kHX * kHY; e2 += kAX * kAY) {
      const int hy = e2 / kHX, hx = e2 - hy * kHX;
      const int gx = x0 - 2 + hx, gy = y0 - 2 + hy;
      const bool ok = (gx >= 0) & (gx < nx) & (gy >= 0) & (gy < ny);
      cp_async_elem<T>(&dst[hy][hx], ok ? ps + gx + nx * gy : p, ok);
    }
  } else {
    for (int e2 = tid; e2 < kHX * kHY; e2 += kAX * kAY) (&dst[0][0])[e2] = (T)0;
  }
  cp_async_commit();
}

// One plane step of the z-march, unrolled by the ring size so that every
// ring / window index is a compile-time constant.  On entry planes s and s+1
// are in flight; the step issues plane s + 2, waits for plane s, and outputs
// plane z = s - 2.
template <typename T, int EPI, int M>
__device__ __forceinline__ void apply_step(const CoefT<T> &c, const T *__restrict__ p, const DataView<T> &dv,
                                           const EpiArgs<T> &e, ApplySmem<T> &sm, int s, int x0, int y0, int z0,
                                           int z1, int tx, int ty, int tid, bool own, bool col_deep, int i, int j,
                                           T (&P)[kRing], T (&Cx)[kRing], T (&Cy)[kRing], T (&S)[kRing], T &local) {
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int sxy = nx * ny;
  constexpr int MP = (M + kPrefetch) % kRing;
  if (s + kPrefetch <= z1 + 1)
    stage_plane<T>(c, p, sm.ring[MP], s + kPrefetch, x0, y0, tid);
  else
    cp_async_commit();  // keep one group per step
  cp_async_wait<kPrefetch>();
  __syncthreads();
  {
    const int hx = tx + 2, hy = ty + 2;
    const T(&pl)[kHY][kHX] = sm.ring[M];
    const T p0 = pl[hy][hx];
    const T ex = pl[hy][hx - 2] + pl[hy][hx + 2], ey = pl[hy - 2][hx] + pl[hy + 2][hx];
    const T d4x = ex - (T)4 * (pl[hy][hx - 1] + pl[hy][hx + 1]) + (T)6 * p0;
    const T d4y = ey - (T)4 * (pl[hy - 1][hx] + pl[hy + 1][hx]) + (T)6 * p0;
    const T corners = (pl[hy - 2][hx - 2] + pl[hy - 2][hx + 2]) + (pl[hy + 2][hx - 2] + pl[hy + 2][hx + 2]);
    const T cxy = corners - (T)2 * (ex + ey) + (T)4 * p0;
    P[M] = p0;
    Cx[M] = ex - (T)2 * p0;
    Cy[M] = ey - (T)2 * p0;
    S[M] = c.xx_int * d4x + c.yy_int * d4y + c.xy * cxy;
  }
  const int z = s - 2;
  if (z >= z0 && z < nz && own) {
    constexpr int m0 = (M + kRing - 4) % kRing, m1 = (M + kRing - 3) % kRing, m2 = (M + kRing - 2) % kRing,
                  m3 = (M + kRing - 1) % kRing;
    // window: plane z-2 -> m0, z-1 -> m1, z -> m2, z+1 -> m3, z+2 -> M
    const int g = i + nx * j + sxy * z;
    T q;
    if (col_deep && z >= 3 && z <= nz - 4) {
      const T d4z = (P[m0] + P[M]) - (T)4 * (P[m1] + P[m3]) + (T)6 * P[m2];
      q = c.ridge2 * P[m2] + S[m2] + c.zz_int * d4z + c.xz * ((Cx[m0] + Cx[M]) - (T)2 * Cx[m2]) +
          c.yz * ((Cy[m0] + Cy[M]) - (T)2 * Cy[m2]);
    } else {
      const int hx = tx + 2, hy = ty + 2;
      auto pr = [&](int dz, int dy, int dx) -> T {
        const int slot = dz == -2 ? m0 : dz == -1 ? m1 : dz == 0 ? m2 : dz == 1 ? m3 : M;
        return sm.ring[slot][hy + dy][hx + dx];
      };
      q = shell_node<T>(c, pr, i, j, z);
    }
    if (dv.enabled) q += data_term<T>(dv, g);
    local += epilogue<T, EPI>(e, g, P[m2], q);
  }
}

// Returns the block's sum of the epilogue's per-node contributions (p.q for
// EPI_STORE) through the deterministic grid reduction when `dot_out` is set.
// `zc` is the z chunk of one block (gridDim.z = ceil(nz / zc)).
template <typename T, int EPI>
__global__ void __launch_bounds__(kAX * kAY) fd_apply_kernel(CoefT<T> c, const T *__restrict__ p, DataView<T> dv,
                                                             EpiArgs<T> e, int zc, const int *done,
                                                             double *partials, unsigned int *ticket,
                                                             double *dot_out) {
  if (done && *done) return;
  __shared__ ApplySmem<T> sm;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + kAX * ty;
  const int x0 = blockIdx.x * kAX, y0 = blockIdx.y * kAY, z0 = blockIdx.z * zc;
  const int z1 = min(z0 + zc, nz);
  const int i = x0 + tx, j = y0 + ty;
  const bool own = (i < nx) & (j < ny);
  const bool col_deep = (i >= 3) & (i <= nx - 4) & (j >= 3) & (j <= ny - 4);
  T P[kRing], Cx[kRing], Cy[kRing], S[kRing];
#pragma unroll
  for (int w = 0; w < kRing; ++w) P[w] = Cx[w] = Cy[w] = S[w] = (T)0;
  T local = 0;
  const int s0 = z0 - 2;
  // prologue: planes s0 and s0 + 1 in flight
  stage_plane<T>(c, p, sm.ring[0], s0, x0, y0, tid);
  stage_plane<T>(c, p, sm.ring[1], s0 + 1, x0, y0, tid);
  for (int s = s0; s <= z1 + 1; s += kRing) {
#define LS_STEP(MM)                                                                                                  \
  if (s + MM > z1 + 1) break;                                                                                        \
  apply_step<T, EPI, MM>(c, p, dv, e, sm, s + MM, x0, y0, z0, z1, tx, ty, tid, own, col_deep, i, j, P, Cx, Cy, S, \
                         local);
    LS_STEP(0) LS_STEP(1) LS_STEP(2) LS_STEP(3) LS_STEP(4) LS_STEP(5) LS_STEP(6) LS_STEP(7)
#undef LS_STEP
  }
  cp_async_wait<0>();
  if (dot_out) {
    double tot;
    const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (grid_sum_ex<kAX * kAY>((double)local, partials, ticket, &tot, tid, bid, gridDim.x * gridDim.y * gridDim.z))
      *dot_out = tot;
  }
}

// z chunk giving at least ~2 waves of blocks (short chunks cost halo re-reads,
// long ones serialise the march)
inline int apply_zchunk(int nx, int ny, int nz, int sms) {
  const int gxy = ((nx + kAX - 1) / kAX) * ((ny + kAY - 1) / kAY);
  const int want_blocks = 6 * sms;
  int zc = (int)(((int64_t)nz * gxy + want_blocks - 1) / want_blocks);
  if (zc < 4) zc = 4;
  if (zc > 32) zc = 32;
  return zc;
}

inline dim3 apply_grid(int nx, int ny, int nz, int zc) {
  return dim3((nx + kAX - 1) / kAX, (ny + kAY - 1) / kAY, (nz + zc - 1) / zc);
}

// s_r = w_r^2 (a_r . p)  (no reduction)
template <typename T>
__global__ void rows_kernel(int64_t nrows, int width, const int32_t *__restrict__ cols, const T *__restrict__ a,
                            const T *__restrict__ w2, const T *__restrict__ p, T *__restrict__ s, const int *done) {
  if (done && *done) return;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    T acc = 0;
    for (int k = 0; k < width; ++k) {
      const int32_t col = cols[r * width + k];
      if (col >= 0) acc += a[r * width + k] * p[col];
    }
    s[r] = w2[r] * acc;
  }
}

}  // namespace ls
