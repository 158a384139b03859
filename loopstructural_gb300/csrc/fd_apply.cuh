// Fused matrix-free application of the FD normal operator
//     q = (sum_f w_f^2 R_f^T R_f + A_d^T W A_d + ridge^2 I) p
// with a per-use epilogue, as one z-marching kernel.
//
// Tiling: a block of 32 x 8 threads owns a 32 x 8 x 8 node tile; the tile and
// a 2-node halo are staged in shared memory in one cp.async burst.  Every
// thread forms, for its own (x, y) column and each staged plane, the in-plane
// quantities of the composite deep-interior stencil
//     S(s)  = a_x d4_x p + a_y d4_y p + b_xy C_x C_y p      (12 shared reads)
//     Cx(s) = C_x p,  Cy(s) = C_y p,  P(s) = p
// in register windows over z, so that at plane z
//     q = ridge^2 P + S(z) + a_z d4_z P + b_xz C_z Cx + b_yz C_z Cy
// needs no further memory traffic (d4 = (1,-4,6,-4,1), C = (1,0,-2,0,1) at
// stride 2; a = w^2/6, b = w^2/4).  Nodes within 3 of a face evaluate the exact
// two-pass sum branch-free from the staged neighbourhood (shell_node).
//
// Data rows: the touched nodes are marked in a bit mask (x-fastest words); a
// touched node adds sum_e a_e s_row(e) over its incidence list, where
// s_row = w^2 (a_row . p) was produced by the rows kernel launched just before.
#pragma once

#include <algorithm>
#include <cassert>

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
  const T *qd;               // optional: per-touched-node totals from data_nodes_warp_kernel
  int enabled;
  // optional 27-point form of data rows confined to one cell (coarse
  // multigrid levels): q += sum_o k27[o][rank] p(node + o) at marked nodes
  const uint32_t *kmask;
  const int32_t *krank;
  const T *k27;  // 27 x knt, offset o = 9 (dz+1) + 3 (dy+1) + (dx+1)
  int64_t knt;
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

// Epilogue operands read at the output node, loaded ahead of the stencil
// (software prefetch) so that their latency overlaps the arithmetic.
template <typename T>
struct EpiIn {
  T x, r, dinv;
};

template <typename T, int EPI>
__device__ __forceinline__ EpiIn<T> epi_load(const EpiArgs<T> &e, int g) {
  EpiIn<T> v{};
  if (EPI == EPI_CHEB) {
    v.x = e.x[g];
    v.r = e.r[g];
    v.dinv = e.dinv[g];
  } else if (EPI == EPI_RESID) {
    v.r = e.b[g];
    v.dinv = e.dinv[g];
  }
  return v;
}

template <typename T, int EPI>
__device__ __forceinline__ T epi_store(const EpiArgs<T> &e, int g, T p_own, T q, const EpiIn<T> &v) {
  if (EPI == EPI_STORE) {
    e.q[g] = q;
    return p_own * q;
  } else if (EPI == EPI_CHEB) {
    e.x[g] = v.x + p_own;
    const T rn = v.r - q;
    e.r[g] = rn;
    e.d_out[g] = e.c1 * p_own + e.c2 * v.dinv * rn;
    return (T)0;
  } else {
    const T rn = v.r - q;  // v.r holds b
    e.r[g] = rn;
    e.d_out[g] = e.c2 * v.dinv * rn;
    return (T)0;
  }
}

template <typename T, int EPI>
__device__ __forceinline__ T epilogue(const EpiArgs<T> &e, int g, T p_own, T q) {
  return epi_store<T, EPI>(e, g, p_own, q, epi_load<T, EPI>(e, g));
}

// Data term at node g whose mask word has been loaded already.
template <typename T>
__device__ __forceinline__ T data_term_w(const DataView<T> &dv, int g, uint32_t word) {
  const uint32_t bit = 1u << (g & 31);
  if (!(word & bit)) return (T)0;
  const int rank = __ldg(dv.word_rank + (g >> 5)) + __popc(word & (bit - 1u));
  if (dv.qd) return dv.qd[rank];
  T acc = 0;
  const int64_t e1 = __ldg(dv.inc_ptr + rank + 1);
  for (int64_t e = __ldg(dv.inc_ptr + rank); e < e1; ++e) acc += __ldg(dv.inc_a + e) * __ldg(dv.s_rows + __ldg(dv.inc_row + e));
  return acc;
}

template <typename T>
__device__ __forceinline__ T data_term(const DataView<T> &dv, int g) {
  const uint32_t word = __ldg(dv.mask + (g >> 5));
  const uint32_t bit = 1u << (g & 31);
  if (!(word & bit)) return (T)0;
  const int rank = __ldg(dv.word_rank + (g >> 5)) + __popc(word & (bit - 1u));
  if (dv.qd) return dv.qd[rank];
  T acc = 0;
  const int64_t e1 = __ldg(dv.inc_ptr + rank + 1);
  for (int64_t e = __ldg(dv.inc_ptr + rank); e < e1; ++e) acc += __ldg(dv.inc_a + e) * __ldg(dv.s_rows + __ldg(dv.inc_row + e));
  return acc;
}

template <typename T, typename PR>
__device__ __forceinline__ T k27_term_w(const DataView<T> &dv, int g, uint32_t word, const PR &pr) {
  const uint32_t bit = 1u << (g & 31);
  if (!(word & bit)) return (T)0;
  const int rank = __ldg(dv.krank + (g >> 5)) + __popc(word & (bit - 1u));
  T acc = 0;
#pragma unroll
  for (int o = 0; o < 27; ++o) acc += __ldg(dv.k27 + (int64_t)o * dv.knt + rank) * pr(o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1);
  return acc;
}

template <typename T, typename PR>
__device__ __forceinline__ T k27_term(const DataView<T> &dv, int g, const PR &pr) {
  return k27_term_w<T>(dv, g, __ldg(dv.kmask + (g >> 5)), pr);
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
// Template flags BY / BZ / BX = false declare the node deep along y / z / x
// (index in [3, n-4]: every row centre around it interior, none on a border
// layer), so that those factors are compile-time constants; the result is the
// same.
template <typename T, typename PR, bool BY = true, bool BZ = true, bool BX = true>
__device__ __forceinline__ T shell_node(const CoefT<T> &c, const PR &pr, int i, int j, int k) {
  T ix[3], bx[3], iy[3], by[3], iz[3], bz[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    ix[d] = BX ? ind_i<T>(i + d - 1, c.nx) : (T)1;
    bx[d] = BX ? ind_b<T>(i + d - 1, c.nx) : (T)0;
    iy[d] = BY ? ind_i<T>(j + d - 1, c.ny) : (T)1;
    by[d] = BY ? ind_b<T>(j + d - 1, c.ny) : (T)0;
    iz[d] = BZ ? ind_i<T>(k + d - 1, c.nz) : (T)1;
    bz[d] = BZ ? ind_b<T>(k + d - 1, c.nz) : (T)0;
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

// Output planes per block (TZ; the block stages TZ + 4 planes of 432 nodes):
// 8 or 4 in FP32 (20.8 / 13.8 KB of shared memory; 4 on grids too small to
// fill the GPU with 8-plane tiles), 8 in FP64 (41.5 KB).  Deeper FP32 tiles
// stage fewer halo planes but their fully unrolled plane loop outgrows the
// instruction cache and spills under the 4-blocks-per-SM register budget
// (measured: 16-plane tiles 95 us, 8-plane tiles 80 us per Chebyshev apply
// at 200^3).
template <typename T, int TZ_>
struct Tile {
  static constexpr int TZ = TZ_;
  static constexpr int SZ = TZ + 4;
  static constexpr int PLANE = kHY * kHX;  // 432 staged nodes per plane
};

// Operator modes.  FULL: every node of the grid, boundary nodes through the
// exact shell sum.  DEEP: only the deep box [3, n-4]^3, composite stencil
// without a branch; the boundary shell is left to fd_point_kernel.
enum ApplyMode { MODE_FULL = 0, MODE_DEEP = 1 };

// The deep box is split off when every axis has at least this many nodes.
constexpr int kSplitMin = 24;
inline bool apply_split(int nx, int ny, int nz) { return nx >= kSplitMin && ny >= kSplitMin && nz >= kSplitMin; }

// Asynchronous global -> shared copy of one element (cp.async); a zero source
// size fills zeros (outside the grid).
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
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Block = 32 x 8 threads owning a 32 x 8 x TZ output tile.  The tile and a
// 2-node halo ((32+4) x (8+4) x (TZ+4)) are staged in one cp.async burst (each
// thread copies the same one or two in-plane positions of every plane), then
// one barrier.  Each thread walks its own column through the staged planes in
// a fully unrolled loop: the in-plane quantities P, Cx, Cy of plane s are
// formed when s is reached and the output of plane s-2 is emitted as soon as
// they are, so only a 5-plane window stays live in registers.
// Returns the block's sum of the epilogue contributions (p.q for EPI_STORE)
// through the deterministic grid reduction when `dot_out` is set.
template <typename T, int EPI, int MODE, int TZ_>
__global__ void __launch_bounds__(kAX * kAY, MODE == MODE_DEEP ? 4 : 1)
    fd_apply_kernel(CoefT<T> c, const T *__restrict__ p, DataView<T> dv, EpiArgs<T> e, const int *done,
                    double *partials, unsigned int *ticket, double *dot_out) {
  if (done && *done) return;
  using TL = Tile<T, TZ_>;
  constexpr int TZ = TL::TZ, SZ = TL::SZ, PLANE = TL::PLANE;
  __shared__ T sm[SZ][kHY][kHX];
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int org = MODE == MODE_DEEP ? 3 : 0;  // first node of the covered box
  const int xe = MODE == MODE_DEEP ? nx - 3 : nx, ye = MODE == MODE_DEEP ? ny - 3 : ny,
            ze = MODE == MODE_DEEP ? nz - 3 : nz;  // one past the last covered node
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + kAX * ty;
  const int x0 = org + blockIdx.x * kAX, y0 = org + blockIdx.y * kAY, z0 = org + blockIdx.z * TZ;
  const int sxy = nx * ny;  // node counts stay below 2^31
  const int i = x0 + tx, j = y0 + ty;
  const bool col_in = (i < xe) & (j < ye);
  const int gcol = j * nx + i;
  // mask words of the column's output nodes, loaded before the staging burst
  // and reduced to one bit per output plane while it is in flight
  uint32_t mw[TZ];
#pragma unroll
  for (int oz = 0; oz < TZ; ++oz) {
    const int g = (z0 + oz) * sxy + gcol;
    const bool ok = col_in & (z0 + oz < ze);
    mw[oz] = (dv.enabled && ok) ? __ldg(dv.mask + (g >> 5)) : 0u;
  }
  uint32_t dbits = 0u;
  // ---- stage the tile ----
  {
    int off[2];
    bool vxy[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int e2 = tid + u * kAX * kAY;
      const int hy = e2 / kHX, hx = e2 - hy * kHX;
      const int gx = x0 - 2 + hx, gy = y0 - 2 + hy;
      vxy[u] = (e2 < PLANE) & (gx >= 0) & (gx < nx) & (gy >= 0) & (gy < ny);
      off[u] = vxy[u] ? gy * nx + gx : 0;
    }
    T *base = &sm[0][0][0];
#pragma unroll
    for (int hz = 0; hz < SZ; ++hz) {
      const int gz = z0 - 2 + hz;
      const bool vz = (gz >= 0) & (gz < nz);
      const T *src = p + (vz ? gz * sxy : 0);
      cp_async_elem<T>(base + hz * PLANE + tid, src + off[0], vz & vxy[0]);
      if (tid + kAX * kAY < PLANE) cp_async_elem<T>(base + hz * PLANE + tid + kAX * kAY, src + off[1], vz & vxy[1]);
    }
  }
  cp_async_commit();
#pragma unroll
  for (int oz = 0; oz < TZ; ++oz) {
    const int g = (z0 + oz) * sxy + gcol;
    dbits |= ((mw[oz] >> (g & 31)) & 1u) << oz;
  }
  cp_async_wait_all();
  __syncthreads();
  T local = 0;
  if (col_in) {
    const bool col_deep = MODE == MODE_DEEP || ((i >= 3) & (i <= nx - 4) & (j >= 3) & (j <= ny - 4));
    const int hx = tx + 2, hy = ty + 2;
    T P[SZ], Cx[SZ], Cy[SZ];
    EpiIn<T> pre[TZ];
#pragma unroll
    for (int hz = 0; hz < SZ; ++hz) {
      // epilogue operands of output plane hz - 1, three planes ahead of their use
      if (hz >= 1 && hz - 1 < TZ && z0 + hz - 1 < ze) pre[hz - 1] = epi_load<T, EPI>(e, (z0 + hz - 1) * sxy + gcol);
      const T(&pl)[kHY][kHX] = sm[hz];
      const T p0 = pl[hy][hx];
      P[hz] = p0;
      Cx[hz] = (pl[hy][hx - 2] + pl[hy][hx + 2]) - (T)2 * p0;
      Cy[hz] = (pl[hy - 2][hx] + pl[hy + 2][hx]) - (T)2 * p0;
      if (hz >= 4) {
        const int ho = hz - 2;  // staged plane of the output
        const int oz = ho - 2;
        const int z = z0 + oz;
        if (z < ze) {
          const int g = z * sxy + gcol;
          T q;
          if (col_deep & (MODE == MODE_DEEP || ((z >= 3) & (z <= nz - 4)))) {
            const T(&po)[kHY][kHX] = sm[ho];
            const T q0 = P[ho];
            const T ex = po[hy][hx - 2] + po[hy][hx + 2], ey = po[hy - 2][hx] + po[hy + 2][hx];
            const T d4x = ex - (T)4 * (po[hy][hx - 1] + po[hy][hx + 1]) + (T)6 * q0;
            const T d4y = ey - (T)4 * (po[hy - 1][hx] + po[hy + 1][hx]) + (T)6 * q0;
            const T corners = (po[hy - 2][hx - 2] + po[hy - 2][hx + 2]) + (po[hy + 2][hx - 2] + po[hy + 2][hx + 2]);
            const T d4z = (P[ho - 2] + P[ho + 2]) - (T)4 * (P[ho - 1] + P[ho + 1]) + (T)6 * q0;
            q = c.ridge2 * q0 + c.xx_int * d4x + c.yy_int * d4y + c.zz_int * d4z +
                c.xy * (corners - (T)2 * (ex + ey) + (T)4 * q0) +
                c.xz * ((Cx[ho - 2] + Cx[ho + 2]) - (T)2 * Cx[ho]) + c.yz * ((Cy[ho - 2] + Cy[ho + 2]) - (T)2 * Cy[ho]);
          } else {
            auto pr = [&](int dz, int dy, int dx) -> T { return sm[ho + dz][hy + dy][hx + dx]; };
            q = shell_node<T>(c, pr, i, j, z);
          }
          if ((dbits >> oz) & 1u) q += data_term<T>(dv, g);
          local += epi_store<T, EPI>(e, g, P[ho], q, pre[oz]);
        }
      }
    }
  }
  if (dot_out) {
    double tot;
    const unsigned int bid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    if (grid_sum_ex<kAX * kAY, T>(local, partials, ticket, &tot, tid, bid, gridDim.x * gridDim.y * gridDim.z))
      *dot_out = tot;
  }
}

template <typename T, int TZ>
inline dim3 apply_grid(int nx, int ny, int nz, int mode) {
  if (mode == MODE_DEEP) {
    nx -= 6;
    ny -= 6;
    nz -= 6;
  }
  return dim3((nx + kAX - 1) / kAX, (ny + kAY - 1) / kAY, (nz + TZ - 1) / TZ);
}

// Boundary shell of a split grid: nodes with some coordinate in {0,1,2,n-3,n-2,n-1}
// (all axes >= 7), enumerated in three slabs: the 6 z-planes; then, for
// 3 <= k <= nz-4, the 6 y-rows; then, for 3 <= j <= ny-4, the 6 x-columns.
__host__ __device__ inline int64_t shell_count(int nx, int ny, int nz) {
  return (int64_t)nx * ny * nz - (int64_t)(nx - 6) * (ny - 6) * (nz - 6);
}
__device__ __forceinline__ void shell_node_index(int64_t s, int nx, int ny, int nz, int &i, int &j, int &k) {
  const int64_t zs = 6 * (int64_t)nx * ny, ys = 6 * (int64_t)nx * (nz - 6);
  if (s < zs) {
    const int t = (int)(s / ((int64_t)nx * ny));
    const int rem = (int)(s - (int64_t)t * nx * ny);
    k = t < 3 ? t : nz - 6 + t;
    j = rem / nx;
    i = rem - j * nx;
  } else if (s < zs + ys) {
    const int64_t u = s - zs;
    const int kk = (int)(u / (6 * nx));
    const int rem = (int)(u - (int64_t)kk * 6 * nx);
    const int t = rem / nx;
    k = 3 + kk;
    j = t < 3 ? t : ny - 6 + t;
    i = rem - t * nx;
  } else {
    const int64_t u = s - zs - ys;
    const int kk = (int)(u / (6 * (ny - 6)));
    const int rem = (int)(u - (int64_t)kk * 6 * (ny - 6));
    const int jj = rem / 6, t = rem - jj * 6;
    k = 3 + kk;
    j = 3 + jj;
    i = t < 3 ? t : nx - 6 + t;
  }
}

// The exact operator node by node (one thread per node, neighbours straight
// from L1/L2), with the data term and the epilogue: the boundary shell of a
// split grid (ALL = false), or every node of a small grid (ALL = true), where
// a thread per node exposes more parallelism than the staged tiles.
template <typename T, int EPI, bool ALL>
__global__ void __launch_bounds__(256) fd_point_kernel(CoefT<T> c, const T *__restrict__ p, DataView<T> dv,
                                                       EpiArgs<T> e, const int *done, double *partials,
                                                       unsigned int *ticket, double *dot_out) {
  if (done && *done) return;
  const int nx = c.nx, ny = c.ny, nz = c.nz;
  const int64_t ns = ALL ? (int64_t)nx * ny * nz : shell_count(nx, ny, nz);
  T local = 0;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    if (ALL) {
      k = (int)(s / ((int64_t)nx * ny));
      const int rem = (int)(s - (int64_t)k * nx * ny);
      j = rem / nx;
      i = rem - j * nx;
    } else {
      shell_node_index(s, nx, ny, nz, i, j, k);
    }
    // neighbours at offsets -2..2: per-axis validity bits, one predicated load each
    unsigned vx = 0u, vy = 0u, vz = 0u;
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
      vx |= (unsigned)((i + d >= 0) & (i + d < nx)) << (d + 2);
      vy |= (unsigned)((j + d >= 0) & (j + d < ny)) << (d + 2);
      vz |= (unsigned)((k + d >= 0) & (k + d < nz)) << (d + 2);
    }
    const int g = (k * ny + j) * nx + i;
    const int sxy = nx * ny;
    auto pr = [&](int dz, int dy, int dx) -> T {
      const bool ok = (vz >> (dz + 2)) & (vy >> (dy + 2)) & (vx >> (dx + 2)) & 1u;
      return ok ? __ldg(p + (g + dz * sxy + dy * nx + dx)) : (T)0;
    };
    T q = shell_node<T>(c, pr, i, j, k);
    if (dv.enabled) q += data_term<T>(dv, g);
    local += epilogue<T, EPI>(e, g, __ldg(p + g), q);
  }
  if (dot_out) {
    double tot;
    if (grid_sum<256, T>(local, partials, ticket, &tot)) *dot_out = tot;
  }
}

// Grids with fewer nodes than this run the node-per-thread kernel alone.
constexpr int64_t kPointMaxNodes = 300000;

template <typename T, int EPI, int MODE>
inline void launch_tiles(const CoefT<T> &c, const T *p, const DataView<T> &dv, const EpiArgs<T> &e, const int *done,
                         double *partials, unsigned int *ticket, double *dot, int sms, cudaStream_t st) {
  const dim3 blk(kAX, kAY);
  if constexpr (sizeof(T) == 8) {
    fd_apply_kernel<T, EPI, MODE, 8><<<apply_grid<T, 8>(c.nx, c.ny, c.nz, MODE), blk, 0, st>>>(
        c, p, dv, e, done, partials, ticket, dot);
  } else {
    const dim3 g8 = apply_grid<T, 8>(c.nx, c.ny, c.nz, MODE);
    if ((int64_t)g8.x * g8.y * g8.z >= 4 * (int64_t)sms) {
      fd_apply_kernel<T, EPI, MODE, 8><<<g8, blk, 0, st>>>(c, p, dv, e, done, partials, ticket, dot);
    } else {
      fd_apply_kernel<T, EPI, MODE, 4><<<apply_grid<T, 4>(c.nx, c.ny, c.nz, MODE), blk, 0, st>>>(
          c, p, dv, e, done, partials, ticket, dot);
    }
  }
}

template <typename T, int EPI>
inline int launch_operator_k(const CoefT<T> &c, const T *p, const DataView<T> &dv, const EpiArgs<T> &e,
                             const int *done, double *partials, unsigned int *ticket_main, double *dot_main,
                             unsigned int *ticket_shell, double *dot_shell, int max_blocks, cudaStream_t st) {
  const int64_t n = (int64_t)c.nx * c.ny * c.nz;
  const int sms = max_blocks / 8;
  if (n <= kPointMaxNodes) {
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, max_blocks));
    fd_point_kernel<T, EPI, true><<<gs, 256, 0, st>>>(c, p, dv, e, done, partials, ticket_main, dot_main);
    return 1;
  }
  if (apply_split(c.nx, c.ny, c.nz)) {
    launch_tiles<T, EPI, MODE_DEEP>(c, p, dv, e, done, partials, ticket_main, dot_main, sms, st);
    const int64_t ns = shell_count(c.nx, c.ny, c.nz);
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((ns + 255) / 256, max_blocks));
    fd_point_kernel<T, EPI, false><<<gs, 256, 0, st>>>(c, p, dv, e, done, partials, ticket_shell, dot_shell);
    return 2;
  }
  launch_tiles<T, EPI, MODE_FULL>(c, p, dv, e, done, partials, ticket_main, dot_main, sms, st);
  return 1;
}

// q = N_reg p (+ data term) with an epilogue: one node-per-thread kernel on
// small grids; the deep-box kernel plus the shell kernel on split grids; else
// one staged full-grid kernel.  The epilogue sums land in dot_main (full grid
// / deep box) and dot_shell (shell; untouched otherwise).  Returns the number
// of kernels launched.  Used on the finest level, whose data rows are in row
// form (the coarse levels' 27-point form is applied by fd_galerkin.cuh).
template <typename T, int EPI>
inline int launch_operator(const CoefT<T> &c, const T *p, const DataView<T> &dv, const EpiArgs<T> &e, const int *done,
                           double *partials, unsigned int *ticket_main, double *dot_main, unsigned int *ticket_shell,
                           double *dot_shell, int max_blocks, cudaStream_t st) {
  assert(dv.k27 == nullptr);  // the 27-point data form exists on Galerkin levels only (fd_galerkin.cuh)
  return launch_operator_k<T, EPI>(c, p, dv, e, done, partials, ticket_main, dot_main, ticket_shell, dot_shell,
                                   max_blocks, st);
}

// Data term of the touched nodes with one warp per node (coarse multigrid
// levels, where many Galerkin rows pile up on each node): qd[rank] = sum_e a_e s_row(e)
template <typename T>
__global__ void data_nodes_warp_kernel(int64_t ntouched, const int64_t *__restrict__ inc_ptr,
                                       const int32_t *__restrict__ inc_row, const T *__restrict__ inc_a,
                                       const T *__restrict__ s_rows, T *__restrict__ qd, const int *done) {
  if (done && *done) return;
  const int lane = threadIdx.x & 31;
  for (int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; t < ntouched;
       t += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    T acc = 0;
    for (int64_t e = inc_ptr[t] + lane; e < inc_ptr[t + 1]; e += 32) acc += inc_a[e] * s_rows[inc_row[e]];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) qd[t] = acc;
  }
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
