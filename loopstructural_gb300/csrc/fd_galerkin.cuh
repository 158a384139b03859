// Galerkin coarse operators of the FD regularisation, G_l = P^T G_{l-1} P
// (G_0 = N_reg), for the coarse multigrid levels.
//
// Every regularisation family is a tensor product of per-axis operators: the
// row stencil ((1,-2,1), (-1,0,1) or the identity), the row-existence mask of
// the axis (interior 1..n-2, border layers 1 and n-2, or none) and the
// trilinear prolongation P = Px (x) Py (x) Pz.  Hence
//     G = sum_f w_f  Tx_f (x) Ty_f (x) Tz_f,
// with five kinds of banded 1-D coarse matrices per axis (bandwidth 2):
//     D2I = P^T D2^T I D2 P,  D1I = P^T D1^T I D1 P,  MI = P^T I P,
//     D2B = P^T D2^T B D2 P,  M0 = P^T P
// and the families (weights w_f = the composite coefficients of the fine
// stencil, fd_stencil.cuh):
//     xx: D2I MI MI   yy: MI D2I MI   zz: MI MI D2I
//     xy: D1I D1I MI  xz: D1I MI D1I  yz: MI D1I D1I
//     x-border: D2B M0 M0  (y, z alike)   ridge: M0 M0 M0.
// Coarsening keeps this form: each 1-D table becomes P^T T P (still
// bandwidth 2).  Away from the faces every 1-D row equals the interior row, so
// G is a constant, symmetric 125-point stencil there (staged-tile kernel); the
// nodes near a face (two per side) take precomputed face and edge stencils
// (the stencil of a node with one or two axes in their bands depends only on
// its band rows) and corners the tensor-product sum from the tables
// (node-per-thread shell kernel).  Levels of at most kG1ExplicitMax nodes store
// every node's explicit 125-point stencil (evaluated from the tables at setup)
// and run one warp per node: one launch, no staging, which is what small
// grids are bound by.  A rediscretised coarse operator would weight the border
// layers much more than G does (P annihilates second differences centred on
// odd fine nodes); at 200^3 the Galerkin hierarchy needs 137 instead of 213
// iterations to rtol 1e-10.
#pragma once

#include "fd_apply.cuh"

namespace ls {

enum G1Kind { G1_D2I = 0, G1_D1I = 1, G1_MI = 2, G1_D2B = 3, G1_M0 = 4, G1_KINDS = 5 };
constexpr int kG1Families = 10;
constexpr int64_t kG1ExplicitMax = 50000;
constexpr int kG1MaxBand = 6;  // face stencils kept for up to 3 band rows per side

struct G1Op {
  int nx, ny, nz;
  int lo[3], hi[3];                  // interior box (inclusive), per axis
  const float *t[3];                 // per axis: [kind][index][5] (offsets -2..2)
  float w[kG1Families];              // family weights
  float c[3][5][5];                  // interior stencil c(|dz|, dy, dx); c(-dz) = c(dz)
  const float *shell_coef;           // small levels: 125 x n explicit stencils of every node
  const float *full_coef;            // small levels: shell_coef plus the folded 27-point data term
  // face nodes (one axis in its boundary band): the stencil depends only on
  // that axis' band row -- face_coef[(axis * kG1MaxBand + row) * 125 + o],
  // row = index (low side) or kG1MaxBand/2 + (n - 1 - index) (high side)
  const float *face_coef;
  // edge nodes (two axes in their bands, the third interior): the stencil
  // depends only on the two band rows -- edge_coef[((pair * kG1MaxBand + ra)
  // * kG1MaxBand + rb) * 125 + o], pair 0 = (x, y), 1 = (x, z), 2 = (y, z),
  // ra / rb the band rows of the lower / higher axis
  const float *edge_coef;
};

// band row of coordinate x on axis a (see face_coef), or -1 when the node is
// interior along a or its side's band is wider than the stored rows
__host__ __device__ __forceinline__ int g1_band_row(const G1Op &g, int a, int x, int n) {
  if (x < g.lo[a]) return g.lo[a] <= kG1MaxBand / 2 ? x : -1;
  if (x > g.hi[a]) return n - 1 - g.hi[a] <= kG1MaxBand / 2 ? kG1MaxBand / 2 + (n - 1 - x) : -1;
  return -1;
}

// 1-D kinds of family f along axis a
__host__ __device__ __forceinline__ int g1_kind(int f, int a) {
  // rows: xx yy zz xy xz yz bx by bz ridge ; columns: x y z
  constexpr int K[kG1Families][3] = {{G1_D2I, G1_MI, G1_MI}, {G1_MI, G1_D2I, G1_MI}, {G1_MI, G1_MI, G1_D2I},
                                     {G1_D1I, G1_D1I, G1_MI}, {G1_D1I, G1_MI, G1_D1I}, {G1_MI, G1_D1I, G1_D1I},
                                     {G1_D2B, G1_M0, G1_M0},  {G1_M0, G1_D2B, G1_M0},  {G1_M0, G1_M0, G1_D2B},
                                     {G1_M0, G1_M0, G1_M0}};
  return K[f][a];
}

// Nodes outside the interior box, enumerated as: the z-planes below lo_z /
// above hi_z; then, inside [lo_z, hi_z], the y-rows below lo_y / above hi_y;
// then the x-columns below lo_x / above hi_x.
__host__ __device__ inline int64_t box_shell_count(const G1Op &g) {
  const int64_t bx = g.hi[0] - g.lo[0] + 1, by = g.hi[1] - g.lo[1] + 1, bz = g.hi[2] - g.lo[2] + 1;
  const int64_t inner = (bx > 0 && by > 0 && bz > 0) ? bx * by * bz : 0;
  return (int64_t)g.nx * g.ny * g.nz - inner;
}
__device__ __forceinline__ void box_shell_index(const G1Op &g, int64_t s, int &i, int &j, int &k) {
  const int nx = g.nx, ny = g.ny;
  const int zout = g.lo[2] + (g.nz - 1 - g.hi[2]);
  const int64_t zs = (int64_t)nx * ny * zout;
  const int yout = g.lo[1] + (ny - 1 - g.hi[1]);
  const int64_t ys = (int64_t)nx * yout * (g.hi[2] - g.lo[2] + 1);
  if (s < zs) {
    const int t = (int)(s / ((int64_t)nx * ny));
    const int rem = (int)(s - (int64_t)t * nx * ny);
    k = t < g.lo[2] ? t : g.hi[2] + 1 + (t - g.lo[2]);
    j = rem / nx;
    i = rem - j * nx;
  } else if (s < zs + ys) {
    const int64_t u = s - zs;
    const int per = nx * yout;
    const int kk = (int)(u / per);
    const int rem = (int)(u - (int64_t)kk * per);
    const int t = rem / nx;
    k = g.lo[2] + kk;
    j = t < g.lo[1] ? t : g.hi[1] + 1 + (t - g.lo[1]);
    i = rem - t * nx;
  } else {
    const int64_t u = s - zs - ys;
    const int xout = g.lo[0] + (nx - 1 - g.hi[0]);
    const int per = xout * (g.hi[1] - g.lo[1] + 1);
    const int kk = (int)(u / per);
    const int rem = (int)(u - (int64_t)kk * per);
    const int jj = rem / xout, t = rem - jj * xout;
    k = g.lo[2] + kk;
    j = g.lo[1] + jj;
    i = t < g.lo[0] ? t : g.hi[0] + 1 + (t - g.lo[0]);
  }
}

// G p at one node from the 1-D tables (nodes near a face); PR(dz, dy, dx)
// returns p at the offset (0 outside the grid).
template <typename PR>
__device__ __forceinline__ float g1_node(const G1Op &g, int i, int j, int k, const PR &pr) {
  float tx[G1_KINDS][5];
#pragma unroll
  for (int t = 0; t < G1_KINDS; ++t)
#pragma unroll
    for (int d = 0; d < 5; ++d) tx[t][d] = __ldg(g.t[0] + ((size_t)t * g.nx + i) * 5 + d);
  float acc = 0.f;
#pragma unroll 1
  for (int dz = -2; dz <= 2; ++dz) {
    float tz[G1_KINDS];
#pragma unroll
    for (int t = 0; t < G1_KINDS; ++t) tz[t] = __ldg(g.t[2] + ((size_t)t * g.nz + k) * 5 + dz + 2);
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
      float ty[G1_KINDS];
#pragma unroll
      for (int t = 0; t < G1_KINDS; ++t) ty[t] = __ldg(g.t[1] + ((size_t)t * g.ny + j) * 5 + dy + 2);
      float r[5];
#pragma unroll
      for (int dx = -2; dx <= 2; ++dx) r[dx + 2] = pr(dz, dy, dx);
      float ax[G1_KINDS];
#pragma unroll
      for (int t = 0; t < G1_KINDS; ++t)
        ax[t] = tx[t][0] * r[0] + tx[t][1] * r[1] + tx[t][2] * r[2] + tx[t][3] * r[3] + tx[t][4] * r[4];
#pragma unroll
      for (int f = 0; f < kG1Families; ++f) acc += g.w[f] * ty[g1_kind(f, 1)] * tz[g1_kind(f, 2)] * ax[g1_kind(f, 0)];
    }
  }
  return acc;
}

// Interior box: staged 32 x 8 x TZ tiles (2-node halo) as in fd_apply_kernel;
// per staged plane the three in-plane sums S_m = sum c(m, dy, dx) p, and
// q(z) = S_0(z) + S_1(z-1) + S_1(z+1) + S_2(z-2) + S_2(z+2).
template <int EPI, bool K27, int TZ>
__global__ void __launch_bounds__(kAX * kAY, 4) g1_apply_kernel(G1Op g, const float *__restrict__ p,
                                                                DataView<float> dv, EpiArgs<float> e,
                                                                const int *done) {
  if (done && *done) return;
  constexpr int SZ = TZ + 4, PLANE = kHY * kHX;
  __shared__ float sm[SZ][kHY][kHX];
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int xe = g.hi[0] + 1, ye = g.hi[1] + 1, ze = g.hi[2] + 1;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + kAX * ty;
  const int x0 = g.lo[0] + blockIdx.x * kAX, y0 = g.lo[1] + blockIdx.y * kAY, z0 = g.lo[2] + blockIdx.z * TZ;
  const int sxy = nx * ny;
  const int i = x0 + tx, j = y0 + ty;
  const bool col_in = (i < xe) & (j < ye);
  const int gcol = j * nx + i;
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
    float *base = &sm[0][0][0];
#pragma unroll
    for (int hz = 0; hz < SZ; ++hz) {
      const int gz = z0 - 2 + hz;
      const bool vz = (gz >= 0) & (gz < nz);
      const float *src = p + (vz ? gz * sxy : 0);
      cp_async_elem<float>(base + hz * PLANE + tid, src + off[0], vz & vxy[0]);
      if (tid + kAX * kAY < PLANE) cp_async_elem<float>(base + hz * PLANE + tid + kAX * kAY, src + off[1], vz & vxy[1]);
    }
  }
  cp_async_commit();
  cp_async_wait_all();
  __syncthreads();
  if (!col_in) return;
  const int hx = tx + 2, hy = ty + 2;
  float S0[SZ], S1[SZ], S2[SZ];
  EpiIn<float> pre[TZ];
#pragma unroll
  for (int hz = 0; hz < SZ; ++hz) {
    if (hz >= 2 && hz - 2 < TZ && z0 + hz - 2 < ze) pre[hz - 2] = epi_load<float, EPI>(e, (z0 + hz - 2) * sxy + gcol);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
#pragma unroll
    for (int dy = 0; dy < 5; ++dy)
#pragma unroll
      for (int dx = 0; dx < 5; ++dx) {
        const float v = sm[hz][hy + dy - 2][hx + dx - 2];
        a0 += g.c[0][dy][dx] * v;
        a1 += g.c[1][dy][dx] * v;
        a2 += g.c[2][dy][dx] * v;
      }
    S0[hz] = a0;
    S1[hz] = a1;
    S2[hz] = a2;
    if (hz >= 4) {
      const int ho = hz - 2, oz = ho - 2, z = z0 + oz;
      if (z < ze) {
        const int gi = z * sxy + gcol;
        float q = S0[ho] + (S1[ho - 1] + S1[ho + 1]) + (S2[ho - 2] + S2[ho + 2]);
        if (dv.enabled) q += data_term<float>(dv, gi);
        if (K27) {
          auto pk = [&](int dz, int dy, int dx) -> float { return sm[ho + dz][hy + dy][hx + dx]; };
          q += k27_term<float>(dv, gi, pk);
        }
        epi_store<float, EPI>(e, gi, sm[ho][hy][hx], q, pre[oz]);
      }
    }
  }
}

// The explicit 125-point stencils of the nodes outside the interior box
// (setup): coef[o][s], o = 25 (dz+2) + 5 (dy+2) + (dx+2).
__global__ void g1_coef_kernel(G1Op g, float *__restrict__ coef) {
  const int64_t ns = box_shell_count(g);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_shell_index(g, s, i, j, k);
    for (int o = 0; o < 125; ++o) {
      const int dz = o / 25 - 2, dy = (o / 5) % 5 - 2, dx = o % 5 - 2;
      double acc = 0.0;
      for (int f = 0; f < kG1Families; ++f)
        acc += (double)g.w[f] * g.t[0][((size_t)g1_kind(f, 0) * g.nx + i) * 5 + dx + 2] *
               g.t[1][((size_t)g1_kind(f, 1) * g.ny + j) * 5 + dy + 2] *
               g.t[2][((size_t)g1_kind(f, 2) * g.nz + k) * 5 + dz + 2];
      coef[(size_t)o * ns + s] = (float)acc;
    }
  }
}

// Nodes outside the interior box, one thread per node: explicit stencils
// (EXPLICIT, small levels whose every node is stored) or the tensor-product
// sum from the tables.
template <int EPI, bool K27, bool EXPLICIT>
__global__ void __launch_bounds__(256) g1_shell_kernel(G1Op g, const float *__restrict__ p, DataView<float> dv,
                                                       EpiArgs<float> e, const int *done) {
  if (done && *done) return;
  __shared__ float fc[EXPLICIT ? 1 : 3 * kG1MaxBand * 125];
  if (!EXPLICIT) {
    for (int t = threadIdx.x; t < 3 * kG1MaxBand * 125; t += blockDim.x) fc[t] = __ldg(g.face_coef + t);
    __syncthreads();
  }
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  const int64_t ns = box_shell_count(g);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    int i, j, k;
    box_shell_index(g, s, i, j, k);
    unsigned vx = 0u, vy = 0u, vz = 0u;
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
      vx |= (unsigned)((i + d >= 0) & (i + d < nx)) << (d + 2);
      vy |= (unsigned)((j + d >= 0) & (j + d < ny)) << (d + 2);
      vz |= (unsigned)((k + d >= 0) & (k + d < nz)) << (d + 2);
    }
    const int gi = (k * ny + j) * nx + i;
    const int sxy = nx * ny;
    auto pr = [&](int dz, int dy, int dx) -> float {
      const bool ok = (vz >> (dz + 2)) & (vy >> (dy + 2)) & (vx >> (dx + 2)) & 1u;
      return ok ? __ldg(p + (gi + dz * sxy + dy * nx + dx)) : 0.f;
    };
    float q = 0.f;
    if (EXPLICIT) {
#pragma unroll
      for (int o = 0; o < 125; ++o)
        q += __ldg(g.shell_coef + (size_t)o * ns + s) * pr(o / 25 - 2, (o / 5) % 5 - 2, o % 5 - 2);
    } else {
      // axes in their boundary band and the band row of each: face nodes
      // read their stencil from shared memory, edge nodes from edge_coef
      // (one loop over generic addresses for both, so that a warp holding
      // both kinds does not run it twice); corners and nodes of wider bands
      // sum the tables.  Selects rather than an indexed array, which would
      // sit in local memory.
      int nb = 0, axis = 0, out = 0, r0 = 0, r1 = 0, r2 = 0;
      bool ok = true;
      if (i < g.lo[0] || i > g.hi[0]) { ++nb; axis = 0; r0 = g1_band_row(g, 0, i, nx); ok &= r0 >= 0; } else out = 0;
      if (j < g.lo[1] || j > g.hi[1]) { ++nb; axis = 1; r1 = g1_band_row(g, 1, j, ny); ok &= r1 >= 0; } else out = 1;
      if (k < g.lo[2] || k > g.hi[2]) { ++nb; axis = 2; r2 = g1_band_row(g, 2, k, nz); ok &= r2 >= 0; } else out = 2;
      const float *c = nullptr;
      if (ok && nb == 1) {
        c = fc + (axis * kG1MaxBand + (axis == 0 ? r0 : axis == 1 ? r1 : r2)) * 125;
      } else if (ok && nb == 2 && g.edge_coef) {
        const int ra = out == 0 ? r1 : r0, rb = out == 2 ? r1 : r2;
        c = g.edge_coef + (((2 - out) * kG1MaxBand + ra) * kG1MaxBand + rb) * 125;
      }
      if (c) {
#pragma unroll
        for (int o = 0; o < 125; ++o) q += c[o] * pr(o / 25 - 2, (o / 5) % 5 - 2, o % 5 - 2);
      } else {
        q = g1_node(g, i, j, k, pr);
      }
    }
    if (dv.enabled) q += data_term<float>(dv, gi);
    if (K27) q += k27_term<float>(dv, gi, pr);
    epilogue<float, EPI>(e, gi, __ldg(p + gi), q);
  }
}

// Explicit levels: the stencils node-major (kG1Row floats per node, the 125
// offsets then zeros) with the 27-point data term of the marked nodes folded
// in, so that one sum covers both.
constexpr int kG1Row = 128;
__global__ void g1_fold_k27_kernel(G1Op g, const uint32_t *__restrict__ kmask, const int32_t *__restrict__ krank,
                                   const float *__restrict__ k27, int64_t knt, float *__restrict__ full) {
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    float *row = full + (size_t)s * kG1Row;
    for (int o = 0; o < 125; ++o) row[o] = g.shell_coef[(size_t)o * n + s];
    for (int o = 125; o < kG1Row; ++o) row[o] = 0.f;
    if (!k27 || knt == 0) continue;
    const uint32_t word = kmask[s >> 5], bit = 1u << (s & 31);
    if (!(word & bit)) continue;
    const int rank = krank[s >> 5] + __popc(word & (bit - 1u));
    for (int o = 0; o < 27; ++o) {
      const int dz = o / 9 - 1, dy = (o / 3) % 3 - 1, dx = o % 3 - 1;
      row[25 * (dz + 2) + 5 * (dy + 2) + (dx + 2)] += k27[(size_t)o * knt + rank];
    }
  }
}

// Explicit levels (every node's stencil stored; small grids): one warp per
// node, lane l < 25 sums stencil row (dz, dy) = (l / 5 - 2, l % 5 - 2) -- five
// x-adjacent coefficients and values -- and the rows meet by shuffles.  One
// thread per node cannot hide the latency of its 250 loads on grids this
// small, and the node-major rows keep a warp's coefficient loads in one
// 512-byte span.
template <int EPI>
__global__ void __launch_bounds__(256) g1_explicit_kernel(G1Op g, const float *__restrict__ p, DataView<float> dv,
                                                          EpiArgs<float> e, const int *done) {
  if (done && *done) return;
  const int nx = g.nx, ny = g.ny, nz = g.nz, sxy = nx * ny;
  const int n = sxy * nz;
  const int lane = threadIdx.x & 31;
  const int s = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (s >= n) return;  // uniform across the warp
  const int k = s / sxy, rem = s - k * sxy, j = rem / nx, i = rem - j * nx;
  float acc = 0.f;
  if (lane < 25) {
    const int dz = lane / 5 - 2, dy = lane % 5 - 2;
    if ((k + dz >= 0) & (k + dz < nz) & (j + dy >= 0) & (j + dy < ny)) {
      const float *c = g.full_coef + (size_t)s * kG1Row + 5 * lane;
      const float *pp = p + (s + dz * sxy + dy * nx);
#pragma unroll
      for (int dx = -2; dx <= 2; ++dx)
        if ((i + dx >= 0) & (i + dx < nx)) acc += __ldg(c + dx + 2) * __ldg(pp + dx);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    if (dv.enabled) acc += data_term<float>(dv, s);
    epilogue<float, EPI>(e, s, __ldg(p + s), acc);
  }
}

// diagonal of G (FP64 output, added to by the data term afterwards)
__global__ void g1_diag_kernel(G1Op g, double *__restrict__ diag) {
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(s / ((int64_t)g.nx * g.ny));
    const int rem = (int)(s - (int64_t)k * g.nx * g.ny);
    const int j = rem / g.nx, i = rem - j * g.nx;
    double acc = 0.0;
    for (int f = 0; f < kG1Families; ++f)
      acc += (double)g.w[f] * g.t[0][((size_t)g1_kind(f, 0) * g.nx + i) * 5 + 2] *
             g.t[1][((size_t)g1_kind(f, 1) * g.ny + j) * 5 + 2] * g.t[2][((size_t)g1_kind(f, 2) * g.nz + k) * 5 + 2];
    diag[s] = acc;
  }
}

// parts: bit 0 the interior kernel, bit 1 the boundary kernel
template <int EPI, bool K27>
inline int launch_g1_k(const G1Op &g, const float *p, const DataView<float> &dv, const EpiArgs<float> &e,
                       const int *done, int sms, cudaStream_t st, int parts = 3) {
  int launches = 0;
  const int bx = g.hi[0] - g.lo[0] + 1, by = g.hi[1] - g.lo[1] + 1, bz = g.hi[2] - g.lo[2] + 1;
  if ((parts & 1) && bx > 0 && by > 0 && bz > 0) {
    const dim3 blk(kAX, kAY);
    const dim3 g8((bx + kAX - 1) / kAX, (by + kAY - 1) / kAY, (bz + 7) / 8);
    if ((int64_t)g8.x * g8.y * g8.z >= 4 * (int64_t)sms) {
      g1_apply_kernel<EPI, K27, 8><<<g8, blk, 0, st>>>(g, p, dv, e, done);
    } else {
      const dim3 g4((bx + kAX - 1) / kAX, (by + kAY - 1) / kAY, (bz + 3) / 4);
      g1_apply_kernel<EPI, K27, 4><<<g4, blk, 0, st>>>(g, p, dv, e, done);
    }
    ++launches;
  }
  const int64_t ns = box_shell_count(g);
  if ((parts & 2) && ns > 0 && g.full_coef) {
    g1_explicit_kernel<EPI><<<(int)((ns * 32 + 255) / 256), 256, 0, st>>>(g, p, dv, e, done);
    ++launches;
  } else if ((parts & 2) && ns > 0) {
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((ns + 255) / 256, 8 * (int64_t)sms));
    if (g.shell_coef)
      g1_shell_kernel<EPI, K27, true><<<gs, 256, 0, st>>>(g, p, dv, e, done);
    else
      g1_shell_kernel<EPI, K27, false><<<gs, 256, 0, st>>>(g, p, dv, e, done);
    ++launches;
  }
  return launches;
}

// q = (G + data term) p with an epilogue; returns the number of launches
template <int EPI>
inline int launch_g1(const G1Op &g, const float *p, const DataView<float> &dv, const EpiArgs<float> &e,
                     const int *done, int sms, cudaStream_t st, int parts = 3) {
  if (dv.k27) return launch_g1_k<EPI, true>(g, p, dv, e, done, sms, st, parts);
  return launch_g1_k<EPI, false>(g, p, dv, e, done, sms, st, parts);
}

}  // namespace ls
