// FD constraint assembly on the GPU (K1 point rows, interface pair rows and
// K2 explicit regularisation indices).
//
// Parity: column indices are bit-identical to the reference COO; values
// follow the reference's floating-point evaluation order (no FMA contraction:
// this file is compiled with -fmad=false) so they agree to ~1 ulp.
#include <math.h>

#include "ls_common.cuh"

namespace ls {
namespace {

struct GridArgs {
  double origin[3], step[3], lo[3], hi[3];
  int64_t n[3], cells[3];
};

GridArgs make_grid_args(const ls_grid3 &g) {
  GridArgs a;
  for (int d = 0; d < 3; ++d) {
    a.origin[d] = g.origin[d];
    a.step[d] = g.step[d];
    a.n[d] = g.nsteps[d];
    a.cells[d] = g.nsteps[d] - 1;
    // S:287-293 inside(): tolerance eps * 32 * max(|max - origin|, 1)
    double mx = g.origin[d] + (double)a.cells[d] * g.step[d];
    double ext = fabs(mx - g.origin[d]);
    if (ext < 1.0) ext = 1.0;
    double tol = 2.220446049250313e-16 * 32.0 * ext;
    a.lo[d] = g.origin[d] - tol;
    a.hi[d] = mx + tol;
  }
  return a;
}

__device__ __forceinline__ bool point_inside(const GridArgs &g, double x, double y, double z) {
  return (x >= g.lo[0]) & (x <= g.hi[0]) & (y >= g.lo[1]) & (y <= g.hi[1]) & (z >= g.lo[2]) & (z <= g.hi[2]);
}

// S:251-282 cell index, S:386-412 corners, G:126-146 clipped local coords.
__device__ __forceinline__ void locate(const GridArgs &g, const double p[3], int64_t idc[8], double l[3]) {
  int64_t c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double x = p[d] - g.origin[d];
    int64_t ci = (int64_t)floor(x / g.step[d]);
    if (ci < 0) ci = 0;
    if (ci > g.cells[d] - 1) ci = g.cells[d] - 1;
    c[d] = ci;
    double co = g.origin[d] + g.step[d] * (double)ci;
    double lc = (p[d] - co) / g.step[d];
    l[d] = fmin(fmax(lc, 0.0), 1.0);
  }
  const int64_t nx = g.n[0], nxy = g.n[0] * g.n[1];
  const int64_t g0 = c[0] + nx * c[1] + nxy * c[2];
  idc[0] = g0;
  idc[1] = g0 + 1;
  idc[2] = g0 + nx;
  idc[3] = g0 + nx + 1;
  idc[4] = g0 + nxy;
  idc[5] = g0 + nxy + 1;
  idc[6] = g0 + nxy + nx;
  idc[7] = g0 + nxy + nx + 1;
}

// G:90-124 (same operation order)
__device__ __forceinline__ void trilinear(const double l[3], double a[8]) {
  const double x = l[0], y = l[1], z = l[2];
  a[0] = (1 - x) * (1 - y) * (1 - z);
  a[1] = x * (1 - y) * (1 - z);
  a[2] = (1 - x) * y * (1 - z);
  a[4] = (1 - x) * (1 - y) * z;
  a[5] = x * (1 - y) * z;
  a[6] = (1 - x) * y * z;
  a[3] = x * y * (1 - z);
  a[7] = x * y * z;
}

// G:393-454 element gradient T (3 x 8) divided by the step
__device__ __forceinline__ void element_gradient(const double l[3], const double step[3], double T[3][8]) {
  const double x = l[0], y = l[1], z = l[2];
  T[0][0] = (1 - z) * (y - 1);
  T[0][1] = (1 - y) * (1 - z);
  T[0][2] = -y * (1 - z);
  T[0][4] = -(1 - y) * z;
  T[0][5] = (1 - y) * z;
  T[0][6] = -y * z;
  T[0][3] = y * (1 - z);
  T[0][7] = y * z;
  T[1][0] = (x - 1) * (1 - z);
  T[1][1] = -x * (1 - z);
  T[1][2] = (1 - x) * (1 - z);
  T[1][4] = -(1 - x) * z;
  T[1][5] = -x * z;
  T[1][6] = (1 - x) * z;
  T[1][3] = x * (1 - z);
  T[1][7] = x * z;
  T[2][0] = -(1 - x) * (1 - y);
  T[2][1] = -x * (1 - y);
  T[2][2] = -(1 - x) * y;
  T[2][4] = (1 - x) * (1 - y);
  T[2][5] = x * (1 - y);
  T[2][6] = (1 - x) * y;
  T[2][3] = -x * y;
  T[2][7] = x * y;
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int k = 0; k < 8; ++k) T[d][k] = T[d][k] / step[d];
}

// numpy's add.reduce of 8 contiguous values (pairwise block of 8)
__device__ __forceinline__ double sumsq8(const double a[8]) {
  double r = ((a[0] * a[0] + a[1] * a[1]) + (a[2] * a[2] + a[3] * a[3])) +
             ((a[4] * a[4] + a[5] * a[5]) + (a[6] * a[6] + a[7] * a[7]));
  return 0.0 + r;
}

// DI:361-366 row normalisation
__device__ __forceinline__ void normalise8(double a[8], double &b) {
  double len = sqrt(sumsq8(a));
  if (len > 0) {
    b = b / len;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = a[k] / len;
  }
}

__device__ __forceinline__ double norm3_seq(double a, double b, double c) {
  return sqrt(((0.0 + a * a) + b * b) + c * c);
}

__device__ __forceinline__ void store_row(int64_t row, const int64_t idc[8], const double a[8], double b, double w,
                                          int64_t *d_idc, double *d_a, double *d_b, double *d_w, int32_t *nan_flag) {
  bool bad = isnan(b);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    d_idc[row * 8 + k] = idc[k];
    d_a[row * 8 + k] = a[k];
    bad |= isnan(a[k]);
  }
  d_b[row] = b;
  d_w[row] = w;
  if (bad) *nan_flag = 1;
}

__global__ void inside_flags_kernel(GridArgs g, const double *__restrict__ pts, int64_t n, int64_t ld,
                                    int32_t *__restrict__ flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *p = pts + i * ld;
    flag[i] = point_inside(g, p[0], p[1], p[2]) ? 1 : 0;
  }
}

// Single-block exclusive scan of int32 flags into int64 slots; writes the
// total to *count.  Setup-time helper (n up to a few million points).
__global__ void __launch_bounds__(1024) scan_flags_kernel(const int32_t *__restrict__ flag, int64_t n,
                                                          int64_t *__restrict__ slot, int64_t *__restrict__ count) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < n; base += 1024) {
    int64_t i = base + threadIdx.x;
    int64_t v = (i < n) ? flag[i] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    int64_t excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
    if (i < n) slot[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = carry;
}

template <int KIND>
__global__ void point_rows_kernel(GridArgs g, const double *__restrict__ pts, int64_t n, int64_t ld, double weight,
                                  const int32_t *__restrict__ flag, const int64_t *__restrict__ slot,
                                  int64_t *__restrict__ d_idc, double *__restrict__ d_a, double *__restrict__ d_b,
                                  double *__restrict__ d_w, int32_t *__restrict__ nan_flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const double *p = pts + i * ld;
    const int64_t s = slot[i];
    double pos[3] = {p[0], p[1], p[2]};
    int64_t idc[8];
    double l[3];
    locate(g, pos, idc, l);
    if (KIND == LS_ROWS_VALUE) {  // FD:236-269
      double a[8];
      trilinear(l, a);
      double b = p[3];
      normalise8(a, b);
      store_row(s, idc, a, b, weight * p[4], d_idc, d_a, d_b, d_w, nan_flag);
    } else if (KIND == LS_ROWS_NORM) {  // FD:403-476
      double T[3][8];
      element_gradient(l, g.step, T);
      const double pw = (ld > 6) ? p[6] : 1.0;
      const double w = (weight / 3.0) * pw;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double b = p[3 + d];
        normalise8(T[d], b);
        store_row((int64_t)d * n + s, idc, T[d], b, w, d_idc, d_a, d_b, d_w, nan_flag);
      }
    } else if (KIND == LS_ROWS_GRADIENT) {  // FD:342-401 + get_vectors (M:276-298)
      double T[3][8];
      element_gradient(l, g.step, T);
      double gv[3] = {p[3], p[4], p[5]};
      double gn = norm3_seq(gv[0], gv[1], gv[2]);
#pragma unroll
      for (int d = 0; d < 3; ++d) gv[d] = gv[d] / gn;
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int k = 0; k < 8; ++k) T[d][k] = T[d][k] / gn;
      double len = norm3_seq(gv[0], gv[1], gv[2]);
      double nv[3] = {gv[0] / len, gv[1] / len, gv[2] / len};
      double len2 = norm3_seq(nv[0], nv[1], nv[2]);
      double nn[3] = {nv[0] / len2, nv[1] / len2, nv[2] / len2};
      double strike_deg = (-atan2(nn[1], nn[0])) * (180.0 / 3.141592653589793);
      double srad = strike_deg * (3.141592653589793 / 180.0);
      double sv[3] = {sin(-srad), -cos(-srad), 0.0};
      double sl = norm3_seq(sv[0], sv[1], sv[2]);
#pragma unroll
      for (int d = 0; d < 3; ++d) sv[d] = sv[d] / sl;
      double dv[3] = {sv[1] * nv[2] - sv[2] * nv[1], sv[2] * nv[0] - sv[0] * nv[2], sv[0] * nv[1] - sv[1] * nv[0]};
      double dl = norm3_seq(dv[0], dv[1], dv[2]);
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        dv[d] = dv[d] / dl * len;
        sv[d] = sv[d] * len;
      }
      double as[8], ad[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        as[k] = (sv[0] * T[0][k] + sv[1] * T[1][k]) + sv[2] * T[2][k];
        ad[k] = (dv[0] * T[0][k] + dv[1] * T[1][k]) + dv[2] * T[2][k];
      }
      double b0 = 0.0, b1 = 0.0;
      normalise8(as, b0);
      normalise8(ad, b1);
      store_row(s, idc, as, b0, weight, d_idc, d_a, d_b, d_w, nan_flag);
      store_row(n + s, idc, ad, b1, weight, d_idc, d_a, d_b, d_w, nan_flag);
    } else {  // LS_ROWS_TANGENT / LS_ROWS_ORTHOGONAL, FD:478-539
      double T[3][8];
      element_gradient(l, g.step, T);
      double v[3] = {p[3], p[4], p[5]};
      double vn = norm3_seq(v[0], v[1], v[2]);
      if (vn > 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) v[d] = v[d] / vn;
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int k = 0; k < 8; ++k) T[d][k] = T[d][k] / vn;
      }
      double a[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = (v[0] * T[0][k] + v[1] * T[1][k]) + v[2] * T[2][k];
      double b = (KIND == LS_ROWS_ORTHOGONAL) ? p[6] : 0.0;  // FD:535 b_ = zeros + b
      normalise8(a, b);
      store_row(s, idc, a, b, weight, d_idc, d_a, d_b, d_w, nan_flag);
    }
  }
}

__global__ void pair_rows_kernel(GridArgs g, const double *__restrict__ pts, int64_t ld,
                                 const int64_t *__restrict__ pairs, int64_t npairs, double weight,
                                 int64_t *__restrict__ d_idc, double *__restrict__ d_a, double *__restrict__ d_b,
                                 double *__restrict__ d_w) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < npairs;
       r += (int64_t)gridDim.x * blockDim.x) {
    double a[16];
    int64_t idc[16];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const double *p = pts + pairs[2 * r + h] * ld;
      double pos[3] = {p[0], p[1], p[2]};
      double l[3];
      locate(g, pos, idc + 8 * h, l);
      trilinear(l, a + 8 * h);
    }
#pragma unroll
    for (int k = 8; k < 16; ++k) a[k] = -a[k];
    // numpy pairwise sum of 16 squares: r[j] = a[j]^2 + a[8+j]^2, then the 8-tree
    double q[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) q[k] = a[k] * a[k] + a[8 + k] * a[8 + k];
    double len = sqrt(0.0 + (((q[0] + q[1]) + (q[2] + q[3])) + ((q[4] + q[5]) + (q[6] + q[7]))));
    double b = 0.0;
    if (len > 0) {
      b = b / len;
#pragma unroll
      for (int k = 0; k < 16; ++k) a[k] = a[k] / len;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      d_idc[r * 16 + k] = idc[k];
      d_a[r * 16 + k] = a[k];
    }
    d_b[r] = b;
    d_w[r] = weight;
  }
}

// ---------------------------------------------------------------------------
// K2: explicit regularisation indices
// ---------------------------------------------------------------------------
struct RegShape {
  int64_t rows;
  int taps;
  bool valid;
};

RegShape reg_shape(const ls_grid3 &g, int fam) {
  const int64_t nx = g.nsteps[0], ny = g.nsteps[1], nz = g.nsteps[2];
  RegShape s{0, 0, true};
  if (fam >= LS_REG_DXY && fam <= LS_REG_DZZ) {
    s.taps = (fam <= LS_REG_DXZ) ? 4 : 3;
    if (nx >= 3 && ny >= 3 && nz >= 3) s.rows = (nx - 2) * (ny - 2) * (nz - 2);
  } else if (fam >= LS_REG_DX_LOWER && fam <= LS_REG_DZ_UPPER) {
    s.taps = 3;
    const int axis = (fam - LS_REG_DX_LOWER) / 2;
    const int64_t n[3] = {nx, ny, nz};
    if (n[axis] >= 3) s.rows = n[(axis + 1) % 3] * n[(axis + 2) % 3];
  } else {
    s.valid = false;
  }
  return s;
}

__global__ void reg_rows_kernel(int64_t nx, int64_t ny, int64_t nz, int fam, int64_t rows, int64_t *__restrict__ idc) {
  const int64_t nxy = nx * ny;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j, k;
    if (fam <= LS_REG_DZZ) {  // interior nodes in ascending gi (G:176-190)
      const int64_t mx = nx - 2, my = ny - 2;
      i = 1 + r % mx;
      j = 1 + (r / mx) % my;
      k = 1 + r / (mx * my);
    } else {  // FD:636-641 boundary layer nodes in ascending gi
      const int axis = (fam - LS_REG_DX_LOWER) / 2;
      const bool upper = ((fam - LS_REG_DX_LOWER) & 1) != 0;
      if (axis == 0) {
        i = upper ? nx - 2 : 1;
        j = r % ny;
        k = r / ny;
      } else if (axis == 1) {
        j = upper ? ny - 2 : 1;
        i = r % nx;
        k = r / nx;
      } else {
        k = upper ? nz - 2 : 1;
        i = r % nx;
        j = r / nx;
      }
    }
    const int64_t gi = i + nx * j + nxy * k;
    int64_t *o = idc + r * ((fam <= LS_REG_DXZ) ? 4 : 3);
    switch (fam) {
      case LS_REG_DXY:  // taps (dx,dy): (-1,-1) (+1,-1) (-1,+1) (+1,+1)
        o[0] = gi - 1 - nx; o[1] = gi + 1 - nx; o[2] = gi - 1 + nx; o[3] = gi + 1 + nx;
        break;
      case LS_REG_DYZ:  // (dz,dy): (-1,-1) (-1,+1) (+1,-1) (+1,+1)
        o[0] = gi - nxy - nx; o[1] = gi - nxy + nx; o[2] = gi + nxy - nx; o[3] = gi + nxy + nx;
        break;
      case LS_REG_DXZ:  // (dz,dx): (-1,-1) (-1,+1) (+1,-1) (+1,+1)
        o[0] = gi - nxy - 1; o[1] = gi - nxy + 1; o[2] = gi + nxy - 1; o[3] = gi + nxy + 1;
        break;
      case LS_REG_DXX: case LS_REG_DX_LOWER: case LS_REG_DX_UPPER:
        o[0] = gi - 1; o[1] = gi; o[2] = gi + 1;
        break;
      case LS_REG_DYY: case LS_REG_DY_LOWER: case LS_REG_DY_UPPER:
        o[0] = gi - nx; o[1] = gi; o[2] = gi + nx;
        break;
      default:
        o[0] = gi - nxy; o[1] = gi; o[2] = gi + nxy;
        break;
    }
  }
}

// Directional regularisation weights (FD:1207-1337): at every interior node m
// (1 <= i, j, k <= n - 2, the centres of the interior families) the row
// weights rw_f = w * c_f(v(m)), c = (vx^2, vy^2, vz^2, 2 vx vy, 2 vx vz,
// 2 vy vz) in the reference's evaluation order; rows with |rw| > 0 (not zero,
// not NaN) add s_f^2 rw^2 to omega[f][m] (s_f^2 = 1/6 for dxx/dyy/dzz, whose
// normalised taps are (1, -2, 1)/sqrt(6); 1/4 for the cross families, whose
// normalised taps are +-1/2) and count as a row of family f.
__global__ void dir_weights_kernel(int nx, int ny, int nz, const double *__restrict__ vec, int64_t ld, double w,
                                   double *__restrict__ omega, unsigned long long *__restrict__ counts) {
  const int64_t n = (int64_t)nx * ny * nz;
  unsigned long long cnt[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || k < 1 || k > nz - 2) continue;
    const double vx = vec[g * ld], vy = vec[g * ld + 1], vz = vec[g * ld + 2];
    const double c[6] = {vx * vx, vy * vy, vz * vz, 2.0 * vx * vy, 2.0 * vx * vz, 2.0 * vy * vz};
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const double rw = w * c[f];
      if (fabs(rw) > 0.0) {
        omega[f * n + g] += (f < 3 ? 1.0 / 6.0 : 0.25) * (rw * rw);
        ++cnt[f];
      }
    }
  }
  if (counts)
#pragma unroll
    for (int f = 0; f < 6; ++f)
      if (cnt[f]) atomicAdd(counts + f, cnt[f]);
}

// Node coordinate along one axis as numpy's linspace(o, max, n) makes it
// (S:233-245 nodes): x_i = i * ((max - o) / (n - 1)) + o, the last node
// exactly max = o + cells * h.  This translation unit is built without FMA
// contraction, so each step rounds as numpy's does.
struct LinAxis {
  double o, step, mx;
  int n;
};

__host__ LinAxis lin_axis(const ls_grid3 &g, int d) {
  LinAxis a;
  a.o = g.origin[d];
  a.n = (int)g.nsteps[d];
  a.mx = g.origin[d] + (double)(g.nsteps[d] - 1) * g.step[d];
  a.step = (a.mx - a.o) / (double)(a.n - 1);
  return a;
}

__device__ __forceinline__ double lin_at(const LinAxis &a, int i) {
  return i == a.n - 1 ? a.mx : (double)i * a.step + a.o;
}

// Regularisation weight scale (FD:66-90 compute_weighting over the normal
// constraints, FD:416-444 / P1:52-69): scale[m] += 1 + alpha exp(-d^2 /
// (2 sigma^2)), d the distance from node m to the nearest point.  Brute force
// over tiles of points in shared memory: an FP32 pass for the smallest
// distance, then the exact FP64 distance (squared differences summed x, y,
// z in turn, then the square root, as a KD-tree query reports it) of every
// point within a margin of it, so the nearest point is found exactly.
constexpr int kWsTile = 256;

__global__ void __launch_bounds__(kWsTile) weight_scale_kernel(LinAxis ax, LinAxis ay, LinAxis az,
                                                               const double *__restrict__ pts, int64_t npts,
                                                               int64_t ld, double alpha, double sigma, double extent,
                                                               double *__restrict__ scale) {
  __shared__ float sf[3][kWsTile];
  __shared__ double sd[3][kWsTile];
  const int nx = ax.n, ny = ay.n;
  const int64_t n = (int64_t)nx * ny * az.n;
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (g < n) {
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    px = lin_at(ax, i);
    py = lin_at(ay, j);
    pz = lin_at(az, k);
  }
  // FP32 coordinates relative to the grid origin
  const float fx = (float)(px - ax.o), fy = (float)(py - ay.o), fz = (float)(pz - az.o);
  float best32 = INFINITY;
  for (int64_t t0 = 0; t0 < npts; t0 += kWsTile) {
    __syncthreads();
    const int64_t q = t0 + threadIdx.x;
    if (q < npts) {
      sf[0][threadIdx.x] = (float)(pts[q * ld] - ax.o);
      sf[1][threadIdx.x] = (float)(pts[q * ld + 1] - ay.o);
      sf[2][threadIdx.x] = (float)(pts[q * ld + 2] - az.o);
    }
    __syncthreads();
    const int m = (int)(npts - t0 < kWsTile ? npts - t0 : kWsTile);
    for (int u = 0; u < m; ++u) {
      const float dx = fx - sf[0][u], dy = fy - sf[1][u], dz = fz - sf[2][u];
      best32 = fminf(best32, dx * dx + dy * dy + dz * dz);
    }
  }
  // candidates: FP32 distance within a margin of the smallest (rounding of
  // coordinates of magnitude `extent` to FP32 and of the FP32 sums)
  const double b = sqrt((double)best32);
  const double lim = b + 1e-5 * (extent + b) + 1e-30;
  const float lim2 = (float)(lim * lim);
  double best = INFINITY;
  for (int64_t t0 = 0; t0 < npts; t0 += kWsTile) {
    __syncthreads();
    const int64_t q = t0 + threadIdx.x;
    if (q < npts) {
      sd[0][threadIdx.x] = pts[q * ld];
      sd[1][threadIdx.x] = pts[q * ld + 1];
      sd[2][threadIdx.x] = pts[q * ld + 2];
      sf[0][threadIdx.x] = (float)(sd[0][threadIdx.x] - ax.o);
      sf[1][threadIdx.x] = (float)(sd[1][threadIdx.x] - ay.o);
      sf[2][threadIdx.x] = (float)(sd[2][threadIdx.x] - az.o);
    }
    __syncthreads();
    const int m = (int)(npts - t0 < kWsTile ? npts - t0 : kWsTile);
    for (int u = 0; u < m; ++u) {
      const float dx = fx - sf[0][u], dy = fy - sf[1][u], dz = fz - sf[2][u];
      if (dx * dx + dy * dy + dz * dz <= lim2) {
        const double ex = px - sd[0][u], ey = py - sd[1][u], ez = pz - sd[2][u];
        double d2 = ex * ex;
        d2 = d2 + ey * ey;
        d2 = d2 + ez * ez;
        best = fmin(best, d2);
      }
    }
  }
  if (g < n) {
    const double d = sqrt(best);
    scale[g] += 1.0 + alpha * exp(-(d * d) / (2.0 * (sigma * sigma)));
  }
}

// Interior regularisation families with a per-node scale (FD:668-672 with
// use_regularisation_weight_scale): the row centred at interior node m has
// weight scale_m w_f, i.e. omega[f][m] += s_f^2 (scale_m w_f)^2 in the
// directional-term weight planes (f = dxx, dyy, dzz, dxy, dxz, dyz; s_f^2 =
// 1/6, 1/4: the squared row normalisation).
__global__ void scaled_weights_kernel(int nx, int ny, int nz, const double *__restrict__ scale, double w0, double w1,
                                      double w2, double w3, double w4, double w5, double *__restrict__ omega) {
  const int64_t n = (int64_t)nx * ny * nz;
  const double w[6] = {w0, w1, w2, w3, w4, w5};
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || k < 1 || k > nz - 2) continue;
    const double sc = scale[g];
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const double rw = sc * w[f];
      omega[f * n + g] += (f < 3 ? 1.0 / 6.0 : 0.25) * (rw * rw);
    }
  }
}

int check_grid(const ls_grid3 *g) {
  LS_ARG_CHECK(g != nullptr, "grid is NULL");
  for (int d = 0; d < 3; ++d) {
    LS_ARG_CHECK(g->nsteps[d] >= 2, "every axis needs at least 2 nodes");
    LS_ARG_CHECK(g->step[d] > 0.0, "step must be positive");
  }
  return LS_OK;
}

}  // namespace
}  // namespace ls

using namespace ls;

extern "C" int ls_fd_point_rows(const ls_grid3 *grid, int kind, const double *d_pts, int64_t npts, int64_t ld,
                                double weight, int64_t *d_idc, double *d_a, double *d_b, double *d_w,
                                int64_t *h_count, int32_t *h_nan, void *stream) {
  LS_TRY(check_grid(grid));
  LS_ARG_CHECK(kind >= LS_ROWS_VALUE && kind <= LS_ROWS_ORTHOGONAL, "unknown row kind");
  LS_ARG_CHECK(npts >= 0, "npts < 0");
  const int64_t min_ld = (kind == LS_ROWS_VALUE) ? 5 : (kind == LS_ROWS_ORTHOGONAL ? 7 : 6);
  LS_ARG_CHECK(ld >= min_ld, "ld too small for the row kind");
  LS_ARG_CHECK(h_count != nullptr && h_nan != nullptr, "h_count / h_nan NULL");
  *h_count = 0;
  *h_nan = 0;
  if (npts == 0) return LS_OK;
  LS_ARG_CHECK(d_pts && d_idc && d_a && d_b && d_w, "NULL device buffer");
  cudaStream_t s = as_stream(stream);
  GridArgs g = make_grid_args(*grid);
  int32_t *flag = nullptr;
  int64_t *slot = nullptr;
  int64_t *cnt = nullptr;
  int32_t *nanf = nullptr;
  LS_CUDA_TRY(cudaMallocAsync((void **)&flag, npts * sizeof(int32_t), s));
  LS_CUDA_TRY(cudaMallocAsync((void **)&slot, npts * sizeof(int64_t), s));
  LS_CUDA_TRY(cudaMallocAsync((void **)&cnt, 2 * sizeof(int64_t), s));
  nanf = (int32_t *)(cnt + 1);
  LS_CUDA_TRY(cudaMemsetAsync(cnt, 0, 2 * sizeof(int64_t), s));
  const int blk = 256, grd = stream_grid(npts, blk);
  inside_flags_kernel<<<grd, blk, 0, s>>>(g, d_pts, npts, ld, flag);
  scan_flags_kernel<<<1, 1024, 0, s>>>(flag, npts, slot, cnt);
  switch (kind) {
    case LS_ROWS_VALUE:
      point_rows_kernel<LS_ROWS_VALUE><<<grd, blk, 0, s>>>(g, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w, nanf);
      break;
    case LS_ROWS_NORM:
      point_rows_kernel<LS_ROWS_NORM><<<grd, blk, 0, s>>>(g, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w, nanf);
      break;
    case LS_ROWS_GRADIENT:
      point_rows_kernel<LS_ROWS_GRADIENT><<<grd, blk, 0, s>>>(g, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w, nanf);
      break;
    case LS_ROWS_TANGENT:
      point_rows_kernel<LS_ROWS_TANGENT><<<grd, blk, 0, s>>>(g, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w, nanf);
      break;
    default:
      point_rows_kernel<LS_ROWS_ORTHOGONAL><<<grd, blk, 0, s>>>(g, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w, nanf);
      break;
  }
  LS_CUDA_TRY(cudaGetLastError());
  int64_t host[2] = {0, 0};
  LS_CUDA_TRY(cudaMemcpyAsync(host, cnt, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LS_CUDA_TRY(cudaFreeAsync(flag, s));
  LS_CUDA_TRY(cudaFreeAsync(slot, s));
  LS_CUDA_TRY(cudaFreeAsync(cnt, s));
  LS_CUDA_TRY(cudaStreamSynchronize(s));
  *h_count = host[0];
  *h_nan = ((int32_t *)&host[1])[0] != 0 ? 1 : 0;
  return LS_OK;
}

extern "C" int ls_fd_pair_rows(const ls_grid3 *grid, const double *d_pts, int64_t ld, const int64_t *d_pairs,
                               int64_t npairs, double weight, int64_t *d_idc, double *d_a, double *d_b, double *d_w,
                               void *stream) {
  LS_TRY(check_grid(grid));
  LS_ARG_CHECK(ld >= 3 && npairs >= 0, "bad ld / npairs");
  if (npairs == 0) return LS_OK;
  LS_ARG_CHECK(d_pts && d_pairs && d_idc && d_a && d_b && d_w, "NULL device buffer");
  GridArgs g = make_grid_args(*grid);
  cudaStream_t s = as_stream(stream);
  pair_rows_kernel<<<stream_grid(npairs, 128), 128, 0, s>>>(g, d_pts, ld, d_pairs, npairs, weight, d_idc, d_a, d_b, d_w);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_reg_shape(const ls_grid3 *grid, int family, int64_t *h_rows, int32_t *h_taps) {
  LS_TRY(check_grid(grid));
  RegShape sh = reg_shape(*grid, family);
  LS_ARG_CHECK(sh.valid, "unknown regularisation family");
  if (h_rows) *h_rows = sh.rows;
  if (h_taps) *h_taps = sh.taps;
  return LS_OK;
}

extern "C" int ls_fd_reg_rows(const ls_grid3 *grid, int family, int64_t *d_idc, void *stream) {
  LS_TRY(check_grid(grid));
  RegShape sh = reg_shape(*grid, family);
  LS_ARG_CHECK(sh.valid, "unknown regularisation family");
  if (sh.rows == 0) return LS_OK;
  LS_ARG_CHECK(d_idc != nullptr, "NULL device buffer");
  cudaStream_t s = as_stream(stream);
  reg_rows_kernel<<<stream_grid(sh.rows, 256), 256, 0, s>>>(grid->nsteps[0], grid->nsteps[1], grid->nsteps[2], family,
                                                          sh.rows, d_idc);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_weight_scale(const ls_grid3 *grid, const double *d_pts, int64_t npts, int64_t ld, double alpha,
                                  double sigma, double *d_scale, void *stream) {
  LS_TRY(check_grid(grid));
  LS_ARG_CHECK(ld >= 3, "ld < 3");
  LS_ARG_CHECK(npts >= 0, "npts < 0");
  LS_ARG_CHECK(d_scale != nullptr && (npts == 0 || d_pts != nullptr), "NULL device buffer");
  LS_ARG_CHECK(sigma > 0.0, "sigma must be positive");
  if (npts == 0) return LS_OK;
  const int64_t n = grid->nsteps[0] * grid->nsteps[1] * grid->nsteps[2];
  LS_ARG_CHECK(n < (int64_t)2000000000, "grid too large");
  const LinAxis ax = lin_axis(*grid, 0), ay = lin_axis(*grid, 1), az = lin_axis(*grid, 2);
  double extent = 1.0;
  for (int d = 0; d < 3; ++d)
    extent = fmax(extent, fabs(grid->origin[d]) + (double)(grid->nsteps[d] - 1) * grid->step[d]);
  cudaStream_t s = as_stream(stream);
  const int64_t blocks = (n + kWsTile - 1) / kWsTile;
  weight_scale_kernel<<<(unsigned)blocks, kWsTile, 0, s>>>(ax, ay, az, d_pts, npts, ld, alpha, sigma, extent, d_scale);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_scaled_weights(const ls_grid3 *grid, const double *d_scale, const double h_w[6], double *d_omega,
                                    void *stream) {
  LS_TRY(check_grid(grid));
  LS_ARG_CHECK(d_scale != nullptr && d_omega != nullptr && h_w != nullptr, "NULL argument");
  const int64_t n = grid->nsteps[0] * grid->nsteps[1] * grid->nsteps[2];
  LS_ARG_CHECK(n < (int64_t)2000000000, "grid too large");
  cudaStream_t s = as_stream(stream);
  scaled_weights_kernel<<<stream_grid(n, 256), 256, 0, s>>>((int)grid->nsteps[0], (int)grid->nsteps[1],
                                                            (int)grid->nsteps[2], d_scale, h_w[0], h_w[1], h_w[2],
                                                            h_w[3], h_w[4], h_w[5], d_omega);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_directional_weights(const ls_grid3 *grid, const double *d_vec, int64_t ld, double weight,
                                         double *d_omega, int64_t *h_counts, void *stream) {
  LS_TRY(check_grid(grid));
  LS_ARG_CHECK(ld >= 3, "ld < 3");
  LS_ARG_CHECK(d_vec != nullptr && d_omega != nullptr, "NULL device buffer");
  const int64_t n = grid->nsteps[0] * grid->nsteps[1] * grid->nsteps[2];
  LS_ARG_CHECK(n < (int64_t)2000000000, "grid too large");
  cudaStream_t s = as_stream(stream);
  unsigned long long *cnt = nullptr;
  LS_CUDA_TRY(cudaMallocAsync((void **)&cnt, 6 * sizeof(unsigned long long), s));
  LS_CUDA_TRY(cudaMemsetAsync(cnt, 0, 6 * sizeof(unsigned long long), s));
  dir_weights_kernel<<<stream_grid(n, 256), 256, 0, s>>>((int)grid->nsteps[0], (int)grid->nsteps[1],
                                                        (int)grid->nsteps[2], d_vec, ld, weight, d_omega, cnt);
  LS_CUDA_TRY(cudaGetLastError());
  unsigned long long host[6] = {0, 0, 0, 0, 0, 0};
  LS_CUDA_TRY(cudaMemcpyAsync(host, cnt, sizeof(host), cudaMemcpyDeviceToHost, s));
  LS_CUDA_TRY(cudaFreeAsync(cnt, s));
  LS_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_counts)
    for (int f = 0; f < 6; ++f) h_counts[f] = (int64_t)host[f];
  return LS_OK;
}
