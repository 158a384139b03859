// K7: value / gradient of the trilinear FD field at points or on a lattice.
// G:295-391 (StructuredGrid.evaluate_value / evaluate_gradient) with the
// interpolator-level conventions of DI:1342-1379.  Sums follow numpy's
// pairwise order for 8 terms, so results agree with the reference to ~1 ulp.
// Compiled with -fmad=false: the point kernel keeps numpy's evaluation order
// for value parity; the lattice kernel writes its FMAs explicitly.
#include <math.h>

#include <algorithm>

#include "ls_common.cuh"

namespace ls {
namespace {

struct EvalGrid {
  double origin[3], step[3], lo[3], hi[3];
  int64_t n[3], cells[3];
};

EvalGrid make_eval_grid(const ls_grid3 &g) {
  EvalGrid a;
  for (int d = 0; d < 3; ++d) {
    a.origin[d] = g.origin[d];
    a.step[d] = g.step[d];
    a.n[d] = g.nsteps[d];
    a.cells[d] = g.nsteps[d] - 1;
    double mx = g.origin[d] + (double)a.cells[d] * g.step[d];
    double ext = fabs(mx - g.origin[d]);
    if (ext < 1.0) ext = 1.0;
    double tol = 2.220446049250313e-16 * 32.0 * ext;
    a.lo[d] = g.origin[d] - tol;
    a.hi[d] = mx + tol;
  }
  return a;
}

__device__ __forceinline__ double sum8(const double v[8]) {
  return 0.0 + (((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7])));
}

__device__ __forceinline__ void eval_one(const EvalGrid &g, const double *__restrict__ c, double px, double py,
                                         double pz, double *value, double *grad) {
  const bool nanrow = isnan(px) | isnan(py) | isnan(pz);
  const bool inside = (px >= g.lo[0]) & (px <= g.hi[0]) & (py >= g.lo[1]) & (py <= g.hi[1]) & (pz >= g.lo[2]) &
                      (pz <= g.hi[2]);
  if (!inside) {
    if (value) *value = nanrow ? 0.0 : __longlong_as_double(0x7ff8000000000000LL);
    if (grad) grad[0] = grad[1] = grad[2] = 0.0;
    return;
  }
  const double p[3] = {px, py, pz};
  int64_t ci[3];
  double l[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double x = p[d] - g.origin[d];
    int64_t k = (int64_t)floor(x / g.step[d]);
    if (k < 0) k = 0;
    if (k > g.cells[d] - 1) k = g.cells[d] - 1;
    ci[d] = k;
    double co = g.origin[d] + g.step[d] * (double)k;
    l[d] = fmin(fmax((p[d] - co) / g.step[d], 0.0), 1.0);
  }
  const int64_t nx = g.n[0], nxy = g.n[0] * g.n[1];
  const int64_t g0 = ci[0] + nx * ci[1] + nxy * ci[2];
  double cv[8];
  cv[0] = c[g0];
  cv[1] = c[g0 + 1];
  cv[2] = c[g0 + nx];
  cv[3] = c[g0 + nx + 1];
  cv[4] = c[g0 + nxy];
  cv[5] = c[g0 + nxy + 1];
  cv[6] = c[g0 + nxy + nx];
  cv[7] = c[g0 + nxy + nx + 1];
  const double x = l[0], y = l[1], z = l[2];
  if (value) {
    double a[8];
    a[0] = (1 - x) * (1 - y) * (1 - z);
    a[1] = x * (1 - y) * (1 - z);
    a[2] = (1 - x) * y * (1 - z);
    a[4] = (1 - x) * (1 - y) * z;
    a[5] = x * (1 - y) * z;
    a[6] = (1 - x) * y * z;
    a[3] = x * y * (1 - z);
    a[7] = x * y * z;
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = a[k] * cv[k];
    *value = sum8(a);
  }
  if (grad) {
    double T[8];
    T[0] = (1 - z) * (y - 1);
    T[1] = (1 - y) * (1 - z);
    T[2] = -y * (1 - z);
    T[4] = -(1 - y) * z;
    T[5] = (1 - y) * z;
    T[6] = -y * z;
    T[3] = y * (1 - z);
    T[7] = y * z;
#pragma unroll
    for (int k = 0; k < 8; ++k) T[k] = T[k] * cv[k];
    grad[0] = sum8(T) / g.step[0];
    T[0] = (x - 1) * (1 - z);
    T[1] = -x * (1 - z);
    T[2] = (1 - x) * (1 - z);
    T[4] = -(1 - x) * z;
    T[5] = -x * z;
    T[6] = (1 - x) * z;
    T[3] = x * (1 - z);
    T[7] = x * z;
#pragma unroll
    for (int k = 0; k < 8; ++k) T[k] = T[k] * cv[k];
    grad[1] = sum8(T) / g.step[1];
    T[0] = -(1 - x) * (1 - y);
    T[1] = -x * (1 - y);
    T[2] = -(1 - x) * y;
    T[4] = (1 - x) * (1 - y);
    T[5] = x * (1 - y);
    T[6] = (1 - x) * y;
    T[3] = -x * y;
    T[7] = x * y;
#pragma unroll
    for (int k = 0; k < 8; ++k) T[k] = T[k] * cv[k];
    grad[2] = sum8(T) / g.step[2];
  }
}

__global__ void eval_points_kernel(EvalGrid g, const double *__restrict__ c, const double *__restrict__ pts,
                                   int64_t n, int64_t ld, double *__restrict__ value, double *__restrict__ grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *p = pts + i * ld;
    double v, gr[3];
    eval_one(g, c, p[0], p[1], p[2], value ? &v : nullptr, grad ? gr : nullptr);
    if (value) value[i] = v;
    if (grad) {
      grad[3 * i] = gr[0];
      grad[3 * i + 1] = gr[1];
      grad[3 * i + 2] = gr[2];
    }
  }
}

// per-axis part of the point location: inside flag, cell index, local coordinate
struct AxisLoc {
  double l;
  int64_t cell;
  bool inside;
};

__device__ __forceinline__ AxisLoc locate_axis(const EvalGrid &g, int d, double p) {
  AxisLoc a;
  a.inside = (p >= g.lo[d]) & (p <= g.hi[d]);
  int64_t k = (int64_t)floor((p - g.origin[d]) / g.step[d]);
  if (k < 0) k = 0;
  if (k > g.cells[d] - 1) k = g.cells[d] - 1;
  a.cell = k;
  const double co = g.origin[d] + g.step[d] * (double)k;
  a.l = fmin(fmax((p - co) / g.step[d], 0.0), 1.0);
  return a;
}

// ---------------------------------------------------------------------------
// Lattice evaluation.  GB300 runs FP64 arithmetic at a small fraction of its
// FP32 rate, so this kernel is built to spend as few FP64 operations per
// lattice point as possible (the point kernel above keeps the reference's
// operation order for parity; here sums are regrouped, agreeing to a few ulp):
//  * the trilinear weight factorises as w_x(a) * w_yz(b, k): the x location of
//    every lattice x index is computed once per block (each thread keeps its
//    own), the y / z part once per lattice row (RowCoef, one lane per row);
//  * row collapse: along one lattice row the y / z interpolation is done once
//    per grid node, E(i) = sum w_yz c(i, ., .), and likewise its y / z
//    derivatives, into shared memory; each lattice point is then a lerp of two
//    neighbouring entries (value, d/dy, d/dz: 2 FP64 ops each; d/dx: 1).
//    This needs the chunk's node span to fit the buffer, i.e. a lattice at
//    least about as dense as the grid in x; otherwise (sparse lattices) each
//    point gathers its 8 coefficients and reuses the row weights (~24 ops).
// Block: 256 threads = one chunk of 256 consecutive lattice x indices; the
// block walks a strided set of lattice rows (b, k) for that chunk.
constexpr int kLatThreads = 256;
constexpr int kLatRowBatch = 32;
constexpr int kLatMaxSpan = 2 * kLatThreads + 2;

struct RowCoef {
  double w[4];    // value weights of the 4 x-lines (by + 2 bz): wy(by) * wz(bz)
  double gy[2];   // d/dy weights of the z = cz / cz + 1 line pairs: (1 - lz) / hy, lz / hy
  double gz[2];   // d/dz weights of the y = cy / cy + 1 line pairs: (1 - ly) / hz, ly / hz
  int64_t base;   // node index of (0, cy, cz)
  int inside;
};

__device__ RowCoef row_coef(const EvalGrid &g, double py, double pz) {
  const AxisLoc ly = locate_axis(g, 1, py), lz = locate_axis(g, 2, pz);
  RowCoef r;
  const double y = ly.l, z = lz.l;
  r.w[0] = (1 - y) * (1 - z);
  r.w[1] = y * (1 - z);
  r.w[2] = (1 - y) * z;
  r.w[3] = y * z;
  r.gy[0] = (1 - z) / g.step[1];
  r.gy[1] = z / g.step[1];
  r.gz[0] = (1 - y) / g.step[2];
  r.gz[1] = y / g.step[2];
  r.base = g.n[0] * (ly.cell + g.n[1] * lz.cell);
  r.inside = ly.inside & lz.inside;
  return r;
}

__global__ void __launch_bounds__(kLatThreads) eval_lattice_kernel(EvalGrid g, const double *__restrict__ c,
                                                                   double ox, double oy, double oz, double hx,
                                                                   double hy, double hz, int64_t n0, int64_t n1,
                                                                   int64_t n2, double *__restrict__ value,
                                                                   double *__restrict__ grad) {
  __shared__ RowCoef rc[kLatRowBatch];
  __shared__ double buf[2][3][kLatMaxSpan];  // E, dE/dy, dE/dz per node, double-buffered over rows
  __shared__ int span_lo, span_hi;
  const int tid = threadIdx.x;
  const int64_t a = blockIdx.y * (int64_t)kLatThreads + tid;
  const bool active = a < n0;
  // x location of this thread's lattice index, once for every row
  AxisLoc lx = {0.0, 0, false};
  if (active) lx = locate_axis(g, 0, ox + hx * (double)a);
  if (tid == 0) {
    span_lo = 0x7fffffff;
    span_hi = -1;
  }
  __syncthreads();
  if (active) {
    atomicMin(&span_lo, (int)lx.cell);
    atomicMax(&span_hi, (int)lx.cell + 1);
  }
  __syncthreads();
  const int lo = span_lo, span = span_hi - span_lo + 1;
  const bool collapse = span <= kLatMaxSpan;
  const double inv_hx = 1.0 / g.step[0];
  const int64_t nx = g.n[0], nxy = g.n[0] * g.n[1];
  const int64_t rows = n1 * n2;
  int parity = 0;
  for (int64_t t0 = blockIdx.x; t0 < rows; t0 += (int64_t)gridDim.x * kLatRowBatch) {
    __syncthreads();  // the previous batch's coefficients are no longer read
    if (tid < kLatRowBatch) {
      const int64_t r = t0 + (int64_t)tid * gridDim.x;
      if (r < rows) rc[tid] = row_coef(g, oy + hy * (double)(r % n1), oz + hz * (double)(r / n1));
    }
    __syncthreads();
    for (int q = 0; q < kLatRowBatch; ++q) {
      const int64_t r = t0 + (int64_t)q * gridDim.x;
      if (r >= rows) break;  // uniform across the block
      const RowCoef &R = rc[q];
      const int64_t out = a + n0 * r;
      if (collapse) {
        if (R.inside) {
          for (int m = tid; m < span; m += kLatThreads) {
            const double *p = c + R.base + lo + m;
            const double c00 = __ldg(p), c10 = __ldg(p + nx), c01 = __ldg(p + nxy), c11 = __ldg(p + nxy + nx);
            buf[parity][0][m] = fma(R.w[3], c11, fma(R.w[2], c01, fma(R.w[1], c10, R.w[0] * c00)));
            buf[parity][1][m] = fma(R.gy[1], c11 - c01, R.gy[0] * (c10 - c00));
            buf[parity][2][m] = fma(R.gz[1], c11 - c10, R.gz[0] * (c01 - c00));
          }
        }
        __syncthreads();
        if (!active) {
          parity ^= 1;
          continue;
        }
        if (!(R.inside & lx.inside)) {
          if (value) value[out] = __longlong_as_double(0x7ff8000000000000LL);
          if (grad) grad[3 * out] = grad[3 * out + 1] = grad[3 * out + 2] = 0.0;
          parity ^= 1;
          continue;
        }
        const int m = (int)lx.cell - lo;
        const double e0 = buf[parity][0][m], de = buf[parity][0][m + 1] - e0;
        if (value) value[out] = fma(lx.l, de, e0);
        if (grad) {
          const double y0 = buf[parity][1][m], z0 = buf[parity][2][m];
          grad[3 * out] = de * inv_hx;
          grad[3 * out + 1] = fma(lx.l, buf[parity][1][m + 1] - y0, y0);
          grad[3 * out + 2] = fma(lx.l, buf[parity][2][m + 1] - z0, z0);
        }
        parity ^= 1;
      } else {
        if (!active) continue;
        if (!(R.inside & lx.inside)) {
          if (value) value[out] = __longlong_as_double(0x7ff8000000000000LL);
          if (grad) grad[3 * out] = grad[3 * out + 1] = grad[3 * out + 2] = 0.0;
          continue;
        }
        const double *p = c + R.base + lx.cell;
        double e[4], d[4];
        const int64_t off[4] = {0, nx, nxy, nxy + nx};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const double c0 = __ldg(p + off[j]);
          d[j] = __ldg(p + off[j] + 1) - c0;
          e[j] = fma(lx.l, d[j], c0);
        }
        if (value) value[out] = fma(R.w[3], e[3], fma(R.w[2], e[2], fma(R.w[1], e[1], R.w[0] * e[0])));
        if (grad) {
          grad[3 * out] = fma(R.w[3], d[3], fma(R.w[2], d[2], fma(R.w[1], d[1], R.w[0] * d[0]))) * inv_hx;
          grad[3 * out + 1] = fma(R.gy[1], e[3] - e[2], R.gy[0] * (e[1] - e[0]));
          grad[3 * out + 2] = fma(R.gz[1], e[3] - e[1], R.gz[0] * (e[2] - e[0]));
        }
      }
    }
  }
}

// Transpose of the point evaluation: out[node] += sum over the points of the
// trilinear weight of the node times gv[i] (+ the shape-function gradient
// times gg[i], 3 per point).  Points outside the support contribute nothing.
// FP64 atomics: the summation order varies run to run at the ulp level.
__global__ void eval_adjoint_kernel(EvalGrid g, const double *__restrict__ pts, int64_t n, int64_t ld,
                                    const double *__restrict__ gv, const double *__restrict__ gg,
                                    double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *p = pts + i * ld;
    AxisLoc l[3];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      l[d] = locate_axis(g, d, p[d]);
      inside &= l[d].inside;
    }
    if (!inside) continue;
    const double x = l[0].l, y = l[1].l, z = l[2].l;
    const double v = gv ? gv[i] : 0.0;
    const double gx = gg ? gg[3 * i] / g.step[0] : 0.0, gy = gg ? gg[3 * i + 1] / g.step[1] : 0.0,
                 gz = gg ? gg[3 * i + 2] / g.step[2] : 0.0;
    const int64_t nx = g.n[0], nxy = g.n[0] * g.n[1];
    const int64_t g0 = l[0].cell + nx * l[1].cell + nxy * l[2].cell;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
      const double wx = bx ? x : 1 - x, wy = by ? y : 1 - y, wz = bz ? z : 1 - z;
      const double dx = bx ? 1.0 : -1.0, dy = by ? 1.0 : -1.0, dz = bz ? 1.0 : -1.0;
      const double c = v * wx * wy * wz + gx * dx * wy * wz + gy * wx * dy * wz + gz * wx * wy * dz;
      atomicAdd(out + g0 + bx + nx * by + nxy * bz, c);
    }
  }
}

// Field jets at points: out[11 i ..] = (u, du/dx, du/dy, du/dz, d2u/dxdy,
// d2u/dxdz, d2u/dydz, lx, ly, lz, inside) of the trilinear interpolant of c
// (second derivatives along one axis vanish); local coordinates in [0, 1];
// all 0 outside the support.  The inputs of the adjoint with respect to point
// positions and normal vectors.
__global__ void eval_jets_kernel(EvalGrid g, const double *__restrict__ c, const double *__restrict__ pts, int64_t n,
                                 int64_t ld, double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *p = pts + i * ld;
    AxisLoc l[3];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      l[d] = locate_axis(g, d, p[d]);
      inside &= l[d].inside;
    }
    double *o = out + 11 * i;
    if (!inside) {
#pragma unroll
      for (int k = 0; k < 11; ++k) o[k] = 0.0;
      continue;
    }
    const int64_t nx = g.n[0], nxy = g.n[0] * g.n[1];
    const int64_t g0 = l[0].cell + nx * l[1].cell + nxy * l[2].cell;
    double u = 0, ux = 0, uy = 0, uz = 0, uxy = 0, uxz = 0, uyz = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int bx = k & 1, by = (k >> 1) & 1, bz = (k >> 2) & 1;
      const double cv = c[g0 + bx + nx * by + nxy * bz];
      const double wx = bx ? l[0].l : 1 - l[0].l, wy = by ? l[1].l : 1 - l[1].l, wz = bz ? l[2].l : 1 - l[2].l;
      const double dx = (bx ? 1.0 : -1.0) / g.step[0], dy = (by ? 1.0 : -1.0) / g.step[1],
                   dz = (bz ? 1.0 : -1.0) / g.step[2];
      u += wx * wy * wz * cv;
      ux += dx * wy * wz * cv;
      uy += wx * dy * wz * cv;
      uz += wx * wy * dz * cv;
      uxy += dx * dy * wz * cv;
      uxz += dx * wy * dz * cv;
      uyz += wx * dy * dz * cv;
    }
    o[0] = u;
    o[1] = ux;
    o[2] = uy;
    o[3] = uz;
    o[4] = uxy;
    o[5] = uxz;
    o[6] = uyz;
    o[7] = l[0].l;
    o[8] = l[1].l;
    o[9] = l[2].l;
    o[10] = 1.0;
  }
}

// ---------------------------------------------------------------------------
// Fault displacement (the caller of K7 for faulted features).
struct FaultDev {
  EvalGrid grid[3];
  const double *c[3];
  double to_local[3][3][4];
  double to_world[3][3][3];
  double displacement, scale;
  int steps, has_function;
  ls_fault_profile prof[3];
};

__device__ __forceinline__ double cubic_at(const double *w, double v) {
  return w[0] * pow(v, 3.0) + w[1] * pow(v, 2.0) + w[2] * v + w[3];
}

// one cubic with its limits and clamp (FF:123-140)
__device__ double cubic_profile(const ls_fault_profile &p, int k, double v) {
  double e = cubic_at(p.w[k], v);
  if (v > p.lim[k][1]) e = cubic_at(p.w[k], p.lim[k][1]);
  if (v < p.lim[k][0]) e = cubic_at(p.w[k], p.lim[k][0]);
  if (e > p.clamp[k][1]) e = p.clamp[k][1];
  if (e < p.clamp[k][0]) e = p.clamp[k][0];
  return e;
}

__device__ double profile_at(const ls_fault_profile &p, double v) {
  switch (p.kind) {
    case LS_PROFILE_ZEROS: return 0.0;
    case LS_PROFILE_SMOOTH_PEAK: return (v >= -1.0 && v <= 1.0) ? pow(v, 4.0) - 2.0 * pow(v, 2.0) + 1.0 : 0.0;
    case LS_PROFILE_CUBIC: return cubic_profile(p, 0, v);
    case LS_PROFILE_COMPOSITE: return v > 0.0 ? cubic_profile(p, 0, v) : (v < 0.0 ? cubic_profile(p, 1, v) : 0.0);
    default: return 1.0;
  }
}

// frame coordinate k at world point w (NaN outside its support); with grad,
// also its world-frame gradient (0 outside)
__device__ double frame_value(const FaultDev &f, int k, const double w[3], double *grad) {
  double l[3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    l[a] = f.to_local[k][a][0] * w[0] + f.to_local[k][a][1] * w[1] + f.to_local[k][a][2] * w[2] +
           f.to_local[k][a][3];
  double v, gl[3];
  eval_one(f.grid[k], f.c[k], l[0], l[1], l[2], &v, grad ? gl : nullptr);
  if (grad) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
      grad[a] = f.to_world[k][a][0] * gl[0] + f.to_world[k][a][1] * gl[1] + f.to_world[k][a][2] * gl[2];
  }
  return v;
}

// displacement of FS:352-362 / FS:399-410 for frame coordinates (gx, gy, gz)
__device__ double fault_d(const FaultDev &f, double gx, double gy, double gz) {
  const bool ok = !isnan(gx) && !isnan(gy) && !isnan(gz);
  if (!ok) return 0.0;
  if (f.has_function)
    return f.scale * profile_at(f.prof[0], gx) * profile_at(f.prof[1], gy) * profile_at(f.prof[2], gz);
  return gx > 0.0 ? 1.0 : 0.0;
}

__global__ void fault_apply_kernel(FaultDev f, double *__restrict__ pts, int64_t n, int64_t ld) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double *p = pts + i * ld;
    double w[3] = {p[0], p[1], p[2]};
    double gx = frame_value(f, 0, w, nullptr), gy = frame_value(f, 1, w, nullptr), gz = frame_value(f, 2, w, nullptr);
    if (!(fabs(fault_d(f, gx, gy, gz)) > 0.0)) continue;  // unaffected by this fault
    const double inv_steps = 1.0 / (double)f.steps;
    for (int s = 0; s < f.steps; ++s) {
      double g[3];
      if (s > 0) {
        gx = frame_value(f, 0, w, nullptr);
        gz = frame_value(f, 2, w, nullptr);
      }
      gy = frame_value(f, 1, w, g);
      const double d = fault_d(f, gx, gy, gz) * f.displacement;
      const bool ok = !isnan(gx) && !isnan(gy) && !isnan(gz);
      const double mag = ok ? sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) : 0.0;
      const double scale = inv_steps * d;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const double ga = mag > 0.0 ? g[a] / mag : g[a];
        w[a] += ga * scale;
      }
    }
    p[0] = w[0];
    p[1] = w[1];
    p[2] = w[2];
  }
}

// gradient of the linear interpolant over one tetrahedron: M g = df with
// M rows v_k - v_0, df_k = f_k - f_0 (k = 1..3), by cofactors
__global__ void tetra_gradient_kernel(const double *__restrict__ tet, const double *__restrict__ val, int64_t n,
                                      double *__restrict__ grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *t = tet + 12 * i;
    const double *f = val + 4 * i;
    double m[3][3], r[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int a = 0; a < 3; ++a) m[k][a] = t[3 * (k + 1) + a] - t[a];
      r[k] = f[k + 1] - f[0];
    }
    // cofactor matrix C, det = row 0 . C row 0; inverse = C^T / det
    const double c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1], c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2],
                 c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    const double c10 = m[0][2] * m[2][1] - m[0][1] * m[2][2], c11 = m[0][0] * m[2][2] - m[0][2] * m[2][0],
                 c12 = m[0][1] * m[2][0] - m[0][0] * m[2][1];
    const double c20 = m[0][1] * m[1][2] - m[0][2] * m[1][1], c21 = m[0][2] * m[1][0] - m[0][0] * m[1][2],
                 c22 = m[0][0] * m[1][1] - m[0][1] * m[1][0];
    const double det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
    const double inv = det != 0.0 ? 1.0 / det : __longlong_as_double(0x7ff8000000000000LL);
    double *o = grad + 3 * i;
    o[0] = (c00 * r[0] + c10 * r[1] + c20 * r[2]) * inv;
    o[1] = (c01 * r[0] + c11 * r[1] + c21 * r[2]) * inv;
    o[2] = (c02 * r[0] + c12 * r[1] + c22 * r[2]) * inv;
  }
}

}  // namespace
}  // namespace ls

using namespace ls;

extern "C" int ls_fault_apply(const ls_fault *fault, double *d_pts, int64_t npts, int64_t ld, void *stream) {
  LS_ARG_CHECK(fault != nullptr, "NULL fault");
  LS_ARG_CHECK(npts >= 0 && ld >= 3, "bad npts / ld");
  LS_ARG_CHECK(fault->steps >= 1, "steps must be >= 1");
  if (npts == 0) return LS_OK;
  LS_ARG_CHECK(d_pts != nullptr, "NULL points");
  FaultDev f;
  for (int k = 0; k < 3; ++k) {
    const ls_fault_field &fr = fault->frame[k];
    LS_ARG_CHECK(fr.d_c != nullptr, "NULL frame field");
    for (int d = 0; d < 3; ++d) LS_ARG_CHECK(fr.grid.nsteps[d] >= 2 && fr.grid.step[d] > 0.0, "bad frame grid");
    f.grid[k] = make_eval_grid(fr.grid);
    f.c[k] = fr.d_c;
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 4; ++b) f.to_local[k][a][b] = fr.to_local[a][b];
      for (int b = 0; b < 3; ++b) f.to_world[k][a][b] = fr.to_world[a][b];
    }
    f.prof[k] = fault->profile[k];
    LS_ARG_CHECK(f.prof[k].kind >= LS_PROFILE_ONES && f.prof[k].kind <= LS_PROFILE_COMPOSITE, "unknown profile kind");
  }
  f.displacement = fault->displacement;
  f.scale = fault->scale;
  f.steps = fault->steps;
  f.has_function = fault->has_function;
  cudaStream_t s = as_stream(stream);
  fault_apply_kernel<<<stream_grid(npts, 128), 128, 0, s>>>(f, d_pts, npts, ld);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_tetra_gradient(const double *d_tetra, const double *d_values, int64_t n, double *d_grad,
                                 void *stream) {
  LS_ARG_CHECK(n >= 0, "n < 0");
  if (n == 0) return LS_OK;
  LS_ARG_CHECK(d_tetra && d_values && d_grad, "NULL argument");
  tetra_gradient_kernel<<<stream_grid(n, 256), 256, 0, as_stream(stream)>>>(d_tetra, d_values, n, d_grad);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_eval_jets(const ls_grid3 *grid, const double *d_c, const double *d_pts, int64_t npts, int64_t ld,
                               double *d_out, void *stream) {
  LS_ARG_CHECK(grid && d_c && d_out, "NULL argument");
  LS_ARG_CHECK(npts >= 0 && ld >= 3, "bad npts / ld");
  if (npts == 0) return LS_OK;
  LS_ARG_CHECK(d_pts != nullptr, "NULL points");
  EvalGrid g = make_eval_grid(*grid);
  cudaStream_t s = as_stream(stream);
  eval_jets_kernel<<<stream_grid(npts, 256), 256, 0, s>>>(g, d_c, d_pts, npts, ld, d_out);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_eval_adjoint(const ls_grid3 *grid, const double *d_pts, int64_t npts, int64_t ld,
                                  const double *d_gvalue, const double *d_ggrad, double *d_out, void *stream) {
  LS_ARG_CHECK(grid && d_out, "NULL argument");
  LS_ARG_CHECK(npts >= 0 && ld >= 3, "bad npts / ld");
  if (npts == 0 || (!d_gvalue && !d_ggrad)) return LS_OK;
  LS_ARG_CHECK(d_pts != nullptr, "NULL points");
  EvalGrid g = make_eval_grid(*grid);
  cudaStream_t s = as_stream(stream);
  eval_adjoint_kernel<<<stream_grid(npts, 256), 256, 0, s>>>(g, d_pts, npts, ld, d_gvalue, d_ggrad, d_out);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_eval_points(const ls_grid3 *grid, const double *d_c, const double *d_pts, int64_t npts, int64_t ld,
                                 double *d_value, double *d_grad, void *stream) {
  LS_ARG_CHECK(grid && d_c, "NULL argument");
  LS_ARG_CHECK(npts >= 0 && ld >= 3, "bad npts / ld");
  if (npts == 0 || (!d_value && !d_grad)) return LS_OK;
  LS_ARG_CHECK(d_pts != nullptr, "NULL points");
  EvalGrid g = make_eval_grid(*grid);
  cudaStream_t s = as_stream(stream);
  eval_points_kernel<<<stream_grid(npts, 256), 256, 0, s>>>(g, d_c, d_pts, npts, ld, d_value, d_grad);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_fd_eval_lattice(const ls_grid3 *grid, const double *d_c, const double lat_origin[3],
                                  const double lat_step[3], const int64_t lat_n[3], double *d_value, double *d_grad,
                                  void *stream) {
  LS_ARG_CHECK(grid && d_c && lat_origin && lat_step && lat_n, "NULL argument");
  LS_ARG_CHECK(lat_n[0] >= 0 && lat_n[1] >= 0 && lat_n[2] >= 0, "negative lattice size");
  const int64_t total = lat_n[0] * lat_n[1] * lat_n[2];
  if (total == 0 || (!d_value && !d_grad)) return LS_OK;
  EvalGrid g = make_eval_grid(*grid);
  cudaStream_t s = as_stream(stream);
  const int64_t chunks = (lat_n[0] + kLatThreads - 1) / kLatThreads;
  LS_ARG_CHECK(chunks <= 65535, "lattice x extent above 16.7 M");
  LS_ARG_CHECK(g.n[0] < (int64_t)0x7fffffff, "grid x extent too large");
  // enough blocks to fill every SM several times over; each walks a strided
  // set of lattice rows of its x chunk
  const int64_t rows = lat_n[1] * lat_n[2];
  const int64_t want = (int64_t)sm_count() * 8;
  const int64_t per_chunk = std::max<int64_t>(1, std::min<int64_t>(rows, (want + chunks - 1) / chunks));
  const dim3 lgrid((unsigned)per_chunk, (unsigned)chunks, 1);
  eval_lattice_kernel<<<lgrid, kLatThreads, 0, s>>>(g, d_c, lat_origin[0], lat_origin[1], lat_origin[2], lat_step[0],
                                                    lat_step[1], lat_step[2], lat_n[0], lat_n[1], lat_n[2], d_value,
                                                    d_grad);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}
