// The FD regularisation part of the normal operator, sum_f w_f^2 R_f^T R_f,
// evaluated per node from its coordinates.
//
// Families and their normalised taps (OP:10-43 masks, row-normalised by
// DI:361-366):
//   dxx / dyy / dzz : (1, -2, 1) / sqrt(6) along one axis, rows at the
//                     interior nodes (all axes in [1, n-2], G:176-190)
//   dx/dy/dz_lower/upper (FD:1052-1144): the same taps, rows at EVERY node
//                     whose index along that axis is 1 (lower) or n-2 (upper)
//   dxy / dxz / dyz : +-1/2 at the four diagonal neighbours in a plane, sign
//                     -1 where both offsets agree, rows at the interior nodes.
// Rows of the same taps at the same centre add in the normal equations, so a
// node carries one combined weight alpha_g per stencil shape g:
//   alpha_xx(c) = [interior] w_dxx^2 + ([i == 1] + [i == nx-2]) w_dx^2
// and  N_reg p (c) = sum_g sum_o m_g(o) alpha_g(c - o) (m_g . p)(c - o).
#pragma once

#include <stdint.h>

#include "../../include/ls_gb300.h"

namespace ls {

struct StencilCoef {
  int64_t nx, ny, nz;
  // alpha / 6 for the (1,-2,1) shapes (taps carry 1/sqrt(6) each)
  double xx_int, yy_int, zz_int;
  double xx_bdr, yy_bdr, zz_bdr;  // 0 when the border family is disabled or the axis has < 3 nodes
  // alpha / 4 for the diagonal shapes (taps carry 1/2 each)
  double xy, xz, yz;
  double ridge2;
};

inline StencilCoef make_stencil_coef(const ls_grid3 &g, double w_dxx, double w_dyy, double w_dzz, double w_dxy,
                                     double w_dyz, double w_dxz, double w_dx, double w_dy, double w_dz, double ridge) {
  StencilCoef c;
  c.nx = g.nsteps[0];
  c.ny = g.nsteps[1];
  c.nz = g.nsteps[2];
  c.xx_int = w_dxx * w_dxx / 6.0;
  c.yy_int = w_dyy * w_dyy / 6.0;
  c.zz_int = w_dzz * w_dzz / 6.0;
  c.xx_bdr = (c.nx >= 3) ? w_dx * w_dx / 6.0 : 0.0;
  c.yy_bdr = (c.ny >= 3) ? w_dy * w_dy / 6.0 : 0.0;
  c.zz_bdr = (c.nz >= 3) ? w_dz * w_dz / 6.0 : 0.0;
  c.xy = w_dxy * w_dxy * 0.25;
  c.xz = w_dxz * w_dxz * 0.25;
  c.yz = w_dyz * w_dyz * 0.25;
  c.ridge2 = ridge * ridge;
  return c;
}

__host__ __device__ __forceinline__ bool is_interior(const StencilCoef &c, int64_t i, int64_t j, int64_t k) {
  return i >= 1 && i <= c.nx - 2 && j >= 1 && j <= c.ny - 2 && k >= 1 && k <= c.nz - 2;
}

__host__ __device__ __forceinline__ bool in_grid(const StencilCoef &c, int64_t i, int64_t j, int64_t k) {
  return i >= 0 && i < c.nx && j >= 0 && j < c.ny && k >= 0 && k < c.nz;
}

// combined weight of the (1,-2,1) rows along `axis` centred at (i,j,k)
__host__ __device__ __forceinline__ double alpha_axis(const StencilCoef &c, int axis, int64_t i, int64_t j, int64_t k) {
  if (!in_grid(c, i, j, k)) return 0.0;
  double a = 0.0;
  const bool inter = is_interior(c, i, j, k);
  if (axis == 0) {
    if (inter) a += c.xx_int;
    a += c.xx_bdr * (double)((i == 1) + (i == c.nx - 2));
  } else if (axis == 1) {
    if (inter) a += c.yy_int;
    a += c.yy_bdr * (double)((j == 1) + (j == c.ny - 2));
  } else {
    if (inter) a += c.zz_int;
    a += c.zz_bdr * (double)((k == 1) + (k == c.nz - 2));
  }
  return a;
}

template <typename T>
__device__ __forceinline__ T stencil_apply_node(const StencilCoef &c, const T *__restrict__ p, int64_t g, int64_t i,
                                                int64_t j, int64_t k) {
  const int64_t sx = 1, sy = c.nx, sz = c.nx * c.ny;
  T acc = (T)c.ridge2 * p[g];
  // (1,-2,1) shapes: row at c' = c - o e_axis, o in {-1,0,1}; tap weight kappa(o)
  const int64_t strides[3] = {sx, sy, sz};
#pragma unroll
  for (int axis = 0; axis < 3; ++axis) {
    const int64_t st = strides[axis];
#pragma unroll
    for (int o = -1; o <= 1; ++o) {
      const int64_t ci = i - (axis == 0 ? o : 0), cj = j - (axis == 1 ? o : 0), ck = k - (axis == 2 ? o : 0);
      const double al = alpha_axis(c, axis, ci, cj, ck);
      if (al != 0.0) {
        const int64_t gc = g - o * st;
        const T s = p[gc - st] - (T)2 * p[gc] + p[gc + st];
        const T kap = (o == 0) ? (T)-2 : (T)1;
        acc += kap * (T)al * s;
      }
    }
  }
  // diagonal shapes in the planes (x,y), (x,z), (y,z); sign -1 when offsets agree
  const double wxy = c.xy, wxz = c.xz, wyz = c.yz;
#pragma unroll
  for (int plane = 0; plane < 3; ++plane) {
    const double w = plane == 0 ? wxy : (plane == 1 ? wxz : wyz);
    if (w == 0.0) continue;
    const int64_t s1 = plane == 2 ? sy : sx;
    const int64_t s2 = plane == 0 ? sy : sz;
#pragma unroll
    for (int a = -1; a <= 1; a += 2) {
#pragma unroll
      for (int b = -1; b <= 1; b += 2) {
        // row centre c' = c - (a, b) in the plane
        int64_t ci = i, cj = j, ck = k;
        if (plane == 0) { ci -= a; cj -= b; }
        else if (plane == 1) { ci -= a; ck -= b; }
        else { cj -= a; ck -= b; }
        if (!is_interior(c, ci, cj, ck)) continue;
        const int64_t gc = g - a * s1 - b * s2;
        const T e = -p[gc - s1 - s2] + p[gc + s1 - s2] + p[gc - s1 + s2] - p[gc + s1 + s2];
        const T sg = (a == b) ? (T)-1 : (T)1;
        acc += sg * (T)w * e;
      }
    }
  }
  return acc;
}

// Coefficients in the arithmetic type of the kernel (FP32 kernels must not
// touch the FP64 pipe: GB300's FP64 rate is a small fraction of FP32).
template <typename T>
struct CoefT {
  int nx, ny, nz;
  T xx_int, yy_int, zz_int, xx_bdr, yy_bdr, zz_bdr, xy, xz, yz, ridge2;
};

template <typename T>
inline CoefT<T> coef_as(const StencilCoef &c) {
  CoefT<T> o;
  o.nx = (int)c.nx;
  o.ny = (int)c.ny;
  o.nz = (int)c.nz;
  o.xx_int = (T)c.xx_int;
  o.yy_int = (T)c.yy_int;
  o.zz_int = (T)c.zz_int;
  o.xx_bdr = (T)c.xx_bdr;
  o.yy_bdr = (T)c.yy_bdr;
  o.zz_bdr = (T)c.zz_bdr;
  o.xy = (T)c.xy;
  o.xz = (T)c.xz;
  o.yz = (T)c.yz;
  o.ridge2 = (T)c.ridge2;
  return o;
}

template <typename T>
__device__ __forceinline__ T alpha_axis32(const CoefT<T> &c, int axis, int i, int j, int k) {
  if (i < 0 || i >= c.nx || j < 0 || j >= c.ny || k < 0 || k >= c.nz) return (T)0;
  const bool inter = (i >= 1) & (i <= c.nx - 2) & (j >= 1) & (j <= c.ny - 2) & (k >= 1) & (k <= c.nz - 2);
  if (axis == 0) return (inter ? c.xx_int : (T)0) + c.xx_bdr * (T)((i == 1) + (i == c.nx - 2));
  if (axis == 1) return (inter ? c.yy_int : (T)0) + c.yy_bdr * (T)((j == 1) + (j == c.ny - 2));
  return (inter ? c.zz_int : (T)0) + c.zz_bdr * (T)((k == 1) + (k == c.nz - 2));
}

// Exact two-pass evaluation at any node (boundary shell).
template <typename T>
__device__ __forceinline__ T stencil_node_general(const CoefT<T> &c, const T *__restrict__ p, int g, int i, int j,
                                                  int k) {
  const int sy = c.nx, sz = c.nx * c.ny;
  T acc = c.ridge2 * __ldg(p + g);
  const int strides[3] = {1, sy, sz};
#pragma unroll
  for (int axis = 0; axis < 3; ++axis) {
    const int st = strides[axis];
#pragma unroll
    for (int o = -1; o <= 1; ++o) {
      const int ci = i - (axis == 0 ? o : 0), cj = j - (axis == 1 ? o : 0), ck = k - (axis == 2 ? o : 0);
      const T al = alpha_axis32<T>(c, axis, ci, cj, ck);
      if (al != (T)0) {
        const int gc = g - o * st;
        const T s = __ldg(p + gc - st) - (T)2 * __ldg(p + gc) + __ldg(p + gc + st);
        acc += ((o == 0) ? (T)-2 : (T)1) * al * s;
      }
    }
  }
#pragma unroll
  for (int plane = 0; plane < 3; ++plane) {
    const T w = plane == 0 ? c.xy : (plane == 1 ? c.xz : c.yz);
    if (w == (T)0) continue;
    const int s1 = plane == 2 ? sy : 1;
    const int s2 = plane == 0 ? sy : sz;
#pragma unroll
    for (int a = -1; a <= 1; a += 2) {
#pragma unroll
      for (int b = -1; b <= 1; b += 2) {
        int ci = i, cj = j, ck = k;
        if (plane == 0) { ci -= a; cj -= b; }
        else if (plane == 1) { ci -= a; ck -= b; }
        else { cj -= a; ck -= b; }
        if (!((ci >= 1) & (ci <= c.nx - 2) & (cj >= 1) & (cj <= c.ny - 2) & (ck >= 1) & (ck <= c.nz - 2))) continue;
        const int gc = g - a * s1 - b * s2;
        const T e = -__ldg(p + gc - s1 - s2) + __ldg(p + gc + s1 - s2) + __ldg(p + gc - s1 + s2) - __ldg(p + gc + s1 + s2);
        acc += ((a == b) ? (T)-1 : (T)1) * w * e;
      }
    }
  }
  return acc;
}

// Deep interior (every index in [3, n-4]): all contributing rows carry the
// interior weights, and the two-pass sum collapses to the composite stencil
//   ridge^2 p + sum_a (w_a^2/6) d4_a p + sum_{a<b} (w_ab^2/4) C_a C_b p,
// d4 = (1,-4,6,-4,1) and C = (1,0,-2,0,1) (stride-2 second difference).
template <typename T>
__device__ __forceinline__ T stencil_node_deep(const CoefT<T> &c, const T *__restrict__ p, int g) {
  const int sy = c.nx, sz = c.nx * c.ny;
  const T p0 = __ldg(p + g);
  auto d4 = [&](int s) {
    return (__ldg(p + g - 2 * s) + __ldg(p + g + 2 * s)) - (T)4 * (__ldg(p + g - s) + __ldg(p + g + s)) + (T)6 * p0;
  };
  auto cc = [&](int s1, int s2) {
    const T corners = (__ldg(p + g - 2 * s1 - 2 * s2) + __ldg(p + g + 2 * s1 - 2 * s2)) +
                      (__ldg(p + g - 2 * s1 + 2 * s2) + __ldg(p + g + 2 * s1 + 2 * s2));
    const T edges = (__ldg(p + g - 2 * s1) + __ldg(p + g + 2 * s1)) + (__ldg(p + g - 2 * s2) + __ldg(p + g + 2 * s2));
    return corners - (T)2 * edges + (T)4 * p0;
  };
  T acc = c.ridge2 * p0;
  acc += c.xx_int * d4(1);
  acc += c.yy_int * d4(sy);
  acc += c.zz_int * d4(sz);
  acc += c.xy * cc(1, sy);
  acc += c.xz * cc(1, sz);
  acc += c.yz * cc(sy, sz);
  return acc;
}

template <typename T>
__device__ __forceinline__ bool is_deep(const CoefT<T> &c, int i, int j, int k) {
  return (i >= 3) & (i <= c.nx - 4) & (j >= 3) & (j <= c.ny - 4) & (k >= 3) & (k <= c.nz - 4);
}

template <typename T>
__device__ __forceinline__ T stencil_node32(const CoefT<T> &c, const T *__restrict__ p, int g, int i, int j, int k) {
  return is_deep(c, i, j, k) ? stencil_node_deep<T>(c, p, g) : stencil_node_general<T>(c, p, g, i, j, k);
}

// diagonal of the stencil part + ridge^2
__host__ __device__ __forceinline__ double stencil_diag_node(const StencilCoef &c, int64_t i, int64_t j, int64_t k) {
  double d = c.ridge2;
  for (int axis = 0; axis < 3; ++axis)
    for (int o = -1; o <= 1; ++o) {
      const double al = alpha_axis(c, axis, i - (axis == 0 ? o : 0), j - (axis == 1 ? o : 0), k - (axis == 2 ? o : 0));
      d += (o == 0 ? 4.0 : 1.0) * al;
    }
  for (int plane = 0; plane < 3; ++plane) {
    const double w = plane == 0 ? c.xy : (plane == 1 ? c.xz : c.yz);
    if (w == 0.0) continue;
    for (int a = -1; a <= 1; a += 2)
      for (int b = -1; b <= 1; b += 2) {
        int64_t ci = i, cj = j, ck = k;
        if (plane == 0) { ci -= a; cj -= b; }
        else if (plane == 1) { ci -= a; ck -= b; }
        else { cj -= a; ck -= b; }
        if (is_interior(c, ci, cj, ck)) d += w;
      }
  }
  return d;
}

}  // namespace ls
