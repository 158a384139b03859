// Directional (anisotropic) second-derivative regularisation, matrix-free.
//
// FD:1207-1337 minimise_directional_gradient_change adds, for a direction
// field v sampled at every node and a weight w, the six interior
// second-derivative families again (the masks of OP:28-35 at every node with
// 1 <= i, j, k <= n - 2) with a per-row weight w * c_f(v(m)),
//     c = (vx^2, vy^2, vz^2, 2 vx vy, 2 vx vz, 2 vy vz),
// dropping rows whose weight is not > 0 in magnitude.  In the normal
// equations these rows contribute
//     sum_f D_f^T diag(W_f) D_f,   W_f(m) = s_f^2 sum_terms (w c_f(v(m)))^2
// with D_f the raw integer stencil -- (1, -2, 1) along one axis (f = 0..2:
// dxx, dyy, dzz) or the corner pattern du * dv in one plane (f = 3..5: dxy,
// dxz, dyz) -- and s_f the row normalisation of DI:361-366 (1/sqrt(6) and
// 1/2).  W (6 planes of n values, family-major) is zero off the interior.
//
// The term is applied as its own node-per-thread kernel after the fused
// isotropic operator: it adds D^T W D p to the operator's stored result and
// then runs the caller's epilogue (store, Chebyshev step or residual).
#pragma once

#include "fd_apply.cuh"
#include "fd_galerkin.cuh"

namespace ls {

template <typename T>
struct DirView {
  int nx, ny, nz;
  const T *w;  // 6 x n, family-major
};

constexpr int kDirFamilies = 6;

// (sum_f D_f^T W_f D_f p) at node (i, j, k).  The 25 distinct p values the
// 21 rows around the node touch (offsets within 2 along each axis and the
// (+-2, +-2) corners of the three planes) are loaded once (0 outside the
// grid: they only meet rows whose centre is not interior, whose weight is 0).
template <typename T>
__device__ __forceinline__ T dir_node(const DirView<T> &d, const T *__restrict__ p, int i, int j, int k) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t n = (int64_t)nx * ny * nz;
  const int g = (k * ny + j) * nx + i;
  const int st[3] = {1, nx, nx * ny};
  const int c[3] = {i, j, k}, lim[3] = {nx, ny, nz};
  auto inb = [&](int a, int off) { return c[a] + off >= 0 && c[a] + off < lim[a]; };
  // is the row centre (i, j, k) + (a0, a1, a2) an interior node?
  auto interior = [&](int a0, int a1, int a2) {
    return (i + a0 >= 1) & (i + a0 <= nx - 2) & (j + a1 >= 1) & (j + a1 <= ny - 2) & (k + a2 >= 1) & (k + a2 <= nz - 2);
  };
  const T pc = __ldg(p + g);
  T acc = 0;
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    T v[5];
#pragma unroll
    for (int o = -2; o <= 2; ++o) v[o + 2] = o == 0 ? pc : (inb(f, o) ? __ldg(p + g + o * st[f]) : (T)0);
#pragma unroll
    for (int t = -1; t <= 1; ++t) {  // node g is tap t of the row centred at m = g - t e_f
      if (interior(f == 0 ? -t : 0, f == 1 ? -t : 0, f == 2 ? -t : 0)) {
        const T D = v[1 - t] - (T)2 * v[2 - t] + v[3 - t];
        acc += (t == 0 ? (T)-2 : (T)1) * __ldg(d.w + f * n + (g - t * st[f])) * D;
      }
    }
  }
#pragma unroll
  for (int f = 3; f < 6; ++f) {
    const int u = (f == 5) ? 1 : 0, v = (f == 3) ? 1 : 2;
    const int su = st[u], sv = st[v];
    T q[3][3];  // q[a][b] = p at (2a - 2) e_u + (2b - 2) e_v
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        const int ou = 2 * a - 2, ov = 2 * b - 2;
        q[a][b] = (ou == 0 && ov == 0) ? pc
                                       : ((inb(u, ou) && inb(v, ov)) ? __ldg(p + g + ou * su + ov * sv) : (T)0);
      }
#pragma unroll
    for (int du = -1; du <= 1; du += 2)
#pragma unroll
      for (int dv = -1; dv <= 1; dv += 2) {  // node g is tap (du, dv) of the row centred at g - du e_u - dv e_v
        const int a0 = (u == 0 ? -du : 0), a1 = (u == 1 ? -du : 0) + (v == 1 ? -dv : 0), a2 = (v == 2 ? -dv : 0);
        if (interior(a0, a1, a2)) {
          // the row centre sits at (-du, -dv); its taps at (-du +- 1, -dv +- 1)
          // are q[(3 - du) / 2 or (1 - du) / 2][(3 - dv) / 2 or (1 - dv) / 2]
          const int ap = (3 - du) / 2, am = (1 - du) / 2, bp = (3 - dv) / 2, bm = (1 - dv) / 2;
          const T D = q[ap][bp] - q[ap][bm] - q[am][bp] + q[am][bm];
          acc += (T)(du * dv) * __ldg(d.w + f * n + (g - du * su - dv * sv)) * D;
        }
      }
  }
  return acc;
}

// q = qin + D^T W D p, then the epilogue.  With EPI_STORE, p . (D^T W D p)
// (the directional share of p . q only) lands in *dot_out.  qin may alias e.q.
template <typename T, int EPI>
__global__ void __launch_bounds__(256) dir_apply_kernel(DirView<T> d, const T *__restrict__ p, const T *qin,
                                                        EpiArgs<T> e, const int *done, double *partials,
                                                        unsigned int *ticket, double *dot_out) {
  if (done && *done) return;
  const int nx = d.nx, ny = d.ny;
  const int64_t n = (int64_t)nx * ny * d.nz;
  T local = 0;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)s;
    const int k = g / (nx * ny);
    const int rem = g - k * nx * ny;
    const int j = rem / nx;
    const int i = rem - j * nx;
    const T dq = dir_node<T>(d, p, i, j, k);
    const T pg = __ldg(p + g);
    epilogue<T, EPI>(e, g, pg, qin[g] + dq);
    if (EPI == EPI_STORE) local += pg * dq;
  }
  if (dot_out) {
    double tot;
    if (grid_sum<256, T>(local, partials, ticket, &tot)) *dot_out = tot;
  }
}

// diag += diagonal of sum_f D_f^T W_f D_f
template <typename T>
__global__ void dir_diag_kernel(DirView<T> d, double *__restrict__ diag) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int g = (int)s;
    const int k = g / (nx * ny);
    const int rem = g - k * nx * ny;
    const int j = rem / nx;
    const int i = rem - j * nx;
    const int c[3] = {i, j, k}, hi[3] = {nx - 2, ny - 2, nz - 2}, st[3] = {1, nx, nx * ny};
    double acc = 0.0;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const int u = f < 3 ? f : (f == 5 ? 1 : 0);
      const int v = f < 3 ? f : (f == 3 ? 1 : 2);
#pragma unroll
      for (int a = -1; a <= 1; ++a)
#pragma unroll
        for (int b = -1; b <= 1; ++b) {
          // pure families: centre offset a along the axis (b unused); cross: (a, b) corners
          if (f < 3 && b != 0) continue;
          if (f >= 3 && (a == 0 || b == 0)) continue;
          int m3[3] = {c[0], c[1], c[2]};
          m3[u] -= a;
          if (f >= 3) m3[v] -= b;
          bool ok = true;
#pragma unroll
          for (int x = 0; x < 3; ++x) ok &= (m3[x] >= 1) & (m3[x] <= hi[x]);
          if (!ok) continue;
          const int m = m3[0] * st[0] + m3[1] * st[1] + m3[2] * st[2];
          const double tap2 = (f < 3 && a == 0) ? 4.0 : 1.0;
          acc += tap2 * (double)d.w[f * n + m];
        }
    }
    diag[g] += acc;
  }
}

// ---------------------------------------------------------------------------
// Coarse multigrid levels.  The Galerkin product P^T D_f^T diag(W_f) D_f P of
// a family with constant unit weight over the interior rows is the tensor
// product Tx_f (x) Ty_f (x) Tz_f of the level's 1-D Galerkin tables
// (fd_galerkin.cuh: D2I / D1I / MI kinds, family order xx yy zz xy xz yz).
// With varying weights the coarse term is approximated by
//     sum_f S_f (Tx_f (x) Ty_f (x) Tz_f) S_f,   S_f = diag(sqrt(Wc_f)),
// Wc_f the full-weighting average of the finer level's weights over its rows
// (exact for constant weights; symmetric positive semi-definite always).  It
// is applied in three 1-D passes (x with the S_f scaling folded in, y, then z
// with the second S_f, the sum over families and the epilogue).
// ---------------------------------------------------------------------------
struct DirCoarse {
  int nx, ny, nz;
  const float *t[3];  // the level's 1-D tables, per axis [kind][index][5] (offsets -2..2)
  const float *sw;    // 6 x n: sqrt of the averaged weights
};

// Wc = average of the fine weights over the fine rows (mass) in the
// full-weighting window of each coarse node; mc = mass / 8; swc = sqrt(Wc).
// mf == nullptr: the fine level is the finest, whose rows are its interior nodes.
__global__ void dir_average_kernel(int fnx, int fny, int fnz, const float *__restrict__ wf, const float *__restrict__ mf,
                                   int cnx, int cny, int cnz, float *__restrict__ wc, float *__restrict__ mc,
                                   float *__restrict__ swc) {
  const int64_t fn = (int64_t)fnx * fny * fnz, cn = (int64_t)cnx * cny * cnz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < cn; s += (int64_t)gridDim.x * blockDim.x) {
    const int ck = (int)(s / ((int64_t)cnx * cny));
    const int rem = (int)(s - (int64_t)ck * cnx * cny);
    const int cj = rem / cnx, ci = rem - cj * cnx;
    float msum = 0.f, wsum[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c3 = -1; c3 <= 1; ++c3)
      for (int b = -1; b <= 1; ++b)
        for (int a = -1; a <= 1; ++a) {
          const int fi = 2 * ci + a, fj = 2 * cj + b, fk = 2 * ck + c3;
          if (fi < 0 || fj < 0 || fk < 0 || fi >= fnx || fj >= fny || fk >= fnz) continue;
          const int64_t fg = ((int64_t)fk * fny + fj) * fnx + fi;
          float m;
          if (mf)
            m = mf[fg];
          else
            m = (fi >= 1 && fi <= fnx - 2 && fj >= 1 && fj <= fny - 2 && fk >= 1 && fk <= fnz - 2) ? 1.f : 0.f;
          if (m == 0.f) continue;
          const float wt = (a ? 0.5f : 1.f) * (b ? 0.5f : 1.f) * (c3 ? 0.5f : 1.f) * m;
          msum += wt;
#pragma unroll
          for (int f = 0; f < 6; ++f) wsum[f] += wt * wf[f * fn + fg];
        }
    mc[s] = 0.125f * msum;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const float w = msum > 0.f ? wsum[f] / msum : 0.f;
      wc[f * cn + s] = w;
      swc[f * cn + s] = sqrtf(w);
    }
  }
}

// pass 1 (x): u_f = Tx_f (S_f p)
__global__ void __launch_bounds__(256) dir_coarse_x_kernel(DirCoarse d, const float *__restrict__ p,
                                                           float *__restrict__ u, const int *done) {
  if (done && *done) return;
  const int nx = d.nx;
  const int64_t n = (int64_t)nx * d.ny * d.nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(s % nx);
    float sp[5];
#pragma unroll
    for (int o = -2; o <= 2; ++o) sp[o + 2] = (i + o >= 0 && i + o < nx) ? __ldg(p + s + o) : 0.f;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const float *t = d.t[0] + ((size_t)g1_kind(f, 0) * nx + i) * 5;
      const float *sw = d.sw + f * n + s;
      float acc = 0.f;
#pragma unroll
      for (int o = -2; o <= 2; ++o)
        if (i + o >= 0 && i + o < nx) acc += __ldg(t + o + 2) * __ldg(sw + o) * sp[o + 2];
      u[f * n + s] = acc;
    }
  }
}

// pass 2 (y): v_f = Ty_f u_f
__global__ void __launch_bounds__(256) dir_coarse_y_kernel(DirCoarse d, const float *__restrict__ u,
                                                           float *__restrict__ v, const int *done) {
  if (done && *done) return;
  const int nx = d.nx, ny = d.ny;
  const int64_t n = (int64_t)nx * ny * d.nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)((s / nx) % ny);
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const float *t = d.t[1] + ((size_t)g1_kind(f, 1) * ny + j) * 5;
      const float *uf = u + f * n + s;
      float acc = 0.f;
#pragma unroll
      for (int o = -2; o <= 2; ++o)
        if (j + o >= 0 && j + o < ny) acc += __ldg(t + o + 2) * uf[(int64_t)o * nx];
      v[f * n + s] = acc;
    }
  }
}

// pass 3 (z): q = qin + sum_f S_f Tz_f v_f, then the epilogue (qin may alias e.q)
template <int EPI>
__global__ void __launch_bounds__(256) dir_coarse_z_kernel(DirCoarse d, const float *__restrict__ v,
                                                           const float *__restrict__ p, const float *qin,
                                                           EpiArgs<float> e, const int *done) {
  if (done && *done) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t sxy = (int64_t)nx * ny, n = sxy * nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(s / sxy);
    float acc = 0.f;
#pragma unroll
    for (int f = 0; f < 6; ++f) {
      const float *t = d.t[2] + ((size_t)g1_kind(f, 2) * nz + k) * 5;
      const float *vf = v + f * n + s;
      float a = 0.f;
#pragma unroll
      for (int o = -2; o <= 2; ++o)
        if (k + o >= 0 && k + o < nz) a += __ldg(t + o + 2) * vf[o * sxy];
      acc += __ldg(d.sw + f * n + s) * a;
    }
    epilogue<float, EPI>(e, (int)s, __ldg(p + s), qin[s] + acc);
  }
}

// diag += sum_f Wc_f * Tx_f(i, i) Ty_f(j, j) Tz_f(k, k)
__global__ void dir_coarse_diag_kernel(DirCoarse d, const float *__restrict__ wc, double *__restrict__ diag) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(s / ((int64_t)nx * ny));
    const int rem = (int)(s - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    double acc = 0.0;
#pragma unroll
    for (int f = 0; f < 6; ++f)
      acc += (double)wc[f * n + s] * d.t[0][((size_t)g1_kind(f, 0) * nx + i) * 5 + 2] *
             d.t[1][((size_t)g1_kind(f, 1) * ny + j) * 5 + 2] * d.t[2][((size_t)g1_kind(f, 2) * nz + k) * 5 + 2];
    diag[s] += acc;
  }
}

__global__ void dir_to_f32_kernel(int64_t count, const double *__restrict__ a, float *__restrict__ b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

}  // namespace ls
