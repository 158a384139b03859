// P1 (structured TetMesh, 5 tetrahedra per cell) on the GPU: face table and
// constant-gradient face rows (K3), barycentric point location with value /
// normal rows, and evaluation.
//
// Reference: T = packages/loop_common/src/loop_common/supports/_3d_structured_tetra.py,
//            P1 = packages/loop_interpolation/src/loop_interpolation/_p1interpolator.py
// Tet t lives in cell t / 5 (x fastest) with local index t % 5; its corner
// numbers come from the even / odd masks (T:28-34).  Compiled with -fmad=false
// and written in the reference's operation order, so indices are bit-exact and
// values agree to ~1 ulp (face rows up to the row sign, which follows the
// order of the three shared nodes: the reference orders them with an unstable
// sort; here they are ascending).
#include <math.h>

#include "ls_common.cuh"

namespace ls {
namespace {

__constant__ int kMaskEven[5][4] = {{7, 1, 2, 4}, {6, 2, 4, 7}, {5, 1, 4, 7}, {0, 1, 2, 4}, {3, 1, 2, 7}};
__constant__ int kMaskOdd[5][4] = {{0, 6, 5, 3}, {7, 3, 5, 6}, {4, 0, 5, 6}, {2, 0, 3, 6}, {1, 0, 3, 5}};
// T:664-712 neighbour tables: [odd][local-1][3][dx, dy, dz, neighbour local]
__constant__ int kNb[2][4][3][4] = {
    {{{-1, 0, 0, 1}, {0, 1, 0, 2}, {0, 0, 1, 3}},
     {{1, 0, 0, 2}, {0, -1, 0, 1}, {0, 0, 1, 4}},
     {{-1, 0, 0, 4}, {0, -1, 0, 3}, {0, 0, -1, 2}},
     {{1, 0, 0, 3}, {0, 1, 0, 4}, {0, 0, -1, 1}}},
    {{{1, 0, 0, 1}, {0, 1, 0, 2}, {0, 0, 1, 4}},
     {{-1, 0, 0, 2}, {0, -1, 0, 1}, {0, 0, 1, 3}},
     {{-1, 0, 0, 4}, {0, 1, 0, 3}, {0, 0, -1, 1}},
     {{1, 0, 0, 3}, {0, -1, 0, 4}, {0, 0, -1, 2}}}};

struct MeshArgs {
  int64_t n[3];      // nodes per axis
  int64_t cells[3];  // cells per axis
  double origin[3], step[3];
  double lo[3], hi[3];      // tolerant inside
  double smax[3];           // strict inside upper bound origin + step * cells (T:264-272)
  double ls_step[3];        // np.linspace spacing of the node coordinates
  double ls_stop[3];
};

MeshArgs make_mesh_args(const ls_grid3 &g) {
  MeshArgs a;
  for (int d = 0; d < 3; ++d) {
    a.n[d] = g.nsteps[d];
    a.cells[d] = g.nsteps[d] - 1;
    a.origin[d] = g.origin[d];
    a.step[d] = g.step[d];
    const double mx = g.origin[d] + (double)a.cells[d] * g.step[d];
    double ext = fabs(mx - g.origin[d]);
    if (ext < 1.0) ext = 1.0;
    const double tol = 2.220446049250313e-16 * 32.0 * ext;
    a.lo[d] = g.origin[d] - tol;
    a.hi[d] = mx + tol;
    a.smax[d] = g.origin[d] + g.step[d] * (double)a.cells[d];
    a.ls_stop[d] = mx;
    a.ls_step[d] = (a.n[d] > 1) ? (mx - g.origin[d]) / (double)(a.n[d] - 1) : 0.0;
  }
  return a;
}

__device__ __forceinline__ void cell_of(const MeshArgs &m, int64_t cell, int64_t c[3]) {
  c[0] = cell % m.cells[0];
  c[1] = (cell / m.cells[0]) % m.cells[1];
  c[2] = cell / (m.cells[0] * m.cells[1]);
}

__device__ __forceinline__ int64_t corner_gi(const MeshArgs &m, const int64_t c[3], int k) {
  return (c[0] + (k & 1)) + m.n[0] * ((c[1] + ((k >> 1) & 1)) + m.n[1] * (c[2] + (k >> 2)));
}

__device__ __forceinline__ void tet_nodes(const MeshArgs &m, int64_t t, int64_t nodes[4], int corners[4]) {
  const int64_t cell = t / 5;
  const int local = (int)(t % 5);
  int64_t c[3];
  cell_of(m, cell, c);
  const bool even = ((c[0] + c[1] + c[2]) % 2) == 0;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    corners[v] = even ? kMaskEven[local][v] : kMaskOdd[local][v];
    nodes[v] = corner_gi(m, c, corners[v]);
  }
}

// T:626-740
__device__ __forceinline__ void tet_neighbours(const MeshArgs &m, int64_t t, int64_t nb[4]) {
  const int64_t cell = t / 5;
  const int local = (int)(t % 5);
  if (local == 0) {
    nb[0] = t + 1;
    nb[1] = t + 2;
    nb[2] = t + 3;
    nb[3] = t + 4;
    return;
  }
  int64_t c[3];
  cell_of(m, cell, c);
  const int odd = ((c[0] + c[1] + c[2]) % 2) == 1;
  nb[0] = 5 * cell;
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const int *tb = kNb[odd][local - 1][e];
    const int64_t x = c[0] + tb[0], y = c[1] + tb[1], z = c[2] + tb[2];
    const bool ok = x >= 0 && y >= 0 && z >= 0 && x < m.cells[0] && y < m.cells[1] && z < m.cells[2];
    nb[1 + e] = ok ? (x + y * m.cells[0] + z * m.cells[0] * m.cells[1]) * 5 + tb[3] : -1;
  }
}

// node coordinate as np.linspace produces it (T shared_element_norm uses support.nodes)
__device__ __forceinline__ double ls_coord(const MeshArgs &m, int d, int64_t i) {
  if (i == m.n[d] - 1) return m.ls_stop[d];
  return (double)i * m.ls_step[d] + m.origin[d];
}

// node coordinate as node_indexes_to_position produces it (origin + step * idx)
__device__ __forceinline__ double ix_coord(const MeshArgs &m, int d, int64_t i) {
  return m.origin[d] + m.step[d] * (double)i;
}

// 3 x 4 shape-function gradient of a tet from its corner numbers (T:421-486):
// grad = inv(M)^T [[-1,1,0,0],[-1,0,1,0],[-1,0,0,1]], M columns = edges p_e - p_0
__device__ __forceinline__ void tet_gradient(const MeshArgs &m, const int64_t c[3], const int corners[4],
                                             double grad[3][4]) {
  double p[4][3];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int k = corners[v];
    p[v][0] = ix_coord(m, 0, c[0] + (k & 1));
    p[v][1] = ix_coord(m, 1, c[1] + ((k >> 1) & 1));
    p[v][2] = ix_coord(m, 2, c[2] + (k >> 2));
  }
  double M[3][3];  // M[d][e]
#pragma unroll
  for (int e = 0; e < 3; ++e)
#pragma unroll
    for (int d = 0; d < 3; ++d) M[d][e] = p[e + 1][d] - p[0][d];
  // inverse by cofactors: inv[e][d] = cof[d][e] / det
  double cof[3][3];
  cof[0][0] = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  cof[0][1] = -(M[1][0] * M[2][2] - M[1][2] * M[2][0]);
  cof[0][2] = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  cof[1][0] = -(M[0][1] * M[2][2] - M[0][2] * M[2][1]);
  cof[1][1] = M[0][0] * M[2][2] - M[0][2] * M[2][0];
  cof[1][2] = -(M[0][0] * M[2][1] - M[0][1] * M[2][0]);
  cof[2][0] = M[0][1] * M[1][2] - M[0][2] * M[1][1];
  cof[2][1] = -(M[0][0] * M[1][2] - M[0][2] * M[1][0]);
  cof[2][2] = M[0][0] * M[1][1] - M[0][1] * M[1][0];
  const double det = M[0][0] * cof[0][0] + M[0][1] * cof[0][1] + M[0][2] * cof[0][2];
  // grad[d][k] = sum_e inv[e][d] I[e][k];  inv[e][d] = cof[d][e] / det
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double a0 = cof[d][0] / det, a1 = cof[d][1] / det, a2 = cof[d][2] / det;
    grad[d][0] = -a0 - a1 - a2;
    grad[d][1] = a0;
    grad[d][2] = a1;
    grad[d][3] = a2;
  }
}

// ---------------------------------------------------------------------------
// face table: faces of tet i are its neighbours j < i, ascending (T:120-184)
// ---------------------------------------------------------------------------
__global__ void face_count_kernel(MeshArgs m, int64_t ntet, int32_t *__restrict__ count) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntet; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t nb[4];
    tet_neighbours(m, t, nb);
    int cnt = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e) cnt += (nb[e] >= 0 && nb[e] < t);
    count[t] = cnt;
  }
}

// device-wide exclusive scan of int32 counts (single block, setup-time)
__global__ void __launch_bounds__(1024) scan_counts_kernel(const int32_t *__restrict__ cnt, int64_t n,
                                                           int64_t *__restrict__ off, int64_t *__restrict__ total) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = (i < n) ? cnt[i] : 0;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t t = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warp_tot[lane] = t;
    }
    __syncthreads();
    const int64_t excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0) + carry;
    if (i < n) off[i] = excl;
    __syncthreads();
    if (threadIdx.x == 1023) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// numpy pairwise order for the L2 norm of 8 values
__device__ __forceinline__ double norm8(const double a[8]) {
  const double r = ((a[0] * a[0] + a[1] * a[1]) + (a[2] * a[2] + a[3] * a[3])) +
                   ((a[4] * a[4] + a[5] * a[5]) + (a[6] * a[6] + a[7] * a[7]));
  return sqrt(0.0 + r);
}

// faces of tet i and their rows (P1:115-166): const = [n . grad_i, -n . grad_j],
// n the face normal, or vec[face] when given (P1:129-130, the directional
// regularisation of P1:172-178)
__global__ void face_rows_kernel(MeshArgs m, int64_t ntet, const int64_t *__restrict__ off, double weight,
                                 const double *__restrict__ vec, int64_t *__restrict__ pairs,
                                 int64_t *__restrict__ shared, int64_t *__restrict__ idc, double *__restrict__ a,
                                 double *__restrict__ b, double *__restrict__ w) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntet; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t nb[4];
    tet_neighbours(m, t, nb);
    // ascending neighbour ids below t
    int64_t js[4];
    int nj = 0;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (nb[e] >= 0 && nb[e] < t) js[nj++] = nb[e];
    for (int x = 1; x < nj; ++x)
      for (int y = x; y > 0 && js[y - 1] > js[y]; --y) {
        const int64_t tmp = js[y];
        js[y] = js[y - 1];
        js[y - 1] = tmp;
      }
    if (nj == 0) continue;
    int64_t ni[4];
    int ci_[4];
    tet_nodes(m, t, ni, ci_);
    int64_t cell_i[3];
    cell_of(m, t / 5, cell_i);
    double gi[3][4];
    tet_gradient(m, cell_i, ci_, gi);
    int64_t f = off[t];
    for (int q = 0; q < nj; ++q, ++f) {
      const int64_t j = js[q];
      int64_t nj4[4];
      int cj_[4];
      tet_nodes(m, j, nj4, cj_);
      int64_t cell_j[3];
      cell_of(m, j / 5, cell_j);
      double gj[3][4];
      tet_gradient(m, cell_j, cj_, gj);
      // three shared nodes, ascending
      int64_t sh[3];
      int ns = 0;
      for (int u = 0; u < 4; ++u)
        for (int v = 0; v < 4; ++v)
          if (ni[u] == nj4[v] && ns < 3) sh[ns++] = ni[u];
      for (int x = 1; x < ns; ++x)
        for (int y = x; y > 0 && sh[y - 1] > sh[y]; --y) {
          const int64_t tmp = sh[y];
          sh[y] = sh[y - 1];
          sh[y - 1] = tmp;
        }
      // face normal from linspace node coordinates (T:186-194)
      double P[3][3];
      for (int v = 0; v < 3; ++v) {
        const int64_t g = sh[v];
        P[v][0] = ls_coord(m, 0, g % m.n[0]);
        P[v][1] = ls_coord(m, 1, (g / m.n[0]) % m.n[1]);
        P[v][2] = ls_coord(m, 2, g / (m.n[0] * m.n[1]));
      }
      const double v1[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
      const double v2[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
      double nrm[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
      if (vec) {
        nrm[0] = vec[3 * f];
        nrm[1] = vec[3 * f + 1];
        nrm[2] = vec[3 * f + 2];
      }
      double row[8];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        row[k] = (nrm[0] * gi[0][k] + nrm[1] * gi[1][k]) + nrm[2] * gi[2][k];
        row[4 + k] = -((nrm[0] * gj[0][k] + nrm[1] * gj[1][k]) + nrm[2] * gj[2][k]);
      }
      const double len = norm8(row);
      if (len > 0)
#pragma unroll
        for (int k = 0; k < 8; ++k) row[k] = row[k] / len;
      if (pairs) {
        pairs[2 * f] = t;
        pairs[2 * f + 1] = j;
      }
      if (shared)
        for (int v = 0; v < 3; ++v) shared[3 * f + v] = sh[v];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        idc[8 * f + k] = ni[k];
        idc[8 * f + 4 + k] = nj4[k];
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) a[8 * f + k] = row[k];
      b[f] = 0.0;
      w[f] = weight;
    }
  }
}

// ---------------------------------------------------------------------------
// point location (T:274-365): barycentric coordinates in the 5 candidate tets,
// the last containing tet wins, strict inside test
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double a[3], const double b[3], double o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// returns the tet (or -1) and its barycentric coordinates / corner numbers
__device__ __forceinline__ int64_t locate(const MeshArgs &m, const double pos[3], double bc[4], int corners[4],
                                          int64_t cell[3]) {
  bool inside = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) inside &= (pos[d] >= m.lo[d]) & (pos[d] <= m.hi[d]);
  int64_t c[3] = {0, 0, 0};
  if (inside)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int64_t k = (int64_t)floor((pos[d] - m.origin[d]) / m.step[d]);
      if (k < 0) k = 0;
      if (k > m.cells[d] - 1) k = m.cells[d] - 1;
      c[d] = k;
    }
  const bool even = ((c[0] + c[1] + c[2]) % 2) == 0;
  int found = -1;
  double best[4] = {0, 0, 0, 0};
  for (int lt = 0; lt < 5; ++lt) {
    double V[4][3];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int k = even ? kMaskEven[lt][v] : kMaskOdd[lt][v];
      V[v][0] = ix_coord(m, 0, c[0] + (k & 1));
      V[v][1] = ix_coord(m, 1, c[1] + ((k >> 1) & 1));
      V[v][2] = ix_coord(m, 2, c[2] + (k >> 2));
    }
    double vap[3], vbp[3], vab[3], vac[3], vad[3], vbc[3], vbd[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      vap[d] = pos[d] - V[0][d];
      vbp[d] = pos[d] - V[1][d];
      vab[d] = V[1][d] - V[0][d];
      vac[d] = V[2][d] - V[0][d];
      vad[d] = V[3][d] - V[0][d];
      vbc[d] = V[2][d] - V[1][d];
      vbd[d] = V[3][d] - V[1][d];
    }
    double t1[3];
    cross3(vbd, vbc, t1);
    const double va = dot3(vbp, t1) / 6.0;
    cross3(vac, vad, t1);
    const double vb = dot3(vap, t1) / 6.0;
    const double vol = dot3(vab, t1) / 6.0;
    cross3(vad, vab, t1);
    const double vc = dot3(vap, t1) / 6.0;
    cross3(vab, vac, t1);
    const double vd = dot3(vap, t1) / 6.0;
    const double cc[4] = {va / vol, vb / vol, vc / vol, vd / vol};
    if ((cc[0] >= 0) & (cc[1] >= 0) & (cc[2] >= 0) & (cc[3] >= 0)) {
      found = lt;
#pragma unroll
      for (int v = 0; v < 4; ++v) best[v] = cc[v];
    }
  }
  bool strict = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) strict &= (pos[d] > m.origin[d]) & (pos[d] < m.smax[d]);
  if (!(inside && found >= 0 && strict)) return -1;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    bc[v] = best[v];
    corners[v] = even ? kMaskEven[found][v] : kMaskOdd[found][v];
  }
  cell[0] = c[0];
  cell[1] = c[1];
  cell[2] = c[2];
  return found + 5 * (c[0] + m.cells[0] * c[1] + m.cells[0] * m.cells[1] * c[2]);
}

__global__ void locate_kernel(MeshArgs m, const double *__restrict__ pts, int64_t n, int64_t ld,
                              int64_t *__restrict__ tet, double *__restrict__ bc, int32_t *__restrict__ flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pos[3] = {pts[i * ld], pts[i * ld + 1], pts[i * ld + 2]};
    double c[4];
    int corners[4];
    int64_t cell[3];
    const int64_t t = locate(m, pos, c, corners, cell);
    if (tet) tet[i] = t;
    if (bc)
      for (int v = 0; v < 4; ++v) bc[4 * i + v] = t >= 0 ? c[v] : __longlong_as_double(0x7ff8000000000000LL);
    if (flag) flag[i] = t >= 0 ? 1 : 0;
  }
}

// volume of a tetrahedron, |det(edges)| / 6 (T:81-95 element_size)
__device__ __forceinline__ double tet_volume(const MeshArgs &m, const int64_t c[3], const int corners[4]) {
  double p[4][3];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int k = corners[v];
    p[v][0] = ix_coord(m, 0, c[0] + (k & 1));
    p[v][1] = ix_coord(m, 1, c[1] + ((k >> 1) & 1));
    p[v][2] = ix_coord(m, 2, c[2] + (k >> 2));
  }
  double e[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int d = 0; d < 3; ++d) e[r][d] = p[r + 1][d] - p[0][d];
  const double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                     e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                     e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
  return fabs(det) / 6;
}

// value (P1:98-113), normal (P1:73-96) or gradient-orthogonal (P1:248-296;
// KIND 2, b = 0, the tangent rows of DI:668-682; KIND 3, b = column 6) rows of
// the inside points at slot[i]
template <int KIND>
__global__ void p1_point_rows_kernel(MeshArgs m, const double *__restrict__ pts, int64_t n, int64_t ld, double weight,
                                     const int32_t *__restrict__ flag, const int64_t *__restrict__ slot,
                                     int64_t *__restrict__ idc, double *__restrict__ a, double *__restrict__ b,
                                     double *__restrict__ w) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[i]) continue;
    const double *p = pts + i * ld;
    const double pos[3] = {p[0], p[1], p[2]};
    double c[4];
    int corners[4];
    int64_t cell[3];
    locate(m, pos, c, corners, cell);
    int64_t nodes[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) nodes[v] = corner_gi(m, cell, corners[v]);
    const int64_t s = slot[i];
    if (KIND == 0) {  // value: barycentric row, weight column ignored
      const double len = sqrt(((((0.0 + c[0] * c[0]) + c[1] * c[1]) + c[2] * c[2]) + c[3] * c[3]));
      double bb = p[3];
      double row[4] = {c[0], c[1], c[2], c[3]};
      if (len > 0) {
        bb = bb / len;
        for (int v = 0; v < 4; ++v) row[v] = row[v] / len;
      }
      for (int v = 0; v < 4; ++v) {
        idc[4 * s + v] = nodes[v];
        a[4 * s + v] = row[v];
      }
      b[s] = bb;
      w[s] = weight;
    } else if (KIND >= 2) {  // v/|v| . grad phi, weight w * volume of the tetrahedron
      double g[3][4];
      tet_gradient(m, cell, corners, g);
      double v[3] = {p[3], p[4], p[5]};
      const double vn = sqrt(((0.0 + v[0] * v[0]) + v[1] * v[1]) + v[2] * v[2]);
      if (vn > 0)
        for (int d = 0; d < 3; ++d) v[d] = v[d] / vn;
      double row[4];
      for (int k = 0; k < 4; ++k) row[k] = (v[0] * g[0][k] + v[1] * g[1][k]) + v[2] * g[2][k];
      double bb = KIND == 3 ? p[6] : 0.0;
      const double len =
          sqrt(((((0.0 + row[0] * row[0]) + row[1] * row[1]) + row[2] * row[2]) + row[3] * row[3]));
      if (len > 0) {
        bb = bb / len;
        for (int v2 = 0; v2 < 4; ++v2) row[v2] = row[v2] / len;
      }
      for (int v2 = 0; v2 < 4; ++v2) {
        idc[4 * s + v2] = nodes[v2];
        a[4 * s + v2] = row[v2];
      }
      b[s] = bb;
      w[s] = weight * tet_volume(m, cell, corners);
    } else {  // normal: 3 gradient rows per point, point-major
      double g[3][4];
      tet_gradient(m, cell, corners, g);
      for (int d = 0; d < 3; ++d) {
        const int64_t r = 3 * s + d;
        const double len =
            sqrt(((((0.0 + g[d][0] * g[d][0]) + g[d][1] * g[d][1]) + g[d][2] * g[d][2]) + g[d][3] * g[d][3]));
        double bb = p[3 + d];
        double row[4] = {g[d][0], g[d][1], g[d][2], g[d][3]};
        if (len > 0) {
          bb = bb / len;
          for (int v = 0; v < 4; ++v) row[v] = row[v] / len;
        }
        for (int v = 0; v < 4; ++v) {
          idc[4 * r + v] = nodes[v];
          a[4 * r + v] = row[v];
        }
        b[r] = bb;
        w[r] = weight;
      }
    }
  }
}

// evaluation (T:208-262): NaN outside for value and gradient; a NaN input row
// gives value 0 at the interpolator level (DI:1342-1362)
__global__ void p1_eval_kernel(MeshArgs m, const double *__restrict__ cvec, const double *__restrict__ pts, int64_t n,
                               int64_t ld, double *__restrict__ value, double *__restrict__ grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pos[3] = {pts[i * ld], pts[i * ld + 1], pts[i * ld + 2]};
    const bool nanrow = isnan(pos[0]) | isnan(pos[1]) | isnan(pos[2]);
    double c[4];
    int corners[4];
    int64_t cell[3];
    const int64_t t = nanrow ? -1 : locate(m, pos, c, corners, cell);
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
    if (t < 0) {
      if (value) value[i] = nanrow ? 0.0 : qnan;
      if (grad) grad[3 * i] = grad[3 * i + 1] = grad[3 * i + 2] = qnan;
      continue;
    }
    double cv[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) cv[v] = cvec[corner_gi(m, cell, corners[v])];
    if (value) value[i] = (((0.0 + c[0] * cv[0]) + c[1] * cv[1]) + c[2] * cv[2]) + c[3] * cv[3];
    if (grad) {
      double g[3][4];
      tet_gradient(m, cell, corners, g);
      for (int d = 0; d < 3; ++d)
        grad[3 * i + d] = (((0.0 + g[d][0] * cv[0]) + g[d][1] * cv[1]) + g[d][2] * cv[2]) + g[d][3] * cv[3];
    }
  }
}

int check_mesh(const ls_grid3 *g) {
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

extern "C" int ls_p1_face_count(const ls_grid3 *mesh, int64_t *h_faces) {
  LS_TRY(check_mesh(mesh));
  LS_ARG_CHECK(h_faces != nullptr, "NULL output");
  // closed form: 4 internal faces per cell + 2 triangles per interior cell face
  const int64_t cx = mesh->nsteps[0] - 1, cy = mesh->nsteps[1] - 1, cz = mesh->nsteps[2] - 1;
  *h_faces = 4 * cx * cy * cz + 2 * ((cx - 1) * cy * cz + cx * (cy - 1) * cz + cx * cy * (cz - 1));
  return LS_OK;
}

namespace {
int face_rows(const ls_grid3 *mesh, double weight, const double *d_vec, int64_t *d_pairs, int64_t *d_shared,
              int64_t *d_idc, double *d_a, double *d_b, double *d_w, void *stream) {
  LS_TRY(check_mesh(mesh));
  LS_ARG_CHECK(d_idc && d_a && d_b && d_w, "NULL device buffer");
  const MeshArgs m = make_mesh_args(*mesh);
  const int64_t ntet = 5 * m.cells[0] * m.cells[1] * m.cells[2];
  cudaStream_t s = as_stream(stream);
  int32_t *cnt = nullptr;
  int64_t *off = nullptr;
  LS_CUDA_TRY(cudaMallocAsync((void **)&cnt, ntet * sizeof(int32_t), s));
  LS_CUDA_TRY(cudaMallocAsync((void **)&off, (ntet + 1) * sizeof(int64_t), s));
  face_count_kernel<<<stream_grid(ntet, 256), 256, 0, s>>>(m, ntet, cnt);
  scan_counts_kernel<<<1, 1024, 0, s>>>(cnt, ntet, off, off + ntet);
  face_rows_kernel<<<stream_grid(ntet, 128), 128, 0, s>>>(m, ntet, off, weight, d_vec, d_pairs, d_shared, d_idc, d_a,
                                                         d_b, d_w);
  LS_CUDA_TRY(cudaGetLastError());
  LS_CUDA_TRY(cudaFreeAsync(cnt, s));
  LS_CUDA_TRY(cudaFreeAsync(off, s));
  return LS_OK;
}
}  // namespace

extern "C" int ls_p1_face_rows(const ls_grid3 *mesh, double weight, int64_t *d_pairs, int64_t *d_shared,
                               int64_t *d_idc, double *d_a, double *d_b, double *d_w, void *stream) {
  return face_rows(mesh, weight, nullptr, d_pairs, d_shared, d_idc, d_a, d_b, d_w, stream);
}

extern "C" int ls_p1_face_rows_directional(const ls_grid3 *mesh, double weight, const double *d_vec, int64_t *d_idc,
                                           double *d_a, double *d_b, double *d_w, void *stream) {
  LS_ARG_CHECK(d_vec != nullptr, "NULL direction buffer");
  return face_rows(mesh, weight, d_vec, nullptr, nullptr, d_idc, d_a, d_b, d_w, stream);
}

extern "C" int ls_p1_locate(const ls_grid3 *mesh, const double *d_pts, int64_t npts, int64_t ld, int64_t *d_tet,
                            double *d_bc, void *stream) {
  LS_TRY(check_mesh(mesh));
  LS_ARG_CHECK(npts >= 0 && ld >= 3, "bad npts / ld");
  if (npts == 0) return LS_OK;
  const MeshArgs m = make_mesh_args(*mesh);
  cudaStream_t s = as_stream(stream);
  locate_kernel<<<stream_grid(npts, 128), 128, 0, s>>>(m, d_pts, npts, ld, d_tet, d_bc, nullptr);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

extern "C" int ls_p1_point_rows(const ls_grid3 *mesh, int kind, const double *d_pts, int64_t npts, int64_t ld,
                                double weight, int64_t *d_idc, double *d_a, double *d_b, double *d_w,
                                int64_t *h_count, void *stream) {
  LS_TRY(check_mesh(mesh));
  LS_ARG_CHECK(kind == LS_ROWS_VALUE || kind == LS_ROWS_NORM || kind == LS_ROWS_TANGENT || kind == LS_ROWS_ORTHOGONAL,
               "P1 rows: kind must be VALUE, NORM, TANGENT or ORTHOGONAL");
  LS_ARG_CHECK(ld >= (kind == LS_ROWS_VALUE ? 4 : kind == LS_ROWS_ORTHOGONAL ? 7 : 6), "ld too small for the row kind");
  LS_ARG_CHECK(h_count != nullptr, "h_count NULL");
  *h_count = 0;
  if (npts == 0) return LS_OK;
  const MeshArgs m = make_mesh_args(*mesh);
  cudaStream_t s = as_stream(stream);
  int32_t *flag = nullptr;
  int64_t *slot = nullptr;
  LS_CUDA_TRY(cudaMallocAsync((void **)&flag, npts * sizeof(int32_t), s));
  LS_CUDA_TRY(cudaMallocAsync((void **)&slot, (npts + 1) * sizeof(int64_t), s));
  locate_kernel<<<stream_grid(npts, 128), 128, 0, s>>>(m, d_pts, npts, ld, nullptr, nullptr, flag);
  scan_counts_kernel<<<1, 1024, 0, s>>>(flag, npts, slot, slot + npts);
  const int grd = stream_grid(npts, 128);
  if (kind == LS_ROWS_VALUE)
    p1_point_rows_kernel<0><<<grd, 128, 0, s>>>(m, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w);
  else if (kind == LS_ROWS_NORM)
    p1_point_rows_kernel<1><<<grd, 128, 0, s>>>(m, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w);
  else if (kind == LS_ROWS_TANGENT)
    p1_point_rows_kernel<2><<<grd, 128, 0, s>>>(m, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w);
  else
    p1_point_rows_kernel<3><<<grd, 128, 0, s>>>(m, d_pts, npts, ld, weight, flag, slot, d_idc, d_a, d_b, d_w);
  LS_CUDA_TRY(cudaGetLastError());
  int64_t cnt = 0;
  LS_CUDA_TRY(cudaMemcpyAsync(&cnt, slot + npts, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  LS_CUDA_TRY(cudaFreeAsync(flag, s));
  LS_CUDA_TRY(cudaFreeAsync(slot, s));
  LS_CUDA_TRY(cudaStreamSynchronize(s));
  *h_count = cnt;
  return LS_OK;
}

extern "C" int ls_p1_eval_points(const ls_grid3 *mesh, const double *d_c, const double *d_pts, int64_t npts,
                                 int64_t ld, double *d_value, double *d_grad, void *stream) {
  LS_TRY(check_mesh(mesh));
  LS_ARG_CHECK(d_c != nullptr && npts >= 0 && ld >= 3, "bad argument");
  if (npts == 0 || (!d_value && !d_grad)) return LS_OK;
  const MeshArgs m = make_mesh_args(*mesh);
  cudaStream_t s = as_stream(stream);
  p1_eval_kernel<<<stream_grid(npts, 128), 128, 0, s>>>(m, d_c, d_pts, npts, ld, d_value, d_grad);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}
