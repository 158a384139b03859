// Isosurface extraction on the StructuredGrid node values (the solved
// coefficients): the level set {f = iso} of the piecewise-linear interpolant
// over the Freudenthal (Kuhn) triangulation of every cell.
//
// Reference: DI:1395-1405 `surfaces(value)` contours the support's VTK image
// with pyvista (marching cubes), and LoopIsosurfacer (utils/_surface.py)
// samples the field and calls skimage's marching_cubes.  Neither library is
// available here; this is a table-free marching-tetrahedra formulation on the
// same node values, watertight and without the ambiguous cases of marching
// cubes.
//
// Triangulation: cell (i, j, k) is split into the 6 tetrahedra along its main
// diagonal, one per axis permutation (a, b, c): corners 0, e_a, e_a + e_b,
// e_a + e_b + e_c.  Every tetrahedron edge joins a node p to p + d with d one
// of the 7 directions {x, y, z, xy, xz, yz, xyz} (non-negative components),
// and adjacent cells split their shared face along the same diagonal, so the
// surface is closed.
//
// A vertex lies on every crossing edge (one endpoint > iso, the other <= iso,
// both finite) at the linear-interpolation point; vertices are numbered by
// (node, direction) -- node offset from a scan of per-node crossing counts,
// plus the rank of the direction in the node's 7-bit crossing mask -- so each
// is emitted once and shared by the triangles around the edge.  Each
// tetrahedron with 1 or 3 vertices above iso gives one triangle, with 2 a
// quadrilateral split in two; triangles are wound so that their normal points
// towards increasing f.  Vertex normals: the central-difference node
// gradients interpolated along the edge, normalised (one-sided next to NaN
// nodes; the edge direction where no gradient is left).
//
// Passes: classify (node masks, per-cell triangle counts), two exclusive
// scans (3-phase, multi-block), emit.
#include <math.h>

#include "ls_common.cuh"

struct ls_iso {
  ls_grid3 grid;
  int64_t n = 0;
  double iso = 0.0;
  const double *values = nullptr;  // borrowed: valid until ls_iso_copy returns
  uint8_t *mask = nullptr;         // per node: crossing edges (bit = direction)
  uint8_t *tcount = nullptr;       // per cell anchor node: triangles
  int64_t *voff = nullptr;         // exclusive scan of popc(mask)
  int64_t *toff = nullptr;         // exclusive scan of tcount
  int64_t *tile = nullptr;         // scan scratch
  int64_t nverts = 0, ntris = 0;
};

namespace ls {
namespace {

constexpr int kDirs = 7;
// direction index -> corner bitmask (bit 0 = +x, bit 1 = +y, bit 2 = +z)
__constant__ int kDirBits[kDirs] = {1, 2, 4, 3, 5, 6, 7};
// corner bitmask -> direction index (-1: not a direction)
__constant__ int kBitsDir[8] = {-1, 0, 1, 3, 2, 4, 5, 6};
// the 6 Freudenthal tetrahedra as corner bitmasks, one per axis permutation
__constant__ int kTet[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};

struct IsoGrid {
  int nx, ny, nz;
  double o[3], h[3];
};

IsoGrid iso_grid(const ls_grid3 &g) {
  IsoGrid r;
  r.nx = (int)g.nsteps[0];
  r.ny = (int)g.nsteps[1];
  r.nz = (int)g.nsteps[2];
  for (int d = 0; d < 3; ++d) {
    r.o[d] = g.origin[d];
    r.h[d] = g.step[d];
  }
  return r;
}

__device__ __forceinline__ bool above(double f, double iso) { return f > iso; }

// pass 1: crossing masks of the node's 7 forward edges; triangle count of the
// cell anchored at the node (0 for nodes on an upper face)
__global__ void iso_classify_kernel(IsoGrid gr, const double *__restrict__ f, double iso, uint8_t *__restrict__ mask,
                                    uint8_t *__restrict__ tcount) {
  const int nx = gr.nx, ny = gr.ny, nz = gr.nz;
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    const double f0 = f[g];
    unsigned m = 0u;
#pragma unroll
    for (int d = 0; d < kDirs; ++d) {
      const int b = kDirBits[d];
      const int di = b & 1, dj = (b >> 1) & 1, dk = (b >> 2) & 1;
      if (i + di >= nx || j + dj >= ny || k + dk >= nz) continue;
      const double f1 = f[g + di + (int64_t)nx * (dj + (int64_t)ny * dk)];
      if (isnan(f0) || isnan(f1)) continue;
      if (above(f0, iso) != above(f1, iso)) m |= 1u << d;
    }
    mask[g] = (uint8_t)m;
    unsigned tris = 0u;
    if (i + 1 < nx && j + 1 < ny && k + 1 < nz) {
      double c[8];
      bool bad = false;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        c[b] = f[g + (b & 1) + (int64_t)nx * (((b >> 1) & 1) + (int64_t)ny * ((b >> 2) & 1))];
        bad |= isnan(c[b]);
      }
      if (!bad) {
#pragma unroll
        for (int t = 0; t < 6; ++t) {
          int ka = 0;
#pragma unroll
          for (int v = 0; v < 4; ++v) ka += above(c[kTet[t][v]], iso) ? 1 : 0;
          tris += (ka == 1 || ka == 3) ? 1u : (ka == 2 ? 2u : 0u);
        }
      }
    }
    tcount[g] = (uint8_t)tris;
  }
}

// ---- exclusive scan (3 phases) of per-node counts ----------------------------
constexpr int kScanThreads = 256, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

template <bool POPC>
__device__ __forceinline__ int64_t scan_item(const uint8_t *a, int64_t idx, int64_t n) {
  if (idx >= n) return 0;
  return POPC ? __popc((unsigned)a[idx]) : (int64_t)a[idx];
}

template <int BLOCK>
__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *total) {
  __shared__ int64_t warp_tot[BLOCK / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t t = lane < BLOCK / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < BLOCK / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  const int64_t excl = x - v + (warp > 0 ? warp_tot[warp - 1] : 0);
  *total = warp_tot[BLOCK / 32 - 1];
  __syncthreads();
  return excl;
}

template <bool POPC>
__global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(const uint8_t *__restrict__ a, int64_t n,
                                                                      int64_t *__restrict__ tile) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t s = 0;
#pragma unroll
  for (int u = 0; u < kScanItems; ++u) s += scan_item<POPC>(a, base + u, n);
  int64_t total;
  block_exclusive_scan<kScanThreads>(s, &total);
  if (threadIdx.x == 0) tile[blockIdx.x] = total;
}

// exclusive scan of the tile sums in place (one block); tile[ntiles] = total
__global__ void __launch_bounds__(1024) scan_tiles_kernel(int64_t *__restrict__ tile, int64_t ntiles) {
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b = 0; b < ntiles; b += 1024) {
    const int64_t idx = b + threadIdx.x;
    const int64_t v = idx < ntiles ? tile[idx] : 0;
    int64_t total;
    const int64_t ex = block_exclusive_scan<1024>(v, &total);
    if (idx < ntiles) tile[idx] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile[ntiles] = carry;
}

template <bool POPC>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint8_t *__restrict__ a, int64_t n,
                                                                  const int64_t *__restrict__ tile,
                                                                  int64_t *__restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems], s = 0;
#pragma unroll
  for (int u = 0; u < kScanItems; ++u) {
    v[u] = scan_item<POPC>(a, base + u, n);
    s += v[u];
  }
  int64_t total;
  int64_t run = block_exclusive_scan<kScanThreads>(s, &total) + tile[blockIdx.x];
#pragma unroll
  for (int u = 0; u < kScanItems; ++u) {
    if (base + u < n) out[base + u] = run;
    run += v[u];
  }
}

// ---- pass 3: vertices and triangles ---------------------------------------------
struct EmitArgs {
  IsoGrid gr;
  const double *f;
  double iso;
  const uint8_t *mask;
  const uint8_t *tcount;
  const int64_t *voff;
  const int64_t *toff;
  double *verts;    // V x 3
  double *normals;  // V x 3 (may be null)
  int64_t *tris;    // T x 3
};

// gradient at node (i, j, k): central differences, one-sided on faces and
// next to NaN nodes, 0 along an axis with no finite pair
__device__ void node_gradient(const EmitArgs &a, int i, int j, int k, double g[3]) {
  const int nx = a.gr.nx, ny = a.gr.ny, nz = a.gr.nz;
  const int c[3] = {i, j, k}, lim[3] = {nx, ny, nz};
  const int64_t st[3] = {1, nx, (int64_t)nx * ny};
  const int64_t p = i + (int64_t)nx * (j + (int64_t)ny * k);
  const double fp = a.f[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double fm = c[d] > 0 ? a.f[p - st[d]] : NAN;
    const double fq = c[d] + 1 < lim[d] ? a.f[p + st[d]] : NAN;
    double v = 0.0;
    if (!isnan(fm) && !isnan(fq))
      v = (fq - fm) / (2.0 * a.gr.h[d]);
    else if (!isnan(fq) && !isnan(fp))
      v = (fq - fp) / a.gr.h[d];
    else if (!isnan(fm) && !isnan(fp))
      v = (fp - fm) / a.gr.h[d];
    g[d] = v;
  }
}

__device__ __forceinline__ int64_t vertex_id(const EmitArgs &a, int64_t p, int dir) {
  const unsigned m = a.mask[p];
  return a.voff[p] + __popc(m & ((1u << dir) - 1u));
}

__global__ void iso_emit_kernel(EmitArgs a) {
  const int nx = a.gr.nx, ny = a.gr.ny, nz = a.gr.nz;
  const int64_t n = (int64_t)nx * ny * nz;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(g / ((int64_t)nx * ny));
    const int rem = (int)(g - (int64_t)k * nx * ny);
    const int j = rem / nx, i = rem - j * nx;
    // vertices on this node's crossing edges
    const unsigned m = a.mask[g];
    if (m) {
      const double f0 = a.f[g];
      double g0[3];
      if (a.normals) node_gradient(a, i, j, k, g0);
      int64_t vid = a.voff[g];
      for (int d = 0; d < kDirs; ++d) {
        if (!(m & (1u << d))) continue;
        const int b = kDirBits[d];
        const int di = b & 1, dj = (b >> 1) & 1, dk = (b >> 2) & 1;
        const double f1 = a.f[g + di + (int64_t)nx * (dj + (int64_t)ny * dk)];
        const double t = (a.iso - f0) / (f1 - f0);
        a.verts[3 * vid + 0] = a.gr.o[0] + a.gr.h[0] * ((double)i + t * di);
        a.verts[3 * vid + 1] = a.gr.o[1] + a.gr.h[1] * ((double)j + t * dj);
        a.verts[3 * vid + 2] = a.gr.o[2] + a.gr.h[2] * ((double)k + t * dk);
        if (a.normals) {
          double g1[3];
          node_gradient(a, i + di, j + dj, k + dk, g1);
          double nv[3], len = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            nv[c] = g0[c] + t * (g1[c] - g0[c]);
            len += nv[c] * nv[c];
          }
          if (!(len > 0.0)) {  // no usable node gradient: the edge direction, towards increasing f
            const double s = f1 > f0 ? 1.0 : -1.0;
            nv[0] = s * di / a.gr.h[0];
            nv[1] = s * dj / a.gr.h[1];
            nv[2] = s * dk / a.gr.h[2];
            len = nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2];
          }
          len = 1.0 / sqrt(len);
#pragma unroll
          for (int c = 0; c < 3; ++c) a.normals[3 * vid + c] = nv[c] * len;
        }
        ++vid;
      }
    }
    // triangles of the cell anchored here
    if (!a.tcount[g]) continue;
    double c[8];
#pragma unroll
    for (int b = 0; b < 8; ++b) c[b] = a.f[g + (b & 1) + (int64_t)nx * (((b >> 1) & 1) + (int64_t)ny * ((b >> 2) & 1))];
    int64_t out = a.toff[g];
    for (int t = 0; t < 6; ++t) {
      int A[4], B[4], na = 0, nb = 0;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int cb = kTet[t][v];
        if (above(c[cb], a.iso))
          A[na++] = cb;
        else
          B[nb++] = cb;
      }
      if (na == 0 || nb == 0) continue;
      // vertex id and position of the crossing edge between corners u and w
      // (the position recomputed from the same two values the owning node
      // interpolates, so no other thread's output is read)
      auto edge = [&](int u, int w, double pos[3]) -> int64_t {
        const int lo = u < w ? u : w, hi = u < w ? w : u;  // the chain is monotone: lo is a subset of hi
        const int db = hi & ~lo;
        const int64_t p = g + (lo & 1) + (int64_t)nx * (((lo >> 1) & 1) + (int64_t)ny * ((lo >> 2) & 1));
        const double tt = (a.iso - c[lo]) / (c[hi] - c[lo]);
        const int base[3] = {i + (lo & 1), j + ((lo >> 1) & 1), k + ((lo >> 2) & 1)};
#pragma unroll
        for (int q = 0; q < 3; ++q) pos[q] = a.gr.o[q] + a.gr.h[q] * ((double)base[q] + tt * ((db >> q) & 1));
        return vertex_id(a, p, kBitsDir[db]);
      };
      // gradient of the linear interpolant on the tetrahedron (physical units):
      // along its chain 0 -> e_a -> e_a + e_b -> 1 each step adds one axis
      double grad[3];
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        const int from = kTet[t][s], to = kTet[t][s + 1];
        const int ax = (to & ~from) == 1 ? 0 : ((to & ~from) == 2 ? 1 : 2);
        grad[ax] = (c[to] - c[from]) / a.gr.h[ax];
      }
      int64_t tri[2][3];
      double P[4][3];
      int ntri;
      if (na == 1 || nb == 1) {
        const int apex = na == 1 ? A[0] : B[0];
        const int *other = na == 1 ? B : A;
        tri[0][0] = edge(apex, other[0], P[0]);
        tri[0][1] = edge(apex, other[1], P[1]);
        tri[0][2] = edge(apex, other[2], P[2]);
        ntri = 1;
      } else {  // quadrilateral e(a0,b0) e(a0,b1) e(a1,b1) e(a1,b0)
        const int64_t q0 = edge(A[0], B[0], P[0]), q1 = edge(A[0], B[1], P[1]);
        const int64_t q2 = edge(A[1], B[1], P[2]), q3 = edge(A[1], B[0], P[3]);
        tri[0][0] = q0, tri[0][1] = q1, tri[0][2] = q2;
        tri[1][0] = q0, tri[1][1] = q2, tri[1][2] = q3;
        ntri = 2;
      }
      for (int r = 0; r < ntri; ++r) {
        // winding: normal along +grad f (P indices of the triangle's corners)
        const int i0 = 0, i1 = r == 0 ? 1 : 2, i2 = r == 0 ? 2 : 3;
        const double e1[3] = {P[i1][0] - P[i0][0], P[i1][1] - P[i0][1], P[i1][2] - P[i0][2]};
        const double e2[3] = {P[i2][0] - P[i0][0], P[i2][1] - P[i0][1], P[i2][2] - P[i0][2]};
        const double nrm[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const bool flip = nrm[0] * grad[0] + nrm[1] * grad[1] + nrm[2] * grad[2] < 0.0;
        a.tris[3 * out + 0] = tri[r][0];
        a.tris[3 * out + 1] = flip ? tri[r][2] : tri[r][1];
        a.tris[3 * out + 2] = flip ? tri[r][1] : tri[r][2];
        ++out;
      }
    }
  }
}

int scan_counts(const uint8_t *a, int64_t n, bool popc, int64_t *tile, int64_t *out, int64_t *h_total, cudaStream_t s) {
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (popc)
    scan_tile_sums_kernel<true><<<(unsigned)ntiles, kScanThreads, 0, s>>>(a, n, tile);
  else
    scan_tile_sums_kernel<false><<<(unsigned)ntiles, kScanThreads, 0, s>>>(a, n, tile);
  scan_tiles_kernel<<<1, 1024, 0, s>>>(tile, ntiles);
  if (popc)
    scan_apply_kernel<true><<<(unsigned)ntiles, kScanThreads, 0, s>>>(a, n, tile, out);
  else
    scan_apply_kernel<false><<<(unsigned)ntiles, kScanThreads, 0, s>>>(a, n, tile, out);
  LS_CUDA_TRY(cudaGetLastError());
  LS_CUDA_TRY(cudaMemcpyAsync(h_total, tile + ntiles, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  return LS_OK;
}

}  // namespace
}  // namespace ls

using namespace ls;

extern "C" int ls_iso_destroy(ls_iso *h) {
  if (!h) return LS_OK;
  void *p[] = {h->mask, h->tcount, h->voff, h->toff, h->tile};
  for (void *q : p)
    if (q) cudaFree(q);
  delete h;
  return LS_OK;
}

extern "C" int ls_iso_extract(const ls_grid3 *grid, const double *d_values, double iso, ls_iso **out,
                              int64_t *h_nverts, int64_t *h_ntris, void *stream) {
  LS_ARG_CHECK(grid && d_values && out && h_nverts && h_ntris, "NULL argument");
  LS_ARG_CHECK(isfinite(iso), "iso value must be finite");
  *out = nullptr;
  for (int d = 0; d < 3; ++d) {
    LS_ARG_CHECK(grid->nsteps[d] >= 1, "every axis needs at least 1 node");
    LS_ARG_CHECK(grid->step[d] > 0.0, "step must be positive");
  }
  const int64_t n = grid->nsteps[0] * grid->nsteps[1] * grid->nsteps[2];
  LS_ARG_CHECK(n < ((int64_t)1 << 40), "grid too large");
  cudaStream_t s = as_stream(stream);
  ls_iso *h = new ls_iso();
  h->grid = *grid;
  h->n = n;
  h->iso = iso;
  h->values = d_values;
  auto fail = [&](int st) {
    ls_iso_destroy(h);
    return st;
  };
  const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (cudaMalloc((void **)&h->mask, n) != cudaSuccess || cudaMalloc((void **)&h->tcount, n) != cudaSuccess ||
      cudaMalloc((void **)&h->voff, n * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc((void **)&h->toff, n * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc((void **)&h->tile, (ntiles + 1) * sizeof(int64_t)) != cudaSuccess) {
    set_error("isosurface scratch allocation failed (%lld nodes)", (long long)n);
    return fail(LS_ERR_ALLOC);
  }
  const IsoGrid gr = iso_grid(*grid);
  iso_classify_kernel<<<stream_grid(n, 256), 256, 0, s>>>(gr, d_values, iso, h->mask, h->tcount);
  int st;
  if ((st = scan_counts(h->mask, n, true, h->tile, h->voff, &h->nverts, s)) < 0) return fail(st);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error("isosurface classify failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(LS_ERR_CUDA);
  }
  if ((st = scan_counts(h->tcount, n, false, h->tile, h->toff, &h->ntris, s)) < 0) return fail(st);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error("isosurface scan failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(LS_ERR_CUDA);
  }
  *h_nverts = h->nverts;
  *h_ntris = h->ntris;
  *out = h;
  return LS_OK;
}

extern "C" int ls_iso_copy(ls_iso *h, double *d_verts, double *d_normals, int64_t *d_tris, void *stream) {
  LS_ARG_CHECK(h != nullptr, "NULL handle");
  LS_ARG_CHECK((h->nverts == 0 || d_verts) && (h->ntris == 0 || d_tris), "NULL output buffer");
  if (h->nverts == 0 && h->ntris == 0) return LS_OK;
  cudaStream_t s = as_stream(stream);
  EmitArgs a;
  a.gr = iso_grid(h->grid);
  a.f = h->values;
  a.iso = h->iso;
  a.mask = h->mask;
  a.tcount = h->tcount;
  a.voff = h->voff;
  a.toff = h->toff;
  a.verts = d_verts;
  a.normals = d_normals;
  a.tris = d_tris;
  iso_emit_kernel<<<stream_grid(h->n, 256), 256, 0, s>>>(a);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}
