// Host-side preparation of the data rows for the multigrid hierarchy (plain
// C++, no CUDA: also compiled by the CPU tests).
//
// split_cell_rows separates the finest level's rows into
//   * cell rows: every column inside one 2 x 2 x 2 box of nodes (all point
//     rows) -- returned as (cell = the box's lowest corner, clamped to n - 2 on
//     the upper faces; 8 corner coefficients, corner bits x | y << 1 | z << 2,
//     repeated columns summed; w^2), sorted stably by the Morton code of the
//     cell, so that on every coarser level (cell >> 1 per axis, i.e. code >> 3)
//     each cell's rows are one contiguous run;
//   * the other rows (e.g. interface pairs spanning two cells), unchanged.
#pragma once

#include <algorithm>
#include <climits>
#include <cstdint>
#include <vector>

namespace ls {

struct HostRows {
  int64_t nrows = 0;
  int width = 0;
  std::vector<int64_t> cols;  // nrows * width, -1 = padding
  std::vector<double> a;
  std::vector<double> w2;
};

struct CellRowsHost {
  std::vector<int32_t> ci, cj, ck;
  std::vector<double> c;  // 8 per row
  std::vector<double> w2;
  int64_t nrows() const { return (int64_t)w2.size(); }
};

// bits of v (21 used) spread to every third position
inline uint64_t morton_spread(uint64_t v) {
  uint64_t x = v & 0x1fffffULL;
  x = (x | x << 32) & 0x1f00000000ffffULL;
  x = (x | x << 16) & 0x1f0000ff0000ffULL;
  x = (x | x << 8) & 0x100f00f00f00f00fULL;
  x = (x | x << 4) & 0x10c30c30c30c30c3ULL;
  x = (x | x << 2) & 0x1249249249249249ULL;
  return x;
}

inline uint64_t morton_code(uint32_t i, uint32_t j, uint32_t k) {
  return morton_spread(i) | morton_spread(j) << 1 | morton_spread(k) << 2;
}

// positions 0..n-1 ordered by key, stably (LSD radix sort, 11-bit digits)
inline std::vector<int64_t> stable_key_order(const std::vector<uint64_t> &key) {
  const size_t n = key.size();
  std::vector<uint64_t> k1(key), k2(n);
  std::vector<int64_t> i1(n), i2(n);
  for (size_t t = 0; t < n; ++t) i1[t] = (int64_t)t;
  uint64_t mx = 0;
  for (uint64_t v : key) mx = std::max(mx, v);
  constexpr int kBits = 11, kBuckets = 1 << kBits;
  std::vector<int64_t> cnt(kBuckets + 1);
  for (int shift = 0; shift < 64 && (mx >> shift) != 0; shift += kBits) {
    std::fill(cnt.begin(), cnt.end(), 0);
    for (size_t t = 0; t < n; ++t) ++cnt[((k1[t] >> shift) & (kBuckets - 1)) + 1];
    for (int d = 0; d < kBuckets; ++d) cnt[d + 1] += cnt[d];
    for (size_t t = 0; t < n; ++t) {
      const int64_t pos = cnt[(k1[t] >> shift) & (kBuckets - 1)]++;
      k2[pos] = k1[t];
      i2[pos] = i1[t];
    }
    k1.swap(k2);
    i1.swap(i2);
  }
  return i1;
}

inline void split_cell_rows(const HostRows &rows, int nx, int ny, int nz, CellRowsHost &cells, HostRows &rest) {
  rest = HostRows{};
  rest.width = rows.width;
  cells = CellRowsHost{};
  const int64_t nxy = (int64_t)nx * ny;
  const int lim[3] = {nx, ny, nz};
  CellRowsHost raw;
  std::vector<uint64_t> key;
  raw.ci.reserve(rows.nrows);
  raw.cj.reserve(rows.nrows);
  raw.ck.reserve(rows.nrows);
  raw.c.reserve(8 * rows.nrows);
  raw.w2.reserve(rows.nrows);
  key.reserve(rows.nrows);
  // the corner order of a point row (position_to_cell_corners): column b is
  // corner b of the cell whose lowest corner is column 0
  const int64_t corner[8] = {0, 1, nx, (int64_t)nx + 1, nxy, nxy + 1, nxy + nx, nxy + nx + 1};
  for (int64_t r = 0; r < rows.nrows; ++r) {
    if (rows.width >= 8) {  // fast path: exactly the 8 corners in corner order (+ padding)
      const int64_t *rc = &rows.cols[r * rows.width];
      bool ok = rc[0] >= 0;
      for (int b = 1; b < 8 && ok; ++b) ok = rc[b] - rc[0] == corner[b];
      for (int k = 8; k < rows.width && ok; ++k) ok = rc[k] < 0;
      if (ok) {
        const int z = (int)(rc[0] / nxy), rem = (int)(rc[0] - (int64_t)z * nxy), y = rem / nx, x = rem - y * nx;
        if (x <= nx - 2 && y <= ny - 2 && z <= nz - 2) {
          raw.ci.push_back(x);
          raw.cj.push_back(y);
          raw.ck.push_back(z);
          const double *ra = &rows.a[r * rows.width];
          for (int b = 0; b < 8; ++b) raw.c.push_back(0.0 + ra[b]);
          raw.w2.push_back(rows.w2[r]);
          key.push_back(morton_code((uint32_t)x, (uint32_t)y, (uint32_t)z));
          continue;
        }
      }
    }
    int xyz[64][3];
    double av[64];
    int m = 0;
    bool cell = rows.width <= 64;
    int lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {-1, -1, -1};
    for (int k = 0; k < rows.width && cell; ++k) {
      const int64_t c = rows.cols[r * rows.width + k];
      if (c < 0) continue;
      const int z = (int)(c / nxy), rem = (int)(c - (int64_t)z * nxy), y = rem / nx, x = rem - y * nx;
      const int ax[3] = {x, y, z};
      for (int d = 0; d < 3; ++d) {
        xyz[m][d] = ax[d];
        lo[d] = std::min(lo[d], ax[d]);
        hi[d] = std::max(hi[d], ax[d]);
        if (hi[d] - lo[d] > 1) cell = false;
      }
      av[m++] = rows.a[r * rows.width + k];
    }
    if (m == 0) cell = false;
    if (!cell) {
      rest.cols.insert(rest.cols.end(), rows.cols.begin() + r * rows.width, rows.cols.begin() + (r + 1) * rows.width);
      rest.a.insert(rest.a.end(), rows.a.begin() + r * rows.width, rows.a.begin() + (r + 1) * rows.width);
      rest.w2.push_back(rows.w2[r]);
      ++rest.nrows;
      continue;
    }
    int base[3];
    for (int d = 0; d < 3; ++d) base[d] = std::min(lo[d], lim[d] - 2);  // a box on the upper face ends there
    double c8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int e = 0; e < m; ++e)
      c8[(xyz[e][0] - base[0]) | ((xyz[e][1] - base[1]) << 1) | ((xyz[e][2] - base[2]) << 2)] += av[e];
    raw.ci.push_back(base[0]);
    raw.cj.push_back(base[1]);
    raw.ck.push_back(base[2]);
    raw.c.insert(raw.c.end(), c8, c8 + 8);
    raw.w2.push_back(rows.w2[r]);
    key.push_back(morton_code((uint32_t)base[0], (uint32_t)base[1], (uint32_t)base[2]));
  }
  const std::vector<int64_t> order = stable_key_order(key);
  const size_t n = order.size();
  cells.ci.resize(n);
  cells.cj.resize(n);
  cells.ck.resize(n);
  cells.c.resize(8 * n);
  cells.w2.resize(n);
  for (size_t t = 0; t < n; ++t) {
    const int64_t r = order[t];
    cells.ci[t] = raw.ci[r];
    cells.cj[t] = raw.cj[r];
    cells.ck[t] = raw.ck[r];
    std::copy(raw.c.begin() + 8 * r, raw.c.begin() + 8 * r + 8, cells.c.begin() + 8 * t);
    cells.w2[t] = raw.w2[r];
  }
}

}  // namespace ls
