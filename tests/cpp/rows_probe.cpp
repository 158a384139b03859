// C entry around the multigrid host row split (mg_rows_host.hpp) for the CPU
// tests: built with g++ by tests/test_rows_host_cpu.py.
#include "../../loopstructural_gb300/csrc/mg_rows_host.hpp"

extern "C" int64_t split_rows_probe(int64_t nrows, int width, const int64_t *cols, const double *a, const double *w2,
                                    int nx, int ny, int nz, int32_t *ci, int32_t *cj, int32_t *ck, double *c,
                                    double *cw2, int64_t *rest_nrows, int64_t *rest_cols, double *rest_a,
                                    double *rest_w2) {
  ls::HostRows rows;
  rows.nrows = nrows;
  rows.width = width;
  rows.cols.assign(cols, cols + nrows * width);
  rows.a.assign(a, a + nrows * width);
  rows.w2.assign(w2, w2 + nrows);
  ls::CellRowsHost cells;
  ls::HostRows rest;
  ls::split_cell_rows(rows, nx, ny, nz, cells, rest);
  const int64_t n = cells.nrows();
  std::copy(cells.ci.begin(), cells.ci.end(), ci);
  std::copy(cells.cj.begin(), cells.cj.end(), cj);
  std::copy(cells.ck.begin(), cells.ck.end(), ck);
  std::copy(cells.c.begin(), cells.c.end(), c);
  std::copy(cells.w2.begin(), cells.w2.end(), cw2);
  *rest_nrows = rest.nrows;
  std::copy(rest.cols.begin(), rest.cols.end(), rest_cols);
  std::copy(rest.a.begin(), rest.a.end(), rest_a);
  std::copy(rest.w2.begin(), rest.w2.end(), rest_w2);
  return n;
}
