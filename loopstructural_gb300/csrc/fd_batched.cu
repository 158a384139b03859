// Batched solves of independent FD systems (model ensembles): host worker
// threads each take the next handle and run its setup, then (after every
// setup is done) its solve on the handle's own stream, so up to `concurrency`
// models overlap on the GPU.  The solves are
// independent (per-handle workspaces, thread-local errors and graph capture),
// so results equal those of the same solves run one after another.
#include <algorithm>
#include <atomic>
#include <string>
#include <thread>
#include <vector>

#include "ls_common.cuh"


extern "C" int ls_fd_solve_batched(ls_fd_handle *const *handles, const ls_solve_opts *opts, double *const *d_x,
                                   ls_solve_stats *stats, int64_t count, int concurrency, int *statuses) {
  LS_ARG_CHECK(count >= 0, "negative count");
  if (count == 0) return LS_OK;
  LS_ARG_CHECK(handles && opts && d_x && stats && statuses, "NULL argument");
  for (int64_t i = 0; i < count; ++i) LS_ARG_CHECK(handles[i] && d_x[i], "NULL handle or solution pointer");
  const int workers = (int)std::max<int64_t>(1, std::min<int64_t>(concurrency > 0 ? concurrency : 8, count));
  std::vector<std::string> errors(count);
  // runs fn(i) for every model on `workers` threads, each on the model's device
  auto parallel = [&](auto &&fn) {
    std::atomic<int64_t> next{0};
    auto work = [&]() {
      for (;;) {
        const int64_t i = next.fetch_add(1);
        if (i >= count) break;
        cudaSetDevice(ls_fd_device(handles[i]));
        fn(i);
      }
    };
    std::vector<std::thread> pool;
    pool.reserve(workers);
    for (int t = 0; t < workers; ++t) pool.emplace_back(work);
    for (auto &t : pool) t.join();
  };
  // phase 1: every allocation (multigrid hierarchies) -- no graph is being
  // captured yet, so allocator calls cannot disturb a capture
  parallel([&](int64_t i) {
    statuses[i] = ls_fd_prepare(handles[i], &opts[i]);
    if (statuses[i] < 0) errors[i] = ls_last_error();
  });
  for (int64_t i = 0; i < count; ++i)
    if (statuses[i] < 0) {
      ls::set_error("model %lld: %s", (long long)i, errors[i].c_str());
      return statuses[i];
    }
  // phase 2: the solves (graph captures and replays on per-model streams)
  parallel([&](int64_t i) {
    statuses[i] = ls_fd_solve(handles[i], &opts[i], d_x[i], &stats[i], nullptr);
    if (statuses[i] < 0) errors[i] = ls_last_error();
  });
  for (int64_t i = 0; i < count; ++i)
    if (statuses[i] < 0) {
      ls::set_error("model %lld: %s", (long long)i, errors[i].c_str());
      return statuses[i];
    }
  return LS_OK;
}
