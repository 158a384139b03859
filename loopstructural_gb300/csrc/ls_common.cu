// Error reporting and device queries shared by all translation units.
#include <stdarg.h>

#include "ls_common.cuh"

namespace ls {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cache[dev] = n;
  }
  return cache[dev];
}

}  // namespace ls

extern "C" const char *ls_last_error(void) { return ls::g_err; }
extern "C" int ls_abi_version(void) { return LS_ABI_VERSION; }
