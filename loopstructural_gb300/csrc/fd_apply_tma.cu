// Host side of the TMA-staged finest-level apply (fd_apply_tma.cuh): tensor-map
// encoding through the driver entry point, eligibility, launch geometry.
#include <cudaTypedefs.h>

#include <stdlib.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "fd_apply_tma.cuh"

namespace ls {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;

void resolve_encoder() {
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess && fn != nullptr)
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  cudaGetLastError();  // a failed lookup leaves no sticky error behind
}

bool encode(CUtensorMap *out, const float *base, int nx, int ny, int nz, int kind) {
  if (g_encode == nullptr || (reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * sizeof(float), (cuuint64_t)nx * ny * sizeof(float)};
  const cuuint32_t box[3] = {kind == 0 ? (cuuint32_t)kTmPX : (cuuint32_t)kTmX,
                             kind == 0 ? (cuuint32_t)kTmPY : (cuuint32_t)kTmY, 1u};
  const cuuint32_t estride[3] = {1u, 1u, 1u};
  const CUresult r = g_encode(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box,
                              estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

const CUtensorMap *lookup(TmCache &cache, const float *ptr, int kind) {
  for (const auto &en : cache.entries)
    if (en.ptr == ptr && en.kind == kind) return &en.map;
  TmCache::Entry en;
  en.ptr = ptr;
  en.kind = kind;
  if (!encode(&en.map, ptr, cache.nx, cache.ny, cache.nz, kind)) return nullptr;
  cache.entries.push_back(en);
  return &cache.entries.back().map;
}

template <int EPI, int ZU>
void set_attributes_zu() {
  cudaFuncSetAttribute(fd_tma_apply_kernel<EPI, ZU>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       tm_smem_bytes<EPI>());
  cudaFuncSetAttribute(fd_tma_apply_kernel<EPI, ZU>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

template <int EPI>
void set_attributes() {
  set_attributes_zu<EPI, 1>();
  set_attributes_zu<EPI, 2>();
}

}  // namespace

void tm_setup(TmCache &cache, int nx, int ny, int nz, bool allow) {
  cache.entries.clear();
  cache.nx = nx;
  cache.ny = ny;
  cache.nz = nz;
  std::call_once(g_encode_once, resolve_encoder);
  // rows of a multiple of 16 bytes; every axis long enough for the 5-plane
  // window; extents the launch geometry can address
  cache.enabled = allow && g_encode != nullptr && nx % 4 == 0 && nx >= 8 && ny >= 8 && nz >= 8 &&
                  (int64_t)nx * ny * nz < (int64_t)2000000000;
  // segments per column tile: LS_GB300_TMA_SEGMENTS overrides the one-wave default
  const char *seg = getenv("LS_GB300_TMA_SEGMENTS");
  cache.segments = seg ? std::max(0, atoi(seg)) : 0;
  const char *step = getenv("LS_GB300_TMA_STEP");
  cache.zu = (step && (atoi(step) == 1 || atoi(step) == 2)) ? atoi(step) : 0;
  if (cache.enabled) {
    set_attributes<EPI_STORE>();
    set_attributes<EPI_CHEB>();
    set_attributes<EPI_RESID>();
    cudaGetLastError();
  }
}

template <int EPI>
int tm_launch(TmCache &cache, const CoefT<float> &c, const float *p, const TmData &d, const EpiArgs<float> &e,
              const int *done, double *partials, unsigned int *ticket, double *dot, double *dot_clear, int *fault,
              int max_blocks, cudaStream_t st, int parts) {
  if (!cache.enabled || c.nx != cache.nx || c.ny != cache.ny || c.nz != cache.nz) return 0;
  TmMaps maps;
  const CUtensorMap *mp = lookup(cache, p, 0);
  if (mp == nullptr) return 0;
  maps.p = *mp;
  const float *opnd[3] = {nullptr, nullptr, nullptr};
  if (EPI == EPI_CHEB) {
    opnd[0] = e.x;
    opnd[1] = e.r;
    opnd[2] = e.dinv;
  } else if (EPI == EPI_RESID) {
    opnd[0] = e.b;
    opnd[1] = e.dinv;
  }
  for (int k = 0; k < TmOps<EPI>::n; ++k) {
    const CUtensorMap *m = lookup(cache, opnd[k], 1);
    if (m == nullptr) return 0;
    maps.op[k] = *m;
  }
  const int ntx = (c.nx + kTmX - 1) / kTmX, nty = (c.ny + kTmY - 1) / kTmY;
  const int64_t ntiles = (int64_t)ntx * nty;
  const int64_t slots = (int64_t)kTmBlocksPerSm * sm_count();
  // segments of ~16 planes (several waves of blocks, so that the tiles with
  // boundary columns, which cost more per plane, do not set the makespan), at
  // least enough to fill every SM once
  int64_t nseg = cache.segments > 0
                     ? cache.segments
                     : std::max<int64_t>((c.nz + 15) / 16, std::max<int64_t>(1, slots / std::max<int64_t>(1, ntiles)));
  const int zlen = (int)((c.nz + nseg - 1) / nseg);
  nseg = (c.nz + zlen - 1) / zlen;
  if (ntiles > 0x7fffffff || (dot != nullptr && ntiles * nseg > max_blocks)) return 0;
  int launched = 0;
  if (parts & TM_APPLY) {
    const dim3 grid((unsigned)ntiles, (unsigned)nseg);
    if (cache.zu == 2)
      fd_tma_apply_kernel<EPI, 2><<<grid, kTmThreads, tm_smem_bytes<EPI>(), st>>>(maps, c, e, done, ntx, zlen,
                                                                                   partials, ticket, dot, dot_clear,
                                                                                   fault);
    else
      fd_tma_apply_kernel<EPI, 1><<<grid, kTmThreads, tm_smem_bytes<EPI>(), st>>>(maps, c, e, done, ntx, zlen,
                                                                                   partials, ticket, dot, dot_clear,
                                                                                   fault);
    ++launched;
  }
  if ((parts & TM_DATA) && d.ntouched > 0) {
    rows_kernel<float><<<stream_grid(d.nrows, 256), 256, 0, st>>>(d.nrows, d.width, d.cols, d.a, d.w2, p, d.s, done);
    // the fix-up's dot partials reuse the apply's (it runs after the apply)
    data_fixup_kernel<EPI><<<(int)std::min<int64_t>(stream_grid(d.ntouched, 256), max_blocks > 0 ? max_blocks : 1024),
                             256, 0, st>>>(d.ntouched, d.touched, d.inc_ptr, d.inc_row, d.inc_a, d.s, p, e, done,
                                           partials, ticket, dot);
    launched += 2;
  }
  LS_CUDA_TRY(cudaGetLastError());
  return launched;
}

int tm_autotune(TmCache &cache, const CoefT<float> &c, const float *p, float *q, int *fault, cudaStream_t st) {
  if (!cache.enabled || cache.zu != 0) return LS_OK;
  const TmData none{};
  EpiArgs<float> e{};
  e.q = q;
  cudaEvent_t a, b;
  LS_CUDA_TRY(cudaEventCreate(&a));
  LS_CUDA_TRY(cudaEventCreate(&b));
  float best = 0.f;
  int pick = 1;
  for (int zu = 1; zu <= 2; ++zu) {
    cache.zu = zu;
    int st1 = tm_launch<EPI_STORE>(cache, c, p, none, e, nullptr, nullptr, nullptr, nullptr, nullptr, fault, 0, st,
                                   TM_APPLY);
    if (st1 <= 0) break;  // the maps could not be encoded: the launch path stays off
    cudaEventRecord(a, st);
    for (int r = 0; r < 5; ++r)
      tm_launch<EPI_STORE>(cache, c, p, none, e, nullptr, nullptr, nullptr, nullptr, nullptr, fault, 0, st, TM_APPLY);
    cudaEventRecord(b, st);
    LS_CUDA_TRY(cudaEventSynchronize(b));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (zu == 1 || ms < best) {
      best = ms;
      pick = zu;
    }
  }
  cache.zu = pick;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  LS_CUDA_TRY(cudaGetLastError());
  return LS_OK;
}

#define LS_TM_INST(EPI)                                                                                           \
  template int tm_launch<EPI>(TmCache &, const CoefT<float> &, const float *, const TmData &,                    \
                              const EpiArgs<float> &, const int *, double *, unsigned int *, double *, double *, \
                              int *, int, cudaStream_t, int);
LS_TM_INST(EPI_STORE)
LS_TM_INST(EPI_CHEB)
LS_TM_INST(EPI_RESID)
#undef LS_TM_INST

}  // namespace ls
