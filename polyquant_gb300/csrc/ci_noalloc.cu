// pq_ci_sigma_noalloc: the sigma entry point for callers that may not
// allocate device memory during the compute phase.
//
// pq_ci_sigma converts the caller's column-major vectors into two interleaved
// work vectors that the handle grows with cudaMalloc on demand.  Some hosts
// cannot allow that: a driver whose device memory is entirely pre-reserved by
// its own pool, code that must not trigger the implicit device
// synchronisation of cudaMalloc/cudaFree in a latency-critical loop, or a
// solver that records its iteration into a CUDA graph.  For them this entry
// point uses a fixed scratch array compiled into the library instead.
//
// Limits and rules (also in include/pq_ci.h):
//  * scratch = 2 x 16 MiB in a file-scope __device__ array; every GPU that
//    loads the library holds it until the process exits;
//  * one 4-vector block of the interleaved work vectors must fit 16 MiB:
//    n_dets * width * sizeof(T) <= 16 MiB (width 1, 2 or 4; T = double or
//    float), larger problems are rejected with PQ_ERR_ARG;
//  * the device address of the array is looked up once per CUDA context, on
//    the first call made in that context; make that first call before any
//    stream capture.  A cudaDeviceReset destroys the context and can move the
//    array, so the library must not be used across one;
//  * all calls share the one array: calls that overlap on the GPU (other
//    streams or threads) race and must be serialised by the caller.
// Nothing in the array has to start at zero: each call writes every element
// of the work vectors it reads (the padding lanes included) before use.
#include <cuda.h>  // CUcontext (the type only; the driver call is reached through the runtime)

#include <mutex>
#include <utility>
#include <vector>

#include "pq_internal.h"

namespace pq {

constexpr size_t kNoAllocHalfBytes = size_t(16) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[2 * kNoAllocHalfBytes];

static std::mutex g_noalloc_mu;
// (context, device address of the array in it): a module, and so the array,
// is loaded once per context, so the address is cached per context rather
// than per device ordinal (a driver-API caller may make its own context
// current on a device whose primary context already loaded the library)
static std::vector<std::pair<CUcontext, void *>> g_noalloc_addr;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);

static pq_status current_context(CUcontext *ctx) {
  static CtxGetCurrentFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || !p || q != cudaDriverEntryPointSuccess) {
      set_error("pq_ci_sigma_noalloc: cuCtxGetCurrent not available (%s)", cudaGetErrorString(e));
      return PQ_ERR_CUDA;
    }
    fn = (CtxGetCurrentFn)p;
  }
  *ctx = nullptr;
  if (fn(ctx) != CUDA_SUCCESS) {
    set_error("pq_ci_sigma_noalloc: cuCtxGetCurrent failed");
    return PQ_ERR_CUDA;
  }
  return PQ_OK;
}

// Device address of the scratch array in the current context (looked up once
// per context, with that context current).
static pq_status noalloc_scratch(void **out) {
  int dev = -1;
  PQ_CUDA_TRY(cudaGetDevice(&dev));
  CUcontext ctx = nullptr;
  PQ_TRY(current_context(&ctx));
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (ctx)
    for (const auto &e : g_noalloc_addr)
      if (e.first == ctx) {
        *out = e.second;
        return PQ_OK;
      }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    set_error("pq_ci_sigma_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev, cudaGetErrorString(e));
    return PQ_ERR_CUDA;
  }
  // with no context current before, the lookup made the device's primary context current
  if (!ctx) PQ_TRY(current_context(&ctx));
  for (const auto &c : g_noalloc_addr)
    if (c.first == ctx) {
      *out = c.second;
      return PQ_OK;
    }
  g_noalloc_addr.emplace_back(ctx, p);
  *out = p;
  return PQ_OK;
}

}  // namespace pq

using namespace pq;

extern "C" pq_status pq_ci_sigma_noalloc(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S,
                                         int64_t lds, int32_t precision) {
  clear_error();
  if (!h || !C || !S || nvec < 1 || ldc < h->n_dets || lds < h->n_dets) {
    set_error("pq_ci_sigma_noalloc: bad arguments (nvec=%d, ldc=%lld, lds=%lld)", nvec, (long long)ldc,
              (long long)lds);
    return PQ_ERR_ARG;
  }
  if (precision != PQ_FP64 && precision != PQ_FP32) {
    set_error("pq_ci_sigma_noalloc: precision must be PQ_FP64 or PQ_FP32");
    return PQ_ERR_ARG;
  }
  const size_t esz = precision == PQ_FP64 ? sizeof(double) : sizeof(float);
  const int width = nvec >= 3 ? 4 : nvec;  // widest block this call will use
  const size_t need = esz * (size_t)width * (size_t)h->n_dets;
  if (need > kNoAllocHalfBytes) {
    set_error("pq_ci_sigma_noalloc: %lld determinants x %d vectors x %zu bytes = %zu bytes exceeds the fixed "
              "16 MiB scratch (use pq_ci_sigma)",
              (long long)h->n_dets, width, esz, need);
    return PQ_ERR_ARG;
  }
  void *base = nullptr;
  PQ_TRY(noalloc_scratch(&base));
  void *X = base;
  void *Y = static_cast<unsigned char *>(base) + kNoAllocHalfBytes;
  for (int v0 = 0; v0 < nvec; v0 += 4) {
    int nv = nvec - v0 < 4 ? nvec - v0 : 4;
    int nvp = nv == 1 ? 1 : (nv == 2 ? 2 : 4);
    PQ_TRY(ci_to_il(h, C, ldc, v0, nv, nvp, precision, X));
    PQ_TRY(ci_sigma_il(h, X, Y, nvp, precision, 0.0, /*allow_scratch=*/false));
    PQ_TRY(ci_from_il(h, Y, v0, nv, nvp, precision, S, lds));
  }
  return PQ_OK;
}
