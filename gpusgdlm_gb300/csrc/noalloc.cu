// sgdlm_log_det_noalloc: log|det(I - Gamma_i)| of a batch of draws without any
// device allocation.
//
// Who needs this: code that must not call cudaMalloc -- for example a host
// process that hands this library device buffers owned by another allocator
// (a framework's caching allocator, a memory pool it must stay inside), code
// running where allocation is forbidden or unsafe (inside a latency-critical
// loop, or after the application has reserved all device memory up front).
// Such callers provide the draws, the parental sets and the output arrays; the
// batched LU's per-CTA working matrices come from the static array below.
//
// The array is a file-scope __device__ buffer of kNoAllocScratchBytes (16 MiB)
// that every GPU which loads this library holds until the process exits.  The
// binding limit on m is the LU kernels' shared memory, not the array: the fast
// pass keeps a (m rounded up to 32)-row panel set in shared memory, which fits
// the 227 KB a block may use up to m = 736 (kNoAllocMaxM, checked against the
// kernels' own plan on every call).  A 736-series working matrix takes 2.2 MB,
// so 7 of them fit the array; fewer matrices in flight means fewer CTAs for
// large m.  All calls on a device share the array: it keeps whatever the last
// call left there (each draw's matrix is rebuilt from scratch, so nothing needs
// clearing between calls), and calls whose kernels overlap on the GPU -- on two
// streams, or from two threads -- race on it and must be serialised by the
// caller.
//
// Host code cannot use the array's name as a device address (on the host it
// names a shadow variable), so the first call in each CUDA context looks the
// address up with cudaGetSymbolAddress while that context is current, and
// caches it under the context's process-unique ID (a context created after
// cudaDeviceReset, or a second context on the same device, gets its own
// lookup).  Make that first call outside any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/sgdlm.h"
#include "elimination.hpp"
#include "kernels.hpp"

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr size_t kNoAllocMaxM = 736;
constexpr size_t kSmemLimit = 227 * 1024 - 64;

__device__ __align__(256) unsigned char g_logdet_scratch[kNoAllocScratchBytes];

// (context ID, device address of g_logdet_scratch in that context)
std::vector<std::pair<unsigned long long, void *>> g_scratch_addr;
std::mutex g_scratch_mu;

int reject(int status, const char *msg) {
  fprintf(stderr, "Error: sgdlm_log_det_noalloc: %s\n", msg);
  return status;
}

// ID of the calling thread's current CUDA context (the runtime's primary
// context of the current device once the runtime has initialised it).  The
// driver functions come through the runtime's entry-point query, so the
// library does not link the driver library itself.
bool current_context_id(unsigned long long *id) {
  using GetCurrent = CUresult (*)(CUcontext *);
  using GetId = CUresult (*)(CUcontext, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  if (!get_current || !get_id) {
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
            cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess ||
        q2 != cudaDriverEntryPointSuccess)
      return false;
    get_current = reinterpret_cast<GetCurrent>(f1);
    get_id = reinterpret_cast<GetId>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

}  // namespace

extern "C" int sgdlm_log_det_noalloc(size_t m, size_t max_p, size_t n, const float *d_theta,
                                     const unsigned *d_sp, double *d_log_det, int *d_flags,
                                     void *stream) {
  using namespace sgdlm;
  if (!d_theta || !d_sp || !d_log_det || !d_flags) return reject(SGDLM_ERR_BAD_ARG, "null pointer");
  if (m < 1 || max_p < 1 || n < 1) return reject(SGDLM_ERR_BAD_DIM, "m, max_p and n must be positive");
  if (max_p > 64) return reject(SGDLM_ERR_UNSUPPORTED, "max_p above 64 is not supported");
  if (n > 0x7FFFFFFFu) return reject(SGDLM_ERR_UNSUPPORTED, "n above 2^31 - 1 is not supported");
  if (m > kNoAllocMaxM) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "m = %zu is above this entry point's limit of %zu series (the LU block's shared "
             "memory)", m, kNoAllocMaxM);
    return reject(SGDLM_ERR_UNSUPPORTED, buf);
  }
  const size_t mp = (m + 31) / 32 * 32;
  const size_t slab = mp * mp * sizeof(float);
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return reject(SGDLM_ERR_DEVICE, "no usable current device");
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return reject(SGDLM_ERR_DEVICE, "cannot query the device");
  // no elimination plan here (planning needs host memory and a device upload):
  // the whole matrix is the dense core, scattered straight from d_sp
  LuPlan pl = plan_lu<float>((int)m, (int)max_p, (long)n, sms, (int)m, 0);
  if (pl.smem > kSmemLimit || pl.smem_fallback > kSmemLimit || slab > kNoAllocScratchBytes)
    return reject(SGDLM_ERR_UNSUPPORTED, "m too large for one LU block");
  const long max_ctas = (long)(kNoAllocScratchBytes / slab);
  if (pl.grid > max_ctas) pl.grid = (int)max_ctas;
  if (pl.fb_grid > max_ctas) pl.fb_grid = (int)max_ctas;
  unsigned long long ctx_id = 0;
  if (!current_context_id(&ctx_id)) {
    // no context is current on this thread yet: the runtime's symbol lookup sets
    // up the current device's primary context and makes it current
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_logdet_scratch) != cudaSuccess || !current_context_id(&ctx_id))
      return reject(SGDLM_ERR_DEVICE, "no current CUDA context");
  }
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    for (const auto &e : g_scratch_addr)
      if (e.first == ctx_id) scratch = e.second;
    if (!scratch) {
      const cudaError_t e = cudaGetSymbolAddress(&scratch, g_logdet_scratch);
      if (e != cudaSuccess || !scratch) {
        fprintf(stderr, "Error: sgdlm_log_det_noalloc: cudaGetSymbolAddress: %s\n",
                cudaGetErrorString(e));
        return SGDLM_ERR_DEVICE;
      }
      g_scratch_addr.emplace_back(ctx_id, scratch);
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemsetAsync(d_flags, 0, n * sizeof(int), s) != cudaSuccess)
    return reject(SGDLM_ERR_DEVICE, "cannot clear the flag array");
  const RngKey no_key{0, 0, 0, nullptr};
  const GammaRows no_rows{nullptr, nullptr, nullptr, nullptr};
  EliminationPlan no_plan{};
  no_plan.m = (int)m;
  no_plan.P = (int)max_p;
  no_plan.core_n = (int)m;
  launch_lu<float>(s, pl, (long)n, no_plan, d_sp, d_theta, nullptr, (float *)scratch, d_log_det,
                   d_flags,
                   nullptr, nullptr, no_key, false, nullptr, no_rows);
  launch_lu_fallback<float>(s, pl, (long)n, no_plan, d_sp, d_theta, nullptr, (float *)scratch, d_log_det,
                            d_flags,
                            nullptr, nullptr, no_key, nullptr, no_rows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "Error: sgdlm_log_det_noalloc: %s\n", cudaGetErrorString(e));
    return SGDLM_ERR_DEVICE;
  }
  return SGDLM_OK;
}
