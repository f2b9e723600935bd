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
// that every GPU which loads this library holds until the process exits.  One
// LU working matrix of (m rounded up to 32)^2 floats must fit in it, so m is at
// most 2048; fewer matrices in flight means fewer CTAs for large m.  All calls
// on a device share the array: it keeps whatever the last call left there (each
// draw's matrix is rebuilt from scratch, so nothing needs clearing between
// calls), and calls whose kernels overlap on the GPU -- on two streams, or from
// two threads -- race on it and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (on the host it
// names a shadow variable), so the first call on each device looks the
// address up with cudaGetSymbolAddress while that device is current and caches
// it.  Make that first call outside any stream capture.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/sgdlm.h"
#include "elimination.hpp"
#include "kernels.hpp"

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_logdet_scratch[kNoAllocScratchBytes];

void *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

int reject(int status, const char *msg) {
  fprintf(stderr, "Error: sgdlm_log_det_noalloc: %s\n", msg);
  return status;
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
  const size_t mp = (m + 31) / 32 * 32;
  const size_t slab = mp * mp * sizeof(float);
  if (slab > kNoAllocScratchBytes) {
    char buf[160];
    snprintf(buf, sizeof buf,
             "m = %zu needs a %zu-byte working matrix; the static scratch holds %zu bytes "
             "(m <= 2048)", m, slab, kNoAllocScratchBytes);
    return reject(SGDLM_ERR_UNSUPPORTED, buf);
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return reject(SGDLM_ERR_DEVICE, "no usable current device");
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return reject(SGDLM_ERR_DEVICE, "cannot query the device");
  // no elimination plan here (planning needs host memory and a device upload):
  // the whole matrix is the dense core, scattered straight from d_sp
  LuPlan pl = plan_lu<float>((int)m, (int)max_p, (long)n, sms, (int)m, 0);
  if (pl.smem > 227 * 1024 - 64) return reject(SGDLM_ERR_UNSUPPORTED, "m too large for one LU block");
  const long max_ctas = (long)(kNoAllocScratchBytes / slab);
  if (pl.grid > max_ctas) pl.grid = (int)max_ctas;
  if (pl.fb_grid > max_ctas) pl.fb_grid = (int)max_ctas;
  void *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_logdet_scratch);
      if (e != cudaSuccess) {
        fprintf(stderr, "Error: sgdlm_log_det_noalloc: cudaGetSymbolAddress: %s\n",
                cudaGetErrorString(e));
        return SGDLM_ERR_DEVICE;
      }
      g_scratch_addr[dev] = p;
    }
    scratch = g_scratch_addr[dev];
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
  launch_lu_fallback<float>(s, pl, (long)n, d_sp, d_theta, nullptr, (float *)scratch, d_log_det,
                            d_flags,
                            nullptr, nullptr, no_key, nullptr, no_rows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "Error: sgdlm_log_det_noalloc: %s\n", cudaGetErrorString(e));
    return SGDLM_ERR_DEVICE;
  }
  return SGDLM_OK;
}
