// Per-series state kernels: the conjugate posterior update, the discount prior
// step, the per-series Cholesky factor and the device-side ESS gate.
//
// The reference runs the posterior as 11 launches (six element-wise kernels and
// four pointer-array DgemmBatched calls, rSGDLM/src/SGDLM/SGDLM.cu:10-113).  Here
// one warp owns one series: the P x P covariance is read once, coalesced over
// rows, and every intermediate (A, Q, e) stays in registers or the warp's slice
// of shared memory.  All arithmetic is FP64, as the covariance update
// C = (R - A A' Q) needs it to stay positive definite.
#include <algorithm>

#include "kernels.hpp"

namespace sgdlm {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// rSGDLM/src/SGDLM/SGDLM.cu:10-113 in one pass; the masking follows
// batchedCutOffVector (kernel_functions.cuh:86-95) and the row-AND-column cut of
// batchedCutOffMatrix (kernel_functions.cuh:98-110).
__global__ void k_posterior(int m, int P, const unsigned *__restrict__ p,
                            double *__restrict__ m_t, double *__restrict__ C_t,
                            double *__restrict__ n_t, double *__restrict__ s_t,
                            const double *__restrict__ y, const double *__restrict__ F) {
  extern __shared__ double sh[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + warp;
  if (j >= m) return;
  double *A = sh + (size_t)warp * 3 * P;
  double *Fj = A + P;
  double *mj = Fj + P;
  const unsigned pj = p[j];
  double *Cj = C_t + (size_t)j * P * P;
  double *mt = m_t + (size_t)j * P;

  for (int r = lane; r < P; r += 32) {
    const double v = ((unsigned)r >= pj) ? 0.0 : mt[r];
    mj[r] = v;
    Fj[r] = F[(size_t)j * P + r];
  }
  for (int e = lane; e < P * P; e += 32) {
    const int r = e % P, c = e / P;
    if ((unsigned)r >= pj && (unsigned)c >= pj) Cj[e] = 0.0;
  }
  __syncwarp();
  // A = R F over the full P x P block (cuBLAS gemm at SGDLM.cu:41-43)
  for (int r = lane; r < P; r += 32) {
    double acc = 0.0;
    for (int c = 0; c < P; ++c) acc = fma(Cj[r + P * c], Fj[c], acc);
    A[r] = acc;
  }
  __syncwarp();
  double q = 0.0, fm = 0.0;
  for (int r = lane; r < P; r += 32) {
    q = fma(Fj[r], A[r], q);
    fm = fma(Fj[r], mj[r], fm);
  }
  q = warp_sum(q);
  fm = warp_sum(fm);
  const double Q = s_t[j] + q;         // Q = c + F'A      (SGDLM.cu:47-54)
  const double e = y[j] - fm;          // e = y - F'a      (SGDLM.cu:69-74)
  const double n_new = n_t[j] + 1.0;   // n = r + 1        (SGDLM.cu:78)
  const double e2q = e * e / Q;
  const double sqQ = sqrt(Q);
  for (int r = lane; r < P; r += 32) {
    const double a = A[r] / Q;         // A /= Q           (SGDLM.cu:63)
    mt[r] = mj[r] + e * a;             // m = a + A e      (SGDLM.cu:91)
    A[r] = a * sqQ;                    // A *= sqrt(Q)     (SGDLM.cu:97)
  }
  __syncwarp();
  const double fac = ((n_new - 1.0) + e2q) / n_new;  // kernel_functions.cuh:393-401
  for (int ix = lane; ix < P * P; ix += 32) {
    const int r = ix % P, c = ix / P;
    Cj[ix] = (Cj[ix] - A[r] * A[c]) * fac;  // C = (R - A A') (r + e^2/Q)/n
  }
  if (lane == 0) {
    s_t[j] = s_t[j] * (n_new - 1.0 + e2q) / n_new;  // kernel_functions.cuh:480-487
    n_t[j] = n_new;
  }
}

// r = beta n; inside the leading p x p block W = C (1/Delta - 1) and R = C / Delta
// (batchedMatrixScaleWithDiff, kernel_functions.cuh:259-288; multiply :438-444).
__global__ void k_prior(int m, int P, const unsigned *__restrict__ p,
                        double *__restrict__ C_t, double *__restrict__ n_t,
                        double *__restrict__ W_t, const double *__restrict__ beta,
                        const double *__restrict__ delta) {
  const size_t PP = (size_t)P * P;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= PP * m) return;
  const int j = (int)(idx / PP);
  const int e = (int)(idx % PP);
  const int r = e % P, c = e / P;
  const unsigned pj = p[j];
  if ((unsigned)r < pj && (unsigned)c < pj) {
    const double v = C_t[idx];
    const double d = delta[idx];
    W_t[idx] = v * (1.0 / d - 1.0);
    C_t[idx] = v / d;
  }
  if (e == 0) n_t[j] = n_t[j] * beta[j];
}

// Upper Cholesky factor with the reference's update order
// (kernel_functions.cuh:845-902), warp per series.  Each element receives the
// same sequence of floating-point operations as the reference's one-thread
// loop, so the factor is bit-identical to it.
__global__ void k_cholesky(int m, int P, const unsigned *__restrict__ p,
                           const double *__restrict__ C, double *__restrict__ U64,
                           float *__restrict__ U32) {
  extern __shared__ double sh[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + warp;
  if (j >= m) return;
  double *a = sh + (size_t)warp * P * P;  // a[row + P*col]
  const double *Cj = C + (size_t)j * P * P;
  const int pj = (int)min((unsigned)P, p[j]);
  for (int ix = lane; ix < P * P; ix += 32) {
    const int r = ix % P, c = ix / P;
    a[ix] = (r < pj && c < pj && c >= r) ? Cj[ix] : 0.0;
  }
  __syncwarp();
  for (int n = 0; n < pj; ++n) {
    const double d = sqrt(a[n + P * n]);
    const double inv = 1.0 / d;
    __syncwarp();
    if (lane == 0) a[n + P * n] = d;
    for (int k = n + 1 + lane; k < pj; k += 32) {
      const double v = a[n + P * k] * inv;
      a[n + P * k] = v;
      a[k + P * k] -= v * v;
    }
    __syncwarp();
    const int rem = pj - n - 1;
    for (int q = lane; q < rem * rem; q += 32) {
      const int k = n + 1 + q % rem, l = n + 1 + q / rem;
      if (l > k) a[k + P * l] -= a[n + P * k] * a[n + P * l];
    }
    __syncwarp();
  }
  for (int ix = lane; ix < P * P; ix += 32) {
    const double v = a[ix];
    U64[(size_t)j * P * P + ix] = v;
    if (U32) U32[(size_t)j * P * P + ix] = (float)v;
  }
}

__global__ void k_gate(int m, int P, const double *__restrict__ stats, double threshold,
                       const double *__restrict__ mean_m, const double *__restrict__ mean_C,
                       const double *__restrict__ mean_n, const double *__restrict__ mean_s,
                       double *__restrict__ m_t, double *__restrict__ C_t,
                       double *__restrict__ n_t, double *__restrict__ s_t,
                       double *__restrict__ accepted) {
  const bool accept = stats[1] > threshold;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx == 0 && accepted) *accepted = accept ? 1.0 : 0.0;
  if (!accept) return;
  const size_t PP = (size_t)P * P;
  if (idx < PP * m) C_t[idx] = mean_C[idx];
  if (idx < (size_t)P * m) m_t[idx] = mean_m[idx];
  if (idx < (size_t)m) {
    n_t[idx] = mean_n[idx];
    s_t[idx] = mean_s[idx];
  }
}

__global__ void k_advance_epoch(uint32_t *dev_epoch, uint32_t delta) { *dev_epoch += delta; }

// Evolution-matrix step of the prior (compute_one_step_ahead_prior with G_t,
// SGDLM.cu:151-178): a = G m with the entries >= p zeroed, then R = (G R) G' with
// the entries whose row AND column are >= p zeroed (the cut-offs of
// kernel_functions.cuh:86-110).  One block per series; G, R and G R in shared
// memory; FP64.
__global__ void k_evo_prior(int m, int P, const unsigned *__restrict__ p,
                            double *__restrict__ m_t, double *__restrict__ C_t,
                            const double *__restrict__ G) {
  extern __shared__ double sh[];
  const size_t PP = (size_t)P * P;
  const int j = blockIdx.x;
  double *Gs = sh, *Rs = Gs + PP, *Ts = Rs + PP, *ms = Ts + PP;
  const double *Gj = G + (size_t)j * PP;
  double *Cj = C_t + (size_t)j * PP;
  for (int e = threadIdx.x; e < (int)PP; e += blockDim.x) {
    Gs[e] = Gj[e];
    Rs[e] = Cj[e];
  }
  for (int e = threadIdx.x; e < P; e += blockDim.x) ms[e] = m_t[(size_t)j * P + e];
  __syncthreads();
  const unsigned pj = p[j];
  for (int e = threadIdx.x; e < (int)PP; e += blockDim.x) {  // T = G R
    const int r = e % P, c = e / P;
    double acc = 0.0;
    for (int l = 0; l < P; ++l) acc += Gs[r + P * l] * Rs[l + P * c];
    Ts[e] = acc;
  }
  for (int r = threadIdx.x; r < P; r += blockDim.x) {  // a = G m
    double acc = 0.0;
    for (int l = 0; l < P; ++l) acc += Gs[r + P * l] * ms[l];
    m_t[(size_t)j * P + r] = ((unsigned)r < pj) ? acc : 0.0;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < (int)PP; e += blockDim.x) {  // R = T G'
    const int r = e % P, c = e / P;
    double acc = 0.0;
    for (int l = 0; l < P; ++l) acc += Ts[r + P * l] * Gs[c + P * l];
    Cj[e] = ((unsigned)r >= pj && (unsigned)c >= pj) ? 0.0 : acc;
  }
}

// Converts a double array to the working precision of the draws.
__global__ void k_to_float(size_t n, const double *__restrict__ src, float *__restrict__ dst) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = (float)src[e];
}

}  // namespace

void launch_advance_epoch(cudaStream_t s, uint32_t *dev_epoch, uint32_t delta) {
  k_advance_epoch<<<1, 1, 0, s>>>(dev_epoch, delta);
}

void launch_posterior(cudaStream_t s, int m, int P, const unsigned *p, double *m_t,
                      double *C_t, double *n_t, double *s_t, const double *y,
                      const double *F) {
  const int warps = 4;
  const size_t smem = (size_t)warps * 3 * P * sizeof(double);
  k_posterior<<<(m + warps - 1) / warps, warps * 32, smem, s>>>(m, P, p, m_t, C_t, n_t,
                                                               s_t, y, F);
}

void launch_prior(cudaStream_t s, int m, int P, const unsigned *p, double *C_t,
                  double *n_t, double *W_t, const double *beta, const double *delta) {
  const size_t total = (size_t)P * P * m;
  const int bs = 256;
  k_prior<<<(unsigned)((total + bs - 1) / bs), bs, 0, s>>>(m, P, p, C_t, n_t, W_t, beta,
                                                            delta);
}

void launch_evo_prior(cudaStream_t s, int m, int P, const unsigned *p, double *m_t,
                      double *C_t, const double *G) {
  const size_t smem = (3 * (size_t)P * P + P) * sizeof(double);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_evo_prior, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_evo_prior<<<m, 128, smem, s>>>(m, P, p, m_t, C_t, G);
}

void launch_to_float(cudaStream_t s, size_t n, const double *src, float *dst) {
  k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, dst);
}

void launch_cholesky(cudaStream_t s, int m, int P, const unsigned *p, const double *C,
                     double *U64, float *U32) {
  // one P x P FP64 slice per warp; keep the block under the default 48 KB
  const size_t per_warp = (size_t)P * P * sizeof(double);
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(4, (48 * 1024) / per_warp));
  const size_t smem = (size_t)warps * per_warp;
  k_cholesky<<<(m + warps - 1) / warps, warps * 32, smem, s>>>(m, P, p, C, U64, U32);
}

void launch_gate(cudaStream_t s, int m, int P, const double *stats, double threshold,
                 const double *mean_m, const double *mean_C, const double *mean_n,
                 const double *mean_s, double *m_t, double *C_t, double *n_t,
                 double *s_t, double *accepted) {
  const size_t total = (size_t)P * P * m;
  const int bs = 256;
  k_gate<<<(unsigned)((total + bs - 1) / bs), bs, 0, s>>>(
      m, P, stats, threshold, mean_m, mean_C, mean_n, mean_s, m_t, C_t, n_t, s_t,
      accepted);
}

}  // namespace sgdlm
