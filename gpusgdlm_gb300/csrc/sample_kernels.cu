// Draw generation: (lambda, theta) from the per-series normal-gamma posterior or
// prior, and the multi-step evolution of forecast draws.
//
// The reference samples with four cuRAND calls into HBM caches, a Marsaglia-Tsang
// kernel with atomic slot compaction, a one-thread-per-series Cholesky and a
// pointer-array gemmBatched of batch m*n for theta = U' z
// (rSGDLM/src/SGDLM/SGDLM.cu:623-677).  Here one thread owns one (draw, series)
// pair: its normals come out of Philox in registers, U_j sits in shared memory
// (every thread of the block shares series j, so reads are broadcasts), and the
// block's theta rows are staged in shared memory so the series-major store is one
// contiguous coalesced run.  From the same staged rows the block writes its draws'
// Gamma entries to the draw-major Gamma copy (GammaDraws), which the LU and
// iterative-solve kernels read as one run per draw.
#include "kernels.hpp"
#include "rng.cuh"

namespace sgdlm {
namespace {

constexpr int kSampleThreads = 128;

// The series' Gamma coefficients: k of the c-th entry of its row (gks[c], the k
// with a simultaneous parent, sp[j*P + k] < m*m, in increasing k), their count and
// the row's first position in the CSR order.  One whole warp: lane l tests k = l,
// l + 32 (P <= 64) and places its k by a ballot of the lanes before it.
__device__ __forceinline__ void gamma_row_of(const unsigned *__restrict__ sp, const int *rowptr,
                                             int j, int P, unsigned mm, int *gks, int *gcnt,
                                             int *gq0) {
  const int lane = threadIdx.x & 31;
  int base = 0;
  for (int k0 = 0; k0 < P; k0 += 32) {
    const int k = k0 + lane;
    const bool g = k < P && sp[(size_t)j * P + k] < mm;
    const unsigned mask = __ballot_sync(0xffffffffu, g);
    if (g) gks[base + __popc(mask & ((1u << lane) - 1u))] = k;
    base += __popc(mask);
  }
  if (lane == 0) {
    *gcnt = base;
    *gq0 = rowptr[j];
  }
}

// The block's draws i0 .. i0 + cnt - 1 of series j, staged row by row (P values
// per draw), to their Gamma runs of the draw-major copy (GammaDraws: draw i's run
// at v[i*nnz + q0 ..]).  Consecutive threads take consecutive entries, so a warp
// writes the runs of several draws at once.
template <typename T>
__device__ __forceinline__ void write_gamma_runs(const GammaDraws<T> &gd, int P, long i0, int cnt,
                                                 const T *stage, const int *gks, int gcnt,
                                                 int gq0) {
  const int tot = cnt * gcnt;
  for (int x = threadIdx.x; x < tot; x += blockDim.x) {
    const int t = x / gcnt, c = x - t * gcnt;
    gd.v[(size_t)(i0 + t) * gd.nnz + gq0 + c] = stage[(size_t)t * P + gks[c]];
  }
}

template <typename T, int PMAX>
__global__ void __launch_bounds__(kSampleThreads)
    k_sample(int m, int P, long n, const double *__restrict__ m_t,
             const double *__restrict__ n_t, const double *__restrict__ s_t,
             const T *__restrict__ U, RngKey key, T *__restrict__ lambda,
             T *__restrict__ theta, GammaDraws<T> gd, int *__restrict__ draw_flags,
             const unsigned *__restrict__ p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Us = reinterpret_cast<T *>(smem_raw);  // P*P, U[row + P*col]
  T *ms = Us + P * P;                       // P
  T *stage = ms + P;                        // blockDim.x * P
  __shared__ T ser[3];                      // the series' gamma shape and rate, s_j
  __shared__ int gks[64], gcnt, gq0;        // its Gamma coefficients (gamma_row_of)
  const int j = blockIdx.y;
  // the series' active coefficients: U_j is zero outside its leading pj x pj
  // block (the Cholesky factor's cut), so theta_k = m_k exactly for k >= pj and
  // the normals z_l, l >= pj, are never used; they are not generated (counter-based
  // streams: the others do not move)
  const int pj = p ? min((int)p[j], P) : P;
  for (int e = threadIdx.x; e < P * P; e += blockDim.x) Us[e] = U[(size_t)j * P * P + e];
  for (int e = threadIdx.x; e < P; e += blockDim.x) ms[e] = (T)m_t[(size_t)j * P + e];
  if (gd.v && (threadIdx.x >> 5) == 1)  // warp 1 (thread 0 sets up ser)
    gamma_row_of(gd.sp, gd.rowptr, j, P, (unsigned)m * (unsigned)m, gks, &gcnt, &gq0);
  if (threadIdx.x == 0) {
    // FP64 once per series (FP64 is a narrow pipe on this GPU)
    const double nj = n_t[j], sj = s_t[j];
    ser[0] = (T)(0.5 * nj);
    ser[1] = (T)(0.5 * nj * sj);
    ser[2] = (T)sj;
  }
  __syncthreads();
  const long i0 = (long)blockIdx.x * blockDim.x;
  const long i = i0 + threadIdx.x;
  if (i < n) {
    const uint32_t ep = key_epoch(key);
    const T alpha = ser[0], rate = ser[1];
    bool fail = false;
    const T lam = gamma_mt<T>(alpha, (uint32_t)i, (uint32_t)j, TAG_GAMMA, ep, key.k0,
                              key.k1, false, &fail) / rate;
    T z[PMAX];
#pragma unroll
    for (int q = 0; q < PMAX / 4; ++q) {
      if (4 * q < pj) {
        const U4 r = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_THETA, q), ep, key.k0, key.k1);
        box_muller<T>(r.x, r.y, z[4 * q], z[4 * q + 1]);
        box_muller<T>(r.z, r.w, z[4 * q + 2], z[4 * q + 3]);
      } else {
        z[4 * q] = z[4 * q + 1] = z[4 * q + 2] = z[4 * q + 3] = T(0);
      }
    }
    // theta = m + (U' z) / sqrt(s lambda)   (makeVB_MVN, kernel_functions.cuh:72-83);
    // one reciprocal instead of P divisions (within 1-2 ulp of the quotients)
    const T rden = T(1) / dev_sqrt(ser[2] * lam);
    T *row = stage + (size_t)threadIdx.x * P;
#pragma unroll
    for (int k = 0; k < PMAX; ++k) {
      if (k < P) {
        T acc = T(0);
        if (k < pj) {
#pragma unroll
          for (int l = 0; l <= k; ++l) acc += Us[l + P * k] * z[l];
        }
        row[k] = ms[k] + acc * rden;
      }
    }
    lambda[(size_t)j * n + i] = lam;
    if (fail) atomicOr(&draw_flags[i], DRAW_FLAG_GAMMA_CAP);
  }
  __syncthreads();
  if (gd.v) write_gamma_runs<T>(gd, P, i0, (int)min((long)blockDim.x, n - i0), stage, gks, gcnt, gq0);
  const long cnt = (long)min((long)blockDim.x, n - i0) * P;
  T *dst = theta + ((size_t)j * n + i0) * P;
  if (((size_t)j * n + i0) * P * sizeof(T) % 16 == 0 && cnt * sizeof(T) % 16 == 0 &&
      (reinterpret_cast<uintptr_t>(stage) & 15) == 0) {
    // 16-byte copies (the staged run, its length and its destination are aligned)
    constexpr int W = (int)(16 / sizeof(T));
    for (long e = (long)threadIdx.x * W; e < cnt; e += (long)blockDim.x * W)
      *reinterpret_cast<uint4 *>(dst + e) = *reinterpret_cast<const uint4 *>(stage + e);
  } else {
    for (long e = threadIdx.x; e < cnt; e += blockDim.x) dst[e] = stage[e];
  }
}

// eta ~ Beta(beta r/2, (1-beta) r/2) / beta via two gammas (make_gamma_1 and
// make_beta, kernel_functions.cuh:644-798); lambda *= eta (batchedMultiply
// :458-466); omega ~ N(0, I) scaled by 1/sqrt(c lambda) and cut at p
// (scale_omegas :986-1001); theta += U_W' omega (SGDLM.cu:755-758).
template <typename T, int PMAX>
__global__ void __launch_bounds__(kSampleThreads)
    k_evolve(int m, int P, long n, const unsigned *__restrict__ p,
             const double *__restrict__ r_t, const double *__restrict__ c_t,
             const double *__restrict__ beta, const T *__restrict__ UW, RngKey key,
             bool compat_unscaled, bool compat_no_boost, T *__restrict__ lambda,
             T *__restrict__ theta, GammaDraws<T> gd, int *__restrict__ draw_flags,
             const T *__restrict__ G) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Us = reinterpret_cast<T *>(smem_raw);
  T *Gs = Us + P * P;  // G_j when an evolution matrix is given
  T *stage = Gs + (G ? P * P : 0);
  __shared__ int gks[64], gcnt, gq0;  // the series' Gamma coefficients (gamma_row_of)
  const int j = blockIdx.y;
  if (gd.v && (threadIdx.x >> 5) == 0)
    gamma_row_of(gd.sp, gd.rowptr, j, P, (unsigned)m * (unsigned)m, gks, &gcnt, &gq0);
  const long i0 = (long)blockIdx.x * blockDim.x;
  const long cnt = (long)min((long)blockDim.x, n - i0) * P;
  T *src = theta + ((size_t)j * n + i0) * P;
  for (int e = threadIdx.x; e < P * P; e += blockDim.x) Us[e] = UW[(size_t)j * P * P + e];
  if (G)
    for (int e = threadIdx.x; e < P * P; e += blockDim.x) Gs[e] = G[(size_t)j * P * P + e];
  for (long e = threadIdx.x; e < cnt; e += blockDim.x) stage[e] = src[e];
  __syncthreads();
  const long i = i0 + threadIdx.x;
  if (i < n) {
    const uint32_t ep = key_epoch(key);
    const double bj = beta[j], rj = r_t[j];
    bool fail = false;
    T eta = T(1);
    if (bj != 1.0) {
      const T ga = gamma_mt<T>((T)(0.5 * bj * rj), (uint32_t)i, (uint32_t)j, TAG_BETA_A,
                               ep, key.k0, key.k1, compat_no_boost, &fail);
      const T gb = gamma_mt<T>((T)(0.5 * (1.0 - bj) * rj), (uint32_t)i, (uint32_t)j,
                               TAG_BETA_B, ep, key.k0, key.k1, compat_no_boost,
                               &fail);
      eta = (ga / (ga + gb)) / (T)bj;
    }
    const T lam = lambda[(size_t)j * n + i] * eta;
    lambda[(size_t)j * n + i] = lam;
    T w[PMAX];
#pragma unroll
    for (int q = 0; q < PMAX / 4; ++q) {
      if (4 * q < P) {
        const U4 r = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_OMEGA, q), ep, key.k0, key.k1);
        box_muller<T>(r.x, r.y, w[4 * q], w[4 * q + 1]);
        box_muller<T>(r.z, r.w, w[4 * q + 2], w[4 * q + 3]);
      } else {
        w[4 * q] = w[4 * q + 1] = w[4 * q + 2] = w[4 * q + 3] = T(0);
      }
    }
    // The reference's scale_omegas launch only ever reaches draw 0 of series 0
    // (its z index is always 0), leaving every other omega unscaled; compat mode
    // reproduces that, the default applies the scaling to every draw.
    const bool do_scale = !compat_unscaled || (i == 0 && j == 0);
    if (do_scale) {
      const T den = dev_sqrt((T)c_t[j] * lam);
      const unsigned pj = p[j];
#pragma unroll
      for (int k = 0; k < PMAX; ++k) w[k] = ((unsigned)k < pj) ? w[k] / den : T(0);
    }
    T *row = stage + (size_t)threadIdx.x * P;
    if (G) {
      // theta = G theta over the full max_p x max_p product (SGDLM.cu:729-740)
      T g[PMAX];
#pragma unroll
      for (int k = 0; k < PMAX; ++k) {
        T acc = T(0);
        if (k < P)
          for (int l = 0; l < P; ++l) acc += Gs[k + P * l] * row[l];
        g[k] = acc;
      }
#pragma unroll
      for (int k = 0; k < PMAX; ++k)
        if (k < P) row[k] = g[k];
    }
#pragma unroll
    for (int k = 0; k < PMAX; ++k) {
      if (k < P) {
        T acc = T(0);
#pragma unroll
        for (int l = 0; l <= k; ++l) acc += Us[l + P * k] * w[l];
        row[k] = acc + row[k];
      }
    }
    if (fail) atomicOr(&draw_flags[i], DRAW_FLAG_GAMMA_CAP);
  }
  __syncthreads();
  if (gd.v) write_gamma_runs<T>(gd, P, i0, (int)min((long)blockDim.x, n - i0), stage, gks, gcnt, gq0);
  for (long e = threadIdx.x; e < cnt; e += blockDim.x) src[e] = stage[e];
}

template <typename T> size_t sample_smem(int P) {
  return ((size_t)P * P + P + (size_t)kSampleThreads * P) * sizeof(T);
}

}  // namespace

template <typename T>
void launch_sample(cudaStream_t s, int m, int P, long n, const double *m_t,
                   const double *n_t, const double *s_t, const T *U, RngKey key,
                   T *lambda, T *theta, GammaDraws<T> gd, int *draw_flags, const unsigned *p) {
  dim3 grid((unsigned)((n + kSampleThreads - 1) / kSampleThreads), (unsigned)m);
  const size_t smem = sample_smem<T>(P);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(k_sample<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_sample<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_sample<T, 24>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_sample<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_sample<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  if (P <= 8)
    k_sample<T, 8><<<grid, kSampleThreads, smem, s>>>(m, P, n, m_t, n_t, s_t, U, key,
                                                      lambda, theta, gd, draw_flags, p);
  else if (P <= 16)
    k_sample<T, 16><<<grid, kSampleThreads, smem, s>>>(m, P, n, m_t, n_t, s_t, U, key,
                                                       lambda, theta, gd, draw_flags, p);
  else if (P <= 24)
    k_sample<T, 24><<<grid, kSampleThreads, smem, s>>>(m, P, n, m_t, n_t, s_t, U, key,
                                                       lambda, theta, gd, draw_flags, p);
  else if (P <= 32)
    k_sample<T, 32><<<grid, kSampleThreads, smem, s>>>(m, P, n, m_t, n_t, s_t, U, key,
                                                       lambda, theta, gd, draw_flags, p);
  else
    k_sample<T, 64><<<grid, kSampleThreads, smem, s>>>(m, P, n, m_t, n_t, s_t, U, key,
                                                       lambda, theta, gd, draw_flags, p);
}

template <typename T>
void launch_evolve(cudaStream_t s, int m, int P, long n, const unsigned *p,
                   const double *r_t, const double *c_t, const double *beta,
                   const T *UW, RngKey key, bool compat_unscaled_omega,
                   bool compat_beta_no_boost, T *lambda, T *theta, GammaDraws<T> gd,
                   int *draw_flags, const T *G) {
  dim3 grid((unsigned)((n + kSampleThreads - 1) / kSampleThreads), (unsigned)m);
  const size_t smem =
      ((size_t)P * P * (G ? 2 : 1) + (size_t)kSampleThreads * P) * sizeof(T);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(k_evolve<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_evolve<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_evolve<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_evolve<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
#define SGDLM_EVOLVE(PM)                                                              \
  k_evolve<T, PM><<<grid, kSampleThreads, smem, s>>>(m, P, n, p, r_t, c_t, beta, UW, \
                                                     key, compat_unscaled_omega,      \
                                                     compat_beta_no_boost, lambda,    \
                                                     theta, gd, draw_flags, G)
  if (P <= 8)
    SGDLM_EVOLVE(8);
  else if (P <= 16)
    SGDLM_EVOLVE(16);
  else if (P <= 32)
    SGDLM_EVOLVE(32);
  else
    SGDLM_EVOLVE(64);
#undef SGDLM_EVOLVE
}

template void launch_sample<float>(cudaStream_t, int, int, long, const double *,
                                   const double *, const double *, const float *, RngKey,
                                   float *, float *, GammaDraws<float>, int *, const unsigned *);
template void launch_sample<double>(cudaStream_t, int, int, long, const double *,
                                    const double *, const double *, const double *,
                                    RngKey, double *, double *, GammaDraws<double>, int *,
                                    const unsigned *);
template void launch_evolve<float>(cudaStream_t, int, int, long, const unsigned *,
                                   const double *, const double *, const double *,
                                   const float *, RngKey, bool, bool, float *, float *,
                                   GammaDraws<float>, int *, const float *);
template void launch_evolve<double>(cudaStream_t, int, int, long, const unsigned *,
                                    const double *, const double *, const double *,
                                    const double *, RngKey, bool, bool, double *,
                                    double *, GammaDraws<double>, int *, const double *);

}  // namespace sgdlm
