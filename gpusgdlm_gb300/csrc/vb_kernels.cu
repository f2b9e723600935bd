// Importance weights and the Variational-Bayes refit.
//
// Reference (rSGDLM/src/SGDLM/SGDLM.cu:325-500): the weight sum is one serial
// thread (sumVector, kernel_functions.cuh:26-39); every moment is a
// one-thread-per-output loop over all n draws (meanScalarAndLog :929-946,
// compute_mean_m_t :949-967, meanBatchedVecVecT :1103-1133 with a global
// read-modify-write per draw); V^-1 comes from getrf/getri; and Q_ij =
// lambda (theta - m)' V^-1 (theta - m) is two gemmBatched calls of batch m*n
// whose only consumer is the weighted mean Q_bar_j (compute_mean_Q_t :1088-1100).
//
// Here:
//  * weights are exp(logdet - max) / sum in FP64 (log-sum-exp), three short
//    multi-block launches (max, exponentials, normalisation);
//  * pass A and pass B reduce over draws with one block per (series, chunk of
//    draws; the chunks are sized for the SM count), coalesced over the
//    series-major draw buffers, FP64 chunk partials; pass B for FP32 draws keeps
//    the next 128-draw sub-chunk in flight by cp.async;
//  * Q_bar_j is evaluated as trace(V^-1 V): since V = sum_i w_i theta~_i theta~_i'
//    with the same weights, sum_i w_i theta~_i' V^-1 theta~_i = tr(V^-1 V)
//    exactly, so the m*n quadratic forms of the reference collapse to a p x p
//    trace per series (equal to p_j up to the rounding of V^-1);
//  * the Newton solve for the gamma shape uses the reference's own asymptotic
//    digamma/trigamma series and stopping rule, in FP64.
#include "kernels.hpp"

namespace sgdlm {
namespace {

constexpr int kVbThreads = 256;
constexpr int kSub = 128;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum; every thread gets the result.  `red` needs 32 doubles.
template <typename T> __device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw; ++w) t += red[w];
  return t;
}
__device__ double block_max(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = -INFINITY;
  const int nw = blockDim.x >> 5;
  for (int w = 0; w < nw; ++w) t = fmax(t, red[w]);
  return t;
}

__device__ __forceinline__ bool finite_ld(double v) { return v == v && fabs(v) < INFINITY; }

// out6 = {sum |det|, ESS, max logdet, #finite, sum w^2, 0}.
// A draw whose log|det| is not finite gets weight 0, as detFromLU gives a NaN/Inf
// determinant weight 0 (kernel_functions.cuh:905-926).
// Importance weights over many blocks (FP64; the exponentials spread over the
// SMs instead of one block's FP64 pipe), three launches:
//   1. per block: max and count of the finite log|det|;
//   2. every block combines the maxima (M); e_i = exp(ld_i - M) into w, and the
//      block's sums of e_i and e_i^2;
//   3. every block combines the sums (S, Q); w_i = e_i / S (NaN for every draw when
//      S = 0: the reference divides 0 by 0); block 0 writes
//      out6 = {exp(M) S, 1 / sum w^2, M, count, sum w^2 = Q / S^2, 0}.
// part: 4 doubles per block (max, count, sum e, sum e^2).
constexpr int kWThreads = 256;
__device__ __forceinline__ void w_range(long n, long &b, long &e) {
  const long per = (n + gridDim.x - 1) / gridDim.x;
  b = (long)blockIdx.x * per;
  e = min(n, b + per);
}
__global__ void __launch_bounds__(kWThreads)
    k_w_max(long n, const double *__restrict__ logdet, double *__restrict__ part) {
  __shared__ double red[32];
  long b, e;
  w_range(n, b, e);
  double mx = -INFINITY, cnt = 0.0;
  for (long i = b + threadIdx.x; i < e; i += blockDim.x) {
    const double v = logdet[i];
    if (finite_ld(v)) {
      mx = fmax(mx, v);
      cnt += 1.0;
    }
  }
  mx = block_max(mx, red);
  cnt = block_sum(cnt, red);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x] = mx;
    part[4 * blockIdx.x + 1] = cnt;
  }
}
__global__ void __launch_bounds__(kWThreads)
    k_w_exp(long n, const double *__restrict__ logdet, double *__restrict__ w,
            double *__restrict__ part) {
  __shared__ double red[32];
  double mx = -INFINITY;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) mx = fmax(mx, part[4 * c]);
  mx = block_max(mx, red);
  long b, e;
  w_range(n, b, e);
  double s = 0.0, q = 0.0;
  for (long i = b + threadIdx.x; i < e; i += blockDim.x) {
    const double v = logdet[i];
    const double ei = finite_ld(v) ? exp(v - mx) : 0.0;
    w[i] = ei;
    s += ei;
    q += ei * ei;
  }
  s = block_sum(s, red);
  q = block_sum(q, red);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x + 2] = s;
    part[4 * blockIdx.x + 3] = q;
  }
}
__global__ void __launch_bounds__(kWThreads)
    k_w_norm(long n, double *__restrict__ w, const double *__restrict__ part,
             double *__restrict__ out6) {
  __shared__ double red[32];
  double mx = -INFINITY, cnt = 0.0, s = 0.0, q = 0.0;
  for (int c = threadIdx.x; c < (int)gridDim.x; c += blockDim.x) {
    mx = fmax(mx, part[4 * c]);
    cnt += part[4 * c + 1];
    s += part[4 * c + 2];
    q += part[4 * c + 3];
  }
  mx = block_max(mx, red);
  cnt = block_sum(cnt, red);
  s = block_sum(s, red);
  q = block_sum(q, red);
  long b, e;
  w_range(n, b, e);
  for (long i = b + threadIdx.x; i < e; i += blockDim.x) w[i] = (s > 0.0) ? w[i] / s : NAN;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const double s2 = q / (s * s);
    out6[0] = (s > 0.0) ? exp(mx) * s : 0.0;
    out6[1] = 1.0 / s2;
    out6[2] = mx;
    out6[3] = cnt;
    out6[4] = s2;
    out6[5] = 0.0;
  }
}

template <typename T> __device__ __forceinline__ T tlog(T v);
template <> __device__ __forceinline__ float tlog<float>(float v) { return logf(v); }
template <> __device__ __forceinline__ double tlog<double>(double v) { return log(v); }
template <typename T> __device__ __forceinline__ T tsqrt(T v);
template <> __device__ __forceinline__ float tsqrt<float>(float v) { return sqrtf(v); }
template <> __device__ __forceinline__ double tsqrt<double>(double v) { return sqrt(v); }

// Pass A: per (chunk, series): sum w lambda, sum w log lambda, sum w lambda theta_k.
template <typename T, int PMAX>
__global__ void __launch_bounds__(kVbThreads)
    k_vb_a(int m, int P, long n, long chunk, const double *__restrict__ w,
           const T *__restrict__ lambda, const T *__restrict__ theta,
           double *__restrict__ part_a) {
  __shared__ double red[32];
  const int j = blockIdx.y, c = blockIdx.x;
  const long i0 = (long)c * chunk;
  const long i1 = min(n, i0 + chunk);
  T sl = T(0), sll = T(0);
  T st[PMAX];
#pragma unroll
  for (int k = 0; k < PMAX; ++k) st[k] = T(0);
  const bool vec_rows = (P * sizeof(T)) % 16 == 0 && (reinterpret_cast<uintptr_t>(theta) & 15) == 0;
  for (long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const T wi = (T)w[i];
    const T lam = lambda[(size_t)j * n + i];
    const T wl = wi * lam;
    sl += wl;
    sll += wi * tlog(lam);
    const T *th = theta + ((size_t)j * n + i) * P;
    if (vec_rows) {
      // 16-byte loads of the row (P * sizeof(T) a multiple of 16)
      constexpr int VW = (int)(16 / sizeof(T));
#pragma unroll
      for (int k = 0; k < PMAX; k += VW)
        if (k < P) {
          T t[VW];
          if constexpr (sizeof(T) == 4) {
            const float4 q = *reinterpret_cast<const float4 *>(th + k);
            t[0] = q.x, t[1] = q.y, t[2] = q.z, t[3] = q.w;
          } else {
            const double2 q = *reinterpret_cast<const double2 *>(th + k);
            t[0] = q.x, t[1] = q.y;
          }
#pragma unroll
          for (int e = 0; e < VW; ++e) st[k + e] += wl * t[e];
        }
    } else {
#pragma unroll
      for (int k = 0; k < PMAX; ++k)
        if (k < P) st[k] += wl * th[k];
    }
  }
  // all P + 2 sums in one round: warp shuffles in the working precision, one
  // shared-memory exchange, and thread k adds the eight warps' partials in FP64
  __shared__ T wpart[kVbThreads / 32][PMAX + 2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  sl = warp_sum_t(sl);
  sll = warp_sum_t(sll);
#pragma unroll
  for (int k = 0; k < PMAX; ++k)
    if (k < P) st[k] = warp_sum_t(st[k]);
  if (lane == 0) {
    wpart[warp][0] = sl;
    wpart[warp][1] = sll;
#pragma unroll
    for (int k = 0; k < PMAX; ++k)
      if (k < P) wpart[warp][2 + k] = st[k];
  }
  __syncthreads();
  double *out = part_a + ((size_t)c * m + j) * (P + 2);
  if (threadIdx.x < P + 2) {
    double v = 0.0;
    for (int w8 = 0; w8 < kVbThreads / 32; ++w8) v += (double)wpart[w8][threadIdx.x];
    out[threadIdx.x] = v;
  }
  (void)red;
}

// Combines the chunk partials of pass A: E_w lambda, E_w log lambda, and the
// uncut weighted mean m_bar = sum w lambda theta / sum w lambda over all P
// (compute_mean_m_t, kernel_functions.cuh:949-967).
__global__ void k_vb_a_fin(int m, int P, int chunks, const double *__restrict__ part_a,
                           double *__restrict__ mean_lambda,
                           double *__restrict__ mean_log_lambda,
                           double *__restrict__ mbar_full) {
  // one warp per series, lane k < P + 2 adds partial k over the chunks in order
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= m) return;
  double sl = 0.0;  // E_w lambda: partial 0, lane 0 of the first round
  for (int k0 = 0; k0 < P + 2; k0 += 32) {
    const int k = k0 + lane;
    double v = 0.0;
    if (k < P + 2)
      for (int c = 0; c < chunks; ++c) v += part_a[((size_t)c * m + j) * (P + 2) + k];
    if (k0 == 0) {
      sl = __shfl_sync(0xffffffffu, v, 0);
      if (lane == 0) mean_lambda[j] = v;
      if (lane == 1) mean_log_lambda[j] = v;
    }
    if (k >= 2 && k < P + 2) mbar_full[(size_t)j * P + (k - 2)] = v / sl;
  }
}

// Pass B: per (chunk, series): V = sum w lambda (theta - m_bar)(theta - m_bar)' over
// the leading p x p block (meanBatchedVecVecT, kernel_functions.cuh:1103-1133).
// Draws are staged kSub at a time as X_i = sqrt(w_i lambda_i) (theta_i - m_bar)
// (rows padded to a multiple of 4, padding zero; a thread's theta loads of a
// sub-chunk are all in flight at once).  The upper triangle is cut into 4 x 4
// tiles; thread (tile, group) accumulates its tile over the draws of its group in
// registers in the working precision -- two 16-byte shared loads per draw for 16
// FMAs -- and the groups' partials are added in FP64 at the end.
// four consecutive values from a 16-byte aligned shared address
__device__ __forceinline__ void load4(const float *a, float *v) {
  const float4 q = *reinterpret_cast<const float4 *>(a);
  v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
}
__device__ __forceinline__ void load4(const double *a, double *v) {
  const double2 q0 = reinterpret_cast<const double2 *>(a)[0];
  const double2 q1 = reinterpret_cast<const double2 *>(a)[1];
  v[0] = q0.x, v[1] = q0.y, v[2] = q1.x, v[3] = q1.y;
}

template <typename T, int PMAX>
__global__ void __launch_bounds__(kVbThreads)
    k_vb_b(int m, int P, long n, long chunk, const unsigned *__restrict__ p,
           const double *__restrict__ w, const T *__restrict__ lambda,
           const T *__restrict__ theta, const double *__restrict__ mbar_full,
           double *__restrict__ part_b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int j = blockIdx.y, c = blockIdx.x;
  const int pj = (int)min((unsigned)P, p[j]);
  const int PX = (P + 3) / 4 * 4;  // padded row of X
  const int nb = (pj + 3) / 4, ntiles = nb * (nb + 1) / 2;
  const int G = ntiles > 0 ? kVbThreads / ntiles : 0;  // draw groups
  T *X = reinterpret_cast<T *>(smem_raw);  // kSub * PX
  T *mb = X + (size_t)kSub * PX;           // PX
  T *sc = mb + PX;                         // kSub
  T *red = sc + kSub;                      // G * ntiles * 16 (at the end)
  for (int k = threadIdx.x; k < PX; k += blockDim.x)
    mb[k] = k < P ? (T)mbar_full[(size_t)j * P + k] : T(0);
  // the rows' padding stays zero (the data never writes it)
  if (PX > P)
    for (int e = threadIdx.x; e < kSub * PX; e += blockDim.x)
      if (e % PX >= P) X[e] = T(0);
  // this thread's tile (bx <= by, column-major over the upper triangle) and group
  const int t = G > 0 ? (int)threadIdx.x % ntiles : 0;
  const int g = G > 0 ? (int)threadIdx.x / ntiles : 1 << 30;
  int by = 0;
  while ((by + 1) * (by + 2) / 2 <= t) ++by;
  const int bx = t - by * (by + 1) / 2;
  T acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = T(0);
  __syncthreads();
  const long i0 = (long)c * chunk;
  const long i1 = min(n, i0 + chunk);
  for (long s0 = i0; s0 < i1; s0 += kSub) {
    const int cnt = (int)min((long)kSub, i1 - s0);
    const T *thb = theta + ((size_t)j * n + s0) * P;
    const int tot = cnt * P;
    T v[kSub * PMAX / kVbThreads];
#pragma unroll
    for (int h = 0; h < kSub * PMAX / kVbThreads; ++h) {
      const int e = threadIdx.x + h * kVbThreads;
      v[h] = e < tot ? thb[e] : T(0);
    }
    for (int s = threadIdx.x; s < cnt; s += blockDim.x)
      sc[s] = tsqrt<T>((T)w[s0 + s] * lambda[(size_t)j * n + s0 + s]);
    __syncthreads();
#pragma unroll
    for (int h = 0; h < kSub * PMAX / kVbThreads; ++h) {
      const int e = threadIdx.x + h * kVbThreads;
      if (e < tot) {
        const int s = e / P, k = e - s * P;
        X[s * PX + k] = sc[s] * (v[h] - mb[k]);
      }
    }
    __syncthreads();
    if (g < G) {
      for (int s = g; s < cnt; s += G) {
        T xa[4], xb[4];
        load4(X + s * PX + 4 * bx, xa);
        load4(X + s * PX + 4 * by, xb);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[4 * a + b] += xa[a] * xb[b];
      }
    }
    __syncthreads();
  }
  if (g < G) {
#pragma unroll
    for (int q = 0; q < 16; ++q) red[((size_t)g * ntiles + t) * 16 + q] = acc[q];
  }
  __syncthreads();
  double *out = part_b + ((size_t)c * m + j) * P * P;
  for (int e = threadIdx.x; e < ntiles * 16; e += blockDim.x) {
    const int tt = e / 16, q = e % 16;
    int yy = 0;
    while ((yy + 1) * (yy + 2) / 2 <= tt) ++yy;
    const int xx = tt - yy * (yy + 1) / 2;
    const int x = 4 * xx + q / 4, y = 4 * yy + q % 4;
    if (x <= y && y < pj) {
      double vv = 0.0;
      for (int gg = 0; gg < G; ++gg) vv += (double)red[((size_t)gg * ntiles + tt) * 16 + q];
      out[x + P * y] = vv;
    }
  }
}

// Asynchronous global -> shared copies of 16, 8 or 4 bytes (cp.async), committed
// as groups; wait_group<N> returns when at most N of this thread's groups are in
// flight.
__device__ __forceinline__ void cpa16(void *sm, const void *g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(sm)), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa8(void *sm, const void *g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(sm)), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa4(void *sm, const void *g) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(sm)), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cpa_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Pass B for FP32 draws: the same tiles and sums as k_vb_b, with the draws of the
// next sub-chunk (theta rows, w, lambda) copied into a second shared buffer by
// cp.async while the current one is accumulated, so that a block always has a
// sub-chunk in flight from HBM.
__global__ void __launch_bounds__(kVbThreads)
    k_vb_b_f32(int m, int P, long n, long chunk, const unsigned *__restrict__ p,
               const double *__restrict__ w, const float *__restrict__ lambda,
               const float *__restrict__ theta, const double *__restrict__ mbar_full,
               double *__restrict__ part_b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int j = blockIdx.y, c = blockIdx.x;
  const int pj = (int)min((unsigned)P, p[j]);
  const int PX = (P + 3) / 4 * 4;
  const int RS = (kSub * P + 3) / 4 * 4;  // one raw sub-chunk of theta
  const int nb = (pj + 3) / 4, ntiles = nb * (nb + 1) / 2;
  const int G = ntiles > 0 ? kVbThreads / ntiles : 0;
  double *wbuf = reinterpret_cast<double *>(smem_raw);  // 2 x kSub
  float *raw = reinterpret_cast<float *>(wbuf + 2 * kSub);  // 2 x RS
  float *lbuf = raw + 2 * RS;                               // 2 x kSub
  float *X = lbuf + 2 * kSub;                               // kSub x PX
  float *mb = X + (size_t)kSub * PX;                        // PX
  float *sc = mb + PX;                                      // kSub
  float *red = sc + kSub;                                   // G * ntiles * 16
  const int tid = threadIdx.x;
  for (int k = tid; k < PX; k += blockDim.x) mb[k] = k < P ? (float)mbar_full[(size_t)j * P + k] : 0.f;
  if (PX > P)
    for (int e = tid; e < kSub * PX; e += blockDim.x)
      if (e % PX >= P) X[e] = 0.f;
  const int t = G > 0 ? tid % ntiles : 0;
  const int g = G > 0 ? tid / ntiles : 1 << 30;
  int by = 0;
  while ((by + 1) * (by + 2) / 2 <= t) ++by;
  const int bx = t - by * (by + 1) / 2;
  float acc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) acc[q] = 0.f;
  const long i0 = (long)c * chunk;
  const long i1 = min(n, i0 + chunk);
  const int nsub = i1 > i0 ? (int)((i1 - i0 + kSub - 1) / kSub) : 0;
  const float *lam_j = lambda + (size_t)j * n;
  // the X-build layout: xstep rows at a time, one column per thread (P <= 256)
  const int xstep = (int)blockDim.x / P, xr = tid / P, xk = tid - xr * P;
  __syncthreads();  // mb is filled
  const float mbk = mb[xk];
  auto issue = [&](int sub) {
    const int b = sub & 1;
    const long s0 = i0 + (long)sub * kSub;
    const int cnt = (int)min((long)kSub, i1 - s0);
    const float *src = theta + ((size_t)j * n + s0) * P;
    float *dst = raw + b * RS;
    const int tot = cnt * P;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
      for (int q = tid; q < tot / 4; q += blockDim.x) cpa16(dst + 4 * q, src + 4 * q);
      for (int q = tot / 4 * 4 + tid; q < tot; q += blockDim.x) cpa4(dst + q, src + q);
    } else {
      for (int q = tid; q < tot; q += blockDim.x) cpa4(dst + q, src + q);
    }
    for (int q = tid; q < cnt; q += blockDim.x) {
      cpa8(wbuf + b * kSub + q, w + s0 + q);
      cpa4(lbuf + b * kSub + q, lam_j + s0 + q);
    }
    cpa_commit();
  };
  if (nsub > 0) issue(0);
  if (nsub > 1) issue(1);
  for (int sub = 0; sub < nsub; ++sub) {
    const int b = sub & 1;
    const long s0 = i0 + (long)sub * kSub;
    const int cnt = (int)min((long)kSub, i1 - s0);
    if (sub + 1 < nsub)
      cpa_wait<1>();
    else
      cpa_wait<0>();
    __syncthreads();
    const float *cur = raw + b * RS;
    for (int s = tid; s < cnt; s += blockDim.x)
      sc[s] = sqrtf((float)wbuf[b * kSub + s] * lbuf[b * kSub + s]);
    __syncthreads();
    // thread (xr, xk) fills column xk of rows xr, xr + xstep, ... (no division)
    if (xr < xstep)
      for (int s = xr; s < cnt; s += xstep) X[s * PX + xk] = sc[s] * (cur[s * P + xk] - mbk);
    __syncthreads();
    // buffer b is free: the sub-chunk after next goes into it
    if (sub + 2 < nsub) issue(sub + 2);
    if (g < G) {
      for (int s = g; s < cnt; s += G) {
        float xa[4], xb[4];
        load4(X + s * PX + 4 * bx, xa);
        load4(X + s * PX + 4 * by, xb);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int bb = 0; bb < 4; ++bb) acc[4 * a + bb] += xa[a] * xb[bb];
      }
    }
    __syncthreads();
  }
  if (g < G) {
#pragma unroll
    for (int q = 0; q < 16; ++q) red[((size_t)g * ntiles + t) * 16 + q] = acc[q];
  }
  __syncthreads();
  double *out = part_b + ((size_t)c * m + j) * P * P;
  for (int e = tid; e < ntiles * 16; e += blockDim.x) {
    const int tt = e / 16, q = e % 16;
    int yy = 0;
    while ((yy + 1) * (yy + 2) / 2 <= tt) ++yy;
    const int xx = tt - yy * (yy + 1) / 2;
    const int x = 4 * xx + q / 4, y = 4 * yy + q % 4;
    if (x <= y && y < pj) {
      double vv = 0.0;
      for (int gg = 0; gg < G; ++gg) vv += (double)red[((size_t)gg * ntiles + tt) * 16 + q];
      out[x + P * y] = vv;
    }
  }
}

// The reference's digamma and trigamma (kernel_functions.cuh:1006-1022): the
// asymptotic (Stirling) series truncated after the x^-14 and x^-9 terms, applied
// at any x.  Reproduced as is, including its error at small x.
// The same asymptotic series evaluated in r = 1/x (one division) by Horner's rule.
__device__ __forceinline__ double psi_series_r(double logx, double r) {
  const double t = r * r;
  const double s =
      t * (-1.0 / 12.0 +
           t * (1.0 / 120.0 +
                t * (-1.0 / 252.0 +
                     t * (1.0 / 240.0 +
                          t * (-5.0 / 660.0 + t * (691.0 / 32760.0 + t * (-1.0 / 12.0)))))));
  return logx - 0.5 * r + s;
}
__device__ __forceinline__ double psi1_series_r(double r) {
  const double t = r * r;
  return r + 0.5 * t + t * r * (1.0 / 6.0 + t * (-1.0 / 30.0 + t * (1.0 / 42.0 + t * (-1.0 / 30.0))));
}

// Orders |v| like the serial pivot scan's "v > best": the magnitude's bits as an
// integer (monotone for non-negative doubles), NaN below every number.
__device__ __forceinline__ long long pivot_key(double v) {
  const long long b = __double_as_longlong(v) & 0x7fffffffffffffffLL;
  return b > 0x7ff0000000000000LL ? -1LL : b;
}

// Per-series refit, one warp per series (FP64):
//   V (p x p) from the chunk partials; V^-1 by Gauss-Jordan with partial
//   pivoting; Q_bar = tr(V^-1 V); Newton for n_bar (compute_mean_n_t,
//   kernel_functions.cuh:1025-1068); s_bar (compute_mean_s_t :1071-1085);
//   C_bar = V s_bar inside p x p, zero outside; m_bar cut at p.
__global__ void k_vb_fin(int m, int P, int chunks, const unsigned *__restrict__ p,
                         const double *__restrict__ n_t, const double *__restrict__ s_t,
                         const double *__restrict__ part_b,
                         const double *__restrict__ mean_lambda,
                         const double *__restrict__ mean_log_lambda,
                         const double *__restrict__ mbar_full, double *__restrict__ mean_m,
                         double *__restrict__ mean_C, double *__restrict__ mean_n,
                         double *__restrict__ mean_s, double *__restrict__ mean_Q,
                         int *__restrict__ series_flags) {
  extern __shared__ double sh[];
  const int j = blockIdx.x;
  const int lane = threadIdx.x;
  const int pj = (int)min((unsigned)P, p[j]);
  double *V = sh;                      // P x P, V[x + P*y]
  double *G = V + (size_t)P * P;       // p x 2p augmented [V | I], G[r + pj*c]
  double *f = G + (size_t)2 * P * P;   // multipliers of the current column
  __shared__ int s_bad;
  __shared__ double s_sb;
  if (lane == 0) s_bad = 0;
  for (int e = lane; e < P * P; e += 32) {
    const int x = e % P, y = e / P;
    double v = 0.0;
    if (x < pj && y < pj) {
      const int a = min(x, y), b = max(x, y);
      for (int c = 0; c < chunks; ++c) v += part_b[((size_t)c * m + j) * P * P + a + P * b];
    }
    V[e] = v;
  }
  __syncwarp();
  for (int e = lane; e < pj * 2 * pj; e += 32) {
    const int r = e % pj, cidx = e / pj;
    G[e] = (cidx < pj) ? V[r + P * cidx] : ((cidx - pj) == r ? 1.0 : 0.0);
  }
  __syncwarp();
  // Gauss-Jordan with partial pivoting on [V | I] -> [I | V^-1].  The pivot row is
  // the first row of the largest |entry| at or below the diagonal, as a serial scan
  // with "v > best" finds it (a NaN diagonal entry stays the pivot; NaN below it is
  // never chosen): a warp reduction over integer keys, ties to the lower row.
  double *grow = f + P;  // the normalised pivot row (2p values)
  for (int k = 0; k < pj; ++k) {
    const double dk = G[k + pj * k];
    long long key = -2;
    int idx = k;
    if (lane >= k && lane < pj) {
      key = lane == k ? pivot_key(dk) : pivot_key(G[lane + pj * k]);
      idx = lane;
    }
    if (pj > 32)
      for (int r = lane + 32; r < pj; r += 32) {
        if (r < k) continue;
        const long long kr = pivot_key(G[r + pj * k]);
        if (kr > key) key = kr, idx = r;
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long ko = __shfl_xor_sync(0xffffffffu, key, o);
      const int io = __shfl_xor_sync(0xffffffffu, idx, o);
      if (ko > key || (ko == key && io < idx)) key = ko, idx = io;
    }
    const bool nan_diag = isnan(dk);
    const int pr = nan_diag ? k : idx;
    if (lane == 0 && !((nan_diag ? -1LL : key) > 0)) s_bad = 1;  // |pivot| > 0 fails
    if (pr != k)
      for (int cidx = lane; cidx < 2 * pj; cidx += 32) {
        const double t = G[k + pj * cidx];
        G[k + pj * cidx] = G[pr + pj * cidx];
        G[pr + pj * cidx] = t;
      }
    __syncwarp();
    const double rpiv = 1.0 / G[k + pj * k];
    for (int r = lane; r < pj; r += 32) f[r] = G[r + pj * k];
    __syncwarp();
    for (int cidx = lane; cidx < 2 * pj; cidx += 32) {
      const double gk = G[k + pj * cidx] * rpiv;
      G[k + pj * cidx] = gk;
      grow[cidx] = gk;
    }
    __syncwarp();
    for (int e = lane; e < 2 * pj * pj; e += 32) {
      const int r = e % pj, cidx = e / pj;
      if (r != k) G[e] -= f[r] * grow[cidx];
    }
    __syncwarp();
  }
  // Q_bar = sum_{x,y} Vinv[x][y] V[y][x]
  double q = 0.0;
  for (int e = lane; e < pj * pj; e += 32) {
    const int x = e % pj, y = e / pj;
    q += G[x + pj * (pj + y)] * V[y + P * x];
  }
  q = warp_sum(q);
  if (lane == 0) {
    const double El = mean_lambda[j], Ell = mean_log_lambda[j];
    const double pd = (double)p[j];
    // When the weights collapse onto fewer draws than p_j, V is singular to
    // working precision and V^-1 is noise; tr(V^-1 V) = p_j is then used as is.
    bool singular_v = s_bad != 0 || !(fabs(q - (double)pj) <= 1e-8 * (double)(pj > 0 ? pj : 1));
    if (singular_v) q = (double)pj;
    double mn = n_t[j];
    double fun, dfun, step = 0.0;
    size_t iter = 0;
    const double log2El = log(2 * El), dq = pd - q;
    do {
      mn -= step;
      const double rmn = 1.0 / mn, r = 2.0 * rmn;  // r = 1 / (mn / 2)
      fun = log(mn + dq) - psi_series_r(log(0.5 * mn), r) - dq * rmn - log2El + Ell;
      dfun = 1.0 / (mn + dq) - .5 * psi1_series_r(r) + dq * rmn * rmn;
      step = fun / dfun;
      if (step > mn) step = .5 * mn;
    } while (fabs(fun) > 1e-6 && iter++ < 50);
    int fl = singular_v ? 1 : 0;
    // A non-finite iterate ends the reference's loop through the NaN comparison and
    // would be returned as is; it is treated as non-convergence instead.
    if (iter >= 50 || !(fabs(mn) < INFINITY)) {
      mn = n_t[j];
      fl |= 2;
    }
    double sb = (mn + pd - q) / (mn * El);
    if (sb < 0) {
      sb = s_t[j];
      fl |= 4;
    }
    mean_n[j] = mn;
    mean_s[j] = sb;
    mean_Q[j] = q;
    if (series_flags) series_flags[j] = fl;
    s_sb = sb;
  }
  __syncwarp();
  const double sb = s_sb;
  for (int e = lane; e < P * P; e += 32) {
    const int x = e % P, y = e / P;
    mean_C[(size_t)j * P * P + e] = (x < pj && y < pj) ? V[e] * sb : 0.0;
  }
  for (int k = lane; k < P; k += 32)
    mean_m[(size_t)j * P + k] = (k < pj) ? mbar_full[(size_t)j * P + k] : 0.0;
}

}  // namespace

void vb_chunking(long n, int m, int num_sms, int *chunks, long *chunk_draws) {
  // about two full waves of the second-moment pass (four 256-thread blocks per SM)
  long c = ((long)num_sms * 8 + m / 2) / (m > 0 ? m : 1);
  if (c < 1) c = 1;
  long d = (n + c - 1) / c;
  d = (d + kSub - 1) / kSub * kSub;
  if (d < kSub) d = kSub;
  c = (n + d - 1) / d;
  *chunks = (int)(c < 1 ? 1 : c);
  *chunk_draws = d;
}

void launch_weights(cudaStream_t s, long n, const double *logdet, double *w, double *out6,
                    double *part) {
  long blocks = (n + kWThreads - 1) / kWThreads;
  if (blocks > kWeightBlocks) blocks = kWeightBlocks;
  if (blocks < 1) blocks = 1;
  k_w_max<<<(unsigned)blocks, kWThreads, 0, s>>>(n, logdet, part);
  k_w_exp<<<(unsigned)blocks, kWThreads, 0, s>>>(n, logdet, w, part);
  k_w_norm<<<(unsigned)blocks, kWThreads, 0, s>>>(n, w, part, out6);
}

template <typename T>
void launch_vb(cudaStream_t s, int m, int P, long n, const unsigned *p, const double *n_t,
               const double *s_t, const double *w, const T *lambda, const T *theta,
               VbScratch scr, double *mean_m, double *mean_C, double *mean_n,
               double *mean_s, double *mean_lambda, double *mean_log_lambda,
               double *mean_Q, int *series_flags) {
  const int chunks = scr.chunks;
  const long chunk = scr.chunk_draws;
  dim3 grid((unsigned)chunks, (unsigned)m);
  if (P <= 8)
    k_vb_a<T, 8><<<grid, kVbThreads, 0, s>>>(m, P, n, chunk, w, lambda, theta, scr.part_a);
  else if (P <= 16)
    k_vb_a<T, 16><<<grid, kVbThreads, 0, s>>>(m, P, n, chunk, w, lambda, theta, scr.part_a);
  else if (P <= 32)
    k_vb_a<T, 32><<<grid, kVbThreads, 0, s>>>(m, P, n, chunk, w, lambda, theta, scr.part_a);
  else
    k_vb_a<T, 64><<<grid, kVbThreads, 0, s>>>(m, P, n, chunk, w, lambda, theta, scr.part_a);
  // mbar_full lives in mean_m's slot until the refit overwrites it with the cut mean;
  // a separate buffer keeps the kernels independent.
  double *mbar_full = scr.part_a + (size_t)chunks * m * (P + 2);
  k_vb_a_fin<<<(m + 3) / 4, 128, 0, s>>>(m, P, chunks, scr.part_a, mean_lambda,
                                         mean_log_lambda, mbar_full);
  const size_t PX = (size_t)(P + 3) / 4 * 4;
  const size_t smem_b = ((size_t)kSub * PX + PX + kSub + (size_t)kVbThreads * 16) * sizeof(T);
  const size_t smem_f = ((size_t)P * P * 3 + 3 * (size_t)P) * sizeof(double);
  if (smem_b > 48 * 1024) {
    cudaFuncSetAttribute(k_vb_b<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
    cudaFuncSetAttribute(k_vb_b<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
    cudaFuncSetAttribute(k_vb_b<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
    cudaFuncSetAttribute(k_vb_b<T, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b);
  }
  if (smem_f > 48 * 1024)
    cudaFuncSetAttribute(k_vb_fin, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_f);
#define SGDLM_VB_B(PM)                                                                \
  k_vb_b<T, PM><<<grid, kVbThreads, smem_b, s>>>(m, P, n, chunk, p, w, lambda, theta, mbar_full, \
                                                 scr.part_b)
  bool done_b = false;
  if constexpr (sizeof(T) == 4) {
    const size_t RS = ((size_t)kSub * P + 3) / 4 * 4;
    const size_t smem_a = 2 * kSub * sizeof(double) +
                          (2 * RS + 2 * kSub + (size_t)kSub * PX + PX + kSub + (size_t)kVbThreads * 16) *
                              sizeof(float);
    if (smem_a <= 200 * 1024) {
      if (smem_a > 48 * 1024)
        cudaFuncSetAttribute(k_vb_b_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_a);
      k_vb_b_f32<<<grid, kVbThreads, smem_a, s>>>(m, P, n, chunk, p, w,
                                                  reinterpret_cast<const float *>(lambda),
                                                  reinterpret_cast<const float *>(theta), mbar_full,
                                                  scr.part_b);
      done_b = true;
    }
  }
  if (done_b) {
  } else if (P <= 8)
    SGDLM_VB_B(8);
  else if (P <= 16)
    SGDLM_VB_B(16);
  else if (P <= 32)
    SGDLM_VB_B(32);
  else
    SGDLM_VB_B(64);
#undef SGDLM_VB_B
  k_vb_fin<<<m, 32, smem_f, s>>>(m, P, chunks, p, n_t, s_t, scr.part_b, mean_lambda,
                                 mean_log_lambda, mbar_full, mean_m, mean_C, mean_n,
                                 mean_s, mean_Q, series_flags);
}

template void launch_vb<float>(cudaStream_t, int, int, long, const unsigned *,
                               const double *, const double *, const double *,
                               const float *, const float *, VbScratch, double *, double *,
                               double *, double *, double *, double *, double *, int *);
template void launch_vb<double>(cudaStream_t, int, int, long, const unsigned *,
                                const double *, const double *, const double *,
                                const double *, const double *, VbScratch, double *,
                                double *, double *, double *, double *, double *, double *,
                                int *);

}  // namespace sgdlm
