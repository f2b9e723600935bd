// Kernels of the learned importance proposal (proposal.hpp): features and
// targets of the network, its replay buffer, the proposal's normal-gamma
// parameters, and the density ratios that keep the importance weights exact.
#include <cuda_bf16.h>

#include "kernels.hpp"
#include "proposal.hpp"
#include "rng.cuh"

namespace sgdlm {
namespace {

constexpr uint32_t TAG_REPLAY = 7u;  // Philox tag of the training batches

// One thread per series.
__global__ void k_features(int m, int P, const unsigned *__restrict__ p,
                           const unsigned *__restrict__ sp, const double *__restrict__ m_t,
                           const double *__restrict__ C_t, const double *__restrict__ n_t,
                           const double *__restrict__ s_t, float *__restrict__ X) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int F = proposal_features(P), pj = (int)p[j];
  float *x = X + (size_t)j * F;
  for (int k = 0; k < P; ++k) {
    const double c = C_t[(size_t)j * P * P + (size_t)k * (P + 1)];
    const bool on = k < pj && c > 0.0;
    x[k] = on ? (float)(m_t[(size_t)j * P + k] / sqrt(c)) : 0.f;
    x[P + k] = on ? (float)log(c) : 0.f;
  }
  x[2 * P] = (float)log(n_t[j]);
  x[2 * P + 1] = (float)log(s_t[j]);
  x[2 * P + 2] = (float)pj / (float)P;
  // simultaneous parents q of j: sp holds row j + m * q (< m * m)
  const size_t mm = (size_t)m * m;
  double s1 = 0.0, s2 = 0.0;
  int cnt = 0;
  for (int k = 0; k < P; ++k) {
    const unsigned pos = sp[(size_t)j * P + k];
    if ((size_t)pos >= mm) continue;
    const int q = (int)(pos / (unsigned)m);
    const int pq = (int)p[q];
    double mu = 0.0;
    for (int l = 0; l < pq; ++l) mu += m_t[(size_t)q * P + l];
    mu = pq > 0 ? mu / pq : 0.0;
    s1 += mu;
    s2 += mu * mu;
    ++cnt;
  }
  const double mean = cnt ? s1 / cnt : 0.0;
  x[2 * P + 3] = (float)mean;
  x[2 * P + 4] = cnt ? (float)fmax(s2 / cnt - mean * mean, 0.0) : 0.f;
}

__device__ __forceinline__ float clampf(float v, float lim) { return fminf(fmaxf(v, -lim), lim); }

__global__ void k_targets(int m, int P, const unsigned *__restrict__ p, const double *__restrict__ m_t,
                          const double *__restrict__ C_t, const double *__restrict__ n_t,
                          const double *__restrict__ s_t, const double *__restrict__ vm,
                          const double *__restrict__ vC, const double *__restrict__ vn,
                          const double *__restrict__ vs, float *__restrict__ Y,
                          float *__restrict__ M) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int O = proposal_outputs(P), pj = (int)p[j];
  float *y = Y + (size_t)j * O, *mk = M + (size_t)j * O;
  for (int k = 0; k < P; ++k) {
    const size_t d = (size_t)j * P * P + (size_t)k * (P + 1);
    const double c = C_t[d], cv = vC[d];
    const double dl = (vm[(size_t)j * P + k] - m_t[(size_t)j * P + k]) / sqrt(c);
    const double rh = 0.5 * log(cv / c);
    const bool okd = k < pj && c > 0.0 && isfinite(dl);
    const bool okr = okd && cv > 0.0 && isfinite(rh);
    y[k] = okd ? clampf((float)dl, kDeltaMax) : 0.f;
    mk[k] = okd ? 1.f : 0.f;
    y[P + k] = okr ? clampf((float)rh, kRhoMax) : 0.f;
    mk[P + k] = okr ? 1.f : 0.f;
  }
  const double a = log(vn[j] / n_t[j]), b = log(vs[j] / s_t[j]);
  y[2 * P] = isfinite(a) ? clampf((float)a, kShapeMax) : 0.f;
  mk[2 * P] = isfinite(a) ? 1.f : 0.f;
  y[2 * P + 1] = isfinite(b) ? clampf((float)b, kShapeMax) : 0.f;
  mk[2 * P + 1] = isfinite(b) ? 1.f : 0.f;
}

// One block: copies the m rows into the ring and adds them to the feature sums.
__global__ void k_replay_append(int m, int F, int O, long pos, long cap, const float *__restrict__ X,
                                const float *__restrict__ Y, const float *__restrict__ M,
                                float *__restrict__ bX, float *__restrict__ bY,
                                float *__restrict__ bM, double *__restrict__ fsum) {
  for (long e = threadIdx.x; e < (long)m * F; e += blockDim.x) {
    const long r = (pos + e / F) % cap;
    bX[r * F + e % F] = X[e];
  }
  for (long e = threadIdx.x; e < (long)m * O; e += blockDim.x) {
    const long r = (pos + e / O) % cap;
    bY[r * O + e % O] = Y[e];
    bM[r * O + e % O] = M[e];
  }
  for (int f = threadIdx.x; f < F; f += blockDim.x) {
    double s1 = 0.0, s2 = 0.0;
    for (int j = 0; j < m; ++j) {
      const double v = X[(size_t)j * F + f];
      s1 += v;
      s2 += v * v;
    }
    fsum[f] += s1;
    fsum[F + f] += s2;
  }
  if (threadIdx.x == 0) fsum[2 * F] += (double)m;
}

__device__ __forceinline__ float normalise(float v, int f, int F, const double *fsum) {
  const double c = fsum[2 * F];
  if (c <= 0.0) return v;
  const double mu = fsum[f] / c, var = fsum[F + f] / c - mu * mu;
  return var > 1e-12 ? (float)((v - mu) / sqrt(var)) : 0.f;
}

__global__ void k_normalise(int rows, int F, const double *__restrict__ fsum, float *__restrict__ X) {
  const long n = (long)rows * F;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    X[e] = normalise(X[e], (int)(e % F), F, fsum);
}

__global__ void k_replay_gather(int B, int F, int O, long count, uint32_t k0, uint32_t k1,
                                uint32_t step, const float *__restrict__ bX,
                                const float *__restrict__ bY, const float *__restrict__ bM,
                                const double *__restrict__ fsum, float *__restrict__ X,
                                float *__restrict__ Y, float *__restrict__ M) {
  const int b = blockIdx.x;
  if (b >= B || count <= 0) return;
  const U4 r = philox((uint32_t)b, 0u, tag_sub(TAG_REPLAY, 0u), step, k0, k1);
  const long row = (long)((((uint64_t)r.x << 32) | r.y) % (uint64_t)count);
  for (int f = threadIdx.x; f < F; f += blockDim.x)
    X[(size_t)b * F + f] = normalise(bX[row * F + f], f, F, fsum);
  for (int o = threadIdx.x; o < O; o += blockDim.x) {
    Y[(size_t)b * O + o] = bY[row * O + o];
    M[(size_t)b * O + o] = bM[row * O + o];
  }
}

// One thread per series: the proposal's parameters and the constant part of the
// log density ratio,
//   c_j = [n/2 log(n s/2) - lgamma(n/2) - 1/2 log|C| + p/2 log s]
//       - [n~/2 log(n~ s~/2) - lgamma(n~/2) - 1/2 log|C~| + p/2 log s~],
// log|C| = 2 sum log U_kk, log|C~| = log|C| + 2 sum rho_k (k < p_j).
template <typename T>
__global__ void k_params(int m, int P, const unsigned *__restrict__ p, const float *__restrict__ out,
                         const double *__restrict__ m_t, const double *__restrict__ n_t,
                         const double *__restrict__ s_t, const double *__restrict__ U64,
                         double *__restrict__ mq, double *__restrict__ nq, double *__restrict__ sq,
                         double *__restrict__ Uq64, T *__restrict__ Uq, double *__restrict__ cst) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int O = proposal_outputs(P), pj = (int)p[j];
  const float *o = out + (size_t)j * O;
  const double *U = U64 + (size_t)j * P * P;
  double logdetC = 0.0, sum_rho = 0.0;
  for (int k = 0; k < P; ++k) {
    const double ukk = U[k + (size_t)P * k];
    const bool on = k < pj && ukk > 0.0;
    const double dl = on ? (double)clampf(o[k], kDeltaMax) : 0.0;
    const double rh = on ? (double)clampf(o[P + k], kRhoMax) : 0.0;
    if (on) {
      logdetC += 2.0 * log(ukk);
      sum_rho += rh;
    }
    // sqrt(C_kk) = the norm of column k of U
    double ckk = 0.0;
    for (int l = 0; l <= k; ++l) ckk += U[l + (size_t)P * k] * U[l + (size_t)P * k];
    mq[(size_t)j * P + k] = m_t[(size_t)j * P + k] + dl * sqrt(ckk);
    const double dk = exp(rh);
    for (int l = 0; l < P; ++l) {
      const double v = U[l + (size_t)P * k] * dk;  // U~ = U D: column k scaled
      Uq64[(size_t)j * P * P + l + (size_t)P * k] = v;
      Uq[(size_t)j * P * P + l + (size_t)P * k] = (T)v;
    }
  }
  const double n = n_t[j], s = s_t[j];
  const double a = (double)clampf(o[2 * P], kShapeMax), b = (double)clampf(o[2 * P + 1], kShapeMax);
  const double n2 = n * exp(a), s2 = s * exp(b);
  nq[j] = n2;
  sq[j] = s2;
  const double cp = 0.5 * n * log(0.5 * n * s) - lgamma(0.5 * n) - 0.5 * logdetC + 0.5 * pj * log(s);
  const double cq = 0.5 * n2 * log(0.5 * n2 * s2) - lgamma(0.5 * n2) -
                    0.5 * (logdetC + 2.0 * sum_rho) + 0.5 * pj * log(s2);
  cst[j] = cp - cq;
}

// One block per (chunk of 128 draws, series j): the two quadratic forms by
// forward substitution with U' and U~' (lower triangular), FP64 combination:
//   lr = c_j + (n - n~)/2 log(lambda) - (n s - n~ s~)/2 lambda
//        - lambda/2 (s |U'^-1 (theta - m)|^2 - s~ |U~'^-1 (theta - m~)|^2).
template <typename T, int PMAX>
__global__ void __launch_bounds__(128)
    k_log_ratio(int m, int P, long n, const unsigned *__restrict__ p, const T *__restrict__ theta,
                const T *__restrict__ lambda, const double *__restrict__ m_t,
                const double *__restrict__ n_t, const double *__restrict__ s_t,
                const T *__restrict__ U, const double *__restrict__ mq, const double *__restrict__ nq,
                const double *__restrict__ sq, const T *__restrict__ Uq,
                const double *__restrict__ cst, double *__restrict__ lr) {
  __shared__ T Us[PMAX * PMAX], Uqs[PMAX * PMAX], ms[PMAX], mqs[PMAX], rd[PMAX], rdq[PMAX];
  const int j = blockIdx.y;
  const int pj = (int)p[j];
  for (int e = threadIdx.x; e < P * P; e += blockDim.x) {
    Us[e] = U[(size_t)j * P * P + e];
    Uqs[e] = Uq[(size_t)j * P * P + e];
  }
  for (int e = threadIdx.x; e < P; e += blockDim.x) {
    ms[e] = (T)m_t[(size_t)j * P + e];
    mqs[e] = (T)mq[(size_t)j * P + e];
    // the diagonals' reciprocals, once per series (the solves multiply)
    rd[e] = T(1) / U[(size_t)j * P * P + e + P * e];
    rdq[e] = T(1) / Uq[(size_t)j * P * P + e + P * e];
  }
  __syncthreads();
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T *th = theta + ((size_t)j * n + i) * P;
  T wp[PMAX], wq[PMAX];
  T qp = T(0), qq = T(0);
#pragma unroll
  for (int k = 0; k < PMAX; ++k) {
    if (k < pj) {
      const T t = th[k];
      T ap = t - ms[k], aq = t - mqs[k];
#pragma unroll
      for (int l = 0; l < k; ++l) {
        ap -= Us[l + P * k] * wp[l];
        aq -= Uqs[l + P * k] * wq[l];
      }
      wp[k] = ap * rd[k];
      wq[k] = aq * rdq[k];
      qp += wp[k] * wp[k];
      qq += wq[k] * wq[k];
    } else {
      wp[k] = wq[k] = T(0);
    }
  }
  const T lamt = lambda[(size_t)j * n + i];
  const double lam = (double)lamt;
  const double nn = n_t[j], ss = s_t[j], n2 = nq[j], s2 = sq[j];
  // log(lambda) in the draws' precision: FP32 draws carry 2^-24 of lambda anyway,
  // and the FP64 logarithm is the kernel's most expensive operation on GB300
  const double loglam = (double)dev_log(lamt);
  lr[(size_t)j * n + i] = cst[j] + 0.5 * (nn - n2) * loglam - 0.5 * (nn * ss - n2 * s2) * lam -
                          0.5 * lam * (ss * (double)qp - s2 * (double)qq);
}

__global__ void k_log_weights(int m, long n, const double *__restrict__ logdet,
                              const double *__restrict__ lr, double *__restrict__ logw) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = logdet[i];
  for (int j = 0; j < m; ++j) v += lr[(size_t)j * n + i];
  logw[i] = v;
}

}  // namespace

void launch_proposal_features(cudaStream_t s, int m, int P, const unsigned *p, const unsigned *sp,
                              const double *m_t, const double *C_t, const double *n_t,
                              const double *s_t, float *X) {
  k_features<<<(m + 127) / 128, 128, 0, s>>>(m, P, p, sp, m_t, C_t, n_t, s_t, X);
}

void launch_proposal_targets(cudaStream_t s, int m, int P, const unsigned *p, const double *m_t,
                             const double *C_t, const double *n_t, const double *s_t,
                             const double *vm, const double *vC, const double *vn,
                             const double *vs, float *Y, float *mask) {
  k_targets<<<(m + 127) / 128, 128, 0, s>>>(m, P, p, m_t, C_t, n_t, s_t, vm, vC, vn, vs, Y, mask);
}

void launch_replay_append(cudaStream_t s, int m, int F, int O, long pos, long cap, const float *X,
                          const float *Y, const float *mask, float *bX, float *bY, float *bM,
                          double *fsum) {
  k_replay_append<<<1, 256, 0, s>>>(m, F, O, pos, cap, X, Y, mask, bX, bY, bM, fsum);
}

void launch_normalise(cudaStream_t s, int rows, int F, const double *fsum, float *X) {
  const long n = (long)rows * F;
  const int g = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
  k_normalise<<<g < 1 ? 1 : g, 256, 0, s>>>(rows, F, fsum, X);
}

void launch_replay_gather(cudaStream_t s, int B, int F, int O, long count, uint64_t seed,
                          uint64_t step, const float *bX, const float *bY, const float *bM,
                          const double *fsum, float *X, float *Y, float *mask) {
  k_replay_gather<<<B, 64, 0, s>>>(B, F, O, count, (uint32_t)seed, (uint32_t)(seed >> 32),
                                   (uint32_t)step, bX, bY, bM, fsum, X, Y, mask);
}

template <typename T>
void launch_proposal_params(cudaStream_t s, int m, int P, const unsigned *p, const float *out,
                            const double *m_t, const double *n_t, const double *s_t,
                            const double *U64, double *mq, double *nq, double *sq, double *Uq64,
                            T *Uq, double *cst) {
  k_params<T><<<(m + 127) / 128, 128, 0, s>>>(m, P, p, out, m_t, n_t, s_t, U64, mq, nq, sq, Uq64,
                                              Uq, cst);
}

template <typename T>
void launch_log_ratio(cudaStream_t s, int m, int P, long n, const unsigned *p, const T *theta,
                      const T *lambda, const double *m_t, const double *n_t, const double *s_t,
                      const T *U, const double *mq, const double *nq, const double *sq,
                      const T *Uq, const double *cst, const double *logdet, double *lr,
                      double *logw) {
  const dim3 grid((unsigned)((n + 127) / 128), (unsigned)m);
  if (P <= 8)
    k_log_ratio<T, 8><<<grid, 128, 0, s>>>(m, P, n, p, theta, lambda, m_t, n_t, s_t, U, mq, nq, sq,
                                           Uq, cst, lr);
  else  // P <= kProposalMaxP (checked by the engine)
    k_log_ratio<T, kProposalMaxP><<<grid, 128, 0, s>>>(m, P, n, p, theta, lambda, m_t, n_t, s_t, U,
                                                       mq, nq, sq, Uq, cst, lr);
  k_log_weights<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m, n, logdet, lr, logw);
}

template void launch_proposal_params<float>(cudaStream_t, int, int, const unsigned *, const float *,
                                            const double *, const double *, const double *,
                                            const double *, double *, double *, double *,
                                            double *, float *, double *);
template void launch_proposal_params<double>(cudaStream_t, int, int, const unsigned *,
                                             const float *, const double *, const double *,
                                             const double *, const double *, double *, double *,
                                             double *, double *, double *, double *);
template void launch_log_ratio<float>(cudaStream_t, int, int, long, const unsigned *, const float *,
                                      const float *, const double *, const double *,
                                      const double *, const float *, const double *,
                                      const double *, const double *, const float *,
                                      const double *, const double *, double *, double *);
template void launch_log_ratio<double>(cudaStream_t, int, int, long, const unsigned *,
                                       const double *, const double *, const double *,
                                       const double *, const double *, const double *,
                                       const double *, const double *, const double *,
                                       const double *, const double *, const double *, double *,
                                       double *);

}  // namespace sgdlm
