// The learned importance proposal (no counterpart in the reference, whose
// proposal is the decoupled naive posterior, rSGDLM/src/SGDLM/SGDLM.cu:623-677).
//
// Per series j a small network maps features of the naive normal-gamma posterior
// (m_j, C_j, n_j, s_j) and of its simultaneous parents to a corrected proposal
//   m~ = m + delta (.) sqrt(diag C),   C~ = D C D,  D = diag(exp(rho)),
//   n~ = n exp(a),                     s~ = s exp(b),
// trained online on (naive posterior -> VB-refitted posterior) pairs.  Draws come
// from q~ = prod_j NG(m~_j, C~_j, n~_j, s~_j), and the importance weights stay
// exact density ratios:
//   log w_i = log|det(I - Gamma_i)| + sum_j [log p_j(theta_ij, lambda_ij)
//                                           - log q~_j(theta_ij, lambda_ij)],
// p_j the naive posterior (under the plain proposal the sum vanishes).
//
// Layouts: features X (m x F) and outputs (m x O) row-major per series;
//   F = 2P + 5: m_k / sqrt(C_kk) (P), log C_kk (P), log n, log s, p_j / P, mean
//               and variance over j's simultaneous parents q of mu_q (the mean of
//               q's posterior means over its p_q coefficients); inactive
//               coefficients (k >= p_j) are 0;
//   O = 2P + 2: delta (P), rho (P), a, b.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.hpp"

namespace sgdlm {

constexpr int kMlpHidden = 128;
constexpr int kProposalMaxP = 24;  // largest max_p the learned proposal serves
__host__ __device__ inline int proposal_features(int P) { return 2 * P + 5; }
__host__ __device__ inline int proposal_outputs(int P) { return 2 * P + 2; }

// Bounds applied to the network's outputs before they shape the proposal (the
// weights stay exact ratios whatever the outputs; the bounds keep q~ within a
// reasonable distance of p, so that its tails cover the target's).
constexpr float kDeltaMax = 3.f, kRhoMax = 1.f, kShapeMax = 2.f;

// GELU, x Phi(x), and its derivative Phi(x) + x phi(x).
__device__ __forceinline__ float gelu_f(float x) {
  return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad_f(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

struct MlpLayout {
  int F, H, O;
  long w1, b1, w2, b2, w3, b3, total;
};
MlpLayout mlp_layout(int F, int O);

// Activations of one batch (B rows): pre-activations Z1, Z2 and activations A1,
// A2 (B x H), outputs (B x O), and backward scratch dOut (B x O), dA, dA2 (B x H).
struct MlpActs {
  float *Z1, *A1, *Z2, *A2, *Out, *dOut, *dA, *dA2;
};

void mlp_forward(cudaStream_t s, const MlpLayout &L, int B, const float *X, const float *w,
                 const __nv_bfloat16 *w16, MlpActs a);
// Masked MSE of a.Out against Y and the gradient of every parameter into grad
// (flat layout); the forward must have run on the same X.
void mlp_loss_backward(cudaStream_t s, const MlpLayout &L, int B, const float *X, const float *Y,
                       const float *mask, const __nv_bfloat16 *w16, MlpActs a, float *grad,
                       double *loss);
void mlp_adam(cudaStream_t s, const MlpLayout &L, float *w, __nv_bfloat16 *w16, const float *grad,
              float *m1, float *m2, float lr, long step);
void mlp_refresh_bf16(cudaStream_t s, const MlpLayout &L, const float *w, __nv_bfloat16 *w16);

// Raw features of every series (m x F) from the naive posterior.
void launch_proposal_features(cudaStream_t s, int m, int P, const unsigned *p, const unsigned *sp,
                              const double *m_t, const double *C_t, const double *n_t,
                              const double *s_t, float *X);
// Training targets (m x O) and mask from the naive and the VB-refitted posterior.
void launch_proposal_targets(cudaStream_t s, int m, int P, const unsigned *p, const double *m_t,
                             const double *C_t, const double *n_t, const double *s_t,
                             const double *vm, const double *vC, const double *vn,
                             const double *vs, float *Y, float *mask);
// Appends m rows of (features, targets, mask) at ring position `pos` of a buffer
// of `cap` rows, and adds the features to the running sums (FP64, 2F + 1: sum,
// sum of squares, count) of the normalisation.
void launch_replay_append(cudaStream_t s, int m, int F, int O, long pos, long cap, const float *X,
                          const float *Y, const float *mask, float *bX, float *bY, float *bM,
                          double *fsum);
// Normalises features in place with the running sums (mean 0, sd 1; constant
// features to 0).
void launch_normalise(cudaStream_t s, int rows, int F, const double *fsum, float *X);
// A training batch of B rows drawn uniformly (Philox, keyed by seed and step)
// from the first `count` rows of the buffer, normalised.
void launch_replay_gather(cudaStream_t s, int B, int F, int O, long count, uint64_t seed,
                          uint64_t step, const float *bX, const float *bY, const float *bM,
                          const double *fsum, float *X, float *Y, float *mask);
// Proposal parameters per series from the network's outputs (m x O) and the
// naive posterior with its Cholesky factor U (U'U = C, P x P per series):
// m~ (P x m), n~, s~ (m), U~ = U D in FP64 and T, and per series the constant
// part of log p_j - log q~_j (FP64).
template <typename T>
void launch_proposal_params(cudaStream_t s, int m, int P, const unsigned *p, const float *out,
                            const double *m_t, const double *n_t, const double *s_t,
                            const double *U64, double *mq, double *nq, double *sq, double *Uq64,
                            T *Uq, double *cst);
// log p_j - log q~_j of every (draw, series) (lr, series-major j*n + i) and the
// draws' log weights logw[i] = logdet[i] + sum_j lr[j*n + i]; P <= kProposalMaxP.
template <typename T>
void launch_log_ratio(cudaStream_t s, int m, int P, long n, const unsigned *p, const T *theta,
                      const T *lambda, const double *m_t, const double *n_t, const double *s_t,
                      const T *U, const double *mq, const double *nq, const double *sq,
                      const T *Uq, const double *cst, const double *logdet, double *lr,
                      double *logw);

}  // namespace sgdlm
