// The learned importance proposal's network: a per-series MLP
//   features (F) -> 128 -> GELU -> 128 -> GELU -> outputs (O)
// with BF16 weights and FP32 accumulation, its backward pass, a masked
// mean-squared-error loss and Adam -- hand-written kernels, no library GEMM.
//
// Parameters live as FP32 master copies (what Adam updates) and BF16 copies
// (what the forward and the backward's data gradients multiply by), in one flat
// layout: W1 (H x F, row-major), b1 (H), W2 (H x H), b2 (H), W3 (O x H), b3 (O).
// Activations are row-major (batch x width).
//
// The reference has no counterpart: its proposal is the decoupled naive
// posterior (rSGDLM/src/SGDLM/SGDLM.cu:623-677).
#include <cuda_bf16.h>

#include "kernels.hpp"
#include "proposal.hpp"

namespace sgdlm {
namespace {

constexpr int kTile = 32;

template <typename T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// C[i, j] (+)= sum_k A(i, k) B(k, j), A(i, k) = A[i*sai + k*sak],
// B(k, j) = B[k*sbk + j*sbj], C row-major with leading dimension ldc; 32 x 32
// output tiles, 16 x 16 threads with 2 x 2 outputs each, K in chunks of 32
// staged in shared memory, FP32 accumulation.  Optional epilogue: + bias[j],
// store the pre-activation to Z, apply GELU.
template <typename TB>
__global__ void __launch_bounds__(256)
    k_matmul(int M, int N, int K, const float *__restrict__ A, long sai, long sak,
             const TB *__restrict__ B, long sbk, long sbj, float *__restrict__ C, int ldc,
             const float *__restrict__ bias, float *__restrict__ Z, int gelu, int accumulate) {
  __shared__ float As[kTile][kTile + 1];
  __shared__ float Bs[kTile][kTile + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.y * kTile, j0 = blockIdx.x * kTile;
  float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int k0 = 0; k0 < K; k0 += kTile) {
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
      const int r = e / kTile, c = e % kTile;
      const int i = i0 + r, k = k0 + c;
      As[r][c] = (i < M && k < K) ? A[(long)i * sai + (long)k * sak] : 0.f;
      const int kk = k0 + r, j = j0 + c;
      Bs[r][c] = (kk < K && j < N) ? to_f(B[(long)kk * sbk + (long)j * sbj]) : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < kTile; ++k) {
      const float a0 = As[ty][k], a1 = As[ty + 16][k];
      const float b0 = Bs[k][tx], b1 = Bs[k][tx + 16];
      acc[0][0] = fmaf(a0, b0, acc[0][0]);
      acc[0][1] = fmaf(a0, b1, acc[0][1]);
      acc[1][0] = fmaf(a1, b0, acc[1][0]);
      acc[1][1] = fmaf(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 2; ++u)
#pragma unroll
    for (int v = 0; v < 2; ++v) {
      const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
      if (i >= M || j >= N) continue;
      float x = acc[u][v];
      if (bias) x += bias[j];
      if (accumulate) x += C[(long)i * ldc + j];
      if (Z) Z[(long)i * ldc + j] = x;
      if (gelu) x = gelu_f(x);
      C[(long)i * ldc + j] = x;
    }
}

// dZ = dA * GELU'(Z), in place on dA.
__global__ void k_gelu_backward(long n, const float *__restrict__ Z, float *__restrict__ dA) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    dA[e] *= gelu_grad_f(Z[e]);
}

// Column sums of a row-major B x N matrix (bias gradients): one thread per column.
__global__ void k_colsum(int B, int N, const float *__restrict__ X, float *__restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += X[(long)b * N + j];
  out[j] = s;
}

// Masked mean squared error over B x O outputs: loss = sum mask (o - y)^2 / cnt,
// dO = 2 mask (o - y) / cnt, cnt = sum mask (at least 1).  One block.
__global__ void __launch_bounds__(1024)
    k_mse(long n, const float *__restrict__ O, const float *__restrict__ Y,
          const float *__restrict__ mask, float *__restrict__ dO, double *__restrict__ loss) {
  __shared__ double s_l[32], s_c[32];
  double l = 0.0, c = 0.0;
  for (long e = threadIdx.x; e < n; e += blockDim.x) {
    const double d = (double)O[e] - (double)Y[e];
    l += (double)mask[e] * d * d;
    c += (double)mask[e];
  }
  for (int o = 16; o > 0; o >>= 1) {
    l += __shfl_xor_sync(0xffffffffu, l, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_l[threadIdx.x >> 5] = l;
    s_c[threadIdx.x >> 5] = c;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = blockDim.x >> 5;
    l = threadIdx.x < nw ? s_l[threadIdx.x] : 0.0;
    c = threadIdx.x < nw ? s_c[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      l += __shfl_xor_sync(0xffffffffu, l, o);
      c += __shfl_xor_sync(0xffffffffu, c, o);
    }
    if (threadIdx.x == 0) {
      s_l[0] = l;
      s_c[0] = c > 1.0 ? c : 1.0;
    }
  }
  __syncthreads();
  const double cnt = s_c[0];
  if (threadIdx.x == 0 && loss) *loss = s_l[0] / cnt;
  const float g = (float)(2.0 / cnt);
  for (long e = threadIdx.x; e < n; e += blockDim.x) dO[e] = g * mask[e] * (O[e] - Y[e]);
}

// Adam (Kingma & Ba 2015) on the flat FP32 parameters, bias-corrected with the
// step count t, then the BF16 copy.
__global__ void k_adam(long n, float *__restrict__ w, __nv_bfloat16 *__restrict__ w16,
                       const float *__restrict__ g, float *__restrict__ m1, float *__restrict__ m2,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const float ge = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * ge;
    const float b = b2 * m2[e] + (1.f - b2) * ge * ge;
    m1[e] = a;
    m2[e] = b;
    const float x = w[e] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[e] = x;
    w16[e] = __float2bfloat16_rn(x);
  }
}

__global__ void k_to_bf16(long n, const float *__restrict__ w, __nv_bfloat16 *__restrict__ w16) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    w16[e] = __float2bfloat16_rn(w[e]);
}

template <typename TB>
void matmul(cudaStream_t s, int M, int N, int K, const float *A, long sai, long sak, const TB *B,
            long sbk, long sbj, float *C, int ldc, const float *bias, float *Z, bool gelu,
            bool accumulate) {
  const dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  k_matmul<TB><<<grid, 256, 0, s>>>(M, N, K, A, sai, sak, B, sbk, sbj, C, ldc, bias, Z,
                                    gelu ? 1 : 0, accumulate ? 1 : 0);
}

int grid_for(long n) {
  long g = (n + 255) / 256;
  return (int)(g < 1024 ? (g < 1 ? 1 : g) : 1024);
}

}  // namespace

MlpLayout mlp_layout(int F, int O) {
  MlpLayout L{};
  L.F = F;
  L.H = kMlpHidden;
  L.O = O;
  L.w1 = 0;
  L.b1 = L.w1 + (long)L.H * F;
  L.w2 = L.b1 + L.H;
  L.b2 = L.w2 + (long)L.H * L.H;
  L.w3 = L.b2 + L.H;
  L.b3 = L.w3 + (long)O * L.H;
  L.total = L.b3 + O;
  return L;
}

void mlp_forward(cudaStream_t s, const MlpLayout &L, int B, const float *X, const float *w,
                 const __nv_bfloat16 *w16, MlpActs a) {
  // Z1 = X W1' + b1, A1 = GELU(Z1): W1 is H x F row-major, B(k, j) = W1[j*F + k]
  matmul<__nv_bfloat16>(s, B, L.H, L.F, X, L.F, 1, w16 + L.w1, 1, L.F, a.A1, L.H, w + L.b1, a.Z1,
                        true, false);
  matmul<__nv_bfloat16>(s, B, L.H, L.H, a.A1, L.H, 1, w16 + L.w2, 1, L.H, a.A2, L.H, w + L.b2,
                        a.Z2, true, false);
  matmul<__nv_bfloat16>(s, B, L.O, L.H, a.A2, L.H, 1, w16 + L.w3, 1, L.H, a.Out, L.O, w + L.b3,
                        nullptr, false, false);
}

void mlp_loss_backward(cudaStream_t s, const MlpLayout &L, int B, const float *X, const float *Y,
                       const float *mask, const __nv_bfloat16 *w16, MlpActs a, float *grad,
                       double *loss) {
  const long nO = (long)B * L.O;
  k_mse<<<1, 1024, 0, s>>>(nO, a.Out, Y, mask, a.dOut, loss);
  // layer 3: dW3 (O x H) = dOut' A2; db3 = colsum dOut; dA2 = dOut W3
  matmul<float>(s, L.O, L.H, B, a.dOut, 1, L.O, a.A2, L.H, 1, grad + L.w3, L.H, nullptr, nullptr,
                false, false);
  k_colsum<<<(L.O + 127) / 128, 128, 0, s>>>(B, L.O, a.dOut, grad + L.b3);
  matmul<__nv_bfloat16>(s, B, L.H, L.O, a.dOut, L.O, 1, w16 + L.w3, L.H, 1, a.dA, L.H, nullptr,
                        nullptr, false, false);
  k_gelu_backward<<<grid_for((long)B * L.H), 256, 0, s>>>((long)B * L.H, a.Z2, a.dA);
  // layer 2
  matmul<float>(s, L.H, L.H, B, a.dA, 1, L.H, a.A1, L.H, 1, grad + L.w2, L.H, nullptr, nullptr,
                false, false);
  k_colsum<<<(L.H + 127) / 128, 128, 0, s>>>(B, L.H, a.dA, grad + L.b2);
  matmul<__nv_bfloat16>(s, B, L.H, L.H, a.dA, L.H, 1, w16 + L.w2, L.H, 1, a.dA2, L.H, nullptr,
                        nullptr, false, false);
  k_gelu_backward<<<grid_for((long)B * L.H), 256, 0, s>>>((long)B * L.H, a.Z1, a.dA2);
  // layer 1
  matmul<float>(s, L.H, L.F, B, a.dA2, 1, L.H, X, L.F, 1, grad + L.w1, L.F, nullptr, nullptr,
                false, false);
  k_colsum<<<(L.H + 127) / 128, 128, 0, s>>>(B, L.H, a.dA2, grad + L.b1);
}

void mlp_adam(cudaStream_t s, const MlpLayout &L, float *w, __nv_bfloat16 *w16, const float *grad,
              float *m1, float *m2, float lr, long step) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<grid_for(L.total), 256, 0, s>>>(L.total, w, w16, grad, m1, m2, lr, b1, b2, eps, c1, c2);
}

void mlp_refresh_bf16(cudaStream_t s, const MlpLayout &L, const float *w, __nv_bfloat16 *w16) {
  k_to_bf16<<<grid_for(L.total), 256, 0, s>>>(L.total, w, w16);
}

}  // namespace sgdlm
