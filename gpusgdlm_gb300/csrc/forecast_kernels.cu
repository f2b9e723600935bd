// Forecast solves y_i = (I - Gamma_i)^-1 nu_i of FP32 draws by fixed-point
// (Jacobi) iteration, y <- nu + Gamma_i y, on the sparse Gamma_i itself.
//
// The reference factors every forecast draw's dense (I - Gamma_i) and forms its
// inverse (getrf + getri, rSGDLM/src/SGDLM/SGDLM.cu:594-617): (2/3 + 4/3) m^3
// flop per draw.  (I - Gamma_i) has at most max_p entries per row, and in the
// filtering regime the spectral radius of Gamma_i is well below one, so the
// iteration converges geometrically at O(nnz) per sweep -- a few ten thousand
// flop per draw at m = 400 instead of 10^8.  A draw is solved here when
//   (1) the sweeps from y = nu reach max|dy| <= 2^-20 max|y| within kMaxSweeps
//       (FP32, the draw's Gamma entries and the iterate in shared memory),
//   (2) the FP64 residual r = nu - (I - Gamma_i) y, solved by the same
//       iteration, gives a correction d with max|d| <= 1e-3 max|y| (the rule
//       the factorising path applies to its refinement step); y + d is written.
// Any other draw (slow or no convergence: spectral radius near or above one,
// non-finite values) is appended to `list` and solved by the LU kernels
// (partial pivoting where needed), as every draw was before.
#include <algorithm>

#include "kernels.hpp"

namespace sgdlm {
namespace {

constexpr int kJacThreads = 256;
constexpr int kMaxSweeps = 128;
// The first solve stops at max|dy| <= 2^-20 max|y|; the correction, whose size
// is that of y's error, needs only 2^-10 of its own size: y + d is then within
// about 2^-30 of the solution (FP32 sweeps reach a few ulps, not further).
constexpr float kSweepTol = 9.5367431640625e-07f;   // 2^-20
constexpr float kCorrSweepTol = 9.765625e-04f;      // 2^-10
constexpr double kCorrTol = 1e-3;

struct JacSmem {
  size_t nud, nuf, ya, yb, res, red, rowptr, col, val, total;
  __host__ __device__ JacSmem(int m, int nnz) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o = (o + bytes + 15) & ~(size_t)15;
      return at;
    };
    nud = take((size_t)m * sizeof(double));
    nuf = take((size_t)m * sizeof(float));
    ya = take((size_t)m * sizeof(float));
    yb = take((size_t)m * sizeof(float));
    res = take((size_t)m * sizeof(float));
    red = take(2 * (kJacThreads / 32) * sizeof(float));
    rowptr = take((size_t)(m + 1) * sizeof(int));
    val = take((size_t)nnz * sizeof(float));
    col = take((size_t)nnz * sizeof(unsigned short));
    total = o;
  }
};

// Block-wide maxima of two non-negative values; a NaN counts as infinity.
__device__ __forceinline__ void block_max2f(float &a, float &b, float *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = (a == a) ? a : INFINITY;
  b = (b == b) ? b : INFINITY;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmaxf(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  __syncthreads();
  if (lane == 0) {
    red[2 * warp] = a;
    red[2 * warp + 1] = b;
  }
  __syncthreads();
  a = b = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    a = fmaxf(a, red[2 * w]);
    b = fmaxf(b, red[2 * w + 1]);
  }
}

// One row of a sweep: c_r + sum_e val[e] x[col[e]] over the row's entries.  The
// first kUnroll entries are unrolled with predication, so that all their shared
// loads are independent and in flight together; two accumulators halve the FMA
// chain.  Rows with more entries finish in a plain loop.
constexpr int kUnroll = 24;
__device__ __forceinline__ float sweep_row(float c, int e0, int e1, const unsigned short *col,
                                           const float *val, const float *x) {
  float a0 = c, a1 = 0.f;
#pragma unroll
  for (int q = 0; q < kUnroll; q += 2) {
    if (e0 + q < e1) a0 = fmaf(val[e0 + q], x[col[e0 + q]], a0);
    if (e0 + q + 1 < e1) a1 = fmaf(val[e0 + q + 1], x[col[e0 + q + 1]], a1);
  }
  for (int e = e0 + kUnroll; e < e1; ++e) a0 = fmaf(val[e], x[col[e]], a0);
  return a0 + a1;
}

// Sweeps x <- c + Gamma x from x = c.  Returns whether they converged
// (max|dx| <= tol max|x|, everything finite); *out is the last iterate.
__device__ bool jacobi(int m, const int *rowptr, const unsigned short *col, const float *val,
                       const float *c, float *xa, float *xb, float *red, float tol, float **out) {
  for (int r = threadIdx.x; r < m; r += blockDim.x) xa[r] = c[r];
  __syncthreads();
  float *cur = xa, *nxt = xb;
  for (int it = 1; it <= kMaxSweeps; ++it) {
    float dmax = 0.f, xmax = 0.f;
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
      const float v = sweep_row(c[r], rowptr[r], rowptr[r + 1], col, val, cur);
      nxt[r] = v;
      dmax = fmaxf(dmax, fabsf(v - cur[r]));
      xmax = fmaxf(xmax, fabsf(v));
    }
    float *t = cur;
    cur = nxt;
    nxt = t;
    if ((it & 3) == 0 || it == kMaxSweeps) {
      block_max2f(dmax, xmax, red);  // also the barrier between sweeps
      if (!(xmax < INFINITY)) break;
      if (dmax <= tol * xmax) {
        *out = cur;
        return true;
      }
    } else {
      __syncthreads();
    }
  }
  *out = cur;
  return false;
}

__global__ void __launch_bounds__(kJacThreads)
    k_forecast_jacobi(int m, int P, long n, int nnz, GammaRows rows,
                      const float *__restrict__ theta_dm, const double *__restrict__ nu,
                      double *__restrict__ y, double *__restrict__ logdet, int *__restrict__ list) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const JacSmem L(m, nnz);
  double *nud = reinterpret_cast<double *>(smem_raw + L.nud);
  float *nuf = reinterpret_cast<float *>(smem_raw + L.nuf);
  float *ya = reinterpret_cast<float *>(smem_raw + L.ya);
  float *yb = reinterpret_cast<float *>(smem_raw + L.yb);
  float *res = reinterpret_cast<float *>(smem_raw + L.res);
  float *red = reinterpret_cast<float *>(smem_raw + L.red);
  int *rowptr = reinterpret_cast<int *>(smem_raw + L.rowptr);
  float *val = reinterpret_cast<float *>(smem_raw + L.val);
  unsigned short *col = reinterpret_cast<unsigned short *>(smem_raw + L.col);
  const int tid = threadIdx.x;
  for (int r = tid; r <= m; r += blockDim.x) rowptr[r] = rows.rowptr[r];
  for (int e = tid; e < nnz; e += blockDim.x) col[e] = (unsigned short)rows.ent[e].y;
  const size_t row_len = (size_t)m * P;
  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    // this draw's Gamma entries (from its draw-major theta row) and nu
    const float *th = theta_dm + (size_t)i * row_len;
    for (int e = tid; e < nnz; e += blockDim.x) val[e] = th[__ldg(&rows.ent[e].x)];
    for (int r = tid; r < m; r += blockDim.x) {
      const double v = nu[(size_t)r * n + i];
      nud[r] = v;
      nuf[r] = (float)v;
    }
    __syncthreads();
    float *yv = nullptr;
    bool ok = jacobi(m, rowptr, col, val, nuf, ya, yb, red, kSweepTol, &yv);
    if (ok) {
      // residual in FP64 and its correction by the same iteration
      float *other = (yv == ya) ? yb : ya;
      for (int r = tid; r < m; r += blockDim.x) {
        double v = nud[r] - (double)yv[r];
        const int e1 = rowptr[r + 1];
        for (int e = rowptr[r]; e < e1; ++e) v += (double)val[e] * (double)yv[col[e]];
        res[r] = (float)v;
      }
      __syncthreads();
      // the correction's iterates go to `other` and nuf (nu's FP32 copy is no
      // longer needed); yv keeps y
      float *dv = nullptr;
      ok = jacobi(m, rowptr, col, val, res, other, nuf, red, kCorrSweepTol, &dv);
      float dmax = 0.f, ymax = 0.f;
      for (int r = tid; r < m; r += blockDim.x) {
        dmax = fmaxf(dmax, fabsf(dv[r]));
        ymax = fmaxf(ymax, fabsf(yv[r]));
      }
      block_max2f(dmax, ymax, red);
      ok = ok && ymax < INFINITY && (double)dmax <= kCorrTol * (double)ymax;
      if (ok)
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)yv[r] + (double)dv[r];
    }
    if (tid == 0) {
      if (ok) {
        logdet[i] = NAN;  // no factorisation: no log|det| for this forecast draw
      } else {
        const int q = atomicAdd(list, 1);
        if (q < n) list[1 + q] = (int)i;
      }
    }
    __syncthreads();
  }
}

}  // namespace

JacobiPlan plan_jacobi(int m, int nnz, int num_sms) {
  JacobiPlan jp{};
  if (m < 1 || m > 65535) return jp;
  jp.smem = JacSmem(m, nnz).total;
  if (jp.smem > 100 * 1024) return jp;  // the draws keep the factorising path
  int per_sm = 0;
  cudaFuncSetAttribute(k_forecast_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jp.smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_forecast_jacobi, kJacThreads,
                                                    jp.smem) != cudaSuccess ||
      per_sm < 1) {
    (void)cudaGetLastError();
    return jp;
  }
  jp.grid = num_sms * per_sm;
  jp.nnz = nnz;
  jp.ok = 1;
  return jp;
}

void launch_forecast_jacobi(cudaStream_t s, const JacobiPlan &jp, int m, int P, long n,
                            GammaRows rows, const float *theta_dm, const double *nu, double *y,
                            double *logdet, int *list) {
  const long grid = std::min<long>(jp.grid, n);
  k_forecast_jacobi<<<(unsigned)std::max<long>(grid, 1), kJacThreads, jp.smem, s>>>(
      m, P, n, jp.nnz, rows, theta_dm, nu, y, logdet, list);
}

}  // namespace sgdlm
