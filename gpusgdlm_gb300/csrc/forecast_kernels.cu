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
//       (FP32; one thread per row holds the row's Gamma entries in registers in
//       ELL form, the iterate is in shared memory),
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

constexpr int kJacMaxThreads = 1024;  // one row per thread: m <= 1024
constexpr int kMaxSweeps = 128;
// The first solve stops at max|dy| <= 2^-20 max|y|; the correction, whose size
// is that of y's error, needs only 2^-10 of its own size: y + d is then within
// about 2^-30 of the solution (FP32 sweeps reach a few ulps, not further).
constexpr float kSweepTol = 9.5367431640625e-07f;   // 2^-20
constexpr float kCorrSweepTol = 9.765625e-04f;      // 2^-10
constexpr double kCorrTol = 1e-3;

struct JacSmem {
  size_t nud, nuf, ya, yb, res, red, total;
  __host__ __device__ JacSmem(int m) {
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
    red = take(2 * (kJacMaxThreads / 32) * sizeof(float));
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

// The thread's row r = threadIdx.x in ELL form held in registers: K slots
// (entries beyond the row's length have value 0 and point at the row itself),
// the column indices packed two to a register.
template <int K> struct Row {
  uint32_t col[K / 2];
  float val[K];
  __device__ __forceinline__ int c(int q) const {
    return (int)((col[q >> 1] >> (16 * (q & 1))) & 0xFFFFu);
  }
};

// Sweeps x <- c + Gamma x from x = c over this thread's row r.  Returns whether
// they converged (max|dx| <= tol max|x|, everything finite); *out is the last
// iterate.  wlen: the longest row of this warp, rounded up to even (warp-uniform):
// slots beyond it are padding in every row of the warp (value 0, so skipping them
// leaves every sum unchanged).
template <int K>
__device__ bool jacobi(int m, int r, int wlen, const Row<K> &R, const float *c, float *xa,
                       float *xb, float *red, float tol, float **out) {
  if (r < m) xa[r] = c[r];
  __syncthreads();
  float *cur = xa, *nxt = xb;
  for (int it = 1; it <= kMaxSweeps; ++it) {
    float dmax = 0.f, xmax = 0.f;
    if (r < m) {
      float a0 = c[r], a1 = 0.f;
#pragma unroll
      for (int q = 0; q < K; q += 2) {
        if (q >= wlen) break;
        a0 = fmaf(R.val[q], cur[R.c(q)], a0);
        a1 = fmaf(R.val[q + 1], cur[R.c(q + 1)], a1);
      }
      const float v = a0 + a1;
      nxt[r] = v;
      // fmaxf drops NaN operands: a NaN (an overflowed iterate times a padded
      // zero slot, or inf - inf) must count as divergence, so it becomes infinity
      // here
      const float av = fabsf(v), dv = fabsf(v - cur[r]);
      xmax = (av == av) ? av : INFINITY;
      dmax = (dv == dv) ? dv : INFINITY;
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

template <int K>
__global__ void __launch_bounds__(kJacMaxThreads)
    k_forecast_jacobi(int m, int P, long n, GammaRows rows, const float *__restrict__ theta_g,
                      int nnz,
                      const double *__restrict__ nu, double *__restrict__ y,
                      double *__restrict__ logdet, int *__restrict__ list,
                      const int *__restrict__ order) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const JacSmem L(m);
  double *nud = reinterpret_cast<double *>(smem_raw + L.nud);
  float *nuf = reinterpret_cast<float *>(smem_raw + L.nuf);
  float *ya = reinterpret_cast<float *>(smem_raw + L.ya);
  float *yb = reinterpret_cast<float *>(smem_raw + L.yb);
  float *res = reinterpret_cast<float *>(smem_raw + L.res);
  float *red = reinterpret_cast<float *>(smem_raw + L.red);
  const int tid = threadIdx.x;
  const int r = (tid < m && order) ? order[tid] : tid;  // this thread's row (r >= m: none)
  Row<K> R;
  const int e0 = r < m ? rows.rowptr[r] : 0;
  const int len = r < m ? rows.rowptr[r + 1] - e0 : 0;
  const int wlen = (__reduce_max_sync(0xffffffffu, (unsigned)len) + 1) & ~1;
#pragma unroll
  for (int q = 0; q < K; q += 2) {
    const uint32_t self = (uint32_t)(r < m ? r : 0);
    const uint32_t c0 = q < len ? (uint32_t)rows.ent[e0 + q].y : self;
    const uint32_t c1 = q + 1 < len ? (uint32_t)rows.ent[e0 + q + 1].y : self;
    R.col[q >> 1] = c0 | (c1 << 16);
  }
  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    // this draw's Gamma entries (row r's run of its Gamma copy) and nu
    const float *th = theta_g + (size_t)i * nnz + e0;
#pragma unroll
    for (int q = 0; q < K; ++q) R.val[q] = q < len ? th[q] : 0.f;
    if (r < m) {
      const double v = nu[(size_t)r * n + i];
      nud[r] = v;
      nuf[r] = (float)v;
    }
    __syncthreads();
    float *yv = nullptr;
    bool ok = jacobi<K>(m, r, wlen, R, nuf, ya, yb, red, kSweepTol, &yv);
    if (ok) {
      // residual in FP64 and its correction by the same iteration
      float *other = (yv == ya) ? yb : ya;
      if (r < m) {
        double v = nud[r] - (double)yv[r];
#pragma unroll
        for (int q = 0; q < K; ++q) v += (double)R.val[q] * (double)yv[R.c(q)];
        res[r] = (float)v;
      }
      __syncthreads();
      // the correction's iterates go to `other` and nuf (nu's FP32 copy is no
      // longer needed); yv keeps y
      float *dv = nullptr;
      ok = jacobi<K>(m, r, wlen, R, res, other, nuf, red, kCorrSweepTol, &dv);
      float dmax = 0.f, ymax = 0.f;
      if (r < m) {
        const float ad = fabsf(dv[r]), ay = fabsf(yv[r]);
        dmax = (ad == ad) ? ad : INFINITY;
        ymax = (ay == ay) ? ay : INFINITY;
      }
      block_max2f(dmax, ymax, red);
      ok = ok && ymax < INFINITY && dmax < INFINITY && (double)dmax <= kCorrTol * (double)ymax;
      // thread t writes row t (block_max2f ended on a barrier): a warp's stores are
      // one contiguous run, also when y is page-locked host memory
      if (ok && tid < m) y[(size_t)i * m + tid] = (double)yv[tid] + (double)dv[tid];
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

// ELL widths: the smallest of these that holds the longest row
constexpr int kJacWidths[] = {8, 12, 16, 18, 20, 24, 32};

template <int K> void *jacobi_kernel() { return reinterpret_cast<void *>(k_forecast_jacobi<K>); }
void *jacobi_kernel_for(int K) {
  switch (K) {
    case 8: return jacobi_kernel<8>();
    case 12: return jacobi_kernel<12>();
    case 16: return jacobi_kernel<16>();
    case 18: return jacobi_kernel<18>();
    case 20: return jacobi_kernel<20>();
    case 24: return jacobi_kernel<24>();
    default: return jacobi_kernel<32>();
  }
}

}  // namespace

JacobiPlan plan_jacobi(int m, int max_row, int num_sms) {
  JacobiPlan jp{};
  if (m < 1 || m > kJacMaxThreads || max_row > 32) return jp;
  jp.nnz = 32;
  for (int k : kJacWidths)
    if (max_row <= k) {
      jp.nnz = k;
      break;
    }
  jp.threads = (m + 31) / 32 * 32;
  jp.smem = JacSmem(m).total;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_kernel_for(jp.nnz), jp.threads,
                                                    jp.smem) != cudaSuccess ||
      per_sm < 1) {
    (void)cudaGetLastError();
    return jp;
  }
  jp.grid = num_sms * per_sm;
  jp.ok = 1;
  return jp;
}

void launch_forecast_jacobi(cudaStream_t s, const JacobiPlan &jp, int m, int P, long n,
                            GammaRows rows, const float *theta_g, int nnz, const double *nu,
                            double *y, double *logdet, int *list) {
  const unsigned grid = (unsigned)std::max<long>(std::min<long>(jp.grid, n), 1);
  const unsigned th = (unsigned)jp.threads;
#define SGDLM_JACOBI(K)                                                                    \
  k_forecast_jacobi<K><<<grid, th, jp.smem, s>>>(m, P, n, rows, theta_g, nnz, nu, y, logdet, list, \
                                                 jp.order)
  switch (jp.nnz) {
    case 8: SGDLM_JACOBI(8); break;
    case 12: SGDLM_JACOBI(12); break;
    case 16: SGDLM_JACOBI(16); break;
    case 18: SGDLM_JACOBI(18); break;
    case 20: SGDLM_JACOBI(20); break;
    case 24: SGDLM_JACOBI(24); break;
    default: SGDLM_JACOBI(32); break;
  }
#undef SGDLM_JACOBI
}

}  // namespace sgdlm
