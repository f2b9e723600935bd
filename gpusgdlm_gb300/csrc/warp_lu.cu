// Warp-per-draw LU of (I - Gamma_i) for small systems (m <= 32).
//
// The block LU kernels give a draw a whole CTA and pad its matrix to 32 x 32;
// at m = 6 (the README configuration) that is a CTA of 256 threads for a
// 6 x 6 matrix.  Here one warp owns one draw and lane r one row: the row sits
// in registers (32 values), the LU runs with partial pivoting (getrf semantics:
// the row with the largest |entry| of the column becomes the pivot row, ties to
// the lowest row; cublasXgetrfBatched at rSGDLM/src/SGDLM/SGDLM.cu:276-283), the
// pivot row is broadcast by shuffles, rows are never moved (each lane records
// the position of its pivot), and log|det| is the sum of log|pivot|.  No draw
// needs a redo.  Forecasts solve L U y = P nu with the same factors (the forward
// and back substitutions as shuffle chains), FP32 draws refined three times with an
// FP64 residual of the original rows (kept in shared memory).
#include "kernels.hpp"

namespace sgdlm {
namespace {

constexpr int kWarpLuThreads = 128;
constexpr int kWarpLuWarps = kWarpLuThreads / 32;
constexpr unsigned kAll = 0xffffffffu;

template <typename T> __device__ __forceinline__ T wabs(T v) { return v < T(0) ? -v : v; }

// Solves (P^T L U) x = b for the lane-held factors: lane r holds row r of the
// factored matrix (multipliers in a[c] for c < pos, U's row in a[c] for c >= pos),
// pos its pivot position, prow[k] the lane whose pivot position is k.  b is the
// lane's right-hand side entry (row r); the result is x_lane (column = lane).
template <typename T>
__device__ __forceinline__ T lu_solve(const T (&a)[32], int m, int pos, const int *prow, T b) {
  const int lane = threadIdx.x & 31;
  T acc = b;
#pragma unroll
  for (int c = 0; c < 32; ++c) {
    if (c < m) {
      const T zc = __shfl_sync(kAll, acc, prow[c]);
      if (pos > c) acc -= a[c] * zc;
    }
  }
  T x = T(0);
#pragma unroll
  for (int c = 31; c >= 0; --c) {
    if (c < m) {
      const int src = prow[c];
      const T q = acc / a[c];  // meaningful on the lane whose pivot position is c
      const T xc = __shfl_sync(kAll, q, src);
      if (pos < c) acc -= a[c] * xc;
      if (lane == c) x = xc;
    }
  }
  return x;
}

template <typename T>
__global__ void __launch_bounds__(kWarpLuThreads)
    k_lu_warp(int m, int P, long n, const unsigned *__restrict__ sp, const T *__restrict__ theta_sm,
              double *__restrict__ logdet,
              int *__restrict__ draw_flags, const double *__restrict__ nu, double *__restrict__ y) {
  __shared__ T tile[kWarpLuWarps][32][33];  // the draw's (I - Gamma_i), row-major
  __shared__ int prow_s[kWarpLuWarps][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T(*M)[33] = tile[w];
  int *prow = prow_s[w];
  const size_t mm = (size_t)m * m;
  const long stride = (long)gridDim.x * kWarpLuWarps;
  for (long i = (long)blockIdx.x * kWarpLuWarps + w; i < n; i += stride) {
    // ---- (I - Gamma_i) into the warp's tile, then row `lane` into registers
#pragma unroll
    for (int c = 0; c < 32; ++c) M[lane][c] = (lane == c) ? T(1) : T(0);
    __syncwarp();
    for (int e = lane; e < m * P; e += 32) {
      const unsigned pos = sp[e];
      if ((size_t)pos < mm) {
        const T th = theta_sm[((size_t)(e / P) * n + i) * P + e % P];
        M[pos % (unsigned)m][pos / (unsigned)m] = -th;
      }
    }
    __syncwarp();
    T a[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) a[c] = M[lane][c];
    // ---- LU with partial pivoting, rows in place
    bool done = lane >= m;
    int pos = 32;
    bool singular = false;
    double ld = 0.0;
#pragma unroll
    for (int k = 0; k < 32; ++k) {
      if (k < m) {
        // pivot: the active row with the largest |a[k]| (a NaN wins, and then
        // fails the finiteness check below)
        T v = done ? T(-1) : (a[k] == a[k] ? wabs(a[k]) : T(INFINITY));
        int li = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const T ov = __shfl_xor_sync(kAll, v, o);
          const int oi = __shfl_xor_sync(kAll, li, o);
          if (ov > v || (ov == v && oi < li)) {
            v = ov;
            li = oi;
          }
        }
        const T pv = __shfl_sync(kAll, a[k], li);
        if (!(v > T(0)) || !(wabs(pv) <= T(3.0e38))) singular = true;
        if (lane == 0) {
          prow[k] = li;
          ld += log(fabs((double)pv));
        }
        const bool upd = !done && lane != li;
        if (lane == li) {
          done = true;
          pos = k;
        }
        const T l = upd ? a[k] / pv : T(0);
        if (upd) a[k] = l;
#pragma unroll
        for (int c = k + 1; c < 32; ++c) {
          if (c < m) {
            const T u = __shfl_sync(kAll, a[c], li);
            if (upd) a[c] -= l * u;
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) {
      logdet[i] = singular ? -INFINITY : ld;
      if (singular) atomicOr(&draw_flags[i], DRAW_FLAG_SINGULAR);
    }
    if (y) {
      if (singular) {
        if (lane < m) y[(size_t)i * m + lane] = NAN;
      } else {
        const double nur = lane < m ? nu[(size_t)lane * n + i] : 0.0;
        T x = lu_solve<T>(a, m, pos, prow, (T)nur);
        double yr = (double)x;
        // FP32 factors: three refinements with the FP64 residual nu - (I - Gamma) y
        // (y accumulated in FP64)
        constexpr int kRefine = sizeof(T) == 4 ? 3 : 0;
#pragma unroll 1
        for (int it = 0; it < kRefine; ++it) {
          double res = nur;
#pragma unroll
          for (int c = 0; c < 32; ++c) {
            const double yc = __shfl_sync(kAll, yr, c);
            if (c < m && lane < m) res -= (double)M[lane][c] * yc;
          }
          yr += (double)lu_solve<T>(a, m, pos, prow, (T)res);
        }
        if (lane < m) y[(size_t)i * m + lane] = yr;
      }
    }
    __syncwarp();
  }
}

}  // namespace

template <typename T>
void launch_lu_warp(cudaStream_t s, int m, int P, long n, int num_sms, const unsigned *sp,
                    const T *theta, double *logdet, int *draw_flags,
                    const double *nu, double *y) {
  long blocks = (n + kWarpLuWarps - 1) / kWarpLuWarps;
  const long cap = (long)num_sms * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_lu_warp<T><<<(unsigned)blocks, kWarpLuThreads, 0, s>>>(m, P, n, sp, theta, logdet,
                                                           draw_flags, nu, y);
}

template void launch_lu_warp<float>(cudaStream_t, int, int, long, int, const unsigned *,
                                    const float *, double *, int *, const double *,
                                    double *);
template void launch_lu_warp<double>(cudaStream_t, int, int, long, int, const unsigned *,
                                     const double *, double *, int *,
                                     const double *, double *);

}  // namespace sgdlm
