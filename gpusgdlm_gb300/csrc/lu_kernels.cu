// Batched LU of (I - Gamma_i), one matrix per draw: log|det| for the importance
// weights, and for forecasts the solve y_i = (I - Gamma_i)^-1 nu_i.
//
// The reference zeroes 2*nsim_batch dense m x m FP64 matrices in HBM, scatters
// the parents, calls cublasDgetrfBatched through a pointer array and, for
// forecasts, cublasDgetriBatched plus a gemv on the explicit inverse
// (rSGDLM/src/SGDLM/SGDLM.cu:231-323, 555-620; kernel_functions.cuh:810-842,
// 905-926; HostWrapperImpl.cu:375-377).
//
// Here a persistent CTA owns one draw at a time and one private m_p x m_p slab of
// scratch (m_p = m rounded up to 32; the padding is identity, which changes
// neither det nor the solve).  With one slab per resident CTA the whole working
// set of the LU (about 100 MB at m = 400 in FP32) stays in the 126 MB L2.
// The factorisation is a right-looking blocked LU with 32 x 32 blocks:
//   (a) one warp factors the diagonal block in shared memory;
//   (b) the column panel L = A U^-1 and (c) the row panel U = L^-1 A, one
//       row/column per thread, land in shared memory;
//   (d) the trailing update A -= L U is a register-tiled FMA loop over
//       128 x 128 tiles (8 x 8 per thread) fed from those shared panels.
// (I - Gamma) is diagonally dominant for the parent graphs SGDLM is used with, so
// the blocked pass does not pivot; it checks every multiplier against
// kPivotThreshold and flags the draw when one is larger (or a pivot is zero or
// not finite).  Flagged draws are redone by k_lu_fallback with partial pivoting,
// as getrf would.  |det| does not depend on the pivot order.
//
// For forecasts the right-hand side rides along as an extra column held in
// shared memory, so the factorisation also produces L^-1 nu; a blocked back
// substitution gives y0, an FP64 residual nu - (I - Gamma) y0 is formed from the
// sparse parent list, and one refinement solve with the same factors corrects y0.
#include "kernels.hpp"
#include "rng.cuh"

namespace sgdlm {
namespace {

constexpr int kB = 32;          // LU block size
constexpr int kThreads = 256;   // 16 x 16 thread grid of the trailing update
constexpr double kPivotThreshold = 8.0;


__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T> __device__ __forceinline__ T dabs(T v) { return v < T(0) ? -v : v; }
template <typename T> __device__ __forceinline__ bool finite_t(T v) {
  return v == v && dabs(v) <= (T)3.0e38;
}

// Shared-memory carve-up (all offsets in bytes, 16-byte aligned).
struct Smem {
  int Rmax;
  size_t off_D, off_Lp, off_Up, off_z, off_zu, off_nu, off_res, off_red, total;
  __host__ __device__ Smem(int mp, size_t tsz) {
    Rmax = mp - kB > 0 ? mp - kB : kB;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 15) & ~(size_t)15;
      return at;
    };
    off_D = take((size_t)kB * (kB + 1) * tsz);
    off_Lp = take((size_t)kB * Rmax * tsz);
    off_Up = take((size_t)kB * Rmax * tsz);
    off_z = take((size_t)mp * tsz);
    off_zu = take((size_t)kB * tsz);
    off_nu = take((size_t)mp * sizeof(double));
    off_res = take((size_t)mp * sizeof(double));
    off_red = take(64 * sizeof(double));
    total = o;
  }
};

// Writes the identity plus the scattered -theta entries of draw i into A, and for
// forecasts nu_i into nu (double) and z (working precision).
// fillGammas (kernel_functions.cuh:822-842), batchedComputeNuPlusMu (:1156-1178).
template <typename T>
__device__ void build_system(int m, int P, int mp, long n, long i,
                             const unsigned *__restrict__ sp, const T *__restrict__ theta,
                             T *__restrict__ A, const double *__restrict__ x,
                             const T *__restrict__ lambda, RngKey key, double *nu, T *z) {
  const int tid = threadIdx.x;
  const size_t elems = (size_t)mp * mp;
  const size_t n16 = elems * sizeof(T) / 16;
  uint4 *A16 = reinterpret_cast<uint4 *>(A);
  for (size_t e = tid; e < n16; e += blockDim.x) A16[e] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for (int r = tid; r < mp; r += blockDim.x) A[(size_t)r * mp + r] = T(1);
  const size_t mm = (size_t)m * m;
  for (int e = tid; e < m * P; e += blockDim.x) {
    const unsigned pos = sp[e];
    if ((size_t)pos < mm) {
      const int j = e / P, k = e % P;
      const int row = (int)(pos % (unsigned)m), col = (int)(pos / (unsigned)m);
      A[row + (size_t)mp * col] = -theta[((size_t)j * n + i) * P + k];
    }
  }
  if (x != nullptr) {
    const uint32_t ep = key_epoch(key);
    for (int r = tid; r < mp; r += blockDim.x) {
      double v = 0.0;
      if (r < m) {
        const int j = r;
        const U4 g = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_NU, 0), ep, key.k0, key.k1);
        T z0, z1;
        box_muller<T>(g.x, g.y, z0, z1);
        const T lam = lambda[(size_t)j * n + i];
        v = (double)(z0 / dev_sqrt(lam));
        const T *th = theta + ((size_t)j * n + i) * P;
        for (int k = 0; k < P; ++k)
          if ((size_t)sp[(size_t)j * P + k] >= mm) v += x[(size_t)j * P + k] * (double)th[k];
      }
      nu[r] = v;
      z[r] = (T)v;
    }
  }
  __syncthreads();
}

// 16-byte vectors of the working precision.
template <typename T> struct Vec;
template <> struct Vec<float> {
  static constexpr int W = 4;
  __device__ static __forceinline__ void ld(const float *p, float *o) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  __device__ static __forceinline__ void st(float *p, const float *o) {
    *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
  }
};
template <> struct Vec<double> {
  static constexpr int W = 2;
  __device__ static __forceinline__ void ld(const double *p, double *o) {
    const double2 v = *reinterpret_cast<const double2 *>(p);
    o[0] = v.x; o[1] = v.y;
  }
  __device__ static __forceinline__ void st(double *p, const double *o) {
    *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
  }
};

// Register-tiled trailing update A[r0:, r0:] -= Lp Up over an R x R region.
// 16 x 16 threads; thread (tr, tc) owns rows {tr*W + a, 16W + tr*W + a} and columns
// {tc*4 + b, 64 + tc*4 + b} of a (32W) x 128 tile, so every shared-memory read is a
// 16-byte vector and the 8 threads of each access phase read one contiguous
// 128-byte line (no bank conflicts); global loads are 16-byte vectors, 16 threads
// covering 256 contiguous bytes of a column.
template <typename T>
__device__ __forceinline__ void trailing_update(T *__restrict__ A, int mp, int r0, int R,
                                                const T *__restrict__ Lp,
                                                const T *__restrict__ Up, int Rmax) {
  using V = Vec<T>;
  constexpr int W = V::W;
  constexpr int TM = 2 * W, TN = 8;
  constexpr int tileM = 32 * W, tileN = 128;
  const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
  for (int tile_r = 0; tile_r < R; tile_r += tileM) {
    for (int tile_c = 0; tile_c < R; tile_c += tileN) {
      const int ra = tile_r + tr * W, rb = ra + 16 * W;
      const int ca = tile_c + tc * 4, cb = ca + 64;
      if (ra >= R || ca >= R) continue;  // chunk b lies beyond chunk a
      const bool vb = rb < R, wb = cb < R;
      T acc[TM][TN];
#pragma unroll
      for (int b = 0; b < TN; ++b) {
        const int col = (b < 4) ? (ca + b) : (cb + b - 4);
        const bool cv = (b < 4) || wb;
        T tmp[W];
        if (cv) {
          const T *colp = A + (size_t)mp * (r0 + col) + r0;
          V::ld(colp + ra, tmp);
#pragma unroll
          for (int a = 0; a < W; ++a) acc[a][b] = tmp[a];
          if (vb) {
            V::ld(colp + rb, tmp);
#pragma unroll
            for (int a = 0; a < W; ++a) acc[W + a][b] = tmp[a];
          } else {
#pragma unroll
            for (int a = 0; a < W; ++a) acc[W + a][b] = T(0);
          }
        } else {
#pragma unroll
          for (int a = 0; a < TM; ++a) acc[a][b] = T(0);
        }
      }
#pragma unroll 2
      for (int k = 0; k < kB; ++k) {
        T lv[TM], uv[TN];
        const T *lrow = Lp + k * Rmax;
        const T *urow = Up + k * Rmax;
        V::ld(lrow + ra, lv);
        if (vb) {
          V::ld(lrow + rb, lv + W);
        } else {
#pragma unroll
          for (int a = 0; a < W; ++a) lv[W + a] = T(0);
        }
#pragma unroll
        for (int q = 0; q < 4; q += W) V::ld(urow + ca + q, uv + q);
        if (wb) {
#pragma unroll
          for (int q = 0; q < 4; q += W) V::ld(urow + cb + q, uv + 4 + q);
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) uv[4 + q] = T(0);
        }
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
          for (int b = 0; b < TN; ++b) acc[a][b] -= lv[a] * uv[b];
      }
#pragma unroll
      for (int b = 0; b < TN; ++b) {
        const bool cv = (b < 4) || wb;
        if (!cv) continue;
        const int col = (b < 4) ? (ca + b) : (cb + b - 4);
        T *colp = A + (size_t)mp * (r0 + col) + r0;
        T tmp[W];
#pragma unroll
        for (int a = 0; a < W; ++a) tmp[a] = acc[a][b];
        V::st(colp + ra, tmp);
        if (vb) {
#pragma unroll
          for (int a = 0; a < W; ++a) tmp[a] = acc[W + a][b];
          V::st(colp + rb, tmp);
        }
      }
    }
  }
}

// Unit-lower forward substitution of the 32-vector v (lane r holds v_r) with the
// diagonal block of A at k0 (strictly lower part = L).
template <typename T>
__device__ __forceinline__ T warp_forward_unit(const T *__restrict__ A, int mp, int k0,
                                               T v) {
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < kB; ++c) {
    const T vc = __shfl_sync(0xffffffffu, v, c);
    if (lane > c) v -= A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)] * vc;
  }
  return v;
}

// Upper back substitution of the 32-vector v with the diagonal block at k0.
template <typename T>
__device__ __forceinline__ T warp_backward_upper(const T *__restrict__ A, int mp, int k0,
                                                 T v) {
  const int lane = threadIdx.x & 31;
  for (int c = kB - 1; c >= 0; --c) {
    if (lane == c) v /= A[(size_t)(k0 + c) + (size_t)mp * (k0 + c)];
    const T vc = __shfl_sync(0xffffffffu, v, c);
    if (lane < c) v -= A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)] * vc;
  }
  return v;
}

// Solves U v = v in place (v in shared memory, length mp) with the stored factors.
template <typename T>
__device__ void block_back_solve(const T *__restrict__ A, int mp, T *v) {
  const int tid = threadIdx.x;
  const int nbk = mp / kB;
  for (int kb = nbk - 1; kb >= 0; --kb) {
    const int k0 = kb * kB;
    if (tid < 32) {
      T w = v[k0 + tid];
      w = warp_backward_upper(A, mp, k0, w);
      v[k0 + tid] = w;
    }
    __syncthreads();
    for (int r = tid; r < k0; r += blockDim.x) {
      T acc = T(0);
      for (int c = 0; c < kB; ++c) acc += A[(size_t)r + (size_t)mp * (k0 + c)] * v[k0 + c];
      v[r] -= acc;
    }
    __syncthreads();
  }
}

// Solves L v = v in place (unit lower, stored factors).
template <typename T>
__device__ void block_forward_solve(const T *__restrict__ A, int mp, T *v) {
  const int tid = threadIdx.x;
  const int nbk = mp / kB;
  for (int kb = 0; kb < nbk; ++kb) {
    const int k0 = kb * kB;
    if (tid < 32) {
      T w = v[k0 + tid];
      w = warp_forward_unit(A, mp, k0, w);
      v[k0 + tid] = w;
    }
    __syncthreads();
    for (int r = k0 + kB + tid; r < mp; r += blockDim.x) {
      T acc = T(0);
      for (int c = 0; c < kB; ++c) acc += A[(size_t)r + (size_t)mp * (k0 + c)] * v[k0 + c];
      v[r] -= acc;
    }
    __syncthreads();
  }
}

// res = nu - (I - Gamma) y for the unpermuted system, in FP64, one thread per row
// summing that row's Gamma entries in a fixed order (deterministic).
template <typename T>
__device__ void residual(int m, int P, int mp, long n, long i, GammaRows rows,
                         const T *__restrict__ theta, const double *nu, const T *y,
                         double *res) {
  for (int r = threadIdx.x; r < mp; r += blockDim.x) {
    double v = 0.0;
    if (r < m) {
      v = nu[r] - (double)y[r];
      for (int q = rows.rowptr[r]; q < rows.rowptr[r + 1]; ++q) {
        const int2 ec = rows.ent[q];
        const int j = ec.x / P, k = ec.x % P;
        v += (double)theta[((size_t)j * n + i) * P + k] * (double)y[ec.y];
      }
    }
    res[r] = v;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
    k_lu(int m, int P, int mp, long n, const unsigned *__restrict__ sp,
         const T *__restrict__ theta, T *__restrict__ scratch, double *__restrict__ logdet,
         int *__restrict__ draw_flags, const double *__restrict__ x,
         const T *__restrict__ lambda, RngKey key, bool refine, double *__restrict__ y,
         GammaRows rows) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Smem L(mp, sizeof(T));
  T *D = reinterpret_cast<T *>(smem_raw + L.off_D);
  T *Lp = reinterpret_cast<T *>(smem_raw + L.off_Lp);
  T *Up = reinterpret_cast<T *>(smem_raw + L.off_Up);
  T *z = reinterpret_cast<T *>(smem_raw + L.off_z);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  int *sflag = reinterpret_cast<int *>(smem_raw + L.off_red);
  const int Rmax = L.Rmax;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T *A = scratch + (size_t)blockIdx.x * mp * mp;
  const int nbk = mp / kB;
  const bool solve = (x != nullptr);
  const T tau = (T)kPivotThreshold;

  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    if (tid == 0) *sflag = 0;
    build_system<T>(m, P, mp, n, i, sp, theta, A, x, lambda, key, nu, z);
    double ld = 0.0;  // warp 0's running sum of log|u_kk|
    bool bad = false;
    for (int kb = 0; kb < nbk; ++kb) {
      const int k0 = kb * kB, r0 = k0 + kB, R = mp - r0;
      // (a) diagonal block, warp 0, row per lane
      if (warp == 0) {
        for (int c = 0; c < kB; ++c)
          D[lane * (kB + 1) + c] = A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)];
        __syncwarp();
        for (int k = 0; k < kB; ++k) {
          const T piv = D[k * (kB + 1) + k];
          if (lane > k) {
            const T l = D[lane * (kB + 1) + k] / piv;
            D[lane * (kB + 1) + k] = l;
            if (!(dabs(l) <= tau)) bad = true;
            for (int c = k + 1; c < kB; ++c) D[lane * (kB + 1) + c] -= l * D[k * (kB + 1) + c];
          }
          __syncwarp();
        }
        const T u = D[lane * (kB + 1) + lane];
        if (!(finite_t(u) && u != T(0))) bad = true;
        ld += warp_sum_d(log(fabs((double)u)));
        if (solve)
          for (int c = 0; c < kB; ++c)
            A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)] = D[lane * (kB + 1) + c];
        if (solve) {
          // right-hand side block: z_k <- L_kk^-1 z_k (unit lower, from shared D)
          T w = z[k0 + lane];
          for (int c = 0; c < kB; ++c) {
            const T wc = __shfl_sync(0xffffffffu, w, c);
            if (lane > c) w -= D[lane * (kB + 1) + c] * wc;
          }
          z[k0 + lane] = w;
        }
      }
      __syncthreads();
      // (b) column panel rows r0.. -> Lp and (c) row panel columns r0.. -> Up, solved
      // in place in shared memory (thread t owns column t of Lp or Up); the factors
      // go back to global memory only when a solve needs them later.
      for (int t = tid; t < 2 * R; t += blockDim.x) {
        if (t < R) {
          const int row = r0 + t;
          T *lp = Lp + t;
#pragma unroll 8
          for (int c = 0; c < kB; ++c) lp[c * Rmax] = A[(size_t)row + (size_t)mp * (k0 + c)];
          for (int c = 0; c < kB; ++c) {
            T acc = lp[c * Rmax];
#pragma unroll 4
            for (int cp = 0; cp < c; ++cp) acc -= lp[cp * Rmax] * D[cp * (kB + 1) + c];
            acc = acc / D[c * (kB + 1) + c];
            lp[c * Rmax] = acc;
            if (!(dabs(acc) <= tau)) bad = true;
            if (solve) A[(size_t)row + (size_t)mp * (k0 + c)] = acc;
          }
        } else {
          const int tt = t - R;
          const int col = r0 + tt;
          T *colp = A + (size_t)mp * col + k0;
          T *up = Up + tt;
#pragma unroll
          for (int r = 0; r < kB; r += Vec<T>::W) {
            T v[Vec<T>::W];
            Vec<T>::ld(colp + r, v);
#pragma unroll
            for (int q = 0; q < Vec<T>::W; ++q) up[(r + q) * Rmax] = v[q];
          }
          for (int r = 1; r < kB; ++r) {
            T acc = up[r * Rmax];
#pragma unroll 4
            for (int rp = 0; rp < r; ++rp) acc -= D[r * (kB + 1) + rp] * up[rp * Rmax];
            up[r * Rmax] = acc;
          }
          if (solve) {
#pragma unroll
            for (int r = 0; r < kB; r += Vec<T>::W) {
              T v[Vec<T>::W];
#pragma unroll
              for (int q = 0; q < Vec<T>::W; ++q) v[q] = up[(r + q) * Rmax];
              Vec<T>::st(colp + r, v);
            }
          }
        }
      }
      __syncthreads();
      // (d) trailing update, plus the right-hand side below the block
      if (R > 0) {
        if (solve) {
          for (int t = tid; t < R; t += blockDim.x) {
            T acc = T(0);
            for (int k = 0; k < kB; ++k) acc += Lp[k * Rmax + t] * z[k0 + k];
            z[r0 + t] -= acc;
          }
        }
        trailing_update<T>(A, mp, r0, R, Lp, Up, Rmax);
      }
      __syncthreads();
    }
    if (bad) atomicOr(sflag, 1);
    __syncthreads();
    const bool flagged = (*sflag != 0);
    if (tid == 0) {
      logdet[i] = ld;
      if (flagged) atomicOr(&draw_flags[i], DRAW_FLAG_PIVOT);
    }
    if (solve && !flagged) {
      block_back_solve<T>(A, mp, z);  // z = y0
      if (refine) {
        residual<T>(m, P, mp, n, i, rows, theta, nu, z, res);
        T *d = Up;  // the row-panel buffer (32 x Rmax >= m_p) holds the correction
        for (int r = tid; r < mp; r += blockDim.x) d[r] = (T)res[r];
        __syncthreads();
        block_forward_solve<T>(A, mp, d);
        block_back_solve<T>(A, mp, d);
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)z[r] + (double)d[r];
      } else {
        for (int r = tid; r < m; r += blockDim.x) y[(size_t)i * m + r] = (double)z[r];
      }
    }
    __syncthreads();
  }
}

// Partial-pivoting LU for the draws the blocked pass flagged (getrf semantics).
// Unblocked and slow; it only runs on the rare draws whose (I - Gamma) is not
// diagonally dominant enough for the no-pivot pass.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_lu_fallback(int m, int P, int mp, long n, const unsigned *__restrict__ sp,
                  const T *__restrict__ theta, T *__restrict__ scratch,
                  double *__restrict__ logdet, int *__restrict__ draw_flags,
                  const double *__restrict__ x, const T *__restrict__ lambda, RngKey key,
                  double *__restrict__ y, GammaRows rows) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Smem L(mp, sizeof(T));
  T *z = reinterpret_cast<T *>(smem_raw + L.off_z);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  double *red = reinterpret_cast<double *>(smem_raw + L.off_red);  // 64 doubles
  int *perm = reinterpret_cast<int *>(smem_raw + L.off_Lp);        // mp ints
  T *d = reinterpret_cast<T *>(smem_raw + L.off_Up);               // mp values
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  T *A = scratch + (size_t)blockIdx.x * mp * mp;
  const bool solve = (x != nullptr);
  __shared__ int s_piv;
  __shared__ bool s_singular;

  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    if (!(draw_flags[i] & DRAW_FLAG_PIVOT)) continue;
    build_system<T>(m, P, mp, n, i, sp, theta, A, x, lambda, key, nu, z);
    for (int r = tid; r < mp; r += blockDim.x) perm[r] = r;
    if (tid == 0) s_singular = false;
    __syncthreads();
    double ld = 0.0;
    for (int k = 0; k < mp; ++k) {
      // pivot search over rows k.. of column k
      double best = -1.0;
      int bidx = k;
      for (int r = k + tid; r < mp; r += blockDim.x) {
        const double v = fabs((double)A[(size_t)r + (size_t)mp * k]);
        if (v > best) {
          best = v;
          bidx = r;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
          best = ov;
          bidx = oi;
        }
      }
      if (lane == 0) {
        red[warp] = best;
        red[32 + warp] = (double)bidx;
      }
      __syncthreads();
      if (tid == 0) {
        double b = red[0];
        int bi = (int)red[32];
        for (int w = 1; w < nwarps; ++w) {
          if (red[w] > b || (red[w] == b && (int)red[32 + w] < bi)) {
            b = red[w];
            bi = (int)red[32 + w];
          }
        }
        s_piv = bi;
        if (!(b > 0.0) || !(b <= 3.0e38)) s_singular = true;
      }
      __syncthreads();
      if (s_singular) break;
      const int pr = s_piv;
      if (pr != k) {
        for (int c = tid; c < mp; c += blockDim.x) {
          const T t0 = A[(size_t)k + (size_t)mp * c];
          A[(size_t)k + (size_t)mp * c] = A[(size_t)pr + (size_t)mp * c];
          A[(size_t)pr + (size_t)mp * c] = t0;
        }
        if (tid == 0) {
          const int tp = perm[k];
          perm[k] = perm[pr];
          perm[pr] = tp;
          const T tz = z[k];
          z[k] = z[pr];
          z[pr] = tz;
        }
      }
      __syncthreads();
      const T piv = A[(size_t)k + (size_t)mp * k];
      ld += log(fabs((double)piv));
      for (int r = k + 1 + tid; r < mp; r += blockDim.x)
        A[(size_t)r + (size_t)mp * k] /= piv;
      __syncthreads();
      const int rem = mp - k - 1;
      for (long e = tid; e < (long)rem * rem; e += blockDim.x) {
        const int r = k + 1 + (int)(e % rem), c = k + 1 + (int)(e / rem);
        A[(size_t)r + (size_t)mp * c] -= A[(size_t)r + (size_t)mp * k] * A[(size_t)k + (size_t)mp * c];
      }
      if (solve) {
        for (int r = k + 1 + tid; r < mp; r += blockDim.x)
          z[r] -= A[(size_t)r + (size_t)mp * k] * z[k];
      }
      __syncthreads();
    }
    if (tid == 0) {
      if (s_singular) {
        logdet[i] = -INFINITY;
        atomicOr(&draw_flags[i], DRAW_FLAG_SINGULAR | DRAW_FLAG_REDONE);
      } else {
        logdet[i] = ld;
        atomicOr(&draw_flags[i], DRAW_FLAG_REDONE);
      }
    }
    __syncthreads();
    if (solve) {
      if (s_singular) {
        for (int r = tid; r < m; r += blockDim.x) y[(size_t)i * m + r] = NAN;
      } else {
        block_back_solve<T>(A, mp, z);
        residual<T>(m, P, mp, n, i, rows, theta, nu, z, res);
        for (int r = tid; r < mp; r += blockDim.x) d[r] = (T)res[perm[r]];
        __syncthreads();
        block_forward_solve<T>(A, mp, d);
        block_back_solve<T>(A, mp, d);
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)z[r] + (double)d[r];
      }
    }
    __syncthreads();
  }
}

}  // namespace

template <typename T> LuPlan plan_lu(int m, int P, long n, int num_sms) {
  LuPlan pl{};
  pl.m = m;
  pl.P = P;
  pl.mp = ((m + kB - 1) / kB) * kB;
  pl.block = kThreads;
  pl.smem = Smem(pl.mp, sizeof(T)).total;
  // k_lu_fallback adds a few bytes of static shared memory on top of pl.smem
  int ctas_per_sm = (int)((227u * 1024u) / (pl.smem + 1024));
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  if (ctas_per_sm > 2) ctas_per_sm = 2;
  long grid = (long)num_sms * ctas_per_sm;
  if (grid > n) grid = n;
  if (grid < 1) grid = 1;
  pl.grid = (int)grid;
  pl.scratch_elems_per_cta = (size_t)pl.mp * pl.mp;
  (void)P;
  return pl;
}

template <typename T>
void launch_lu(cudaStream_t s, const LuPlan &pl, long n, const unsigned *sp,
               const T *theta, T *scratch, double *logdet, int *draw_flags,
               const double *x, const T *lambda, RngKey key, bool refine, double *y,
               GammaRows rows) {
  // opt in to exactly the shared memory this plan needs (a failure here shows up
  // as a launch error that the engine reports)
  if (pl.smem > 48 * 1024)
    cudaFuncSetAttribute(k_lu<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  k_lu<T><<<pl.grid, pl.block, pl.smem, s>>>(pl.m, pl.P, pl.mp, n, sp, theta, scratch,
                                             logdet, draw_flags, x, lambda, key, refine, y, rows);
}

template <typename T>
void launch_lu_fallback(cudaStream_t s, const LuPlan &pl, long n, const unsigned *sp,
                        const T *theta, T *scratch, double *logdet, int *draw_flags,
                        const double *x, const T *lambda, RngKey key, double *y,
                        GammaRows rows) {
  if (pl.smem > 48 * 1024)
    cudaFuncSetAttribute(k_lu_fallback<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)pl.smem);
  k_lu_fallback<T><<<pl.grid, pl.block, pl.smem, s>>>(pl.m, pl.P, pl.mp, n, sp, theta,
                                                      scratch, logdet, draw_flags, x,
                                                      lambda, key, y, rows);
}

template LuPlan plan_lu<float>(int, int, long, int);
template LuPlan plan_lu<double>(int, int, long, int);
template void launch_lu<float>(cudaStream_t, const LuPlan &, long, const unsigned *,
                               const float *, float *, double *, int *, const double *,
                               const float *, RngKey, bool, double *, GammaRows);
template void launch_lu<double>(cudaStream_t, const LuPlan &, long, const unsigned *,
                                const double *, double *, double *, int *, const double *,
                                const double *, RngKey, bool, double *, GammaRows);
template void launch_lu_fallback<float>(cudaStream_t, const LuPlan &, long,
                                        const unsigned *, const float *, float *, double *,
                                        int *, const double *, const float *, RngKey,
                                        double *, GammaRows);
template void launch_lu_fallback<double>(cudaStream_t, const LuPlan &, long,
                                         const unsigned *, const double *, double *,
                                         double *, int *, const double *, const double *,
                                         RngKey, double *, GammaRows);

}  // namespace sgdlm
