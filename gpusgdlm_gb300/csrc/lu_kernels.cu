// Batched log|det(I - Gamma_i)| and forecast solves y_i = (I - Gamma_i)^-1 nu_i.
//
// The reference zeroes 2*nsim_batch dense m x m FP64 matrices in HBM, scatters
// the parents, calls cublasDgetrfBatched through a pointer array and, for
// forecasts, cublasDgetriBatched plus a gemv on the explicit inverse
// (rSGDLM/src/SGDLM/SGDLM.cu:231-323, 555-620; kernel_functions.cuh:810-842,
// 905-926; HostWrapperImpl.cu:375-377).
//
// Here a persistent CTA owns one draw at a time and one private slab of scratch.
//  1. Sparse pre-elimination (elimination.hpp): the host planned levels of
//     independent sets; the CTA runs that program over the draw's value slots
//     (in shared memory when they fit), accumulating sum log|pivot| of the
//     eliminated nodes.  The remaining core (about 210 of 400 nodes at m = 400)
//     is written as a dense d_p x d_p matrix through the plan's slot map
//     (d_p = core size rounded up to 32, identity padding).
//  2. Block elimination of the core with 32 x 32 blocks, no chains of
//     dependent scalar solves:
//     (a) one warp inverts the diagonal block D in registers by Gauss-Jordan
//         elimination with 4 x 4 pivot blocks (its pivots are the LU pivots,
//         so they give log|det|), while the other warps stage the column panel
//         C and the row panel B;
//     (b) the multipliers C D^-1 and (c) the trailing update E -= (C D^-1) B:
//         for FP32 draws and d_p <= 224 as tcgen05 MMAs (kind::f16 on a
//         three-way bf16 split of every operand, FP32 accumulation in tensor
//         memory, E's first 128-row tile preloaded while D is inverted, and
//         warp 0 starting the next inversion as soon as the first tile is
//         updated); otherwise register-tiled FMA loops over shared memory.
//     The pass does not pivot: (I - Gamma) is diagonally dominant in the
//     filtering regime.  Every multiplier (the levels', the diagonal blocks'
//     and C D^-1) is checked against kPivotThreshold; a draw with a larger one,
//     or a zero / non-finite pivot, is appended to the redo list and redone by
//     k_lu_fallback: the sparse levels again, then partial pivoting on the
//     dense core (getrf semantics); a draw whose level pivots fail is pivoted
//     over the full matrix.  |det| does not depend on the elimination order.
//  3. Forecasts: the right-hand sides (k_forecast_nu, all draws beforehand) go
//     through the levels' forward program and ride along the block
//     elimination (b2 -= C D^-1 b1); the back solve x1 = D^-1 (b1 - B x2) runs
//     as a pipeline between warps with the stored D^-1, C D^-1 and B, then the
//     levels' backward program (staged in shared memory).  The residual
//     nu - (I - Gamma) y0 from the sparse parent rows (FP64, or double-float
//     FP32 for FP32 draws) drives one refinement solve with the same factors.
#include <algorithm>

#include <cuda_bf16.h>

#include "elimination.hpp"
#include "kernels.hpp"
#include "mma_sync.hpp"
#include "rng.cuh"

namespace sgdlm {
namespace {

constexpr int kB = 32;          // block size
constexpr int kThreads = 256;   // 16 x 16 thread grid of the trailing update
constexpr int kWarps = kThreads / 32;
constexpr double kPivotThreshold = 8.0;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kDs = 36;  // row stride of D^-1 in shared memory (16-byte rows, 4-way store conflicts)
constexpr int kUs = 36;  // stride of the row panel B, stored column by column: B[c][t] at t*kUs + c
constexpr int kGjRows = 224;  // rows of C the panel Gauss-Jordan holds (warps 1..7)
constexpr int kLevFlight = 8;  // chunks of a sparse level in flight per warp
// one super-step of the panel Gauss-Jordan in shared memory: the pivot rows
// (row q, position p at kGjRow q + p; the padding keeps the four writers' 16-byte
// stores on distinct banks), then P^-1 (entry (q, c) at 4 kGjRow + 4q + c)
constexpr int kGjRow = kB + 4;
constexpr int kGjSlot = 4 * kGjRow + 16;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <typename T> __device__ __forceinline__ T dabs(T v) { return v < T(0) ? -v : v; }
template <typename T> __device__ __forceinline__ bool finite_t(T v) {
  return v == v && dabs(v) <= (T)3.0e38;
}
// log|v| in the working precision, returned in double for the FP64 sums
__device__ __forceinline__ double log_abs(float v) { return (double)logf(fabsf(v)); }
__device__ __forceinline__ double log_abs(double v) { return log(fabs(v)); }

// Deterministic block-wide sum (fixed order); `red` holds 32 doubles.
__device__ double block_sum_det(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}
// Block-wide maxima of two non-negative values (a NaN in either counts as
// infinity), over red (at least 2 * warps doubles).
__device__ void block_max2(double &a, double &b, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  a = (a == a) ? a : INFINITY;
  b = (b == b) ? b : INFINITY;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a = fmax(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  __syncthreads();
  if (lane == 0) {
    red[2 * warp] = a;
    red[2 * warp + 1] = b;
  }
  __syncthreads();
  a = b = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    a = fmax(a, red[2 * w]);
    b = fmax(b, red[2 * w + 1]);
  }
}

// Shared-memory carve-up (byte offsets, 16-byte aligned).  dp is the padded
// dense size, m the number of nodes (forecast vectors are node-indexed).  The
// panel buffers Lp (C, column-major, 32 x Rmax) / Up (B, Rmax columns of kUs)
// and the value slots of the sparse levels (nv_smem of them, 0 when they live in
// global memory) share one region: the slots are dead while the panels are in
// use.  prow holds the eight super-steps of the panel Gauss-Jordan.
struct Smem {
  int Rmax, Mpad;
  size_t off_D, off_prow, off_Dt, off_Lp, off_Up, off_vals, off_Lt, off_Ut, part_L, part_U, off_z,
      off_nu, off_res, off_zf, off_yf, off_yd, off_red, off_bsum, total;
  __host__ __device__ Smem(int dp, int m, size_t tsz, int nv_smem, bool tc = false) {
    Rmax = dp - kB > 0 ? dp - kB : kB;
    Mpad = (Rmax + 127) / 128 * 128;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 15) & ~(size_t)15;
      return at;
    };
    off_D = take((size_t)kB * kDs * tsz);
    off_prow = take((size_t)(kB / 4) * kGjSlot * tsz);
    // tensor-core path: D^-1 as the B operand of L = C D^-1 (three bf16 parts of
    // 32 rows x 64 bytes)
    off_Dt = tc ? take((size_t)3 * kB * 64) : o;
    // tensor-core path: three bf16 parts of C D^-1 (Mpad rows) and of B (Rmax
    // columns), each a K-major 32-wide UMMA tile of 64-byte rows
    part_L = (size_t)Mpad * 64;
    part_U = (size_t)Rmax * 64;
    const size_t panels = tc ? 3 * (part_L + part_U) : ((size_t)kB * Rmax + (size_t)Rmax * kUs) * tsz;
    const size_t vals = (((size_t)nv_smem + 3) / 4) * 4 * tsz;
    o = (o + 127) & ~(size_t)127;
    off_Lp = take(panels > vals ? panels : vals);
    off_Up = off_Lp + (size_t)kB * Rmax * tsz;
    off_Lt = off_Lp;
    off_Ut = off_Lp + 3 * part_L;
    off_vals = off_Lp;
    off_z = take((size_t)dp * tsz);
    off_nu = take((size_t)m * sizeof(double));
    off_res = take((size_t)m * sizeof(double));
    off_zf = take((size_t)m * tsz);
    off_yf = take((size_t)m * tsz);
    off_yd = take((size_t)m * tsz);
    off_red = take(64 * sizeof(double));
    off_bsum = take((size_t)kWarps * kB * tsz);
    total = o;
  }
};

// Shared memory of the pivoting redo: the 32-column panel (column-major, stride
// of the factored matrix's order, at most mp), one 128-column chunk of the row
// panel U12, the right-hand side and correction, the row permutation, one
// diagonal block, the FP64 forecast vectors and the node-indexed vectors of the
// levels' solve programs.
constexpr int kFbChunk = 128;
constexpr int kFbRefine = 3;  // refinement steps of the pivoting pass's forecast solves, at most
// ... fewer once a correction is below this fraction of the solution (FP32
// resolution: a further step could only re-round the result)
constexpr double kFbRefineStop = 1e-7;
// Whether a refinement correction dv is below kFbRefineStop of the solution yv
// over the first m entries (uniform over the block: block_max2 ends on a barrier
// and every thread reads the same maxima; a NaN counts as not done).
template <typename T>
__device__ bool refine_done(int m, const T *dv, const T *yv, double *red) {
  double dmax = 0.0, ymax = 0.0;
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    const double ad = fabs((double)dv[r]), ay = fabs((double)yv[r]);
    dmax = (ad == ad && ad > dmax) ? ad : ((ad == ad) ? dmax : INFINITY);
    ymax = (ay == ay && ay > ymax) ? ay : ((ay == ay) ? ymax : INFINITY);
  }
  block_max2(dmax, ymax, red);
  return ymax < INFINITY && dmax <= kFbRefineStop * ymax;
}
// the redo eliminates the sparse levels unpivoted unless a multiplier exceeds this
// (then it pivots over the full matrix)
constexpr double kLevelMultMax = 65536.0;
// the fast pass's forecast of a draw is kept when its refinement correction is at
// most this fraction of the solution (the error left is about its square)
constexpr double kRefineTol = 1e-3;
struct FallbackSmem {
  size_t off_pan, off_U, off_core, off_piv, off_pivabs, off_cand, off_D, off_z, off_d, off_perm,
      off_nu, off_res, off_red, off_zf, off_yf, off_yd, off_crow, off_ccv, off_cci, off_disp,
      total;
  // core_dp > 0: the dense core (core_dp x core_dp) is factored in shared memory,
  // in a region that the full-matrix path's panel buffers share
  __host__ __device__ FallbackSmem(int mp, int m, size_t tsz, int core_dp = 0) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 15) & ~(size_t)15;
      return at;
    };
    const size_t pan_bytes = ((size_t)kB * mp * tsz + 15) & ~(size_t)15;
    const size_t u_bytes = (size_t)kFbChunk * kUs * tsz;
    const size_t core_bytes = (size_t)core_dp * core_dp * tsz;
    const size_t region = core_bytes > pan_bytes + u_bytes ? core_bytes : pan_bytes + u_bytes;
    off_core = off_pan = take(region);
    off_U = off_pan + pan_bytes;
    off_piv = take((size_t)kB * sizeof(int));
    off_pivabs = take((size_t)mp * tsz);
    off_cand = take((size_t)2 * kWarps * (tsz > 4 ? tsz : 4));
    off_crow = take((size_t)2 * kWarps * kB * tsz);
    off_ccv = take((size_t)2 * kWarps * tsz);
    off_cci = take((size_t)2 * kWarps * sizeof(int));
    off_disp = take((size_t)kB * sizeof(int));
    off_D = take((size_t)kB * (kB + 1) * tsz);
    off_z = take((size_t)mp * tsz);
    off_d = take((size_t)mp * tsz);
    off_perm = take((size_t)mp * sizeof(int));
    off_nu = take((size_t)m * sizeof(double));
    off_res = take((size_t)m * sizeof(double));
    off_red = take(64 * sizeof(double));
    off_zf = take((size_t)m * tsz);
    off_yf = take((size_t)m * tsz);
    off_yd = take((size_t)m * tsz);
    total = o;
  }
};

// The draws' theta, series-major (theta[(j*n + i)*P + k], the sampler's layout),
// and, when present, their Gamma entries draw-major (GammaDraws: draw i's entry q
// at g[i*nnz + q], q the CSR position of the entry = its index in the plan's
// level-0 list), so that a draw's Gamma values are one contiguous run.
template <typename T> struct Theta {
  const T *sm, *g;
  int m, P, nnz;
  long n;
  // by theta index e = j*P + k (series-major copy)
  __device__ __forceinline__ T at(long i, int e) const {
    return sm[((size_t)(e / P) * n + i) * P + e % P];
  }
  // Gamma entry q of draw i, whose theta index is e
  __device__ __forceinline__ T gamma(long i, int q, int e) const {
    return g ? g[(size_t)i * nnz + q] : at(i, e);
  }
  __device__ __forceinline__ const T *row(long i, int j) const {
    return sm + ((size_t)j * n + i) * P;
  }
};

// nu_j = z/sqrt(lambda) + sum over external predictors x_jk theta_jk for draw i
// (batchedComputeNuPlusMu, kernel_functions.cuh:1156-1178), into nu (double).
template <typename T>
__device__ void forecast_rhs(int m, int P, long n, long i, GammaRows rows, Theta<T> theta,
                             const double *__restrict__ x,
                             const T *__restrict__ lambda, RngKey key, double *nu) {
  const uint32_t ep = key_epoch(key);
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const U4 g = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_NU, 0), ep, key.k0, key.k1);
    T z0, z1;
    box_muller<T>(g.x, g.y, z0, z1);
    const T lam = lambda[(size_t)j * n + i];
    double v = (double)(z0 / dev_sqrt(lam));
    const T *th = theta.row(i, j);
    for (int q = rows.ext_ptr[j]; q < rows.ext_ptr[j + 1]; ++q) {
      const int k = rows.ext_k[q];
      v += x[(size_t)j * P + k] * (double)th[k];
    }
    nu[j] = v;
  }
}

// The forecast right-hand sides of every (draw, series) pair in one launch (the
// Philox stream of forecast_rhs), written series-major (nu[j*n + i], coalesced
// over draws); the LU kernel then reads its draw's m values in one round instead
// of generating them on its critical path.  FP32 draws: the sum in FP32 with an
// FP32 copy of x (x32; FP64 is a narrow pipe on this GPU, and the normals are
// FP32 already), one conversion for the stored value; FP64 draws: in FP64.
template <typename T>
__global__ void __launch_bounds__(128)
    k_forecast_nu(int m, int P, long n, GammaRows rows, const T *__restrict__ theta,
                  const double *__restrict__ x, const float *__restrict__ x32,
                  const T *__restrict__ lambda, RngKey key, double *__restrict__ nu) {
  const int j = blockIdx.y;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t ep = key_epoch(key);
  const U4 g = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_NU, 0), ep, key.k0, key.k1);
  T z0, z1;
  box_muller<T>(g.x, g.y, z0, z1);
  const T lam = lambda[(size_t)j * n + i];
  const T *th = theta + ((size_t)j * n + i) * P;
  if constexpr (sizeof(T) == 4) {
    float v = z0 / dev_sqrt(lam);
    for (int q = rows.ext_ptr[j]; q < rows.ext_ptr[j + 1]; ++q) {
      const int k = rows.ext_k[q];
      v = fmaf(x32[(size_t)j * P + k], th[k], v);
    }
    nu[(size_t)j * n + i] = (double)v;
  } else {
    double v = (double)(z0 / dev_sqrt(lam));
    for (int q = rows.ext_ptr[j]; q < rows.ext_ptr[j + 1]; ++q) {
      const int k = rows.ext_k[q];
      v += x[(size_t)j * P + k] * (double)th[k];
    }
    nu[(size_t)j * n + i] = v;
  }
}

// Writes the identity plus the scattered -theta entries of draw i into the full
// mp x mp matrix A (fillGammas, kernel_functions.cuh:822-842).
template <typename T>
__device__ void build_full(int m, int P, int mp, long n, long i, const unsigned *__restrict__ sp,
                           Theta<T> theta, T *__restrict__ A) {
  const int tid = threadIdx.x;
  const size_t n16 = (size_t)mp * mp * sizeof(T) / 16;
  uint4 *A16 = reinterpret_cast<uint4 *>(A);
  for (size_t e = tid; e < n16; e += blockDim.x) A16[e] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  for (int r = tid; r < mp; r += blockDim.x) A[(size_t)r * mp + r] = T(1);
  const size_t mm = (size_t)m * m;
  for (int e = tid; e < m * P; e += blockDim.x) {
    const unsigned pos = sp[e];
    if ((size_t)pos < mm) {
      const int row = (int)(pos % (unsigned)m), col = (int)(pos / (unsigned)m);
      A[row + (size_t)mp * col] = -theta.at(i, e);
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

// Two consecutive values (8 or 16 bytes) from shared memory.
template <typename T> struct Pair;
template <> struct Pair<float> {
  __device__ static __forceinline__ void ld(const float *p, float *o) {
    const float2 v = *reinterpret_cast<const float2 *>(p);
    o[0] = v.x; o[1] = v.y;
  }
};
template <> struct Pair<double> {
  __device__ static __forceinline__ void ld(const double *p, double *o) {
    const double2 v = *reinterpret_cast<const double2 *>(p);
    o[0] = v.x; o[1] = v.y;
  }
};

// Register-tiled trailing update A[r0:, r0:] -= Lp B over the rows r0 .. r0+R and
// the C columns r0+c_off .. (a chunk of the R x R trailing matrix; R and C are
// multiples of 32), B (32 x C) read from Up[t * Us + c] with t relative to the
// chunk.  The region is cut exactly into units of 2W rows x 8 columns: rows
// {ra .. ra+W-1, ra+R/2 .. ra+R/2+W-1} and columns {ca .. ca+3, ca+C/2 .. ca+C/2+3},
// handed round-robin to the nthr threads tid = 0 .. nthr-1 (no padded tiles).  Consecutive threads take
// consecutive row groups, so Lp reads are conflict-free 16-byte vectors over one
// contiguous line, B reads see at most two addresses per warp, and the global
// loads and stores of the accumulators are coalesced 16-byte vectors.
template <typename T>
__device__ __forceinline__ void trailing_update(T *__restrict__ A, int mp, int r0, int R,
                                                int c_off, int C, const T *__restrict__ Lp,
                                                const T *__restrict__ Up, int Rmax, int Us = kUs,
                                                int tid = threadIdx.x, int nthr = blockDim.x) {
  using V = Vec<T>;
  constexpr int W = V::W;
  constexpr int TM = 2 * W, TN = 8;
  const int nrg = R / (2 * W), hr = R / 2, hc = C / 2;
  const int nu = nrg * (C / 8);
  T *Abase = A + (size_t)mp * (r0 + c_off) + r0;
  // whole units in full rounds of the block; the rest as quarter units below
  const int full = (nu / nthr) * nthr;
  for (int u = tid; u < full; u += nthr) {
    const int cg = u / nrg, rg = u - cg * nrg;
    const int ra = rg * W, rb = ra + hr;
    const int ca = cg * 4, cb = ca + hc;
    T acc[TM][TN];
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int col = (b < 4) ? (ca + b) : (cb + b - 4);
      const T *colp = Abase + mp * col;
      T tmp[W];
      V::ld(colp + ra, tmp);
#pragma unroll
      for (int a = 0; a < W; ++a) acc[a][b] = tmp[a];
      V::ld(colp + rb, tmp);
#pragma unroll
      for (int a = 0; a < W; ++a) acc[W + a][b] = tmp[a];
    }
#pragma unroll 1
    for (int k2 = 0; k2 < kB; k2 += 2) {
      T u2[TN][2];
#pragma unroll
      for (int b = 0; b < TN; ++b) {
        const int col = (b < 4) ? (ca + b) : (cb + b - 4);
        Pair<T>::ld(Up + col * Us + k2, u2[b]);
      }
#pragma unroll
      for (int kk = 0; kk < 2; ++kk) {
        T lv[TM];
        const T *lrow = Lp + (k2 + kk) * Rmax;
        V::ld(lrow + ra, lv);
        V::ld(lrow + rb, lv + W);
#pragma unroll
        for (int a = 0; a < TM; ++a)
#pragma unroll
          for (int b = 0; b < TN; ++b) acc[a][b] -= lv[a] * u2[b][kk];
      }
    }
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const int col = (b < 4) ? (ca + b) : (cb + b - 4);
      T *colp = Abase + mp * col;
      T tmp[W];
#pragma unroll
      for (int a = 0; a < W; ++a) tmp[a] = acc[a][b];
      V::st(colp + ra, tmp);
#pragma unroll
      for (int a = 0; a < W; ++a) tmp[a] = acc[W + a][b];
      V::st(colp + rb, tmp);
    }
  }
  // the last, partial round: quarter units (W rows x 4 columns) so that every
  // thread gets nearly the same share; consecutive threads take consecutive row
  // groups of the same quarter
  const int nrem = nu - full, nq = 4 * nrem;
  for (int v = tid; v < nq; v += nthr) {
    const int qd = v / nrem, u = full + (v - qd * nrem);
    const int cg = u / nrg, rg = u - cg * nrg;
    const int ra = rg * W + ((qd & 1) ? hr : 0);
    const int ca = cg * 4 + ((qd & 2) ? hc : 0);
    T acc[W][4];
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      T tmp[W];
      V::ld(Abase + mp * (ca + b) + ra, tmp);
#pragma unroll
      for (int a = 0; a < W; ++a) acc[a][b] = tmp[a];
    }
#pragma unroll 1
    for (int k2 = 0; k2 < kB; k2 += 2) {
      T u2[4][2];
#pragma unroll
      for (int b = 0; b < 4; ++b) Pair<T>::ld(Up + (ca + b) * Us + k2, u2[b]);
#pragma unroll
      for (int kk = 0; kk < 2; ++kk) {
        T lv[W];
        V::ld(Lp + (k2 + kk) * Rmax + ra, lv);
#pragma unroll
        for (int a = 0; a < W; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) acc[a][b] -= lv[a] * u2[b][kk];
      }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      T tmp[W];
#pragma unroll
      for (int a = 0; a < W; ++a) tmp[a] = acc[a][b];
      V::st(Abase + mp * (ca + b) + ra, tmp);
    }
  }
}

// Asynchronous global -> shared copies (cp.async), so that the panel staging
// overlaps the Gauss-Jordan steps.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Issues the copies of rows t_begin.. of the column panel C (rows r0.., columns
// k0..k0+31) into Lp[c * Rmax + t] and of the row panel B (rows k0..k0+31,
// columns r0..) into Up[t * kUs + c]; both are 16-byte pieces of contiguous
// global columns.
template <typename T>
__device__ __forceinline__ void stage_panels_async(const T *__restrict__ A, int dp, int k0, int r0,
                                                   int R, int t_begin, T *Lp, T *Up, int Rmax) {
  constexpr int W = Vec<T>::W;
  const int RW = (R - t_begin) / W, nc = kB * RW;
  for (int u = threadIdx.x; u < nc; u += blockDim.x) {
    const int c = u / RW, t = t_begin + (u - c * RW) * W;
    cp_async16(Lp + c * Rmax + t, A + (size_t)(r0 + t) + (size_t)dp * (k0 + c));
  }
  constexpr int QW = kB / W;
  for (int u = threadIdx.x; u < R * QW; u += blockDim.x) {
    const int t = u / QW, q = u - t * QW;
    cp_async16(Up + t * kUs + q * W, A + (size_t)(k0 + q * W) + (size_t)dp * (r0 + t));
  }
}

// Reciprocal on the elimination's critical path.  FP32: the hardware
// approximation refined by one Newton-Raphson step, r' = r + r (1 - x r) (the
// classical quadratically convergent reciprocal iteration), accurate to about
// 1 ulp; FP64: the IEEE quotient.
__device__ __forceinline__ float rcp_fast(float x) {
  const float r = __fdividef(1.0f, x);
  return fmaf(r, fmaf(-x, r, 1.0f), r);
}
__device__ __forceinline__ double rcp_fast(double x) { return 1.0 / x; }

// ---- tensor-core (tcgen05) trailing update for the mixed precision ------------
// E -= L U with L = C D^-1 (R x 32) and U = B (32 x R) split three ways into
// bf16, x = h + m + l (h = bf16(x), m = bf16(x - h), l = bf16(x - h - m)); the six
// products h.h + h.m + m.h + h.l + m.m + l.h accumulate in FP32 into E held in
// tensor memory, which leaves an FP32-level error.  Operands are K-major UMMA
// tiles without swizzle: core matrices of 8 rows x 16 bytes, the four K-chunks of
// a row group 128 bytes apart (LBO) and row groups 512 bytes apart (SBO).
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;  // leading byte offset: next K-chunk
  d |= (uint64_t)(512 >> 4) << 32;  // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;           // descriptor version of tcgen05
  return d;                         // base offset 0, no swizzle
}
// kind::f16 instruction descriptor: D f32, A and B bf16, K-major, M = 128, N
// columns; negate: A negated (D -= A B).
__device__ __forceinline__ uint32_t umma_idesc(int N, bool negate = true) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (negate ? (1u << 13) : 0u) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}
// byte offset of (row n, k) in a K-major 32-wide bf16 tile
__device__ __forceinline__ int umma_off(int n, int k) {
  return (n >> 3) * 512 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ uint32_t bf16_pair(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}
// Writes row n (32 values) of a split operand: three parts, part_bytes apart.
__device__ __forceinline__ void write_split_row(unsigned char *tile, size_t part_bytes, int n,
                                                const float (&x)[kB]) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    uint32_t h[4], mm[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      __nv_bfloat16 hv[2], mv[2], lv[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const float v = x[8 * c + 2 * e + u];
        hv[u] = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(hv[u]);
        mv[u] = __float2bfloat16_rn(r1);
        lv[u] = __float2bfloat16_rn(r1 - __bfloat162float(mv[u]));
      }
      h[e] = bf16_pair(hv[0], hv[1]);
      mm[e] = bf16_pair(mv[0], mv[1]);
      l[e] = bf16_pair(lv[0], lv[1]);
    }
    unsigned char *d = tile + umma_off(n, 8 * c);
    *reinterpret_cast<uint4 *>(d) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(d + part_bytes) = make_uint4(mm[0], mm[1], mm[2], mm[3]);
    *reinterpret_cast<uint4 *>(d + 2 * part_bytes) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// Writes K-chunk c (values 8c .. 8c + 7, given in x) of row n of a split operand.
__device__ __forceinline__ void write_split_chunk(unsigned char *tile, size_t part_bytes, int n,
                                                  int c, const float (&x)[8]) {
  uint32_t h[4], mm[4], l[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    __nv_bfloat16 hv[2], mv[2], lv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const float v = x[2 * e + u];
      hv[u] = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(hv[u]);
      mv[u] = __float2bfloat16_rn(r1);
      lv[u] = __float2bfloat16_rn(r1 - __bfloat162float(mv[u]));
    }
    h[e] = bf16_pair(hv[0], hv[1]);
    mm[e] = bf16_pair(mv[0], mv[1]);
    l[e] = bf16_pair(lv[0], lv[1]);
  }
  unsigned char *d = tile + umma_off(n, 8 * c);
  *reinterpret_cast<uint4 *>(d) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4 *>(d + part_bytes) = make_uint4(mm[0], mm[1], mm[2], mm[3]);
  *reinterpret_cast<uint4 *>(d + 2 * part_bytes) = make_uint4(l[0], l[1], l[2], l[3]);
}

// The CTA's MMA completion barrier and its give-up flag (mma_sync.hpp).
struct MmaSync {
  uint64_t bar;
  int dead;
};

__device__ __forceinline__ bool mma_poll(const MmaSync *ms, uint32_t phase, int polls) {
  uint32_t done = 0;
  for (int it = 0; it < polls && !done; ++it)
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(&ms->bar)), "r"(phase));
  return done != 0;
}

// Bounded wait for the MMAs committed to ms->bar (the rules of mma_sync.hpp): a
// late completion marks the draw bad and is drained so the phase stays in step;
// a completion never seen makes the CTA give the barrier up (ms->dead).
__device__ __forceinline__ void mma_wait(MmaSync *ms, uint32_t &mphase, bool &bad) {
  const bool dead = *reinterpret_cast<volatile int *>(&ms->dead) != 0;
  bool first = false, drained = false;
  if (!dead) {
    first = mma_poll(ms, mphase, kMmaPolls);
    if (!first) drained = mma_poll(ms, mphase, kMmaDrainPolls);
  }
  if (mma_wait_rule(dead, first, drained, mphase, bad) == kMmaLost)
    *reinterpret_cast<volatile int *>(&ms->dead) = 1;
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// Whether the CTA still issues MMAs (it stops once it has given its barrier up).
__device__ __forceinline__ bool mma_live(const MmaSync *ms) {
  return *reinterpret_cast<const volatile int *>(&ms->dead) == 0;
}

// The six split products of one 128-row tile, K = 32 (two K-steps of 16):
// D (+)= A B^T with A = la (three parts, part_a apart) and B = lb (part_b apart).
__device__ __forceinline__ void umma_split_tile(uint32_t d_tmem, uint32_t la, size_t part_a,
                                                uint32_t lb, size_t part_b, uint32_t idesc,
                                                bool accumulate) {
  const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const uint64_t ad = umma_desc(la + (uint32_t)(pa[q] * part_a) + ks * 256);
      const uint64_t bd = umma_desc(lb + (uint32_t)(pb[q] * part_b) + ks * 256);
      const uint32_t acc = (accumulate || ks > 0 || q > 0) ? 1u : 0u;
      asm volatile(
          "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
          "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
          "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
    }
}

// The block multipliers L = C D^-1 (R x 32) on the tensor cores: C split in Lt
// (rows of C, K-major), D^-1 split in Dt (its columns as rows), one 128-row tile
// per 32 columns of tensor memory from column kTmemL (the columns below hold the
// first tile of the trailing update, loaded meanwhile).  Each thread then reads one row of L back,
// checks |L| <= tau (the no-pivot criterion of the rows of C), writes it split
// into Lt (in place of C: the MMAs have completed) as the A operand of the
// trailing update and, when solving, applies it to the right-hand side and keeps
// it in A.  Warp w reads tile w / 4, lanes 32 (w % 4) ..
constexpr int kTmemL = 192;
__device__ void tc_block_multipliers(float *__restrict__ A, int dp, int k0, int r0, int R,
                                     unsigned char *Lt, size_t part_L, const unsigned char *Dt,
                                     uint32_t tmem, MmaSync *mbar, uint32_t &mphase, float tau,
                                     float *z, bool solve, bool &bad) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0 && mma_live(mbar)) {
    for (int mt = 0; mt < R; mt += 128)
      umma_split_tile(tmem + kTmemL + (uint32_t)(mt / 128) * kB, smem_u32(Lt) + (uint32_t)(mt / 8) * 512,
                      part_L, smem_u32(Dt), (size_t)kB * 64, umma_idesc(kB, false), false);
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(&mbar->bar)));
  }
  mma_wait(mbar, mphase, bad);
  const int tile = warp >> 2, quarter = warp & 3;
  if (tile * 128 < R) {
    const int row = tile * 128 + quarter * 32 + lane;
    uint32_t v[kB];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(tmem + ((uint32_t)(quarter * 32) << 16) + kTmemL + (uint32_t)tile * kB));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (row < R) {
      float l[kB];
#pragma unroll
      for (int q = 0; q < kB; ++q) {
        l[q] = __uint_as_float(v[q]);
        bad |= !(fabsf(l[q]) <= tau);
      }
      write_split_row(Lt, part_L, row, l);
      if (solve) {
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < kB; ++q) acc += l[q] * z[k0 + q];
        z[r0 + row] -= acc;
        float *rowp = A + (size_t)(r0 + row) + (size_t)dp * k0;
#pragma unroll
        for (int q = 0; q < kB; ++q) rowp[(size_t)dp * q] = l[q];
      }
    }
  }
  asm volatile("fence.proxy.async.shared::cta;");
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// Named barriers of the tensor-core path (barrier 0 is __syncthreads; 1..8 are
// the Gauss-Jordan super-steps of the FFMA path).
constexpr int kBarRest = 9;       // warps 1..7 (224 threads)
constexpr int kBarQuarter0 = 10;  // warps 0 and 4 (64 threads): tensor-memory lanes 0..31
constexpr int kBarDt = 11;        // warp 0 and warps 1, 2, 3, 5 (160 threads): D^-1 -> Dt
__device__ __forceinline__ void named_arrive_n(int id, int n) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void named_sync_n(int id, int n) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// 16 columns of tensor memory at taddr into v.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}
// The two-tile update's product -L U (this warp's lanes, columns [cb, ce), a
// multiple of 16 wide) is added to E in global memory in 16-column chunks: a
// chunk's E loads and its tensor-memory read are issued together and waited for
// once (8-column chunks, each loaded one chunk ahead, took 1 % longer per VB pass;
// 32-column chunks spill).  Not inlined: its registers stay out of the kernel's
// peak.  Rows at or beyond R are padding: never loaded or stored.
__device__ __noinline__ void tmem_add_e(float *E, int dp, int R, int row, int cb, int ce,
                                        uint32_t tlane) {
  for (int c0 = cb; c0 < ce; c0 += 16) {
    float e[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) e[j] = row < R ? E[(size_t)row + (size_t)dp * (c0 + j)] : 0.f;
    uint32_t v[16];
    tmem_ld16(tlane + (uint32_t)c0, v);
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (row < R) {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        E[(size_t)row + (size_t)dp * (c0 + j)] = __fadd_rn(e[j], __uint_as_float(v[j]));
    }
  }
}

// Single-tile updates (R <= 128) keep E's tile in tensor memory: warps 1..7
// load it into columns 0 .. R-1 while warp 0 inverts the diagonal block
// (tc_preload_tile0), the MMAs put -L U into columns kTmemU .. kTmemU + R - 1
// (free then: the block multipliers there have been read out), and the sum is
// formed from the two in FP32 with round-to-nearest.
constexpr int kTmemU = 128;
__device__ __forceinline__ void e_to_tmem(const float *E, int dp, int R, int row, int cb, int ce,
                                          uint32_t tlane) {
  for (int c0 = cb; c0 < ce; c0 += 16) {
    uint32_t v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j)
      v[j] = __float_as_uint(row < R ? E[(size_t)row + (size_t)dp * (c0 + j)] : 0.f);
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(tlane + (uint32_t)c0),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
        "r"(v[15]));
  }
  asm volatile("tcgen05.wait::st.sync.aligned;");
}
// E = E + (-L U), both in tensor memory, columns [cb, ce) of this warp's lanes,
// stored to global (rows at or beyond R are not stored).
__device__ __noinline__ void tmem_sum_to_e(float *E, int dp, int R, int row, int cb, int ce,
                                           uint32_t tlane) {
  for (int c0 = cb; c0 < ce; c0 += 16) {
    uint32_t e[16], u[16];
    tmem_ld16(tlane + (uint32_t)c0, e);
    tmem_ld16(tlane + (uint32_t)(kTmemU + c0), u);
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (row < R) {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        E[(size_t)row + (size_t)dp * (c0 + j)] = __fadd_rn(__uint_as_float(e[j]), __uint_as_float(u[j]));
    }
  }
}

// This warp's columns of a 128-row tile of E: lanes 32..127 split the columns in
// halves between warps q and q + 4; lanes 0..31 (the next diagonal block's rows)
// give warp 0 the first 32 columns and warp 4 the rest (in halves when the
// update has two tiles).
__device__ __forceinline__ void e_columns(int warp, int R, bool with_warp0, int &cb, int &ce,
                                          bool halves = false) {
  const int quarter = warp & 3, hc = R / 2;
  if (quarter == 0 && !halves) {
    cb = (warp == 0 || !with_warp0) ? 0 : kB;
    ce = warp == 0 ? kB : R;
  } else {
    cb = (warp >> 2) * hc;
    ce = cb + hc;
  }
}

// The first 128-row tile of E[r0:, r0:] into tensor memory (columns 0 .. R-1,
// R <= 128), by warps 1..7 while warp 0 inverts the diagonal block.  after_d:
// warp 4 first waits for warp 0 to have read the diagonal block out of lanes
// 0..31 (the previous trailing update had one tile too; after two tiles the
// update ended on __syncthreads).
__device__ __forceinline__ void tc_preload_tile0(const float *A, int dp, int r0, int R,
                                                 uint32_t tmem, bool after_d) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, quarter = warp & 3;
  const float *E = A + (size_t)r0 + (size_t)dp * r0;
  int cb, ce;
  e_columns(warp, R, false, cb, ce);
  if (warp == 4 && after_d) {
    named_sync_n(kBarQuarter0, 64);
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  if (quarter * 32 < R)
    e_to_tmem(E, dp, R, quarter * 32 + lane, cb, ce, tmem + ((uint32_t)(quarter * 32) << 16));
}

// E[r0:, r0:] (R x R, leading dimension dp, R <= 192) -= L U on the tensor cores,
// 128-row tiles (rows beyond R are padding: loaded as 0, never stored).  One
// thread issues the 12 MMAs of a tile, -L U accumulated from zero in tensor
// memory, and commits them to mbar; the waiting threads spin with a bound
// (mma_sync.hpp) and then form E + (-L U) in FP32 with round-to-nearest.  The
// tensor cores' own accumulation rounds toward zero (their adder aligns and
// truncates); accumulating onto E itself would shrink every entry of E by about
// half an ulp per MMA and bias log|det| (about -8e-5 at m = 400), while on the
// product alone that rounding is as small as the product.  Warp w moves lanes
// 32 (w % 4) .. (columns: e_columns).
// One tile (R <= 128): E was preloaded into columns 0 .. R-1, the product goes to
// columns kTmemU ..; warp 0 forms the next diagonal block (rows and columns
// r0 .. r0 + 31 of the updated matrix) into dnext (shared, row-major, stride
// kDs) instead of storing it and returns, so that the next panel's Gauss-Jordan
// overlaps the rest of this update and the other warps' splits and preload of the
// next panel; warps 1..7 meet on a named barrier at the end.
// Two tiles (R > 128): the product of each tile goes to columns 0 .. R-1 and E
// comes from global memory (tmem_add_e); warp 4 would carry lanes 0..31 alone
// through both tiles, so lanes 0..31 are split in halves as the other quarters,
// warp 0 stashes the next diagonal block from the first tile, and the update ends
// on __syncthreads.
__device__ void tc_trailing_update(float *__restrict__ A, int dp, int r0, int R,
                                   const unsigned char *Lt, const unsigned char *Ut,
                                   size_t part_L, size_t part_U, uint32_t tmem, MmaSync *mbar,
                                   uint32_t &mphase, bool &bad, float *dnext) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3;
  const bool two = R > 128;
  float *E = A + (size_t)r0 + (size_t)dp * r0;
  const uint32_t idesc = umma_idesc(R);
  const uint32_t tlane = tmem + ((uint32_t)(quarter * 32) << 16);
  int cb, ce;
  e_columns(warp, R, true, cb, ce, two);
  if (!two) {
    const int row = quarter * 32 + lane;
    if (tid == 0 && mma_live(mbar)) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      umma_split_tile(tmem + kTmemU, smem_u32(Lt), part_L, smem_u32(Ut), part_U, idesc, false);
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar->bar)));
    }
    mma_wait(mbar, mphase, bad);
    if (warp == 0) {
#pragma unroll
      for (int h = 0; h < kB; h += 16) {
        uint32_t e[16], u[16];
        tmem_ld16(tlane + (uint32_t)h, e);
        tmem_ld16(tlane + (uint32_t)(kTmemU + h), u);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int q = 0; q < 16; q += 4)
          *reinterpret_cast<float4 *>(dnext + lane * kDs + h + q) = make_float4(
              __fadd_rn(__uint_as_float(e[q]), __uint_as_float(u[q])),
              __fadd_rn(__uint_as_float(e[q + 1]), __uint_as_float(u[q + 1])),
              __fadd_rn(__uint_as_float(e[q + 2]), __uint_as_float(u[q + 2])),
              __fadd_rn(__uint_as_float(e[q + 3]), __uint_as_float(u[q + 3])));
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      // warp 4 may overwrite lanes 0..31 now, in the next panel's preload (there
      // is one when R > 32)
      if (R > kB) named_arrive_n(kBarQuarter0, 64);
      __syncwarp();
      return;
    }
    if (quarter * 32 < R) tmem_sum_to_e(E, dp, R, row, cb, ce, tlane);
    asm volatile("tcgen05.fence::before_thread_sync;");
    named_sync_n(kBarRest, kThreads - 32);
    asm volatile("tcgen05.fence::after_thread_sync;");
    return;
  }
  // ---- two tiles: tile 0, rows 0..127
  {
    const int row = quarter * 32 + lane;
    if (tid == 0 && mma_live(mbar)) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      umma_split_tile(tmem, smem_u32(Lt), part_L, smem_u32(Ut), part_U, idesc, false);
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar->bar)));
    }
    if (warp == 0) {
      // the next diagonal block's rows of E into dnext (copied while the MMAs run)
#pragma unroll 8
      for (int q = 0; q < kB; ++q) cp_async4(dnext + lane * kDs + q, E + (size_t)lane + (size_t)dp * q);
      mma_wait(mbar, mphase, bad);
      cp_async_wait_all();
#pragma unroll
      for (int h = 0; h < kB; h += 16) {
        uint32_t v[16];
        tmem_ld16(tlane + (uint32_t)h, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int q = 0; q < 16; q += 4) {
          float4 *dst = reinterpret_cast<float4 *>(dnext + lane * kDs + h + q);
          float4 d = *dst;
          d.x = __fadd_rn(d.x, __uint_as_float(v[q]));
          d.y = __fadd_rn(d.y, __uint_as_float(v[q + 1]));
          d.z = __fadd_rn(d.z, __uint_as_float(v[q + 2]));
          d.w = __fadd_rn(d.w, __uint_as_float(v[q + 3]));
          *dst = d;
        }
      }
      if (kB < ce) tmem_add_e(E, dp, R, row, kB, ce, tlane);  // the rest of warp 0's half
    } else {
      const bool mine = quarter * 32 < R && cb < ce;
      mma_wait(mbar, mphase, bad);
      if (mine) tmem_add_e(E, dp, R, row, cb, ce, tlane);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  // ---- tile 1: rows 128..R-1, all eight warps
  {
    const int row = 128 + quarter * 32 + lane;
    if (tid == 0 && mma_live(mbar)) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      umma_split_tile(tmem, smem_u32(Lt) + (uint32_t)(128 / 8) * 512, part_L, smem_u32(Ut), part_U,
                      idesc, false);
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar->bar)));
    }
    const bool mine = 128 + quarter * 32 < R && cb < ce;
    mma_wait(mbar, mphase, bad);
    if (mine) tmem_add_e(E, dp, R, row, cb, ce, tlane);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
}

// Panel Gauss-Jordan: column elimination of the stacked block column [D; C]
// (D the 32 x 32 diagonal block, C the rows below it) with 4 x 4 pivot blocks,
// in place, giving [D^-1; C D^-1] -- the block inverse and the block multipliers
// of the elimination in one pass.  Warp 0 holds the rows of D, warps 1..7 up to
// 224 rows of C; every thread keeps its row in registers (a[p], column position
// p).  Super-step K (pivot rows c0 = 4K .. 4K+3 of D, pivot columns at positions
// 0..3) right-multiplies by [[P^-1, -P^-1 B], [0, I]]:
//   rows outside the pivot rows:  a[pivot] <- g = a[0..3] P^-1,
//                                 a[p]     <- a[p] - g . M[K][p]
//   pivot row qi:                 a[pivot] <- (P^-1)[qi][*],
//                                 a[p]     <- -(P^-1 M[K][p])[qi]
// and rotates the columns by four positions (a[p-4] <- new a[p], a[28..31] <- the
// new pivot columns), so that every register index is a constant and after
// eight super-steps the columns are back in place.  The pivots of P are the LU
// pivots of D.
//
// Only the rows of D feed the next super-step, so warp 0 runs the eight of them
// alone (gj_diag, warp-synchronous) and publishes super-step K in its own slot
// of shared memory -- the pivot rows M[K][*] at the start of the super-step and
// P^-1 -- with bar.arrive on named barrier 1 + K; the rows of C (gj_rows) wait
// on that barrier only, so they trail warp 0 without a CTA-wide barrier between
// super-steps, and warps 1..7 can do other work (the row panel B) first.  All 256
// threads take part in the eight named barriers of every panel.
// No-pivot check: zero / non-finite pivots, LU multipliers inside P above tau,
// and block multipliers g of the rows still to be eliminated (rows of D below the
// pivot rows, all rows of C) above tau.
constexpr int kGjBar0 = 1;            // named barriers 1 .. 8; barrier 0 is __syncthreads

__device__ __forceinline__ void named_arrive(int id) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(kThreads) : "memory");
}
__device__ __forceinline__ void named_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(kThreads) : "memory");
}

// The update of one super-step for the positions P0 <= p < P1 (multiples of 4):
// a[p - 4] <- base[p] - g . M[K][p] (base = a, or 0 for the pivot rows), M[K] the
// pivot rows in the slot buf.  Positions are updated in increasing order, so the
// shift by four reads every position before it is overwritten.  FP32: packed
// f32x2 FMAs over pairs of positions.
template <int P0, int P1, typename T>
__device__ __forceinline__ void gj_update_range(T (&a)[kB], const T (&g)[4], const T *buf,
                                                bool zero) {
  if constexpr (sizeof(T) == 4) {
    float2 ng[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) ng[q] = make_float2(-g[q], -g[q]);
#pragma unroll
    for (int p = P0; p < P1; p += 4) {
      float4 r[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) r[q] = *reinterpret_cast<const float4 *>(buf + q * kGjRow + p);
      float2 lo = zero ? make_float2(0.f, 0.f) : make_float2(a[p], a[p + 1]);
      float2 hi = zero ? make_float2(0.f, 0.f) : make_float2(a[p + 2], a[p + 3]);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        lo = __ffma2_rn(ng[q], make_float2(r[q].x, r[q].y), lo);
        hi = __ffma2_rn(ng[q], make_float2(r[q].z, r[q].w), hi);
      }
      a[p - 4] = lo.x;
      a[p - 3] = lo.y;
      a[p - 2] = hi.x;
      a[p - 1] = hi.y;
    }
  } else {
#pragma unroll
    for (int p = P0; p < P1; p += 2) {
      T r[4][2];
#pragma unroll
      for (int q = 0; q < 4; ++q) Vec<T>::ld(buf + q * kGjRow + p, r[q]);
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        T v = zero ? T(0) : a[p + u];
#pragma unroll
        for (int q = 0; q < 4; ++q) v = fma(-g[q], r[q][u], v);
        a[p - 4 + u] = v;
      }
    }
  }
}
// The whole update of a super-step and the rotation (the new pivot columns g go
// to positions 28..31).
template <typename T>
__device__ __forceinline__ void gj_update(T (&a)[kB], const T (&g)[4], const T *buf, bool zero) {
  gj_update_range<4, kB>(a, g, buf, zero);
#pragma unroll
  for (int c = 0; c < 4; ++c) a[kB - 4 + c] = g[c];
}

// P^-1 of a 4 x 4 pivot block, in place, by Gauss-Jordan in registers (every
// lane of the warp holds the whole block and computes the same inverse: no
// shuffles in the dependent chain).  det = det P.  Flags zero / non-finite
// pivots and LU multipliers of P above tau.
// Step k; mult collects the largest |LU multiplier| of P (the entries below the
// pivot, scaled: -P[i][k] after the step).
template <int k, typename T>
__device__ __forceinline__ void gj_invert4_step(T (&P)[4][4], T &det, T &mult) {
  {
    const T pk = P[k][k];
    det *= pk;
    const T rp = rcp_fast(pk);
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (j != k) P[k][j] *= rp;
    P[k][k] = rp;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i == k) continue;
      const T f = P[i][k];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j != k) P[i][j] -= f * P[k][j];
      P[i][k] = -f * rp;
      if (i > k) mult = fmax(mult, dabs(P[i][k]));
    }
  }
}
// The check of the pivots uses det = their product: a zero or non-finite pivot
// makes it zero or non-finite (so does an extreme block whose product under- or
// overflows: it goes to the pivoting redo as well).
template <typename T>
__device__ __forceinline__ void gj_invert4(T (&P)[4][4], T tau, bool &bad, T &det) {
  det = T(1);
  T mult = T(0);
  gj_invert4_step<0>(P, det, mult);
  gj_invert4_step<1>(P, det, mult);
  gj_invert4_step<2>(P, det, mult);
  gj_invert4_step<3>(P, det, mult);
  bad |= !(finite_t(det) && det != T(0) && mult <= tau);
}

// The pivot block (positions 0..3 of the slot's four pivot rows) into every lane.
template <typename T>
__device__ __forceinline__ void gj_load_block(const T *buf, T (&P)[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; j += Vec<T>::W) Vec<T>::ld(buf + i * kGjRow + j, &P[i][j]);
}
__device__ __forceinline__ float log_abs_t(float v) { return logf(fabsf(v)); }
__device__ __forceinline__ double log_abs_t(double v) { return log(fabs(v)); }

// P^-1 into its slot (row-major after the pivot rows) for the rows of C.
template <typename T>
__device__ __forceinline__ void gj_put_inverse(const T (&P)[4][4], T *buf) {
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int c = 0; c < 4; c += Vec<T>::W) Vec<T>::st(buf + 4 * kGjRow + 4 * q + c, &P[q][c]);
  }
}

// Warp 0, lane = row of D.  Software-pipelined: super-step K updates positions
// 4..7 first (they are the next pivot block P_{K+1}), the four next pivot rows
// put that block into slot K + 1 and every lane reads it back and inverts it,
// then positions 8..31 are updated and the rest of the pivot rows (and, with
// Publish, P_{K+1}^-1) complete the slot.  With Publish (rows of C trailing on
// the named barriers) the slot is then published.  log|det P| accumulates in T
// on every lane; lane 0 returns the sum.
template <typename T, bool Publish>
__device__ __forceinline__ double gj_diag(T (&a)[kB], T *slots, T tau, bool &bad) {
  using V = Vec<T>;
  const int lane = threadIdx.x & 31;
  T ld = T(0);
  T P[4][4];
  // super-step 0: pivot rows 0..3 and P_0^-1
  if (lane < 4) {
#pragma unroll
    for (int p = 0; p < kB; p += V::W) V::st(slots + lane * kGjRow + p, a + p);
  }
  __syncwarp();
  gj_load_block<T>(slots, P);
  {
    T det;
    gj_invert4<T>(P, tau, bad, det);
    if (Publish) {
      gj_put_inverse<T>(P, slots);
      __syncwarp();
      named_arrive(kGjBar0);
    }
    ld += log_abs_t(det);
  }
#pragma unroll 1
  for (int K = 0; K < kB / 4; ++K) {
    const int c0 = 4 * K;
    const T *buf = slots + K * kGjSlot;
    const bool inK = lane >= c0 && lane < c0 + 4;
    // g = f P^-1, f = this row's pivot-column entries (unit vector for pivot rows)
    T f[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) f[q] = inK ? (q == lane - c0 ? T(1) : T(0)) : a[q];
    T g[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) acc += f[q] * P[q][c];
      g[c] = acc;
    }
    if (lane >= c0 + 4) {
#pragma unroll
      for (int c = 0; c < 4; ++c) bad |= !(dabs(g[c]) <= tau);
    }
    gj_update_range<4, 8>(a, g, buf, inK);  // a[0..3]: the next pivot block's columns
    if (K + 1 < kB / 4) {
      T *nb = slots + (K + 1) * kGjSlot;
      const bool next = lane >= c0 + 4 && lane < c0 + 8;
      if (next) {
#pragma unroll
        for (int p = 0; p < 4; p += V::W) V::st(nb + (lane - c0 - 4) * kGjRow + p, a + p);
      }
      __syncwarp();
      gj_load_block<T>(nb, P);
      T det;
      gj_invert4<T>(P, tau, bad, det);
      gj_update_range<8, kB>(a, g, buf, inK);
#pragma unroll
      for (int c = 0; c < 4; ++c) a[kB - 4 + c] = g[c];
      if (next) {
#pragma unroll
        for (int p = 4; p < kB; p += V::W) V::st(nb + (lane - c0 - 4) * kGjRow + p, a + p);
      }
      if (Publish) gj_put_inverse<T>(P, nb);
      __syncwarp();
      if (Publish) named_arrive(kGjBar0 + K + 1);  // super-step K + 1 is readable by the rows of C
      ld += log_abs_t(det);
    } else {
      gj_update_range<8, kB>(a, g, buf, inK);
#pragma unroll
      for (int c = 0; c < 4; ++c) a[kB - 4 + c] = g[c];
    }
  }
  return lane == 0 ? (double)ld : 0.0;
}

// Warps 1..7, one row of C per thread (active: the row exists).  rows: this warp
// has at least one row; a warp without rows only takes part in the barriers.
template <typename T>
__device__ __forceinline__ void gj_rows(T (&a)[kB], bool active, bool rows, const T *slots, T tau,
                                        bool &bad) {
  using V = Vec<T>;
#pragma unroll 1
  for (int K = 0; K < kB / 4; ++K) {
    named_sync(kGjBar0 + K);
    if (!rows) continue;
    const T *buf = slots + K * kGjSlot;
    T pinv[16];
#pragma unroll
    for (int q = 0; q < 16; q += V::W) V::ld(buf + 4 * kGjRow + q, pinv + q);
    T g[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      T acc = T(0);
#pragma unroll
      for (int q = 0; q < 4; ++q) acc += a[q] * pinv[4 * q + c];
      g[c] = acc;
    }
    if (active) {
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (!(dabs(g[c]) <= tau)) bad = true;
    }
    gj_update<T>(a, g, buf, false);
  }
}

// Back solve of the block elimination, in place on v (length dp, shared):
// x_k = D_k^-1 (v_k - B_k x_{>k}) for k = last .. 0, with D_k^-1 stored in the
// diagonal block and B_k (rows of block k, columns beyond it) untouched in A.
// Column-oriented: as soon as x_k is known, every row above block k subtracts
// A[r][block k] x_k (thread per row, 32 independent loads), so each block costs
// two barriers and one round of loads instead of a dependent chain.
template <typename T>
__device__ void be_back_solve(const T *__restrict__ A, int dp, T *v, T *bsum) {
  const int tid = threadIdx.x, lane = tid & 31;
  for (int kb = dp / kB - 1; kb >= 0; --kb) {
    const int k0 = kb * kB;
    // this thread's first row above the block: its coefficients do not depend on
    // x_k, so their loads are issued before the barrier that publishes x_k
    const bool first = tid < k0;
    T b[kB];
#pragma unroll
    for (int c = 0; c < kB; ++c) b[c] = first ? A[(size_t)tid + (size_t)dp * (k0 + c)] : T(0);
    if (tid < 32) {
      T dinv[kB];
#pragma unroll
      for (int c = 0; c < kB; ++c) dinv[c] = A[(size_t)(k0 + lane) + (size_t)dp * (k0 + c)];
      const T w = v[k0 + lane];
      T xk = T(0);
#pragma unroll
      for (int c = 0; c < kB; ++c) xk += dinv[c] * __shfl_sync(kFull, w, c);
      bsum[lane] = xk;
    }
    __syncthreads();
    if (tid < 32) v[k0 + tid] = bsum[tid];
    if (first) {
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < kB; ++c) acc += b[c] * bsum[c];
      v[tid] -= acc;
    }
    for (int r = tid + blockDim.x; r < k0; r += blockDim.x) {
#pragma unroll
      for (int c = 0; c < kB; ++c) b[c] = A[(size_t)r + (size_t)dp * (k0 + c)];
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < kB; ++c) acc += b[c] * bsum[c];
      v[r] -= acc;
    }
    __syncthreads();
  }
}

// Forward sweep of the block elimination: v_{>k} -= (C_k D_k^-1) v_k, block by block.
template <typename T>
__device__ void be_forward(const T *__restrict__ A, int dp, T *v) {
  for (int kb = 0; kb < dp / kB - 1; ++kb) {
    const int k0 = kb * kB, r0 = k0 + kB;
    for (int t = threadIdx.x; t < dp - r0; t += blockDim.x) {
      T b[kB];
#pragma unroll
      for (int c = 0; c < kB; ++c) b[c] = A[(size_t)(r0 + t) + (size_t)dp * (k0 + c)];
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < kB; ++c) acc += b[c] * v[k0 + c];
      v[r0 + t] -= acc;
    }
    __syncthreads();
  }
}

// The same two sweeps as a pipeline between warps, for d_p <= 256 (warp w owns
// the 32 rows of block w, one per lane): a block's solution is published in
// shared memory and announced on named barrier 1 + block (count: the publishing
// warp and the warps that still need it), so each warp subtracts a later block's
// contribution as soon as that block is solved -- no CTA-wide barrier per block,
// and a warp's coefficients of the next block are loaded while it waits.  The
// named barriers 1..7 are free in the solve phase (the dense phase is over).
// xs: dp values of shared scratch.
// Sum over c of b[c] x[c] for 32 values of x in shared memory (16-byte aligned),
// in four interleaved partial sums.
template <typename T>
__device__ __forceinline__ T dot_block(const T *b, const T *x) {
  using V = Vec<T>;
  T part[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
  for (int c = 0; c < kB; c += V::W) {
    T xv[V::W];
    V::ld(x + c, xv);
#pragma unroll
    for (int e = 0; e < V::W; ++e) part[(c + e) & 3] += b[c + e] * xv[e];
  }
  return (part[0] + part[1]) + (part[2] + part[3]);
}

// Back sweep: the row segments of blocks nb-1 .. w+1 and finally of D_w^-1 are
// one stream of 32-value loads, double-buffered, so that the next segment is in
// flight while the warp waits for a block; D_w^-1 is applied to the warp's
// accumulated values through a broadcast from v (its own rows, free until x is
// written back).
template <typename T>
__device__ void be_back_solve_pipe(const T *__restrict__ A, int dp, T *v, T *xs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nb = dp / kB;
  if (warp >= nb) return;
  const int r = warp * kB + lane;
  T acc = v[r];
  T cur[kB], nxt[kB];
#pragma unroll
  for (int c = 0; c < kB; ++c) cur[c] = A[(size_t)r + (size_t)dp * ((nb - 1) * kB + c)];
  for (int kb = nb - 1; kb > warp; --kb) {
#pragma unroll
    for (int c = 0; c < kB; ++c) nxt[c] = A[(size_t)r + (size_t)dp * ((kb - 1) * kB + c)];
    named_sync_n(1 + kb, (kb + 1) * 32);  // x of block kb is published
    acc -= dot_block<T>(cur, xs + kb * kB);
#pragma unroll
    for (int c = 0; c < kB; ++c) cur[c] = nxt[c];
  }
  // x_w = D_w^-1 acc_w (cur holds row lane of D_w^-1)
  v[r] = acc;
  __syncwarp();
  const T x = dot_block<T>(cur, v + warp * kB);
  __syncwarp();
  xs[r] = x;
  v[r] = x;
  if (warp > 0) named_arrive_n(1 + warp, (warp + 1) * 32);
}

template <typename T>
__device__ void be_forward_pipe(const T *__restrict__ A, int dp, T *v, T *xs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nb = dp / kB;
  if (warp >= nb) return;
  const int r = warp * kB + lane;
  T acc = v[r];
  for (int kb = 0; kb < warp; ++kb) {
    T b[kB];
#pragma unroll
    for (int c = 0; c < kB; ++c) b[c] = A[(size_t)r + (size_t)dp * (kb * kB + c)];
    // block kb is final once its own warp has applied every earlier block
    named_sync_n(1 + kb, (nb - kb) * 32);
#pragma unroll
    for (int c = 0; c < kB; ++c) acc -= b[c] * xs[kb * kB + c];
  }
  xs[r] = acc;
  v[r] = acc;
  if (warp + 1 < nb) named_arrive_n(1 + warp, (nb - warp) * 32);
}

// Copies the 32 x 32 diagonal block at k0 of the stored factors into D (warp 0).
template <typename T>
__device__ __forceinline__ void load_diag_block(const T *__restrict__ A, int mp, int k0, T *D) {
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < kB; ++c) D[lane * (kB + 1) + c] = A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)];
  __syncwarp();
}

// Solves U v = v in place (v in shared memory, length mp) with the triangular
// factors of the pivoting redo.
template <typename T>
__device__ void block_back_solve(const T *__restrict__ A, int mp, T *v, T *D) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int nbk = mp / kB;
  for (int kb = nbk - 1; kb >= 0; --kb) {
    const int k0 = kb * kB;
    if (tid < 32) {
      load_diag_block(A, mp, k0, D);
      T w = v[k0 + lane];
      for (int c = kB - 1; c >= 0; --c) {
        if (lane == c) w /= D[c * (kB + 1) + c];
        const T wc = __shfl_sync(kFull, w, c);
        if (lane < c) w -= D[lane * (kB + 1) + c] * wc;
      }
      v[k0 + lane] = w;
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

// Solves L v = v in place (unit lower, triangular factors of the pivoting redo).
template <typename T>
__device__ void block_forward_solve(const T *__restrict__ A, int mp, T *v, T *D) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int nbk = mp / kB;
  for (int kb = 0; kb < nbk; ++kb) {
    const int k0 = kb * kB;
    if (tid < 32) {
      load_diag_block(A, mp, k0, D);
      T w = v[k0 + lane];
      for (int c = 0; c < kB; ++c) {
        const T wc = __shfl_sync(kFull, w, c);
        if (lane > c) w -= D[lane * (kB + 1) + c] * wc;
      }
      v[k0 + lane] = w;
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

__device__ __forceinline__ int lo16(unsigned w) { return (int)(w & 0xFFFFu); }
__device__ __forceinline__ int hi16(unsigned w) { return (int)(w >> 16); }

// Forward program of one level on the node-indexed vector z: z[r] -= L[r][t] z[t].
// A node's program words are gathered eight at a time so that their loads overlap
// (a node has about ten terms).  The program is read through generic pointers: in
// the global plan, or staged in shared memory for the solve phase.
template <typename T>
__device__ __forceinline__ void level_forward(const EliminationPlan &ep, int lev, const T *vals,
                                              T *z) {
  for (int g = ep.lev_fwd_nodes[lev] + threadIdx.x; g < ep.lev_fwd_nodes[lev + 1]; g += blockDim.x) {
    const int r = ep.fwd_node[g], q1 = ep.fwd_ptr[g + 1];
    T acc = z[r];
    for (int q = ep.fwd_ptr[g]; q < q1; q += 8) {
      unsigned f[8];
#pragma unroll
      for (int h = 0; h < 8; ++h) f[h] = q + h < q1 ? ep.fwd[q + h] : 0u;
#pragma unroll
      for (int h = 0; h < 8; ++h)
        if (q + h < q1) acc -= vals[lo16(f[h])] * z[hi16(f[h])];
    }
    z[r] = acc;
  }
}

// The value slots of draw i before the levels: the constants, the unit diagonal
// and the level-0 entries -theta (each thread's sixteen gathers in flight at once).
template <typename T>
__device__ __forceinline__ void build_slots(const EliminationPlan &ep, int m, long i,
                                            const Theta<T> &theta, T *vals) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    vals[kSlotZero] = T(0);
    vals[kSlotOne] = T(1);
  }
  for (int r = tid; r < m; r += blockDim.x) vals[ep.diag_slot[r]] = T(1);
  for (int k0 = tid; k0 < ep.nnz0; k0 += 16 * kThreads) {
    int e[16], sl[16];
#pragma unroll
    for (int h = 0; h < 16; ++h) {
      const bool ok = k0 + h * kThreads < ep.nnz0;
      e[h] = ok ? (theta.g ? 0 : ep.l0_e[k0 + h * kThreads]) : -1;  // the index only without the Gamma copy
      sl[h] = ok ? ep.l0_slot[k0 + h * kThreads] : 0;
    }
    T th[16];
#pragma unroll
    for (int h = 0; h < 16; ++h) th[h] = e[h] >= 0 ? theta.gamma(i, k0 + h * kThreads, e[h]) : T(0);
#pragma unroll
    for (int h = 0; h < 16; ++h)
      if (e[h] >= 0) vals[sl[h]] = -th[h];
  }
}

// The sparse levels over the value slots `vals` (shared memory, or global when
// they do not fit), as the pivoting redo runs them (k_lu has the same loop
// inline): per level the pivots (sum log|pivot| into ld_part; a zero or
// non-finite pivot sets bad), the multipliers (bad above tau), a barrier, then the
// new entries, and a barrier.  A warp takes chunks c_begin + w + 8i; lane l
// prefetches the term offsets of its warp's chunk i = base + l, so that the term
// loads do not wait on a dependent load; kLevFlight chunks are in flight at a
// time (the plan's words come from L2: the rounds are latency-bound).  With zf,
// the right-hand side's forward program of each level rides along.
template <typename T>
__device__ __forceinline__ void run_levels(const EliminationPlan &ep, T *vals, T tau, bool &bad,
                                           double &ld_part, T *zf) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int lev = 0; lev < ep.nlev; ++lev) {
    for (int q = ep.lev_piv[lev] + tid; q < ep.lev_piv[lev + 1]; q += blockDim.x) {
      const T pv = vals[ep.piv[q]];
      if (!(finite_t(pv) && pv != T(0))) bad = true;
      ld_part += log_abs(pv);
    }
    for (int q = ep.lev_scale[lev] + tid; q < ep.lev_scale[lev + 1]; q += blockDim.x) {
      const unsigned w = ep.scale[q];
      const T l = vals[lo16(w)] / vals[hi16(w)];
      if (!(dabs(l) <= tau)) bad = true;
      vals[lo16(w)] = l;
    }
    __syncthreads();
    // new entries
    const int c_begin = ep.lev_chunk[lev], c_end = ep.lev_chunk[lev + 1];
    const int n_w = (c_begin + warp < c_end) ? (c_end - c_begin - warp + kWarps - 1) / kWarps : 0;
    for (int base = 0; base < n_w; base += 32) {
      int my_t0 = 0, my_t1 = 0;
      if (base + lane < n_w) {
        const int ci = c_begin + warp + (base + lane) * kWarps;
        my_t0 = ep.chunk_tofs[ci];
        my_t1 = ep.chunk_tofs[ci + 1];
      }
      const int n_here = min(32, n_w - base);
      for (int i0 = 0; i0 < n_here; i0 += kLevFlight) {
        unsigned e[kLevFlight];
        int toff[kLevFlight], K[kLevFlight];
#pragma unroll
        for (int h = 0; h < kLevFlight; ++h) {
          const int ii = i0 + h;
          const int t0 = __shfl_sync(kFull, my_t0, ii & 31);
          const int t1 = __shfl_sync(kFull, my_t1, ii & 31);
          const bool ok = ii < n_here;
          const int ch = c_begin + warp + (base + ii) * kWarps;
          e[h] = ok ? __ldg(ep.ent + (size_t)ch * 32 + lane) : kSlotNone;  // none: no store, base 0
          K[h] = ok ? (t1 - t0) >> 5 : 0;
          toff[h] = t0 + lane;
        }
        // the first term's word is loaded before the entry word is first used, so
        // that the two loads from L2 overlap (most entries have one term)
        unsigned w0[kLevFlight];
#pragma unroll
        for (int h = 0; h < kLevFlight; ++h) w0[h] = K[h] > 0 ? __ldg(ep.terms + toff[h]) : 0u;
        T v[kLevFlight];
        int Kmax = 0;
#pragma unroll
        for (int h = 0; h < kLevFlight; ++h) {
          v[h] = vals[hi16(e[h])] - vals[lo16(w0[h])] * vals[hi16(w0[h])];
          Kmax = max(Kmax, K[h]);
        }
#pragma unroll 1
        for (int k = 1; k < Kmax; ++k) {
          unsigned w[kLevFlight];
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h) w[h] = (k < K[h]) ? __ldg(ep.terms + toff[h] + 32 * k) : 0u;
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h) v[h] -= vals[lo16(w[h])] * vals[hi16(w[h])];
        }
#pragma unroll
        for (int h = 0; h < kLevFlight; ++h)
          if ((unsigned)lo16(e[h]) != kSlotNone) vals[lo16(e[h])] = v[h];
      }
    }
    if (zf) level_forward<T>(ep, lev, vals, zf);
    __syncthreads();
  }
}

// The dense core (d_p x d_p, column-major) from the value slots through the
// plan's slot map: four 16-bit slots per 8-byte word of the map, eight words in flight
// per thread.
template <typename T>
__device__ __forceinline__ void scatter_core(const EliminationPlan &ep, int dp, const T *vals,
                                             T *__restrict__ A) {
  using V = Vec<T>;
  constexpr int W = V::W;
  const int tid = threadIdx.x;
  const uint2 *map4 = reinterpret_cast<const uint2 *>(ep.core_map);
  const int nq = dp * dp / 4;
  for (int q0 = tid; q0 < nq; q0 += 8 * kThreads) {
    uint2 w[8];
#pragma unroll
    for (int h = 0; h < 8; ++h) {
      const int q = q0 + h * kThreads;
      w[h] = q < nq ? map4[q] : make_uint2(0u, 0u);
    }
#pragma unroll
    for (int h = 0; h < 8; ++h) {
      const int q = q0 + h * kThreads;
      if (q < nq) {
        T v4[4] = {vals[lo16(w[h].x)], vals[hi16(w[h].x)], vals[lo16(w[h].y)], vals[hi16(w[h].y)]};
#pragma unroll
        for (int g = 0; g < 4; g += W) V::st(A + (size_t)q * 4 + g, v4 + g);
      }
    }
  }
}

template <typename T>
__device__ void levels_forward(const EliminationPlan &ep, const T *vals, T *z) {
  for (int lev = 0; lev < ep.nlev; ++lev) {
    level_forward<T>(ep, lev, vals, z);
    __syncthreads();
  }
}

// Backward program of the sparse levels: y[t] for eliminated nodes from the
// forward-eliminated z and the already known y of later nodes.
template <typename T>
__device__ void levels_backward(const EliminationPlan &ep, const T *vals, const T *z, T *y) {
  for (int lev = ep.nlev - 1; lev >= 0; --lev) {
    for (int g = ep.lev_bwd_nodes[lev] + threadIdx.x; g < ep.lev_bwd_nodes[lev + 1]; g += blockDim.x) {
      const int t = ep.bwd_node[g];
      T acc = z[t];
      for (int q = ep.bwd_ptr[g]; q < ep.bwd_ptr[g + 1]; ++q) {
        const unsigned b = ep.bwd[q];
        acc -= vals[lo16(b)] * y[hi16(b)];
      }
      y[t] = acc / vals[ep.bwd_diag[g]];
    }
    __syncthreads();
  }
}

// res = nu - (I - Gamma) y in FP64, one thread per row summing that row's Gamma
// entries in a fixed order (deterministic); the entries' indices and theta values
// are gathered eight at a time so that their loads overlap.
template <typename T>
__device__ void residual(int m, int P, long n, long i, GammaRows rows, Theta<T> theta,
                         const double *nu, const T *y, double *res) {
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    double v = nu[r] - (double)y[r];
    const int q1 = rows.rowptr[r + 1];
    for (int q0 = rows.rowptr[r]; q0 < q1; q0 += 8) {
      int2 ec[8];
#pragma unroll
      for (int h = 0; h < 8; ++h) ec[h] = (q0 + h < q1) ? rows.ent[q0 + h] : make_int2(-1, 0);
      T th[8];
#pragma unroll
      for (int h = 0; h < 8; ++h)
        th[h] = ec[h].x >= 0 ? theta.gamma(i, q0 + h, ec[h].x) : T(0);
#pragma unroll
      for (int h = 0; h < 8; ++h)
        if (ec[h].x >= 0) v += (double)th[h] * (double)y[ec[h].y];
    }
    res[r] = v;
  }
  __syncthreads();
}

// The refinement's right-hand side, out = nu - (I - Gamma) y rounded to T, for the
// fast pass.  FP64 draws: the FP64 residual above.  FP32 draws: double-float
// arithmetic in FP32 (FP64 is a narrow pipe on this GPU) -- nu_r - y_r in FP64,
// split into two floats; each product theta y is exact as p + e with
// e = fma(theta, y, -p); the sum is compensated with Knuth's TwoSum.  About 48
// bits, ample for a residual that is rounded to FP32 afterwards.
template <typename T>
__device__ void residual_rhs(int m, int P, long n, long i, GammaRows rows, Theta<T> theta,
                             const double *nu, const T *y, double *res, T *out) {
  if constexpr (sizeof(T) == 8) {
    residual<T>(m, P, n, i, rows, theta, nu, y, res);
    for (int r = threadIdx.x; r < m; r += blockDim.x) out[r] = (T)res[r];
  } else {
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
      const double v0 = nu[r] - (double)y[r];
      float sh = (float)v0, sl = (float)(v0 - (double)sh);
      const int q1 = __ldg(rows.rowptr + r + 1);
      for (int q0 = __ldg(rows.rowptr + r); q0 < q1; q0 += 8) {
        int2 ec[8];
#pragma unroll
        for (int h = 0; h < 8; ++h) ec[h] = (q0 + h < q1) ? __ldg(rows.ent + q0 + h) : make_int2(-1, 0);
        float th[8];
#pragma unroll
        for (int h = 0; h < 8; ++h) th[h] = ec[h].x >= 0 ? (float)theta.gamma(i, q0 + h, ec[h].x) : 0.f;
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          if (ec[h].x < 0) continue;
          // explicitly rounded operations: no contraction into FMAs, which would
          // break the error-free transformations
          const float yc = (float)y[ec[h].y];
          const float pr = __fmul_rn(th[h], yc), pe = fmaf(th[h], yc, -pr);
          const float t = __fadd_rn(sh, pr), bb = __fsub_rn(t, sh);
          const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bb)), __fsub_rn(pr, bb));
          sh = t;
          sl = __fadd_rn(sl, __fadd_rn(err, pe));
        }
      }
      out[r] = (T)(sh + sl);
    }
    __syncthreads();
  }
}

// Copies n values between shared and global memory (16-byte vectors; both
// buffers hold n rounded up to 4 values).
template <typename T>
__device__ __forceinline__ void copy_vals(T *__restrict__ dst, const T *__restrict__ src, int n) {
  using V = Vec<T>;
  const int nvec = ((n + 3) / 4) * 4 / V::W;
  for (int q = threadIdx.x; q < nvec; q += blockDim.x) {
    T t[V::W];
    V::ld(src + q * V::W, t);
    V::st(dst + q * V::W, t);
  }
}

// TC: trailing updates on the tensor cores (FP32 draws, d_p <= 224); a separate
// instantiation, so that the FFMA path's register tiles do not weigh on it.
template <typename T, bool TC>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
    k_lu(int m, int P, int dp, size_t per_cta, int vals_smem, int prog_smem, long n,
         EliminationPlan ep,
         const unsigned *__restrict__ sp, const T *__restrict__ theta_sm,
         const T *__restrict__ theta_g, T *__restrict__ scratch,
         double *__restrict__ logdet, int *__restrict__ draw_flags,
         const double *__restrict__ x, const T *__restrict__ lambda, RngKey key, bool refine,
         double *__restrict__ y, GammaRows rows, const double *__restrict__ nu_in,
         int *__restrict__ pivot_list, const int *__restrict__ draw_list) {
  static_assert(!TC || sizeof(T) == 4, "tensor-core path: FP32 draws");
  using V = Vec<T>;
  constexpr int W = V::W;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Theta<T> theta{theta_sm, theta_g, m, P, ep.nnz0, n};
  const Smem L(dp, m, sizeof(T), vals_smem ? ep.nv : 0, TC);
  T *D = reinterpret_cast<T *>(smem_raw + L.off_D);  // D^-1, row-major, stride kB
  T *prow = reinterpret_cast<T *>(smem_raw + L.off_prow);
  T *Lp = reinterpret_cast<T *>(smem_raw + L.off_Lp);
  T *Up = reinterpret_cast<T *>(smem_raw + L.off_Up);
  T *z = reinterpret_cast<T *>(smem_raw + L.off_z);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  T *zf = reinterpret_cast<T *>(smem_raw + L.off_zf);
  T *yf = reinterpret_cast<T *>(smem_raw + L.off_yf);
  T *yd = reinterpret_cast<T *>(smem_raw + L.off_yd);
  double *red = reinterpret_cast<double *>(smem_raw + L.off_red);
  T *bsum = reinterpret_cast<T *>(smem_raw + L.off_bsum);
  const int Rmax = L.Rmax;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T *A = scratch + (size_t)blockIdx.x * per_cta;
  T *vals_g = A + (size_t)dp * dp;
  const bool planned = (ep.core_map != nullptr);
  T *vals = vals_smem ? reinterpret_cast<T *>(smem_raw + L.off_vals) : vals_g;
  const int nbk = dp / kB;
  const bool solve = (x != nullptr);
  const T tau = (T)kPivotThreshold;
  __shared__ int sflag;
  // tensor-core trailing updates (FP32 draws, d_p <= 224): 256 columns of tensor
  // memory for this CTA and the MMA completion barrier
  __shared__ uint32_t s_tmem;
  __shared__ __align__(8) MmaSync s_mbar;
  uint32_t mphase = 0;
  if constexpr (TC) {
    if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
          smem_u32(&s_tmem)));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_mbar.bar)));
      s_mbar.dead = 0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
  }
  const uint32_t tmem = TC ? s_tmem : 0u;

  const long n_todo = draw_list ? min((long)draw_list[0], n) : n;
  for (long it = blockIdx.x; it < n_todo; it += gridDim.x) {
    const long i = draw_list ? (long)draw_list[1 + it] : it;
    if (tid == 0) sflag = 0;
    bool bad = false;
    double ld_part = 0.0;  // this thread's share of sum log|pivot| (levels and core)
    // ---- build: value slots of level 0, forecast right-hand side
    if (planned) {
      if (tid == 0) {
        vals[kSlotZero] = T(0);
        vals[kSlotOne] = T(1);
      }
      for (int r = tid; r < m; r += blockDim.x) vals[ep.diag_slot[r]] = T(1);
      // level-0 values: all of this thread's gathers in flight at once
      for (int k0 = tid; k0 < ep.nnz0; k0 += 16 * kThreads) {
        int e[16], sl[16];
#pragma unroll
        for (int h = 0; h < 16; ++h) {
          const bool ok = k0 + h * kThreads < ep.nnz0;
          e[h] = ok ? (theta.g ? 0 : ep.l0_e[k0 + h * kThreads]) : -1;  // the index only without the Gamma copy
          sl[h] = ok ? ep.l0_slot[k0 + h * kThreads] : 0;
        }
        T th[16];
#pragma unroll
        for (int h = 0; h < 16; ++h) th[h] = e[h] >= 0 ? theta.gamma(i, k0 + h * kThreads, e[h]) : T(0);
#pragma unroll
        for (int h = 0; h < 16; ++h)
          if (e[h] >= 0) vals[sl[h]] = -th[h];
      }
    } else {
      // no plan: the whole matrix is the core, scattered from the parental sets
      build_full<T>(m, P, dp, n, i, sp, theta, A);
    }
    if (solve) {
      if (nu_in) {
        // the right-hand side computed for all draws beforehand (k_forecast_nu)
        for (int r = tid; r < m; r += blockDim.x) {
          const double v = nu_in[(size_t)r * n + i];
          nu[r] = v;
          zf[r] = (T)v;
        }
      } else {
        forecast_rhs<T>(m, P, n, i, rows, theta, x, lambda, key, nu);
        for (int r = tid; r < m; r += blockDim.x) zf[r] = (T)nu[r];
      }
    }
    __syncthreads();
    // ---- sparse levels (the loop of run_levels, kept inline here: through the
    // function this kernel measured 2 % slower)
    for (int lev = 0; lev < ep.nlev; ++lev) {
      for (int q = ep.lev_piv[lev] + tid; q < ep.lev_piv[lev + 1]; q += blockDim.x) {
        const T pv = vals[ep.piv[q]];
        if (!(finite_t(pv) && pv != T(0))) bad = true;
        ld_part += log_abs(pv);
      }
      for (int q = ep.lev_scale[lev] + tid; q < ep.lev_scale[lev + 1]; q += blockDim.x) {
        const unsigned w = ep.scale[q];
        const T l = vals[lo16(w)] / vals[hi16(w)];
        if (!(dabs(l) <= tau)) bad = true;
        vals[lo16(w)] = l;
      }
      __syncthreads();
      // new entries: warp w takes chunks c_begin + w + 8i; lane l prefetches the term
      // offsets of its warp's chunk i = base + l, so that the term loads do not wait
      // on a dependent load; kLevFlight chunks are in flight at a time (the plan's
      // words come from L2: the rounds are latency-bound)
      const int c_begin = ep.lev_chunk[lev], c_end = ep.lev_chunk[lev + 1];
      const int n_w = (c_begin + warp < c_end) ? (c_end - c_begin - warp + kWarps - 1) / kWarps : 0;
      for (int base = 0; base < n_w; base += 32) {
        int my_t0 = 0, my_t1 = 0;
        if (base + lane < n_w) {
          const int ci = c_begin + warp + (base + lane) * kWarps;
          my_t0 = ep.chunk_tofs[ci];
          my_t1 = ep.chunk_tofs[ci + 1];
        }
        const int n_here = min(32, n_w - base);
        for (int i0 = 0; i0 < n_here; i0 += kLevFlight) {
          unsigned e[kLevFlight];
          int toff[kLevFlight], K[kLevFlight];
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h) {
            const int ii = i0 + h;
            const int t0 = __shfl_sync(kFull, my_t0, ii & 31);
            const int t1 = __shfl_sync(kFull, my_t1, ii & 31);
            const bool ok = ii < n_here;
            const int ch = c_begin + warp + (base + ii) * kWarps;
            e[h] = ok ? __ldg(ep.ent + (size_t)ch * 32 + lane) : kSlotNone;  // none: no store, base 0
            K[h] = ok ? (t1 - t0) >> 5 : 0;
            toff[h] = t0 + lane;
          }
          // the first term's word is loaded before the entry word is first used, so
          // that the two loads from L2 overlap (most entries have one term)
          unsigned w0[kLevFlight];
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h) w0[h] = K[h] > 0 ? __ldg(ep.terms + toff[h]) : 0u;
          T v[kLevFlight];
          int Kmax = 0;
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h) {
            v[h] = vals[hi16(e[h])] - vals[lo16(w0[h])] * vals[hi16(w0[h])];
            Kmax = max(Kmax, K[h]);
          }
#pragma unroll 1
          for (int k = 1; k < Kmax; ++k) {
            unsigned w[kLevFlight];
#pragma unroll
            for (int h = 0; h < kLevFlight; ++h) w[h] = (k < K[h]) ? __ldg(ep.terms + toff[h] + 32 * k) : 0u;
#pragma unroll
            for (int h = 0; h < kLevFlight; ++h) v[h] -= vals[lo16(w[h])] * vals[hi16(w[h])];
          }
#pragma unroll
          for (int h = 0; h < kLevFlight; ++h)
            if ((unsigned)lo16(e[h]) != kSlotNone) vals[lo16(e[h])] = v[h];
        }
      }
      if (solve) level_forward<T>(ep, lev, vals, zf);
      __syncthreads();
    }
    // ---- dense core through the slot map; core right-hand side
    if (planned) {
      const uint2 *map4 = reinterpret_cast<const uint2 *>(ep.core_map);
      const int nq = dp * dp / 4;
      for (int q0 = tid; q0 < nq; q0 += 8 * kThreads) {
        uint2 w[8];
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const int q = q0 + h * kThreads;
          w[h] = q < nq ? map4[q] : make_uint2(0u, 0u);
        }
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const int q = q0 + h * kThreads;
          if (q < nq) {
            T v4[4] = {vals[lo16(w[h].x)], vals[hi16(w[h].x)], vals[lo16(w[h].y)], vals[hi16(w[h].y)]};
#pragma unroll
            for (int g = 0; g < 4; g += W) V::st(A + (size_t)q * 4 + g, v4 + g);
          }
        }
      }
      if (solve && vals_smem) copy_vals<T>(vals_g, vals, ep.n_solve);  // what the solves read
    }
    if (solve)
      for (int r = tid; r < dp; r += blockDim.x)
        z[r] = (r < ep.core_n) ? zf[planned ? ep.core_node[r] : r] : T(0);
    __syncthreads();
    if constexpr (TC) {
      {
        // d_p <= 224: warp 0 inverts the diagonal block; the block multipliers
        // L = C D^-1 and the trailing update run on the tensor cores.  Warp 0
        // leaves each trailing update after its first tile with the next diagonal
        // block, so that its Gauss-Jordan overlaps the rest of the update and the
        // other warps' splits of the next panel.
        unsigned char *Lt = smem_raw + L.off_Lt, *Ut = smem_raw + L.off_Ut;
        unsigned char *Dt = smem_raw + L.off_Dt;
        for (int kb = 0; kb < nbk; ++kb) {
          const int k0 = kb * kB, r0 = k0 + kB, R = dp - r0;
          if (warp == 0) {
            // the rows of D (the first panel's from the core, later ones as the
            // previous trailing update left them in shared memory): D^-1 by the
            // warp-synchronous Gauss-Jordan
            T *rowp = A + (size_t)(k0 + lane) + (size_t)dp * k0;
            T a[kB];
            if (kb == 0) {
#pragma unroll
              for (int q = 0; q < kB; ++q) a[q] = rowp[(size_t)dp * q];
            } else {
#pragma unroll
              for (int q = 0; q < kB; q += 4) V::ld(D + lane * kDs + q, a + q);
            }
            ld_part += gj_diag<T, false>(a, prow, tau, bad);
            if (solve) {
#pragma unroll
              for (int q = 0; q < kB; ++q) rowp[(size_t)dp * q] = a[q];
            }
            if (R > 0) {
              // D^-1's rows to shared memory; warps 1, 2, 3, 5 transpose and split
              // them into Dt (its columns as rows) off this warp's chain
#pragma unroll
              for (int q = 0; q < kB; q += 4) V::st(D + lane * kDs + q, a + q);
              __syncwarp();
              named_arrive_n(kBarDt, 160);
            }
          } else {
            // while warp 0 inverts D: the first tile of a single-tile trailing
            // update into tensor memory, and the row panel B (rows k0.., columns
            // r0..) and the rows of C, split, one column of B and one row of C per
            // thread of warps 1..3, 5..7 (warp 4 loads all columns of lanes 0..31)
            if (R > 0 && R <= 128)
              tc_preload_tile0(reinterpret_cast<const float *>(A), dp, r0, R, tmem,
                               kb > 0 && R + kB <= 128);
            if (warp != 4) {
              const int s0 = (warp < 4 ? warp - 1 : warp - 2) * 32 + lane;
              for (int t = s0; t < R; t += kThreads - 64) {
                const float *colp = reinterpret_cast<const float *>(A) + (size_t)k0 + (size_t)dp * (r0 + t);
                float b[kB];
#pragma unroll
                for (int q = 0; q < kB; q += 4) {
                  const float4 v = *reinterpret_cast<const float4 *>(colp + q);
                  b[q] = v.x; b[q + 1] = v.y; b[q + 2] = v.z; b[q + 3] = v.w;
                }
                write_split_row(Ut, L.part_U, t, b);
                const float *rowp = reinterpret_cast<const float *>(A) + (size_t)(r0 + t) + (size_t)dp * k0;
#pragma unroll
                for (int q = 0; q < kB; ++q) b[q] = rowp[(size_t)dp * q];
                write_split_row(Lt, L.part_L, t, b);
              }
            }
            if (R > 0 && (warp <= 3 || warp == 5)) {
              // Dt row n = column n of D^-1: thread (n, c) splits its values 8c .. 8c+7
              named_sync_n(kBarDt, 160);
              const int hidx = (warp == 5 ? 3 : warp - 1) * 32 + lane;
              const int n = hidx & 31, c = hidx >> 5;
              float col[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) col[e] = D[(8 * c + e) * kDs + n];
              write_split_chunk(Dt, (size_t)kB * 64, n, c, col);
            }
          }
          if (R > 0) {
            asm volatile("fence.proxy.async.shared::cta;");
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;");
            tc_block_multipliers(reinterpret_cast<float *>(A), dp, k0, r0, R, Lt, L.part_L, Dt, tmem,
                                 &s_mbar, mphase, tau, reinterpret_cast<float *>(z), solve, bad);
            tc_trailing_update(reinterpret_cast<float *>(A), dp, r0, R, Lt, Ut, L.part_L,
                               L.part_U, tmem, &s_mbar, mphase, bad, reinterpret_cast<float *>(D));
          } else {
            __syncthreads();
          }
        }
      }
    }
    if constexpr (!TC) for (int kb = 0; kb < nbk; ++kb) {
      const int k0 = kb * kB, r0 = k0 + kB, R = dp - r0;
      const int Rg = R < kGjRows ? R : kGjRows;  // rows of C inside the panel Gauss-Jordan
      // (a) the row panel B (and rows of C beyond Rg) in flight while the panel
      // Gauss-Jordan turns [D; C] into [D^-1; C D^-1]
      if (R > 0) stage_panels_async<T>(A, dp, k0, r0, R, Rg, Lp, Up, Rmax);
      {
        const int t = (warp - 1) * 32 + lane;  // row of C (warps 1..7)
        const bool active = (warp == 0) || t < Rg;
        T *rowp = A + (size_t)(warp == 0 ? k0 + lane : r0 + t) + (size_t)dp * k0;
        T a[kB];
#pragma unroll
        for (int q = 0; q < kB; ++q) a[q] = active ? rowp[(size_t)dp * q] : T(0);
        if (warp == 0)
          ld_part += gj_diag<T, true>(a, prow, tau, bad);
        else
          gj_rows<T>(a, active, (warp - 1) * 32 < Rg, prow, tau, bad);
        if (warp == 0) {
#pragma unroll
          for (int q = 0; q < kB; q += W) V::st(D + lane * kDs + q, a + q);
        } else if (active) {
#pragma unroll
          for (int q = 0; q < kB; ++q) Lp[q * Rmax + t] = a[q];
        }
        if (solve && active) {
          // keep D^-1 and C D^-1 for the solves; the right-hand side rides along
#pragma unroll
          for (int q = 0; q < kB; ++q) rowp[(size_t)dp * q] = a[q];
          if (warp > 0) {
            T acc = T(0);
#pragma unroll
            for (int q = 0; q < kB; ++q) acc += a[q] * z[k0 + q];
            z[r0 + t] -= acc;
          }
        }
      }
      cp_async_wait_all();
      __syncthreads();
      if (R > Rg) {
        // (b) rows of C beyond Rg: Lp <- C D^-1 in place; warp (half, quarter) owns
        // 32 rows x 8 columns of each 64-row round, a round reads its rows before
        // writing them.
        const int qc = (warp >> 1) * 8;
        for (int t0 = Rg; t0 < R; t0 += 64) {
          const int t = t0 + (warp & 1) * 32 + lane;
          const bool act = t < R;
          T o[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) o[j] = T(0);
          if (act) {
#pragma unroll 8
            for (int c = 0; c < kB; ++c) {
              const T lv = Lp[c * Rmax + t];
              T dv[8];
#pragma unroll
              for (int j = 0; j < 8; j += W) V::ld(D + c * kDs + qc + j, dv + j);
#pragma unroll
              for (int j = 0; j < 8; ++j) o[j] += lv * dv[j];
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
              if (!(dabs(o[j]) <= tau)) bad = true;
          }
          __syncthreads();
          if (act) {
#pragma unroll
            for (int j = 0; j < 8; ++j) Lp[(qc + j) * Rmax + t] = o[j];
          }
        }
        __syncthreads();
        if (solve) {
          const int RW = (R - Rg) / W;
          for (int u = tid; u < kB * RW; u += blockDim.x) {
            const int c = u / RW, tt = Rg + (u - c * RW) * W;
            T v[W];
            V::ld(Lp + c * Rmax + tt, v);
            V::st(A + (size_t)(r0 + tt) + (size_t)dp * (k0 + c), v);
          }
          for (int tt = Rg + tid; tt < R; tt += blockDim.x) {
            T acc = T(0);
#pragma unroll 8
            for (int c = 0; c < kB; ++c) acc += Lp[c * Rmax + tt] * z[k0 + c];
            z[r0 + tt] -= acc;
          }
        }
      }
      if (R > 0) {
        // (c) trailing update E -= (C D^-1) B
        trailing_update<T>(A, dp, r0, R, 0, R, Lp, Up, Rmax);
      }
      __syncthreads();
    }
    if (bad) atomicOr(&sflag, 1);
    const double ld_total = block_sum_det(ld_part, red);  // contains __syncthreads
    const bool flagged = (sflag != 0);
    if (tid == 0) {
      logdet[i] = ld_total;
      if (flagged) {
        atomicOr(&draw_flags[i], DRAW_FLAG_PIVOT);
        if (pivot_list) {
          const int q = atomicAdd(pivot_list, 1);
          if (q < n) pivot_list[1 + q] = (int)i;
        }
      }
    }
    if (solve && !flagged) {
      EliminationPlan eps = ep;  // the solve programs, staged in shared memory when they fit
      if (planned && vals_smem) {
        copy_vals<T>(vals, vals_g, ep.n_solve);
        if (prog_smem) {
          // after the n_solve value slots in the (now free) union region
          int *sprog = reinterpret_cast<int *>(
              smem_raw + L.off_vals + ((((size_t)ep.n_solve + 3) / 4 * 4 * sizeof(T) + 15) & ~(size_t)15));
          const int4 *src = reinterpret_cast<const int4 *>(ep.prog);
          for (int q = tid; q < ep.prog_len / 4; q += blockDim.x)
            reinterpret_cast<int4 *>(sprog)[q] = src[q];
          auto at = [&](const int *g) { return sprog + (g - ep.prog); };
          eps.lev_fwd_nodes = at(ep.lev_fwd_nodes);
          eps.fwd_node = at(ep.fwd_node);
          eps.fwd_ptr = at(ep.fwd_ptr);
          eps.fwd = reinterpret_cast<const unsigned *>(at(reinterpret_cast<const int *>(ep.fwd)));
          eps.lev_bwd_nodes = at(ep.lev_bwd_nodes);
          eps.bwd_node = at(ep.bwd_node);
          eps.bwd_diag = at(ep.bwd_diag);
          eps.bwd_ptr = at(ep.bwd_ptr);
          eps.bwd = reinterpret_cast<const unsigned *>(at(reinterpret_cast<const int *>(ep.bwd)));
        }
        __syncthreads();
      }
      // core part of y0
      if (dp <= kThreads) {
        be_back_solve_pipe<T>(A, dp, z, bsum);
        __syncthreads();
      } else {
        be_back_solve<T>(A, dp, z, bsum);
      }
      for (int r = tid; r < ep.core_n; r += blockDim.x) yf[planned ? ep.core_node[r] : r] = z[r];
      __syncthreads();
      levels_backward<T>(eps, vals, zf, yf);
      if (refine) {
        residual_rhs<T>(m, P, n, i, rows, theta, nu, yf, res, zf);
        __syncthreads();
        levels_forward<T>(eps, vals, zf);
        for (int r = tid; r < dp; r += blockDim.x)
          z[r] = (r < ep.core_n) ? zf[planned ? ep.core_node[r] : r] : T(0);
        __syncthreads();
        if (dp <= kThreads) {
          be_forward_pipe<T>(A, dp, z, bsum);
          __syncthreads();
          be_back_solve_pipe<T>(A, dp, z, bsum);
          __syncthreads();
        } else {
          be_forward<T>(A, dp, z);
          be_back_solve<T>(A, dp, z, bsum);
        }
        for (int r = tid; r < ep.core_n; r += blockDim.x) yd[planned ? ep.core_node[r] : r] = z[r];
        __syncthreads();
        levels_backward<T>(eps, vals, zf, yd);
        // one refinement step leaves an error of about (correction / solution)^2:
        // a draw whose correction exceeds kRefineTol of its solution (an
        // ill-conditioned (I - Gamma_i), cond * eps not small) goes to the
        // pivoting pass, which refines until it converges
        double dmax = 0.0, ymax = 0.0;
        for (int r = tid; r < m; r += blockDim.x) {
          dmax = fmax(dmax, fabs((double)yd[r]));
          ymax = fmax(ymax, fabs((double)yf[r]));
        }
        block_max2(dmax, ymax, red);
        if (!(dmax <= kRefineTol * ymax)) {
          if (tid == 0) {
            atomicOr(&draw_flags[i], DRAW_FLAG_PIVOT);
            if (pivot_list) {
              const int q = atomicAdd(pivot_list, 1);
              if (q < n) pivot_list[1 + q] = (int)i;
            }
          }
        } else {
          for (int r = tid; r < m; r += blockDim.x)
            y[(size_t)i * m + r] = (double)yf[r] + (double)yd[r];
        }
      } else {
        for (int r = tid; r < m; r += blockDim.x) y[(size_t)i * m + r] = (double)yf[r];
      }
    }
    __syncthreads();
  }
  if constexpr (TC) {
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
  }
}

// Pivoting redo of the draws the fast pass flagged.  The sparse levels' pivots
// are diagonal entries of (I - Gamma) as updated by earlier levels, eliminated
// without pivoting as in the fast pass (their multipliers only feed the
// products of the next levels); the redo pivots where the fast pass's checks
// look: in the dense core, by partial pivoting (getrf semantics on the core:
// at each column the row with the largest |entry| becomes the pivot row).  A
// draw whose level pivots are zero or non-finite, or whose level multipliers
// exceed kLevelMultMax, is factored instead with partial pivoting on the full
// m_p x m_p matrix.  log|det| = sum over the levels' pivots + the core's (the
// levels are a symmetric permutation plus exact block elimination).
//
// Both factorisations are the blocked right-looking LU of pivot_lu (32-column
// panels):
//  (a) the panel (rows k0.., columns k0..k0+31) is factored with partial pivoting
//      in shared memory, three barriers per column (pivot search, row swap,
//      update);
//  (b) the panel's row swaps are applied to the other columns and the right-hand
//      side, and the factors are written back;
//  (c) U12 = L11^-1 A12 by forward substitution, one column per thread, in
//      128-column chunks, each followed by the register-tiled trailing update
//      A22 -= L21 U12 of those columns.
template <typename T> struct FbBufs {
  T *pan, *Uc, *pivabs, *cand_v, *z;
  int *piv, *cand_i, *perm;
  bool *singular;
  // the register panel's exchange: per warp and column parity its best candidate
  // (|value|, row) and that row's 32 values; the displaced rows' positions
  T *crow, *ccv;
  int *cci, *disp;
};

// Factors the Rp x 32 panel pan (column-major, stride N, Rp <= blockDim.x) with
// partial pivoting, one row per thread held in registers and one barrier per
// column: each warp publishes its best candidate for the next column together
// with that row's values while the current column's update runs, so that after
// the barrier every thread knows the pivot row and reads it by broadcast.  Rows
// stay in their registers; warp 0 tracks the row interchanges (b.piv, LAPACK's
// ipiv relative to the panel) and the panel is written back in pivot order.
// pivabs[0..32) receives |u_jj|.  Returns true (uniform) at a zero or
// non-finite pivot column, the panel then left as it was.
template <typename T>
__device__ bool panel_regs(T *__restrict__ pan, int N, int Rp, T *__restrict__ pivabs,
                           const FbBufs<T> &b) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int r = tid;
  const bool row_ok = r < Rp;
  T a[kB];
#pragma unroll
  for (int c = 0; c < kB; ++c) a[c] = row_ok ? pan[c * N + r] : T(0);
  bool done = !row_ok;
  int pos = -1;
  // warp 0's lanes: at = panel row now at position `lane`, dp = position of
  // panel row `lane` (rows >= 32 only move when chosen)
  int at = lane, dp = lane;
  auto key = [](T v) { return v == v ? dabs(v) : T(INFINITY); };
  auto publish = [&](int c, int par) {
    T v = done ? T(-1) : key(a[c]);
    int vi = r;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T ov = __shfl_xor_sync(kFull, v, o);
      const int oi = __shfl_xor_sync(kFull, vi, o);
      if (ov > v || (ov == v && oi < vi)) {
        v = ov;
        vi = oi;
      }
    }
    if (lane == 0) {
      b.ccv[par * kWarps + warp] = v;
      b.cci[par * kWarps + warp] = vi;
    }
    if (vi == r && v >= T(0)) {
      T *dst = b.crow + (size_t)(par * kWarps + warp) * kB;
#pragma unroll
      for (int q = 0; q < kB; ++q) dst[q] = a[q];
    }
  };
  publish(0, 0);
  __syncthreads();
  bool sing = false;
#pragma unroll
  for (int j = 0; j < kB; ++j) {
    const int par = j & 1;
    // the pivot: the best of the warps' candidates (ties -> lowest row)
    T bv = lane < nwarps ? b.ccv[par * kWarps + lane] : T(-2);
    int p = lane < nwarps ? b.cci[par * kWarps + lane] : 0x7fffffff;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      const T ov = __shfl_xor_sync(kFull, bv, o);
      const int oi = __shfl_xor_sync(kFull, p, o);
      if (ov > bv || (ov == bv && oi < p)) {
        bv = ov;
        p = oi;
      }
    }
    bv = __shfl_sync(kFull, bv, 0);  // lanes 0..7 hold the warps' candidates
    p = __shfl_sync(kFull, p, 0);
    sing = sing || !(bv > T(0)) || !(bv <= (T)3.0e38);
    if (!sing) {
      const T *u = b.crow + (size_t)(par * kWarps + (p >> 5)) * kB;
      const T pv = u[j];
      if (tid == 0) pivabs[j] = dabs(pv);
      if (r == p) {
        done = true;
        pos = j;
      } else if (!done) {
        const T l = a[j] / pv;
        a[j] = l;
#pragma unroll
        for (int c = j + 1; c < kB; ++c) a[c] -= l * u[c];
      }
      if (warp == 0) {
        // interchange j <-> q, q the chosen row's current position
        const int q = p < kB ? __shfl_sync(kFull, dp, p) : p;
        const int x = __shfl_sync(kFull, at, j);  // the row leaving position j
        if (lane == x) dp = q;
        if (q < kB && lane == q) at = x;
        if (lane == j) at = p;
        if (p < kB && lane == p) dp = j;
        if (lane == 0) b.piv[j] = q;
      }
      if (j + 1 < kB) publish(j + 1, par ^ 1);
    }
    __syncthreads();
  }
  if (sing) return true;
  if (warp == 0) b.disp[lane] = dp;
  __syncthreads();
  if (row_ok) {
    const int f = done ? pos : (r < kB ? b.disp[r] : r);
#pragma unroll
    for (int c = 0; c < kB; ++c) pan[c * N + f] = a[c];
  }
  __syncthreads();
  return false;
}

// LU with partial pivoting of the N x N column-major matrix A (N a multiple of
// 32) in place; perm records the row permutation and, when `rhs`, z (length N)
// is permuted alongside.  pivabs[0..N) receives |u_jj|.  Returns true (uniform
// over the block) when a pivot column is zero or non-finite.  InSmem: A is in
// shared memory, the panels are factored where they lie and the trailing update
// reads U12 from A; otherwise each panel is staged in b.pan and U12's chunks in
// b.Uc.
template <typename T, bool InSmem>
__device__ bool pivot_lu(T *__restrict__ A, int N, bool rhs, const FbBufs<T> &b) {
  using V = Vec<T>;
  constexpr int W = V::W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int r = tid; r < N; r += blockDim.x) b.perm[r] = r;
  if (tid == 0) *b.singular = false;
  __syncthreads();
  for (int k0 = 0; k0 < N && !*b.singular; k0 += kB) {
    const int Rp = N - k0, r0 = k0 + kB, R = N - r0;
    T *pan = InSmem ? A + (size_t)k0 * N + k0 : b.pan;  // pan[c * N + r]: row k0 + r, column k0 + c
    // (a) the panel, factored with partial pivoting
    if (!InSmem) {
      for (int u = tid; u < kB * (Rp / W); u += blockDim.x) {
        const int c = u / (Rp / W), rw = u - c * (Rp / W);
        T v[W];
        V::ld(A + (size_t)(k0 + rw * W) + (size_t)N * (k0 + c), v);
        V::st(pan + c * N + rw * W, v);
      }
      __syncthreads();
    }
    if (Rp <= (int)blockDim.x) {
      if (panel_regs<T>(pan, N, Rp, b.pivabs + k0, b)) {
        if (tid == 0) *b.singular = true;
        __syncthreads();
      }
    } else
    for (int j = 0; j < kB; ++j) {
      // pivot search in the working precision (ties -> lowest row)
      T best = T(-1);
      int bidx = j;
      for (int r = j + tid; r < Rp; r += blockDim.x) {
        const T v = dabs(pan[j * N + r]);
        if (v > best) {
          best = v;
          bidx = r;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bidx, o);
        if (ov > best || (ov == best && oi < bidx)) {
          best = ov;
          bidx = oi;
        }
      }
      if (lane == 0) {
        b.cand_v[warp] = best;
        b.cand_i[warp] = bidx;
      }
      __syncthreads();
      T bv = b.cand_v[0];
      int p = b.cand_i[0];
      for (int w = 1; w < nwarps; ++w)
        if (b.cand_v[w] > bv || (b.cand_v[w] == bv && b.cand_i[w] < p)) {
          bv = b.cand_v[w];
          p = b.cand_i[w];
        }
      if (!(bv > T(0)) || !(bv <= (T)3.0e38)) {
        if (tid == 0) *b.singular = true;
        break;  // uniform: every thread computed the same bv
      }
      if (p != j && tid < kB) {
        const T t0 = pan[tid * N + j];
        pan[tid * N + j] = pan[tid * N + p];
        pan[tid * N + p] = t0;
      }
      if (tid == 0) b.piv[j] = p;
      __syncthreads();
      const T pv = pan[j * N + j];
      if (tid == 0) b.pivabs[k0 + j] = dabs(pv);
      for (int r = j + 1 + tid; r < Rp; r += blockDim.x) {
        const T l = pan[j * N + r] / pv;
        pan[j * N + r] = l;
        for (int c = j + 1; c < kB; ++c) pan[c * N + r] -= l * pan[c * N + j];
      }
      __syncthreads();
    }
    __syncthreads();
    if (*b.singular) break;
    // (b) the factors back to global; the block's swaps on the other columns, the
    // permutation and the right-hand side
    if (!InSmem) {
      for (int u = tid; u < kB * (Rp / W); u += blockDim.x) {
        const int c = u / (Rp / W), rw = u - c * (Rp / W);
        T v[W];
        V::ld(pan + c * N + rw * W, v);
        V::st(A + (size_t)(k0 + rw * W) + (size_t)N * (k0 + c), v);
      }
    }
    for (int c = tid; c < N - kB; c += blockDim.x) {
      const int col = c < k0 ? c : c + kB;
      T *cp = A + (size_t)N * col;
      for (int j = 0; j < kB; ++j) {
        const int p = b.piv[j];
        if (p != j) {
          const T t0 = cp[k0 + j];
          cp[k0 + j] = cp[k0 + p];
          cp[k0 + p] = t0;
        }
      }
    }
    if (tid == 0) {
      for (int j = 0; j < kB; ++j) {
        const int p = b.piv[j];
        if (p != j) {
          const int tp = b.perm[k0 + j];
          b.perm[k0 + j] = b.perm[k0 + p];
          b.perm[k0 + p] = tp;
          if (rhs) {
            const T tz = b.z[k0 + j];
            b.z[k0 + j] = b.z[k0 + p];
            b.z[k0 + p] = tz;
          }
        }
      }
    }
    __syncthreads();
    // (c) U12 chunk by chunk, each followed by its trailing update
    for (int c_off = 0; c_off < R; c_off += kFbChunk) {
      const int C = min(kFbChunk, R - c_off);
      for (int t = tid; t < C; t += blockDim.x) {
        T *cp = A + (size_t)k0 + (size_t)N * (r0 + c_off + t);
        T xv[kB];
#pragma unroll
        for (int q = 0; q < kB; q += W) V::ld(cp + q, xv + q);
#pragma unroll
        for (int q = 1; q < kB; ++q) {
          T acc = xv[q];
#pragma unroll
          for (int qq = 0; qq < q; ++qq) acc -= pan[qq * N + q] * xv[qq];
          xv[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < kB; q += W) {
          V::st(cp + q, xv + q);
          if (!InSmem) V::st(b.Uc + t * kUs + q, xv + q);
        }
      }
      __syncthreads();
      if (R > 0) {
        if (InSmem)
          trailing_update<T>(A, N, r0, R, c_off, C, pan + kB, A + (size_t)N * (r0 + c_off) + k0, N, N);
        else
          trailing_update<T>(A, N, r0, R, c_off, C, pan + kB, b.Uc, N);
      }
      __syncthreads();
    }
  }
  __syncthreads();
  return *b.singular;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_lu_fallback(int m, int P, int mp, int dp, size_t per_cta, int core_smem, long n,
                  EliminationPlan ep,
                  const unsigned *__restrict__ sp,
                  const T *__restrict__ theta_sm, const T *__restrict__ theta_g,
                  T *__restrict__ scratch,
                  double *__restrict__ logdet, int *__restrict__ draw_flags,
                  const double *__restrict__ x, const T *__restrict__ lambda, RngKey key,
                  double *__restrict__ y, GammaRows rows, const int *__restrict__ pivot_list) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Theta<T> theta{theta_sm, theta_g, m, P, ep.nnz0, n};
  const FallbackSmem L(mp, m, sizeof(T), core_smem ? dp : 0);
  __shared__ bool s_singular;
  __shared__ int s_level_bad;
  FbBufs<T> b;
  b.pan = reinterpret_cast<T *>(smem_raw + L.off_pan);      // pan[c * N + r]
  b.Uc = reinterpret_cast<T *>(smem_raw + L.off_U);         // U12 chunk [t][kUs]
  b.piv = reinterpret_cast<int *>(smem_raw + L.off_piv);    // the panel's pivot rows
  b.pivabs = reinterpret_cast<T *>(smem_raw + L.off_pivabs);
  b.cand_v = reinterpret_cast<T *>(smem_raw + L.off_cand);  // per-warp pivot candidates
  b.cand_i = reinterpret_cast<int *>(b.cand_v + kWarps);
  b.z = reinterpret_cast<T *>(smem_raw + L.off_z);
  b.perm = reinterpret_cast<int *>(smem_raw + L.off_perm);
  b.singular = &s_singular;
  b.crow = reinterpret_cast<T *>(smem_raw + L.off_crow);
  b.ccv = reinterpret_cast<T *>(smem_raw + L.off_ccv);
  b.cci = reinterpret_cast<int *>(smem_raw + L.off_cci);
  b.disp = reinterpret_cast<int *>(smem_raw + L.off_disp);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  double *red = reinterpret_cast<double *>(smem_raw + L.off_red);  // 64 doubles
  T *d = reinterpret_cast<T *>(smem_raw + L.off_d);
  T *D = reinterpret_cast<T *>(smem_raw + L.off_D);
  T *zf = reinterpret_cast<T *>(smem_raw + L.off_zf);  // node-indexed right-hand side
  T *yf = reinterpret_cast<T *>(smem_raw + L.off_yf);  // node-indexed solution
  T *yd = reinterpret_cast<T *>(smem_raw + L.off_yd);  // node-indexed correction
  const int tid = threadIdx.x;
  T *A = scratch + (size_t)blockIdx.x * per_cta;
  T *vals = A + (size_t)dp * dp;  // the levels' value slots (core path)
  const bool solve = (x != nullptr);
  const bool planned = (ep.core_map != nullptr);
  // the levels' value slots fit the core's region (d_p^2 values, rounded copies)
  const bool lvals_smem = planned && core_smem && ((ep.nv + 3) / 4) * 4 <= dp * dp;

  // the flagged draws: the fast pass's list, or all n draws' flags
  const long cnt = pivot_list ? min((long)pivot_list[0], n) : n;
  for (long q = blockIdx.x; q < cnt; q += gridDim.x) {
    const long i = pivot_list ? (long)pivot_list[1 + q] : q;
    if (!(draw_flags[i] & DRAW_FLAG_PIVOT)) continue;
    if (solve) {
      forecast_rhs<T>(m, P, n, i, rows, theta, x, lambda, key, nu);
      __syncthreads();
    }
    double ld_part = 0.0;
    bool core = planned;
    if (planned) {
      // ---- the sparse levels, without pivoting: the value slots in the dense
      // core's shared-memory region while the levels run (the core is formed
      // after them), then copied out for the scatter and the solves
      T *lv = lvals_smem ? reinterpret_cast<T *>(smem_raw + L.off_core) : vals;
      if (tid == 0) s_level_bad = 0;
      build_slots<T>(ep, m, i, theta, lv);
      if (solve)
        for (int r = tid; r < m; r += blockDim.x) zf[r] = (T)nu[r];
      __syncthreads();
      bool bad = false;
      run_levels<T>(ep, lv, (T)kLevelMultMax, bad, ld_part, solve ? zf : nullptr);
      if (lv != vals) {
        copy_vals<T>(vals, lv, ep.nv);
        __syncthreads();
      }
      if (bad) atomicOr(&s_level_bad, 1);
      __syncthreads();
      core = (s_level_bad == 0);
    }
    int N;
    // the matrix factored: the dense core (in shared memory when it fits) or the
    // full matrix (global)
    T *F = (core && core_smem) ? reinterpret_cast<T *>(smem_raw + L.off_core) : A;
    if (core) {
      // ---- dense core through the slot map; its right-hand side
      N = dp;
      scatter_core<T>(ep, dp, vals, F);
      if (solve)
        for (int r = tid; r < dp; r += blockDim.x) b.z[r] = (r < ep.core_n) ? zf[ep.core_node[r]] : T(0);
      __syncthreads();
    } else {
      // ---- the full matrix
      N = mp;
      ld_part = 0.0;
      build_full<T>(m, P, mp, n, i, sp, theta, A);
      if (solve)
        for (int r = tid; r < mp; r += blockDim.x) b.z[r] = (r < m) ? (T)nu[r] : T(0);
      __syncthreads();
    }
    const bool singular = (core && core_smem) ? pivot_lu<T, true>(F, N, solve, b)
                                              : pivot_lu<T, false>(F, N, solve, b);
    if (!singular)
      for (int r = tid; r < N; r += blockDim.x) ld_part += log_abs(b.pivabs[r]);
    const double ld = block_sum_det(ld_part, red);  // contains __syncthreads
    if (tid == 0) {
      const int how = DRAW_FLAG_REDONE | (core ? 0 : DRAW_FLAG_FULL_PIVOT);
      if (singular) {
        logdet[i] = -INFINITY;
        atomicOr(&draw_flags[i], DRAW_FLAG_SINGULAR | how);
      } else {
        logdet[i] = ld;
        atomicOr(&draw_flags[i], how);
      }
    }
    __syncthreads();
    if (solve) {
      if (singular) {
        for (int r = tid; r < m; r += blockDim.x) y[(size_t)i * m + r] = NAN;
      } else if (core) {
        // core solution, then the levels' backward program
        block_forward_solve<T>(F, N, b.z, D);
        block_back_solve<T>(F, N, b.z, D);
        for (int r = tid; r < ep.core_n; r += blockDim.x) yf[ep.core_node[r]] = b.z[r];
        __syncthreads();
        levels_backward<T>(ep, vals, zf, yf);
        // the draws that reach this pass are the ill-conditioned ones: refine up
        // to kFbRefine times (FP64 residual of the working-precision solution),
        // which recovers working-precision accuracy while cond * eps < 1; stop
        // once the correction is below kFbRefineStop of the solution
        for (int it = 0; it < kFbRefine; ++it) {
          if (it > 0) {
            for (int r = tid; r < m; r += blockDim.x) yf[r] += yd[r];
            __syncthreads();
          }
          residual<T>(m, P, n, i, rows, theta, nu, yf, res);
          for (int r = tid; r < m; r += blockDim.x) zf[r] = (T)res[r];
          __syncthreads();
          levels_forward<T>(ep, vals, zf);
          for (int r = tid; r < N; r += blockDim.x) {
            const int pr = b.perm[r];
            d[r] = (pr < ep.core_n) ? zf[ep.core_node[pr]] : T(0);
          }
          __syncthreads();
          block_forward_solve<T>(F, N, d, D);
          block_back_solve<T>(F, N, d, D);
          for (int r = tid; r < ep.core_n; r += blockDim.x) yd[ep.core_node[r]] = d[r];
          __syncthreads();
          levels_backward<T>(ep, vals, zf, yd);
          if (it + 1 < kFbRefine && refine_done<T>(m, yd, yf, red)) break;
        }
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)yf[r] + (double)yd[r];
      } else {
        block_forward_solve<T>(F, N, b.z, D);
        block_back_solve<T>(F, N, b.z, D);
        for (int it = 0; it < kFbRefine; ++it) {
          if (it > 0) {
            for (int r = tid; r < m; r += blockDim.x) b.z[r] += d[r];
            __syncthreads();
          }
          residual<T>(m, P, n, i, rows, theta, nu, b.z, res);
          for (int r = tid; r < N; r += blockDim.x) d[r] = (b.perm[r] < m) ? (T)res[b.perm[r]] : T(0);
          __syncthreads();
          block_forward_solve<T>(F, N, d, D);
          block_back_solve<T>(F, N, d, D);
          if (it + 1 < kFbRefine && refine_done<T>(m, d, b.z, red)) break;
        }
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)b.z[r] + (double)d[r];
      }
    }
    __syncthreads();
  }
}

// Shared memory a CTA may use when `per_sm` CTAs share one SM (228 KB per SM,
// 1 KB of it reserved per CTA; 227 KB at most per CTA).
size_t smem_budget(int per_sm) {
  const size_t b = 233472u / (size_t)per_sm - 1024u;
  return b < 232448u ? b : 232448u;
}

}  // namespace

template <typename T>
LuPlan plan_lu(int m, int P, long n, int num_sms, int core_n, int nv, int n_solve, int prog_len,
               LuOptions opt) {
  LuPlan pl{};
  pl.m = m;
  pl.P = P;
  pl.mp = ((m + kB - 1) / kB) * kB;
  pl.dp = ((core_n + kB - 1) / kB) * kB;
  if (pl.dp < kB) pl.dp = kB;
  pl.block = kThreads;
  // value slots in shared memory when that keeps the target occupancy
  const int target = sizeof(T) == 4 ? 2 : 1;
  // tensor-core path for FP32 draws while the trailing update's first tile (R <= 192
  // columns) and the block multipliers (64 columns) fit the CTA's 256 columns of
  // tensor memory together: d_p <= 224
  pl.tc = (sizeof(T) == 4 && pl.dp <= 224 && opt.allow_tc) ? 1 : 0;
  const size_t with_vals = Smem(pl.dp, m, sizeof(T), nv, pl.tc != 0).total;
  pl.vals_smem = (nv > 0 && with_vals <= smem_budget(target)) ? 1 : 0;
  pl.smem = Smem(pl.dp, m, sizeof(T), pl.vals_smem ? nv : 0, pl.tc != 0).total;
  {
    // the solve programs fit after the solve slots in the union region
    const Smem L(pl.dp, m, sizeof(T), pl.vals_smem ? nv : 0, pl.tc != 0);
    const size_t region = L.off_z - L.off_vals;
    const size_t used = (((size_t)n_solve + 3) / 4 * 4 * sizeof(T) + 15) & ~(size_t)15;
    pl.prog_smem = (pl.vals_smem && prog_len > 0 && used + (size_t)prog_len * 4 <= region) ? 1 : 0;
  }
  // the redo factors the dense core in shared memory when it fits (one CTA per SM)
  pl.fb_core_smem = 0;
  pl.smem_fallback = FallbackSmem(pl.mp, m, sizeof(T)).total;
  if (nv > 0) {
    const size_t with_core = FallbackSmem(pl.mp, m, sizeof(T), pl.dp).total;
    if (with_core + 64 <= smem_budget(1)) {  // 64 bytes: the kernel's static shared memory
      pl.fb_core_smem = 1;
      pl.smem_fallback = with_core;
    }
  }
  int ctas_per_sm = pl.smem <= smem_budget(2) ? 2 : 1;
  if (sizeof(T) == 8) ctas_per_sm = 1;
  long grid = (long)num_sms * ctas_per_sm;
  if (opt.max_grid > 0 && grid > opt.max_grid) grid = opt.max_grid;
  if (grid > n) grid = n;
  if (grid < 1) grid = 1;
  pl.grid = (int)grid;
  pl.scratch_elems_per_cta = (size_t)pl.dp * pl.dp + (((size_t)nv + 3) / 4) * 4;
  const size_t total = pl.scratch_elems_per_cta * pl.grid;
  // the redo needs the dense core and the value slots, or a full m_p x m_p slab,
  // per CTA; it shares the slab array, which grows to one slab per SM for it
  const size_t full = std::max((size_t)pl.mp * pl.mp, pl.scratch_elems_per_cta);
  pl.fb_elems_per_cta = full;
  long fb = num_sms;
  if (fb > n) fb = n;
  if (fb < 1) fb = 1;
  pl.fb_grid = (int)fb;
  pl.scratch_elems_total = std::max(total, (size_t)pl.fb_grid * full);
  return pl;
}

template <typename T>
void launch_lu(cudaStream_t s, const LuPlan &pl, long n, const EliminationPlan &ep,
               const unsigned *sp, const T *theta, const T *theta_g, T *scratch,
               double *logdet, int *draw_flags,
               const double *x, const T *lambda, RngKey key, bool refine, double *y,
               GammaRows rows, const double *nu_in, int *pivot_list, const int *draw_list) {
  // opt in to exactly the shared memory this plan needs (a failure here shows up
  // as a launch error that the engine reports)
  auto run = [&](auto kernel) {
    if (pl.smem > 48 * 1024)
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
    kernel<<<pl.grid, pl.block, pl.smem, s>>>(pl.m, pl.P, pl.dp, pl.scratch_elems_per_cta,
                                              pl.vals_smem, pl.prog_smem, n, ep, sp, theta,
                                              theta_g, scratch,
                                              logdet, draw_flags, x, lambda, key, refine, y, rows,
                                              nu_in, pivot_list, draw_list);
  };
  if constexpr (sizeof(T) == 4) {
    if (pl.tc) {
      run(k_lu<T, true>);
      return;
    }
  }
  run(k_lu<T, false>);
}

template <typename T>
void launch_forecast_nu(cudaStream_t s, int m, int P, long n, GammaRows rows, const T *theta,
                        const double *x, const float *x32, const T *lambda, RngKey key,
                        double *nu) {
  const dim3 grid((unsigned)((n + 127) / 128), (unsigned)m);
  k_forecast_nu<T><<<grid, 128, 0, s>>>(m, P, n, rows, theta, x, x32, lambda, key, nu);
}

template <typename T>
void launch_lu_fallback(cudaStream_t s, const LuPlan &pl, long n, const EliminationPlan &ep,
                        const unsigned *sp, const T *theta, const T *theta_g, T *scratch,
                        double *logdet, int *draw_flags,
                        const double *x, const T *lambda, RngKey key, double *y,
                        GammaRows rows, const int *pivot_list) {
  if (pl.smem_fallback > 48 * 1024)
    cudaFuncSetAttribute(k_lu_fallback<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)pl.smem_fallback);
  k_lu_fallback<T><<<pl.fb_grid, pl.block, pl.smem_fallback, s>>>(
      pl.m, pl.P, pl.mp, pl.dp, pl.fb_elems_per_cta, pl.fb_core_smem, n, ep, sp, theta, theta_g,
      scratch, logdet,
      draw_flags, x, lambda, key, y, rows, pivot_list);
}

template LuPlan plan_lu<float>(int, int, long, int, int, int, int, int, LuOptions);
template LuPlan plan_lu<double>(int, int, long, int, int, int, int, int, LuOptions);
template void launch_lu<float>(cudaStream_t, const LuPlan &, long, const EliminationPlan &,
                               const unsigned *, const float *, const float *, float *,
                               double *, int *,
                               const double *, const float *, RngKey, bool, double *, GammaRows,
                               const double *, int *, const int *);
template void launch_lu<double>(cudaStream_t, const LuPlan &, long, const EliminationPlan &,
                                const unsigned *, const double *, const double *, double *,
                                double *, int *,
                                const double *, const double *, RngKey, bool, double *,
                                GammaRows, const double *, int *, const int *);
template void launch_forecast_nu<float>(cudaStream_t, int, int, long, GammaRows, const float *,
                                        const double *, const float *, const float *, RngKey,
                                        double *);
template void launch_forecast_nu<double>(cudaStream_t, int, int, long, GammaRows,
                                         const double *, const double *, const float *,
                                         const double *, RngKey, double *);
template void launch_lu_fallback<float>(cudaStream_t, const LuPlan &, long,
                                        const EliminationPlan &, const unsigned *,
                                        const float *, const float *, float *, double *, int *,
                                        const double *,
                                        const float *, RngKey, double *, GammaRows, const int *);
template void launch_lu_fallback<double>(cudaStream_t, const LuPlan &, long,
                                         const EliminationPlan &, const unsigned *,
                                         const double *, const double *, double *, double *,
                                         int *,
                                         const double *, const double *, RngKey, double *,
                                         GammaRows, const int *);

}  // namespace sgdlm
