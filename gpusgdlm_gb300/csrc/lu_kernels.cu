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
//     independent sets; the CTA evaluates that program on the draw's values
//     (vals), accumulating sum log|pivot| of the eliminated nodes.  The
//     remaining core (about 260 of 400 nodes at m = 400) is scattered into a
//     dense d_p x d_p matrix (d_p = core size rounded up to 32, identity padding).
//  2. Right-looking blocked LU of the core with 32 x 32 blocks:
//     (a) one warp factors the diagonal block in shared memory;
//     (b) the column panel L = A U^-1 and (c) the row panel U = L^-1 A, solved
//         in place in shared memory (one row / column per thread);
//     (d) the trailing update A -= L U: a register-tiled FMA loop over
//         (32W) x 128 tiles with 16-byte conflict-free shared and global loads.
//     The blocked pass does not pivot: (I - Gamma) is diagonally dominant in the
//     filtering regime.  Every multiplier (sparse levels included) is checked
//     against kPivotThreshold; a draw with a larger one, or a zero / non-finite
//     pivot, is flagged and redone by k_lu_fallback with partial pivoting on the
//     full matrix (getrf semantics).  |det| does not depend on the pivot order.
//  3. Forecasts: the right-hand side goes through the levels' forward program,
//     rides along the core factorisation, is back-substituted through the core
//     and the levels; an FP64 residual nu - (I - Gamma) y0 from the sparse parent
//     rows drives one refinement solve with the same factors.
#include <algorithm>

#include "elimination.hpp"
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

// Shared-memory carve-up (byte offsets, 16-byte aligned).  dp is the padded
// dense size, m the number of nodes (forecast vectors are node-indexed).
struct Smem {
  int Rmax;
  size_t off_D, off_Lp, off_Up, off_z, off_nu, off_res, off_zf, off_yf, off_yd, off_red, total;
  __host__ __device__ Smem(int dp, int m, size_t tsz) {
    Rmax = dp - kB > 0 ? dp - kB : kB;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 15) & ~(size_t)15;
      return at;
    };
    off_D = take((size_t)kB * (kB + 1) * tsz);
    off_Lp = take((size_t)kB * Rmax * tsz);
    off_Up = take((size_t)kB * Rmax * tsz);
    off_z = take((size_t)dp * tsz);
    off_nu = take((size_t)m * sizeof(double));
    off_res = take((size_t)m * sizeof(double));
    off_zf = take((size_t)m * tsz);
    off_yf = take((size_t)m * tsz);
    off_yd = take((size_t)m * tsz);
    off_red = take(64 * sizeof(double));
    total = o;
  }
};

// nu_j = z/sqrt(lambda) + sum over external predictors x_jk theta_jk for draw i
// (batchedComputeNuPlusMu, kernel_functions.cuh:1156-1178), into nu (double).
template <typename T>
__device__ void forecast_rhs(int m, int P, long n, long i, const unsigned *__restrict__ sp,
                             const T *__restrict__ theta, const double *__restrict__ x,
                             const T *__restrict__ lambda, RngKey key, double *nu) {
  const uint32_t ep = key_epoch(key);
  const size_t mm = (size_t)m * m;
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const U4 g = philox((uint32_t)i, (uint32_t)j, tag_sub(TAG_NU, 0), ep, key.k0, key.k1);
    T z0, z1;
    box_muller<T>(g.x, g.y, z0, z1);
    const T lam = lambda[(size_t)j * n + i];
    double v = (double)(z0 / dev_sqrt(lam));
    const T *th = theta + ((size_t)j * n + i) * P;
    for (int k = 0; k < P; ++k)
      if ((size_t)sp[(size_t)j * P + k] >= mm) v += x[(size_t)j * P + k] * (double)th[k];
    nu[j] = v;
  }
}

// Writes the identity plus the scattered -theta entries of draw i into the full
// mp x mp matrix A (fillGammas, kernel_functions.cuh:822-842).
template <typename T>
__device__ void build_full(int m, int P, int mp, long n, long i, const unsigned *__restrict__ sp,
                           const T *__restrict__ theta, T *__restrict__ A) {
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
      const int j = e / P, k = e % P;
      const int row = (int)(pos % (unsigned)m), col = (int)(pos / (unsigned)m);
      A[row + (size_t)mp * col] = -theta[((size_t)j * n + i) * P + k];
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

// Copies the 32 x 32 diagonal block at k0 of the stored factors into D (warp 0).
template <typename T>
__device__ __forceinline__ void load_diag_block(const T *__restrict__ A, int mp, int k0, T *D) {
  const int lane = threadIdx.x & 31;
  for (int c = 0; c < kB; ++c) D[lane * (kB + 1) + c] = A[(size_t)(k0 + lane) + (size_t)mp * (k0 + c)];
  __syncwarp();
}

// Solves U v = v in place (v in shared memory, length mp) with the stored factors.
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
        const T wc = __shfl_sync(0xffffffffu, w, c);
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

// Solves L v = v in place (unit lower, stored factors).
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
        const T wc = __shfl_sync(0xffffffffu, w, c);
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

// Forward program of the sparse levels on the node-indexed vector z.
template <typename T>
__device__ void levels_forward(const EliminationPlan &ep, const T *__restrict__ vals, T *z) {
  for (int lev = 0; lev < ep.nlev; ++lev) {
    for (int g = ep.lev_fwd_nodes[lev] + threadIdx.x; g < ep.lev_fwd_nodes[lev + 1]; g += blockDim.x) {
      const int r = ep.fwd_node[g];
      T acc = z[r];
      for (int q = ep.fwd_ptr[g]; q < ep.fwd_ptr[g + 1]; ++q) {
        const int3 f = ep.fwd[q];
        acc -= vals[f.x] / vals[f.z] * z[f.y];
      }
      z[r] = acc;
    }
    __syncthreads();
  }
}

// Backward program of the sparse levels: y[t] for eliminated nodes from the
// forward-eliminated z and the already known y of later nodes.
template <typename T>
__device__ void levels_backward(const EliminationPlan &ep, const T *__restrict__ vals,
                                const T *z, T *y) {
  for (int lev = ep.nlev - 1; lev >= 0; --lev) {
    for (int g = ep.lev_bwd_nodes[lev] + threadIdx.x; g < ep.lev_bwd_nodes[lev + 1]; g += blockDim.x) {
      const int t = ep.bwd_node[g];
      T acc = z[t];
      for (int q = ep.bwd_ptr[g]; q < ep.bwd_ptr[g + 1]; ++q) {
        const int2 b = ep.bwd[q];
        acc -= vals[b.x] * y[b.y];
      }
      y[t] = acc / vals[ep.bwd_diag[g]];
    }
    __syncthreads();
  }
}

// res = nu - (I - Gamma) y in FP64, one thread per row summing that row's Gamma
// entries in a fixed order (deterministic).
template <typename T>
__device__ void residual(int m, int P, long n, long i, GammaRows rows,
                         const T *__restrict__ theta, const double *nu, const T *y, double *res) {
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    double v = nu[r] - (double)y[r];
    for (int q = rows.rowptr[r]; q < rows.rowptr[r + 1]; ++q) {
      const int2 ec = rows.ent[q];
      const int j = ec.x / P, k = ec.x % P;
      v += (double)theta[((size_t)j * n + i) * P + k] * (double)y[ec.y];
    }
    res[r] = v;
  }
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 2 : 1)
    k_lu(int m, int P, int dp, size_t per_cta, long n, EliminationPlan ep,
         const unsigned *__restrict__ sp, const T *__restrict__ theta, T *__restrict__ scratch,
         double *__restrict__ logdet, int *__restrict__ draw_flags,
         const double *__restrict__ x, const T *__restrict__ lambda, RngKey key, bool refine,
         double *__restrict__ y, GammaRows rows) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Smem L(dp, m, sizeof(T));
  T *D = reinterpret_cast<T *>(smem_raw + L.off_D);
  T *Lp = reinterpret_cast<T *>(smem_raw + L.off_Lp);
  T *Up = reinterpret_cast<T *>(smem_raw + L.off_Up);
  T *z = reinterpret_cast<T *>(smem_raw + L.off_z);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  T *zf = reinterpret_cast<T *>(smem_raw + L.off_zf);
  T *yf = reinterpret_cast<T *>(smem_raw + L.off_yf);
  T *yd = reinterpret_cast<T *>(smem_raw + L.off_yd);
  double *red = reinterpret_cast<double *>(smem_raw + L.off_red);
  const int Rmax = L.Rmax;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T *A = scratch + (size_t)blockIdx.x * per_cta;
  T *vals = A + (size_t)dp * dp;
  const int nbk = dp / kB;
  const bool solve = (x != nullptr);
  const T tau = (T)kPivotThreshold;
  __shared__ int sflag;

  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    if (tid == 0) sflag = 0;
    bool bad = false;
    double ld_part = 0.0;  // this thread's share of sum log|pivot| of the levels
    // ---- build: zero the core, level-0 values, forecast right-hand side
    const bool planned = (ep.core_ent != nullptr);
    if (planned) {
      const size_t n16 = (size_t)dp * dp * sizeof(T) / 16;
      uint4 *A16 = reinterpret_cast<uint4 *>(A);
      for (size_t e = tid; e < n16; e += blockDim.x) A16[e] = make_uint4(0, 0, 0, 0);
      for (int r = tid; r < m; r += blockDim.x) vals[r] = T(1);
      for (int k = tid; k < ep.nnz0; k += blockDim.x) {
        const int e = ep.l0_e[k];
        const int j = e / P, kk = e % P;
        vals[m + k] = -theta[((size_t)j * n + i) * P + kk];
      }
    } else {
      // no plan: the whole matrix is the core, scattered from the parental sets
      build_full<T>(m, P, dp, n, i, sp, theta, A);
    }
    if (solve) forecast_rhs<T>(m, P, n, i, sp, theta, x, lambda, key, nu);
    __syncthreads();
    if (solve) {
      for (int r = tid; r < m; r += blockDim.x) zf[r] = (T)nu[r];
    }
    // ---- sparse levels
    for (int lev = 0; lev < ep.nlev; ++lev) {
      for (int q = ep.lev_entry[lev] + tid; q < ep.lev_entry[lev + 1]; q += blockDim.x) {
        const int base = ep.ent_base[q];
        T v = base >= 0 ? vals[base] : T(0);
        for (int t = ep.ent_tptr[q]; t < ep.ent_tptr[q + 1]; ++t) {
          const int3 tm = ep.terms[t];
          const T l = vals[tm.x] / vals[tm.z];
          if (!(dabs(l) <= tau)) bad = true;
          v -= l * vals[tm.y];
        }
        vals[ep.ent_out[q]] = v;
      }
      for (int q = ep.lev_piv[lev] + tid; q < ep.lev_piv[lev + 1]; q += blockDim.x) {
        const T pv = vals[ep.piv[q]];
        if (!(finite_t(pv) && pv != T(0))) bad = true;
        ld_part += log(fabs((double)pv));
      }
      if (solve) {
        __syncthreads();
        for (int g = ep.lev_fwd_nodes[lev] + tid; g < ep.lev_fwd_nodes[lev + 1]; g += blockDim.x) {
          const int r = ep.fwd_node[g];
          T acc = zf[r];
          for (int q = ep.fwd_ptr[g]; q < ep.fwd_ptr[g + 1]; ++q) {
            const int3 f = ep.fwd[q];
            acc -= vals[f.x] / vals[f.z] * zf[f.y];
          }
          zf[r] = acc;
        }
      }
      __syncthreads();
    }
    // ---- dense core: scatter, identity padding, core right-hand side
    if (planned) {
      for (int q = tid; q < ep.n_core_ent; q += blockDim.x) {
        const int3 ce = ep.core_ent[q];
        A[ce.y + (size_t)dp * ce.z] = vals[ce.x];
      }
      for (int r = ep.core_n + tid; r < dp; r += blockDim.x) A[(size_t)r * dp + r] = T(1);
    }
    if (solve)
      for (int r = tid; r < dp; r += blockDim.x)
        z[r] = (r < ep.core_n) ? zf[planned ? ep.core_node[r] : r] : T(0);
    __syncthreads();
    double ld = 0.0;  // warp 0's running sum of log|u_kk|
    for (int kb = 0; kb < nbk; ++kb) {
      const int k0 = kb * kB, r0 = k0 + kB, R = dp - r0;
      // (a) diagonal block, warp 0, row per lane
      if (warp == 0) {
        for (int c = 0; c < kB; ++c)
          D[lane * (kB + 1) + c] = A[(size_t)(k0 + lane) + (size_t)dp * (k0 + c)];
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
        if (solve) {
          for (int c = 0; c < kB; ++c)
            A[(size_t)(k0 + lane) + (size_t)dp * (k0 + c)] = D[lane * (kB + 1) + c];
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
          for (int c = 0; c < kB; ++c) lp[c * Rmax] = A[(size_t)row + (size_t)dp * (k0 + c)];
          for (int c = 0; c < kB; ++c) {
            T acc = lp[c * Rmax];
#pragma unroll 4
            for (int cp = 0; cp < c; ++cp) acc -= lp[cp * Rmax] * D[cp * (kB + 1) + c];
            acc = acc / D[c * (kB + 1) + c];
            lp[c * Rmax] = acc;
            if (!(dabs(acc) <= tau)) bad = true;
            if (solve) A[(size_t)row + (size_t)dp * (k0 + c)] = acc;
          }
        } else {
          const int tt = t - R;
          const int col = r0 + tt;
          T *colp = A + (size_t)dp * col + k0;
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
        trailing_update<T>(A, dp, r0, R, Lp, Up, Rmax);
      }
      __syncthreads();
    }
    if (bad) atomicOr(&sflag, 1);
    const double ld_levels = block_sum_det(ld_part, red);  // contains __syncthreads
    const bool flagged = (sflag != 0);
    if (tid == 0) {
      logdet[i] = ld + ld_levels;
      if (flagged) atomicOr(&draw_flags[i], DRAW_FLAG_PIVOT);
    }
    if (solve && !flagged) {
      block_back_solve<T>(A, dp, z, D);  // core part of y0
      for (int r = tid; r < ep.core_n; r += blockDim.x) yf[planned ? ep.core_node[r] : r] = z[r];
      __syncthreads();
      levels_backward<T>(ep, vals, zf, yf);
      if (refine) {
        residual<T>(m, P, n, i, rows, theta, nu, yf, res);
        for (int r = tid; r < m; r += blockDim.x) zf[r] = (T)res[r];
        __syncthreads();
        levels_forward<T>(ep, vals, zf);
        T *d = Up;  // the row-panel buffer (32 x Rmax >= d_p) holds the core correction
        for (int r = tid; r < dp; r += blockDim.x)
          d[r] = (r < ep.core_n) ? zf[planned ? ep.core_node[r] : r] : T(0);
        __syncthreads();
        block_forward_solve<T>(A, dp, d, D);
        block_back_solve<T>(A, dp, d, D);
        for (int r = tid; r < ep.core_n; r += blockDim.x) yd[planned ? ep.core_node[r] : r] = d[r];
        __syncthreads();
        levels_backward<T>(ep, vals, zf, yd);
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)yf[r] + (double)yd[r];
      } else {
        for (int r = tid; r < m; r += blockDim.x) y[(size_t)i * m + r] = (double)yf[r];
      }
    }
    __syncthreads();
  }
}

// Partial-pivoting LU of the full matrix for the draws the fast pass flagged
// (getrf semantics).  Unblocked; it runs only on draws whose (I - Gamma) is not
// diagonally dominant enough for the no-pivot pass.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_lu_fallback(int m, int P, int mp, long n, const unsigned *__restrict__ sp,
                  const T *__restrict__ theta, T *__restrict__ scratch,
                  double *__restrict__ logdet, int *__restrict__ draw_flags,
                  const double *__restrict__ x, const T *__restrict__ lambda, RngKey key,
                  double *__restrict__ y, GammaRows rows) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Smem L(mp, m, sizeof(T));
  T *z = reinterpret_cast<T *>(smem_raw + L.off_z);
  double *nu = reinterpret_cast<double *>(smem_raw + L.off_nu);
  double *res = reinterpret_cast<double *>(smem_raw + L.off_res);
  double *red = reinterpret_cast<double *>(smem_raw + L.off_red);  // 64 doubles
  int *perm = reinterpret_cast<int *>(smem_raw + L.off_Lp);        // mp ints
  T *d = reinterpret_cast<T *>(smem_raw + L.off_Up);               // mp values
  T *D = reinterpret_cast<T *>(smem_raw + L.off_D);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  T *A = scratch + (size_t)blockIdx.x * mp * mp;
  const bool solve = (x != nullptr);
  __shared__ int s_piv;
  __shared__ bool s_singular;

  for (long i = blockIdx.x; i < n; i += gridDim.x) {
    if (!(draw_flags[i] & DRAW_FLAG_PIVOT)) continue;
    build_full<T>(m, P, mp, n, i, sp, theta, A);
    if (solve) {
      forecast_rhs<T>(m, P, n, i, sp, theta, x, lambda, key, nu);
      __syncthreads();
      for (int r = tid; r < mp; r += blockDim.x) z[r] = (r < m) ? (T)nu[r] : T(0);
    }
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
      for (int r = k + 1 + tid; r < mp; r += blockDim.x) A[(size_t)r + (size_t)mp * k] /= piv;
      __syncthreads();
      const int rem = mp - k - 1;
      for (long e = tid; e < (long)rem * rem; e += blockDim.x) {
        const int r = k + 1 + (int)(e % rem), c = k + 1 + (int)(e / rem);
        A[(size_t)r + (size_t)mp * c] -= A[(size_t)r + (size_t)mp * k] * A[(size_t)k + (size_t)mp * c];
      }
      if (solve) {
        for (int r = k + 1 + tid; r < mp; r += blockDim.x) z[r] -= A[(size_t)r + (size_t)mp * k] * z[k];
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
        block_back_solve<T>(A, mp, z, D);
        residual<T>(m, P, n, i, rows, theta, nu, z, res);
        for (int r = tid; r < mp; r += blockDim.x) d[r] = (perm[r] < m) ? (T)res[perm[r]] : T(0);
        __syncthreads();
        block_forward_solve<T>(A, mp, d, D);
        block_back_solve<T>(A, mp, d, D);
        for (int r = tid; r < m; r += blockDim.x)
          y[(size_t)i * m + r] = (double)z[r] + (double)d[r];
      }
    }
    __syncthreads();
  }
}

}  // namespace

template <typename T>
LuPlan plan_lu(int m, int P, long n, int num_sms, int core_n, int nv) {
  LuPlan pl{};
  pl.m = m;
  pl.P = P;
  pl.mp = ((m + kB - 1) / kB) * kB;
  pl.dp = ((core_n + kB - 1) / kB) * kB;
  if (pl.dp < kB) pl.dp = kB;
  pl.block = kThreads;
  pl.smem = Smem(pl.dp, m, sizeof(T)).total;
  pl.smem_fallback = Smem(pl.mp, m, sizeof(T)).total;
  int ctas_per_sm = (int)((227u * 1024u) / (pl.smem + 1024));
  if (ctas_per_sm < 1) ctas_per_sm = 1;
  if (ctas_per_sm > 2) ctas_per_sm = 2;
  if (sizeof(T) == 8) ctas_per_sm = 1;
  long grid = (long)num_sms * ctas_per_sm;
  if (grid > n) grid = n;
  if (grid < 1) grid = 1;
  pl.grid = (int)grid;
  pl.scratch_elems_per_cta = (size_t)pl.dp * pl.dp + (((size_t)nv + 3) / 4) * 4;
  const size_t total = pl.scratch_elems_per_cta * pl.grid;
  const size_t full = (size_t)pl.mp * pl.mp;
  long fb = num_sms;
  if (fb > n) fb = n;
  // the redo needs a full m_p x m_p slab per CTA; it shares the slab array
  if ((size_t)fb * full > total) {
    const long fit = (long)(total / full);
    fb = std::max(fit, std::min(fb, 16L));
  }
  if (fb < 1) fb = 1;
  pl.fb_grid = (int)fb;
  pl.scratch_elems_total = std::max(total, (size_t)pl.fb_grid * full);
  return pl;
}

template <typename T>
void launch_lu(cudaStream_t s, const LuPlan &pl, long n, const EliminationPlan &ep,
               const unsigned *sp, const T *theta, T *scratch, double *logdet, int *draw_flags,
               const double *x, const T *lambda, RngKey key, bool refine, double *y,
               GammaRows rows) {
  // opt in to exactly the shared memory this plan needs (a failure here shows up
  // as a launch error that the engine reports)
  if (pl.smem > 48 * 1024)
    cudaFuncSetAttribute(k_lu<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);
  k_lu<T><<<pl.grid, pl.block, pl.smem, s>>>(pl.m, pl.P, pl.dp, pl.scratch_elems_per_cta, n, ep,
                                             sp, theta, scratch, logdet, draw_flags, x, lambda,
                                             key, refine, y, rows);
}

template <typename T>
void launch_lu_fallback(cudaStream_t s, const LuPlan &pl, long n, const unsigned *sp,
                        const T *theta, T *scratch, double *logdet, int *draw_flags,
                        const double *x, const T *lambda, RngKey key, double *y,
                        GammaRows rows) {
  if (pl.smem_fallback > 48 * 1024)
    cudaFuncSetAttribute(k_lu_fallback<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)pl.smem_fallback);
  k_lu_fallback<T><<<pl.fb_grid, pl.block, pl.smem_fallback, s>>>(
      pl.m, pl.P, pl.mp, n, sp, theta, scratch, logdet, draw_flags, x, lambda, key, y, rows);
}

template LuPlan plan_lu<float>(int, int, long, int, int, int);
template LuPlan plan_lu<double>(int, int, long, int, int, int);
template void launch_lu<float>(cudaStream_t, const LuPlan &, long, const EliminationPlan &,
                               const unsigned *, const float *, float *, double *, int *,
                               const double *, const float *, RngKey, bool, double *, GammaRows);
template void launch_lu<double>(cudaStream_t, const LuPlan &, long, const EliminationPlan &,
                                const unsigned *, const double *, double *, double *, int *,
                                const double *, const double *, RngKey, bool, double *,
                                GammaRows);
template void launch_lu_fallback<float>(cudaStream_t, const LuPlan &, long, const unsigned *,
                                        const float *, float *, double *, int *, const double *,
                                        const float *, RngKey, double *, GammaRows);
template void launch_lu_fallback<double>(cudaStream_t, const LuPlan &, long, const unsigned *,
                                         const double *, double *, double *, int *,
                                         const double *, const double *, RngKey, double *,
                                         GammaRows);

}  // namespace sgdlm
