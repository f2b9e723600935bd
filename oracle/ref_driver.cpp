// Runs the reference's own device kernels on the CPU -- TEST INFRASTRUCTURE ONLY.
//
// The reference (lutzgruber/gpuSGDLM) has no CPU implementation and no tests.
// This driver includes its kernel header rSGDLM/src/kernel_functions.cuh
// unchanged, compiled by g++ against the stand-in headers in oracle/ref_shim/,
// and launches each kernel with the grid and block shapes of its call site in
// rSGDLM/src/SGDLM/SGDLM.cu.  An emulated block runs its threads in order;
// kernels that synchronise (the Marsaglia-Tsang samplers) run each thread as a
// ucontext fiber that yields at __syncthreads.  The cuBLAS calls of SGDLM.cu
// (gemmBatched, getrfBatched, getriBatched) are replaced by plain loops, and
// the cuRAND streams by inputs supplied by the caller.
//
// Built by oracle/build_ref.sh into oracle/_ref/ (not committed); its outputs are
// recorded as fixtures by tests/golden/make_golden.py.
#include <ucontext.h>

#include <cstdio>
#include <cstring>
#include <functional>
#include <vector>

#include "cuda_runtime.h"

// Shared memory of the emulated block (the samplers' `extern __shared__ counter`).
unsigned int counter[1 << 16];

#include "kernel_functions.cuh"

thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

namespace {

struct Fiber {
  ucontext_t ctx;
  bool done = false;
  dim3 tid;
};

ucontext_t g_sched;
Fiber *g_cur = nullptr;
std::function<void()> *g_body = nullptr;
bool g_in_fiber = false;

void trampoline() {
  (*g_body)();
  g_cur->done = true;
  swapcontext(&g_cur->ctx, &g_sched);
}

// Launches `body` over grid x block; with barriers, threads are fibers.
void launch(dim3 grid, dim3 block, bool barriers, std::function<void()> body) {
  gridDim = grid;
  blockDim = block;
  const size_t nthr = (size_t)block.x * block.y * block.z;
  const size_t kStack = 64 * 1024;
  std::vector<char> stacks;
  std::vector<Fiber> fibers;
  if (barriers) {
    stacks.resize(nthr * kStack);
    fibers.resize(nthr);
  }
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        blockIdx = dim3(bx, by, bz);
        if (!barriers) {
          for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
              for (unsigned tx = 0; tx < block.x; ++tx) {
                threadIdx = dim3(tx, ty, tz);
                body();
              }
          continue;
        }
        size_t t = 0;
        for (unsigned tz = 0; tz < block.z; ++tz)
          for (unsigned ty = 0; ty < block.y; ++ty)
            for (unsigned tx = 0; tx < block.x; ++tx, ++t) {
              Fiber &f = fibers[t];
              f.done = false;
              f.tid = dim3(tx, ty, tz);
              getcontext(&f.ctx);
              f.ctx.uc_stack.ss_sp = stacks.data() + t * kStack;
              f.ctx.uc_stack.ss_size = kStack;
              f.ctx.uc_link = nullptr;
              makecontext(&f.ctx, trampoline, 0);
            }
        g_body = &body;
        g_in_fiber = true;
        bool live = true;
        while (live) {
          live = false;
          for (auto &f : fibers) {
            if (f.done) continue;
            g_cur = &f;
            threadIdx = f.tid;
            swapcontext(&g_sched, &f.ctx);
            live = true;
          }
        }
        g_in_fiber = false;
      }
}

}  // namespace

void __syncthreads() {
  if (g_in_fiber) swapcontext(&g_cur->ctx, &g_sched);
}
// The emulated block runs one thread at a time, so a plain update is atomic.
unsigned int atomicAdd(unsigned int *addr, unsigned int val) {
  const unsigned int old = *addr;
  *addr = old + val;
  return old;
}

namespace {

unsigned cdiv(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

template <typename T> std::vector<T *> ptrs(T *base, size_t count, size_t stride) {
  std::vector<T *> v(count);
  for (size_t i = 0; i < count; ++i) v[i] = base + i * stride;
  return v;
}

// Partial-pivoting LU and inverse standing in for cublasDgetrfBatched /
// cublasDgetriBatched (column-major n x n).
void getrf(int n, double *A, int *piv) {
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double best = std::fabs(A[k + (size_t)n * k]);
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(A[r + (size_t)n * k]) > best) {
        best = std::fabs(A[r + (size_t)n * k]);
        pr = r;
      }
    piv[k] = pr;
    if (pr != k)
      for (int c = 0; c < n; ++c) std::swap(A[k + (size_t)n * c], A[pr + (size_t)n * c]);
    const double d = A[k + (size_t)n * k];
    if (d == 0.0) continue;
    for (int r = k + 1; r < n; ++r) A[r + (size_t)n * k] /= d;
    for (int c = k + 1; c < n; ++c)
      for (int r = k + 1; r < n; ++r) A[r + (size_t)n * c] -= A[r + (size_t)n * k] * A[k + (size_t)n * c];
  }
}
void getri(int n, const double *LU, const int *piv, double *Ainv) {
  std::vector<double> x(n);
  for (int c = 0; c < n; ++c) {
    for (int r = 0; r < n; ++r) x[r] = (r == c) ? 1.0 : 0.0;
    for (int k = 0; k < n; ++k)
      if (piv[k] != k) std::swap(x[k], x[piv[k]]);
    for (int k = 0; k < n; ++k)
      for (int r = k + 1; r < n; ++r) x[r] -= LU[r + (size_t)n * k] * x[k];
    for (int k = n - 1; k >= 0; --k) {
      x[k] /= LU[k + (size_t)n * k];
      for (int r = 0; r < k; ++r) x[r] -= LU[r + (size_t)n * k] * x[k];
    }
    for (int r = 0; r < n; ++r) Ainv[r + (size_t)n * c] = x[r];
  }
}

const unsigned TPB = THREADS_PER_BLOCK;

}  // namespace

extern "C" {

double ref_psi(double x) { return psi<double>(x); }
double ref_psi1(double x) { return psi1<double>(x); }

// compute_posterior, SGDLM.cu:10-113 (launch shapes at :22-24, :31-34, :58-64,
// :78-79, :84-86, :91-92, :97-99, :107-110).
void ref_posterior(int m, int P, const unsigned *p, double *m_t, double *C_t, double *n_t,
                   double *s_t, const double *y, const double *F) {
  std::vector<double> A((size_t)m * P), Q(m), e(m);
  auto mp = ptrs(m_t, m, P);
  auto Cp = ptrs(C_t, m, (size_t)P * P);
  auto Ap = ptrs(A.data(), m, P);
  dim3 tpb(TPB / P, P), nb(cdiv(m, TPB / P), 1);
  launch(nb, tpb, false, [&] { batchedCutOffVector<double>(m, P, p, mp.data()); });
  launch(dim3(cdiv(m, TPB / P), P), tpb, false,
         [&] { batchedCutOffMatrix<double>(m, P, P, p, p, Cp.data()); });
  for (int j = 0; j < m; ++j)  // gemm A = R F
    for (int r = 0; r < P; ++r) {
      double acc = 0.0;
      for (int c = 0; c < P; ++c) acc += C_t[(size_t)j * P * P + r + P * c] * F[(size_t)j * P + c];
      A[(size_t)j * P + r] = acc;
    }
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] { copy<double>(m, s_t, Q.data()); });
  for (int j = 0; j < m; ++j) {  // gemm Q = F'A + Q
    double acc = 0.0;
    for (int r = 0; r < P; ++r) acc += F[(size_t)j * P + r] * A[(size_t)j * P + r];
    Q[j] = acc + Q[j];
  }
  launch(nb, tpb, false,
         [&] { batchedScale<double>(m, P, Ap.data(), Q.data(), SCALE_TRANSFORMATION_INV); });
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] { copy<double>(m, y, e.data()); });
  for (int j = 0; j < m; ++j) {  // gemm e = -F'm + e
    double acc = 0.0;
    for (int r = 0; r < P; ++r) acc += F[(size_t)j * P + r] * m_t[(size_t)j * P + r];
    e[j] = -acc + e[j];
  }
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] { addScalar<double>(m, n_t, 1.0); });
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false,
         [&] { computeSt<double>(m, s_t, n_t, e.data(), Q.data()); });
  launch(nb, tpb, false,
         [&] { batchedComputeMt<double>(m, P, mp.data(), (const double **)Ap.data(), e.data()); });
  launch(nb, tpb, false,
         [&] { batchedScale<double>(m, P, Ap.data(), Q.data(), SCALE_TRANSFORMATION_SQRT); });
  for (int j = 0; j < m; ++j)  // gemm C = -A A' + C
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r)
        C_t[(size_t)j * P * P + r + P * c] =
            -(A[(size_t)j * P + r] * A[(size_t)j * P + c]) + C_t[(size_t)j * P * P + r + P * c];
  launch(dim3(cdiv(m, TPB / P), P), tpb, false,
         [&] { batchedScaleCt<double>(m, (size_t)P * P, Cp.data(), n_t, e.data(), Q.data()); });
}

// compute_one_step_ahead_prior with G = NULL, SGDLM.cu:115-149.
void ref_prior(int m, int P, const unsigned *p, double *C_t, double *n_t, double *W_t,
               const double *beta, const double *delta) {
  auto Cp = ptrs(C_t, m, (size_t)P * P);
  auto Wp = ptrs(W_t, m, (size_t)P * P);
  auto Dp = ptrs(delta, m, (size_t)P * P);
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] { multiply<double>(m, n_t, beta); });
  dim3 tpb(TPB / P, P), nb(cdiv(m, TPB / P), P);
  launch(nb, tpb, false, [&] {
    batchedMatrixScaleWithDiff<double>(m, P, p, p, Cp.data(), Wp.data(), (const double **)Dp.data(),
                                       SCALE_TRANSFORMATION_INV);
  });
}

// cholesky kernel, launch at SGDLM.cu:648-651.
void ref_cholesky(int m, int P, const unsigned *p, const double *C_t, double *U) {
  auto Cp = ptrs(C_t, m, (size_t)P * P);
  auto Up = ptrs(U, m, (size_t)P * P);
  launch(dim3(1, cdiv(m, TPB)), dim3(1, TPB), false,
         [&] { cholesky<double>(m, P, P, p, (const double **)Cp.data(), Up.data()); });
}

// theta from given lambdas and standard normals (draw-major n x m and n x m x P):
// cholesky, gemm theta = chol' z, makeVB_MVN (SGDLM.cu:647-673).
void ref_thetas(int m, int P, const unsigned *p, const double *m_t, const double *C_t,
                const double *s_t, long n, const double *lambdas, const double *z, double *theta) {
  std::vector<double> U((size_t)m * P * P);
  ref_cholesky(m, P, p, C_t, U.data());
  for (long i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < P; ++k) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += U[(size_t)j * P * P + l + P * k] * z[((size_t)i * m + j) * P + l];
        theta[((size_t)i * m + j) * P + k] = acc;
      }
  auto mp = ptrs(m_t, m, P);
  auto lp = ptrs(lambdas, n, m);
  auto tp = ptrs(theta, n, (size_t)m * P);
  dim3 tpb(1, TPB / P, P), nb((unsigned)n, cdiv(m, TPB / P), 1);
  launch(nb, tpb, false, [&] {
    makeVB_MVN<double>(n, m, P, (const double **)mp.data(), (const double **)lp.data(), s_t, tp.data());
  });
}

// make_gamma2 with caller-supplied uniforms and normals (n_loops * n * m each,
// index j*n_loops*n + k*n + i), launch of curand_manager.cuh:123-139.  gammas is
// draw-major n x m.
void ref_make_gamma2(int m, long n, int n_loops, const double *uniforms, const double *normals,
                     const double *n_t, const double *s_t, double *gammas) {
  auto gp = ptrs(gammas, n, m);
  launch(dim3(cdiv(n, TPB), m), dim3(TPB, 1), true, [&] {
    make_gamma2<double>(m, n, n_loops, nullptr, uniforms, normals, n_t, s_t, gp.data());
  });
}

// make_beta with caller-supplied first gammas in `betas` (draw-major n x m).
void ref_make_beta(int m, long n, int n_loops, const double *uniforms, const double *normals,
                   const double *r_t, const double *beta, double *betas) {
  auto bp = ptrs(betas, n, m);
  launch(dim3(cdiv(n, TPB), m), dim3(TPB, 1), true, [&] {
    make_beta<double>(m, n, n_loops, nullptr, uniforms, normals, r_t, beta, bp.data());
  });
}

// VB_posterior without sampling (SGDLM.cu:231-500) for caller-supplied draws
// (draw-major lambdas n x m, thetas n x m x P), one IS batch of n.  theta is
// overwritten (the reference turns it into sqrt(lambda)(theta - m_bar)).
// aux = {E lambda (m), E log lambda (m), Q_bar (m)}.
void ref_vb(int m, int P, const unsigned *p, const unsigned *sp, const double *n_t,
            const double *s_t, long n, const double *lambdas, double *thetas, double *w,
            double *sum_w, double *mean_m, double *mean_C, double *mean_n, double *mean_s,
            double *aux) {
  const size_t mm = (size_t)m * m;
  std::vector<double> G(mm * n);
  std::vector<int> piv(m);
  auto Gp = ptrs(G.data(), n, mm);
  auto lp = ptrs(lambdas, n, m);
  auto tp = ptrs(thetas, n, (size_t)m * P);
  launch(dim3(cdiv(mm, TPB), (unsigned)n), dim3(TPB, 1), false,
         [&] { batchedInitVector<double>(n, mm, Gp.data()); });
  launch(dim3(cdiv((size_t)m * P, TPB), (unsigned)n), dim3(TPB, 1), false,
         [&] { fillGammas<double>(n, 0, m, P, sp, Gp.data(), (const double **)tp.data()); });
  for (long i = 0; i < n; ++i) getrf(m, Gp[i], piv.data());
  launch(dim3(cdiv(n, TPB)), dim3(TPB), false,
         [&] { detFromLU<double>(n, m, (const double **)Gp.data(), w, 0); });
  launch(dim3(1), dim3(1), false, [&] { sumVector<double>(n, w, sum_w); });
  launch(dim3(cdiv(n, TPB)), dim3(TPB), false,
         [&] { scale<double>(n, w, sum_w, SCALE_TRANSFORMATION_INV); });
  std::vector<double> El(m), Ell(m), Qb(m), Cbuf((size_t)m * P * P), Vinv((size_t)m * P * P),
      Q((size_t)n * m);
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] {
    meanScalarAndLog<double>(n, m, w, (const double **)lp.data(), El.data(), Ell.data());
  });
  auto mbp = ptrs(mean_m, m, P);
  auto mCp = ptrs(mean_C, m, (size_t)P * P);
  auto Cbp = ptrs(Cbuf.data(), m, (size_t)P * P);
  auto Vip = ptrs(Vinv.data(), m, (size_t)P * P);
  launch(dim3(1, cdiv(m, TPB / P)), dim3(P, TPB / P), false, [&] {
    compute_mean_m_t<double>(n, m, P, w, (const double **)lp.data(), El.data(),
                             (const double **)tp.data(), mbp.data());
  });
  launch(dim3(m, cdiv(n, TPB / P), 1), dim3(1, TPB / P, P), false, [&] {
    compute_VB_vector1<double>(n, m, P, (const double **)lp.data(), (const double **)mbp.data(),
                               tp.data());
  });
  launch(dim3(P, cdiv(m, TPB / P), 1), dim3(1, TPB / P, P), false, [&] {
    meanBatchedVecVecT<double>(n, m, P, p, w, (const double **)tp.data(), mCp.data());
  });
  launch(dim3(cdiv(m, TPB / P), 1), dim3(TPB / P, P), false,
         [&] { batchedCutOffVector<double>(m, P, p, mbp.data()); });
  launch(dim3(cdiv(m, TPB / P), P), dim3(TPB / P, P), false,
         [&] { batchedCutOffMatrix<double>(m, P, P, p, p, mCp.data()); });
  launch(dim3(P, cdiv(m, TPB / P)), dim3(P, TPB / P), false,
         [&] { batchedCopy<double>(m, (size_t)P * P, (const double **)mCp.data(), Cbp.data()); });
  launch(dim3(cdiv(m, TPB / P), 1), dim3(TPB / P, P), false,
         [&] { batchedSetOutsideSquareMatrixDiagonal<double>(m, P, p, Cbp.data(), 1.0); });
  std::vector<int> pv(P);
  for (int j = 0; j < m; ++j) {
    getrf(P, Cbp[j], pv.data());
    getri(P, Cbp[j], pv.data(), Vip[j]);
  }
  launch(dim3(cdiv(m, TPB / P), P), dim3(TPB / P, P), false,
         [&] { batchedCutOffMatrix<double>(m, P, P, p, p, Vip.data()); });
  for (long i = 0; i < n; ++i)  // the two gemmBatched of SGDLM.cu:447-457
    for (int j = 0; j < m; ++j) {
      const double *th = thetas + ((size_t)i * m + j) * P;
      double q = 0.0;
      for (int c = 0; c < P; ++c) {
        double t = 0.0;
        for (int r = 0; r < P; ++r) t += th[r] * Vip[j][r + P * c];
        q += t * th[c];
      }
      Q[(size_t)i * m + j] = q;
    }
  auto Qp = ptrs(Q.data(), n, m);
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false,
         [&] { compute_mean_Q_t<double>(n, m, w, (const double **)Qp.data(), Qb.data()); });
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] {
    compute_mean_n_t<double>(m, p, Qb.data(), El.data(), Ell.data(), n_t, mean_n);
  });
  launch(dim3(cdiv(m, TPB)), dim3(TPB), false, [&] {
    compute_mean_s_t<double>(m, p, mean_n, Qb.data(), El.data(), s_t, mean_s);
  });
  launch(dim3(cdiv(m, TPB), (unsigned)(P * P)), dim3(TPB, 1), false, [&] {
    batchedScale<double>(m, P, p, p, mCp.data(), mean_s, SCALE_TRANSFORMATION_NONE);
  });
  for (int j = 0; j < m; ++j) {
    aux[j] = El[j];
    aux[m + j] = Ell[j];
    aux[2 * m + j] = Qb[j];
  }
}

// forecast (SGDLM.cu:538-620) for caller-supplied draws and N(0,1) nus (draw-major
// n x m): batchedComputeNuPlusMu, then y = (I - Gamma)^-1 nu via getrf/getri/gemm.
void ref_forecast(int m, int P, const unsigned *sp, long n, const double *lambdas,
                  const double *thetas, const double *x, const double *nus_in, double *y) {
  const size_t mm = (size_t)m * m;
  std::vector<double> nus(nus_in, nus_in + (size_t)n * m), G(mm), Gi(mm);
  std::vector<int> piv(m);
  auto lp = ptrs(lambdas, n, m);
  auto tp = ptrs(thetas, n, (size_t)m * P);
  auto xp = ptrs(x, m, P);
  auto np = ptrs(nus.data(), n, m);
  launch(dim3(cdiv(n, TPB), m), dim3(TPB, 1), false, [&] {
    batchedComputeNuPlusMu<double>(n, m, P, sp, (const double **)xp.data(), (const double **)tp.data(),
                                   (const double **)lp.data(), np.data());
  });
  for (long i = 0; i < n; ++i) {
    double *Gp1[1] = {G.data()};
    const double *tp1[1] = {tp[i]};
    launch(dim3(cdiv(mm, TPB), 1), dim3(TPB, 1), false,
           [&] { batchedInitVector<double>(1, mm, Gp1); });
    launch(dim3(cdiv((size_t)m * P, TPB), 1), dim3(TPB, 1), false,
           [&] { fillGammas<double>(1, 0, m, P, sp, Gp1, tp1); });
    getrf(m, G.data(), piv.data());
    getri(m, G.data(), piv.data(), Gi.data());
    for (int r = 0; r < m; ++r) {
      double acc = 0.0;
      for (int c = 0; c < m; ++c) acc += Gi[r + (size_t)m * c] * nus[(size_t)i * m + c];
      y[(size_t)i * m + r] = acc;
    }
  }
}

// The omega scaling and theta update of evolve_lambdas_and_thetas
// (SGDLM.cu:710-758) with its launch geometry, for caller-supplied N(0,1) omegas
// (draw-major n x m x P) and already evolved lambdas.
void ref_evolve_theta(int m, int P, const unsigned *p, const double *W_t, const double *c_t,
                      long n, const double *lambdas, const double *omegas_in, double *thetas) {
  std::vector<double> om(omegas_in, omegas_in + (size_t)n * m * P), UW((size_t)m * P * P);
  auto lp = ptrs(lambdas, n, m);
  auto op = ptrs(om.data(), (size_t)n * m, P);
  dim3 tpb(TPB / P, P), nb(cdiv((size_t)n * m + TPB - 1, 1) / (TPB / P), 1);
  nb = dim3((unsigned)(((size_t)n * m + TPB - 1) / tpb.x), 1);
  launch(nb, tpb, false,
         [&] { scale_omegas<double>(n, m, P, p, (const double **)lp.data(), c_t, op.data()); });
  ref_cholesky(m, P, p, W_t, UW.data());
  for (long i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j)
      for (int k = 0; k < P; ++k) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l)
          acc += UW[(size_t)j * P * P + l + P * k] * om[((size_t)i * m + j) * P + l];
        thetas[((size_t)i * m + j) * P + k] = acc + thetas[((size_t)i * m + j) * P + k];
      }
}

// compute_one_step_ahead_prior with an evolution matrix, SGDLM.cu:116-178: r = beta n,
// R = C / Delta and W = R - C inside p x p (batchedMatrixScaleWithDiff), then
// a = G m (gemmBatched, as loops) cut at p (batchedCutOffVector), C_buffer = G R,
// R = C_buffer G' (gemmBatched, as loops), batchedCutOffMatrix with the launch
// shape of SGDLM.cu:170-175.
void ref_evo_prior(int m, int P, const unsigned *p, double *m_t, double *C_t, double *n_t,
                   double *W_t, const double *beta, const double *delta, const double *G) {
  ref_prior(m, P, p, C_t, n_t, W_t, beta, delta);
  const size_t PP = (size_t)P * P;
  std::vector<double> mbuf(m_t, m_t + (size_t)m * P), Cbuf(PP * m);
  for (int j = 0; j < m; ++j)
    for (int r = 0; r < P; ++r) {
      double acc = 0.0;
      for (int l = 0; l < P; ++l) acc += G[j * PP + r + (size_t)P * l] * mbuf[(size_t)j * P + l];
      m_t[(size_t)j * P + r] = acc;
    }
  auto mp = ptrs(m_t, m, P);
  launch(dim3(cdiv(m, TPB / P), 1), dim3(TPB / P, P), false,
         [&] { batchedCutOffVector<double>(m, P, p, mp.data()); });
  for (int j = 0; j < m; ++j)
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += G[j * PP + r + (size_t)P * l] * C_t[j * PP + l + (size_t)P * c];
        Cbuf[j * PP + r + (size_t)P * c] = acc;
      }
  for (int j = 0; j < m; ++j)
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += Cbuf[j * PP + r + (size_t)P * l] * G[j * PP + c + (size_t)P * l];
        C_t[j * PP + r + (size_t)P * c] = acc;
      }
  auto Cp = ptrs(C_t, m, PP);
  launch(dim3(cdiv(m, TPB / P), P), dim3(TPB / P, P), false,
         [&] { batchedCutOffMatrix<double>(m, P, P, p, p, Cp.data()); });
}

// evolve_lambdas_and_thetas with an evolution matrix (SGDLM.cu:729-740): theta = G theta
// (gemmBatched over all n*m draws, as loops) before theta += chol(W)' omega.
void ref_evolve_theta_g(int m, int P, const unsigned *p, const double *W_t, const double *c_t,
                        long n, const double *lambdas, const double *omegas_in, const double *G,
                        double *thetas) {
  const size_t PP = (size_t)P * P;
  std::vector<double> buf(P);
  for (long i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) {
      double *th = thetas + ((size_t)i * m + j) * P;
      for (int l = 0; l < P; ++l) buf[l] = th[l];
      for (int r = 0; r < P; ++r) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += G[j * PP + r + (size_t)P * l] * buf[l];
        th[r] = acc;
      }
    }
  ref_evolve_theta(m, P, p, W_t, c_t, n, lambdas, omegas_in, thetas);
}

}  // extern "C"
