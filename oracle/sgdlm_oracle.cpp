// SGDLM oracle: a plain C++ FP64 restatement of the reference algorithm.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product links or calls this file; it
// is the checker used by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline.  Each function follows the reference file:line given in its comment
// (paths inside lutzgruber/gpuSGDLM, rSGDLM/src/...), sequentially and in FP64.
// Where the reference delegates to cuBLAS (gemm, getrf, getri) the textbook
// operation is written out; where it draws random numbers from cuRAND, the
// oracle regenerates the GB300 library's Philox4x32-10 streams from the same
// (draw, series, tag, sub, epoch) counters, with its own Philox, Box-Muller and
// Marsaglia-Tsang code, so that sampled steps can be compared draw by draw.
//
// The restatement itself is pinned against the reference's own kernel code by
// oracle/ref_driver.cpp (the reference's kernel_functions.cuh compiled for the
// CPU), whose outputs are committed as tests/golden/ fixtures.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- random streams
struct U4 {
  uint32_t x, y, z, w;
};

// Philox4x32-10 (Salmon et al., SC'11).
U4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
  uint32_t c[4] = {c0, c1, c2, c3};
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c[0] = n0;
    c[1] = n1;
    c[2] = n2;
    c[3] = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return U4{c[0], c[1], c[2], c[3]};
}

enum : uint32_t { TAG_GAMMA = 1, TAG_THETA = 2, TAG_NU = 3, TAG_BETA_A = 4, TAG_BETA_B = 5, TAG_OMEGA = 6 };
const int kGammaMaxAttempts = 32;

struct Key {
  uint32_t k0, k1, epoch;
};
Key make_key(uint64_t seed, uint64_t epoch) {
  return Key{(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32), (uint32_t)epoch};
}
U4 draw_block(const Key &k, uint32_t i, uint32_t j, uint32_t tag, uint32_t sub) {
  return philox(i, j, (tag << 24) | (sub & 0xFFFFFFu), k.epoch, k.k0, k.k1);
}

double unif(uint32_t x) { return ((double)x + 0.5) * 2.3283064365386963e-10; }

void box_muller(uint32_t a, uint32_t b, double &z0, double &z1) {
  const double u1 = unif(a), u2 = unif(b);
  const double r = std::sqrt(-2.0 * std::log(u1));
  const double ang = 2.0 * M_PI * u2;
  z0 = r * std::cos(ang);
  z1 = r * std::sin(ang);
}

// Marsaglia & Tsang (2000) with the alpha < 1 boost; the reference's samplers are
// rSGDLM/src/kernel_functions.cuh:569-634 (lambda), :644-798 (Beta), which use
// the same accept/reject test (their squeeze constant 0.331 vs the published
// 0.0331 only short-cuts a subset of the exact log test).
double gamma_mt(double alpha, const Key &k, uint32_t i, uint32_t j, uint32_t tag,
                bool no_boost, bool *failed) {
  const bool boost = alpha < 1.0 && !no_boost;
  const double a = boost ? alpha + 1.0 : alpha;
  const double d = a - 1.0 / 3.0;
  const double c = 1.0 / std::sqrt(9.0 * d);
  double result = alpha, boost_u = 1.0;
  bool ok = false;
  for (int t = 0; t < kGammaMaxAttempts; ++t) {
    const U4 r = draw_block(k, i, j, tag, (uint32_t)t);
    if (t == 0) boost_u = unif(r.w);
    double x, unused;
    box_muller(r.x, r.y, x, unused);
    const double cx = 1.0 + c * x;
    const double v = cx * cx * cx;
    if (v <= 0.0) continue;
    const double u = unif(r.z);
    const double x2 = x * x;
    if (u < 1.0 - 0.0331 * x2 * x2 || std::log(u) < 0.5 * x2 + d * (1.0 - v + std::log(v))) {
      result = d * v;
      ok = true;
      break;
    }
  }
  if (!ok && failed) *failed = true;
  if (boost && ok) result *= std::pow(boost_u, 1.0 / alpha);
  return result;
}

void normals4(const Key &k, uint32_t i, uint32_t j, uint32_t tag, int P, double *z) {
  for (int q = 0; 4 * q < P; ++q) {
    const U4 r = draw_block(k, i, j, tag, (uint32_t)q);
    double a, b, c, d;
    box_muller(r.x, r.y, a, b);
    box_muller(r.z, r.w, c, d);
    const double v[4] = {a, b, c, d};
    for (int t = 0; t < 4 && 4 * q + t < P; ++t) z[4 * q + t] = v[t];
  }
}

// ---------------------------------------------------------------- dense algebra
// Partial-pivoting LU (cublasXgetrfBatched semantics, cublas_manager.cuh:69-77) of
// the column-major n x n matrix A in place; returns sum log|u_kk| and writes the
// row permutation.  Returns -inf on an exactly singular column.
double lu_pp(int n, double *A, int *perm) {
  double ld = 0.0;
  for (int r = 0; r < n; ++r) perm[r] = r;
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double best = std::fabs(A[k + (size_t)n * k]);
    for (int r = k + 1; r < n; ++r) {
      const double v = std::fabs(A[r + (size_t)n * k]);
      if (v > best) {
        best = v;
        pr = r;
      }
    }
    if (!(best > 0.0)) return -std::numeric_limits<double>::infinity();
    if (pr != k) {
      for (int c = 0; c < n; ++c) std::swap(A[k + (size_t)n * c], A[pr + (size_t)n * c]);
      std::swap(perm[k], perm[pr]);
    }
    const double piv = A[k + (size_t)n * k];
    ld += std::log(std::fabs(piv));
    for (int r = k + 1; r < n; ++r) A[r + (size_t)n * k] /= piv;
    for (int c = k + 1; c < n; ++c) {
      const double ukc = A[k + (size_t)n * c];
      if (ukc == 0.0) continue;
      for (int r = k + 1; r < n; ++r) A[r + (size_t)n * c] -= A[r + (size_t)n * k] * ukc;
    }
  }
  return ld;
}

// Solves A x = b with the factors of lu_pp (b overwritten by x).
void lu_solve(int n, const double *LU, const int *perm, double *b) {
  std::vector<double> x(n);
  for (int r = 0; r < n; ++r) x[r] = b[perm[r]];
  for (int c = 0; c < n; ++c)
    for (int r = c + 1; r < n; ++r) x[r] -= LU[r + (size_t)n * c] * x[c];
  for (int c = n - 1; c >= 0; --c) {
    x[c] /= LU[c + (size_t)n * c];
    for (int r = 0; r < c; ++r) x[r] -= LU[r + (size_t)n * c] * x[c];
  }
  for (int r = 0; r < n; ++r) b[r] = x[r];
}

// (I - Gamma_i) of draw i: identity plus -theta at every sp < m*m
// (fillGammas, kernel_functions.cuh:822-842).  theta is series-major.
void build_gamma(int m, int P, const unsigned *sp, long n, long i, const double *theta,
                 double *A) {
  std::fill(A, A + (size_t)m * m, 0.0);
  for (int r = 0; r < m; ++r) A[r + (size_t)m * r] = 1.0;
  const size_t mm = (size_t)m * m;
  for (int j = 0; j < m; ++j)
    for (int k = 0; k < P; ++k) {
      const unsigned pos = sp[(size_t)j * P + k];
      if ((size_t)pos < mm) A[pos] = -theta[((size_t)j * n + i) * P + k];
    }
}

// The reference's digamma/trigamma series (kernel_functions.cuh:1006-1022).
double psi_series(double x) {
  return std::log(x) - 1 / (2 * x) - 1 / (12 * x * x) + 1 / (120 * x * x * x * x) -
         1 / (252 * std::pow(x, 6)) + 1 / (240 * std::pow(x, 8)) - 5 / (660 * std::pow(x, 10)) +
         691 / (32760 * std::pow(x, 12)) - 1 / (12 * std::pow(x, 14));
}
double psi1_series(double x) {
  return 1 / x + 1 / (2 * x * x) + 1 / (6 * x * x * x) - 1 / (30 * std::pow(x, 5)) +
         1 / (42 * std::pow(x, 7)) - 1 / (30 * std::pow(x, 9));
}

int nthreads_eff(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------------------
// Philox block, for the known-answer test.
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  const U4 r = philox(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

double orc_psi(double x) { return psi_series(x); }
double orc_psi1(double x) { return psi1_series(x); }

// Single Marsaglia-Tsang step with given normal x and uniform u (shape alpha >= 1/3):
// returns d*v when accepted, -1 when rejected.  Used to pin the accept/reject
// rule against the reference's make_gamma2 (kernel_functions.cuh:601-625).
double orc_mt_try(double alpha, double x, double u) {
  const double d = alpha - 1.0 / 3.0;
  const double c = 1.0 / std::sqrt(9.0 * d);
  const double cx = 1.0 + c * x;
  const double v = cx * cx * cx;
  if (v <= 0.0) return -1.0;
  const double x2 = x * x;
  if (u < 1.0 - 0.0331 * x2 * x2 || std::log(u) < 0.5 * x2 + d * (1.0 - v + std::log(v)))
    return d * v;
  return -1.0;
}

// compute_posterior, rSGDLM/src/SGDLM/SGDLM.cu:10-113, step by step.
void orc_posterior(int m, int P, const unsigned *p, double *m_t, double *C_t, double *n_t,
                   double *s_t, const double *y, const double *F) {
  std::vector<double> A(P);
  for (int j = 0; j < m; ++j) {
    double *mt = m_t + (size_t)j * P;
    double *C = C_t + (size_t)j * P * P;
    const double *f = F + (size_t)j * P;
    const unsigned pj = p[j];
    for (int k = 0; k < P; ++k)  // batchedCutOffVector (kernel_functions.cuh:86-95)
      if ((unsigned)k >= pj) mt[k] = 0.0;
    for (int c = 0; c < P; ++c)  // batchedCutOffMatrix (kernel_functions.cuh:98-110)
      for (int r = 0; r < P; ++r)
        if ((unsigned)r >= pj && (unsigned)c >= pj) C[r + P * c] = 0.0;
    for (int r = 0; r < P; ++r) {  // A = R F (SGDLM.cu:41-43)
      double acc = 0.0;
      for (int c = 0; c < P; ++c) acc += C[r + P * c] * f[c];
      A[r] = acc;
    }
    double Q = s_t[j];  // Q = c + F'A (SGDLM.cu:47-54)
    for (int r = 0; r < P; ++r) Q += f[r] * A[r];
    for (int r = 0; r < P; ++r) A[r] = A[r] / Q;  // A /= Q (SGDLM.cu:63)
    double e = y[j];  // e = y - F'a (SGDLM.cu:69-74)
    for (int r = 0; r < P; ++r) e -= f[r] * mt[r];
    n_t[j] = n_t[j] + 1.0;                                            // SGDLM.cu:78
    s_t[j] = s_t[j] * (n_t[j] - 1.0 + e * e / Q) / n_t[j];            // kernel_functions.cuh:480-487
    for (int r = 0; r < P; ++r) mt[r] = mt[r] + e * A[r];             // :382-390
    for (int r = 0; r < P; ++r) A[r] = A[r] * std::sqrt(Q);           // SGDLM.cu:97
    for (int c = 0; c < P; ++c)                                       // C = R - A A' (SGDLM.cu:101-103)
      for (int r = 0; r < P; ++r) C[r + P * c] -= A[r] * A[c];
    const double fac = ((n_t[j] - 1) + e * e / Q) / n_t[j];           // :393-401
    for (int q = 0; q < P * P; ++q) C[q] *= fac;
  }
}

// compute_one_step_ahead_prior with G = NULL, SGDLM.cu:115-149.
void orc_prior(int m, int P, const unsigned *p, double *C_t, double *n_t, double *W_t,
               const double *beta, const double *delta) {
  for (int j = 0; j < m; ++j) {
    n_t[j] = n_t[j] * beta[j];  // multiply (kernel_functions.cuh:438-444)
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r) {
        const size_t q = (size_t)j * P * P + r + (size_t)P * c;
        if ((unsigned)r < p[j] && (unsigned)c < p[j]) {  // :259-288, INV branch
          W_t[q] = C_t[q] * (1 / delta[q] - 1.0);
          C_t[q] /= delta[q];
        }
      }
  }
}

// compute_one_step_ahead_prior with an evolution matrix G (SGDLM.cu:116-178): the
// prior above, then a = G m with entries >= p zeroed (batchedCutOffVector,
// kernel_functions.cuh:86-95) and R = G R G' with the entries whose row AND column
// are >= p zeroed (batchedCutOffMatrix :98-110).  W keeps the untransformed
// R - C.
void orc_evo_prior(int m, int P, const unsigned *p, double *m_t, double *C_t, double *n_t,
                   double *W_t, const double *beta, const double *delta, const double *G) {
  orc_prior(m, P, p, C_t, n_t, W_t, beta, delta);
  const size_t PP = (size_t)P * P;
  std::vector<double> mv(P), T(PP);
  for (int j = 0; j < m; ++j) {
    const double *Gj = G + j * PP;
    double *mj = m_t + (size_t)j * P;
    double *Cj = C_t + j * PP;
    for (int l = 0; l < P; ++l) mv[l] = mj[l];
    for (int r = 0; r < P; ++r) {
      double acc = 0.0;
      for (int l = 0; l < P; ++l) acc += Gj[r + (size_t)P * l] * mv[l];
      mj[r] = ((unsigned)r < p[j]) ? acc : 0.0;
    }
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += Gj[r + (size_t)P * l] * Cj[l + (size_t)P * c];
        T[r + (size_t)P * c] = acc;
      }
    for (int c = 0; c < P; ++c)
      for (int r = 0; r < P; ++r) {
        double acc = 0.0;
        for (int l = 0; l < P; ++l) acc += T[r + (size_t)P * l] * Gj[c + (size_t)P * l];
        const bool cut = (unsigned)r >= p[j] && (unsigned)c >= p[j];
        Cj[r + (size_t)P * c] = cut ? 0.0 : acc;
      }
  }
}

// cholesky, kernel_functions.cuh:845-902 (upper U, U'U = C; element (row, col) at
// row + P*col).
void orc_cholesky(int m, int P, const unsigned *p, const double *C, double *U) {
  for (int j = 0; j < m; ++j) {
    const double *Cj = C + (size_t)j * P * P;
    double *a = U + (size_t)j * P * P;
    const int pj = (int)std::min((unsigned)P, p[j]);
    for (int q = 0; q < P * P; ++q) a[q] = 0.0;
    for (int n = 0; n < pj; ++n)
      for (int k = n; k < pj; ++k) a[n + P * k] = Cj[n + P * k];
    for (int n = 0; n < pj; ++n) {
      const double dn = std::sqrt(a[n + P * n]);
      a[n + P * n] = dn;
      const double inv = 1.0 / dn;
      for (int k = n + 1; k < pj; ++k) {
        a[n + P * k] *= inv;
        a[k + P * k] -= a[n + P * k] * a[n + P * k];
      }
      for (int k = n + 1; k < pj; ++k)
        for (int l = k + 1; l < pj; ++l) a[k + P * l] -= a[n + P * k] * a[n + P * l];
    }
  }
}

// sample_lambdas_and_thetas, SGDLM.cu:623-677: lambda ~ Gamma(n/2, rate n s/2)
// (make_gamma2 :569-634), theta = m + U' z / sqrt(s lambda) (gemm :659-662,
// makeVB_MVN :72-83).  Outputs series-major.  Returns the number of capped draws.
long orc_sample(int m, int P, const unsigned *p, const double *m_t, const double *C_t,
                const double *n_t, const double *s_t, long n, uint64_t seed, uint64_t epoch,
                double *lambda, double *theta, int nthreads) {
  const Key key = make_key(seed, epoch);
  std::vector<double> U((size_t)P * P * m);
  orc_cholesky(m, P, p, C_t, U.data());
  long capped = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_eff(nthreads)) reduction(+ : capped)
  for (long i = 0; i < n; ++i) {
    std::vector<double> z(P + 4);
    for (int j = 0; j < m; ++j) {
      bool fail = false;
      const double alpha = 0.5 * n_t[j], rate = 0.5 * n_t[j] * s_t[j];
      const double lam = gamma_mt(alpha, key, (uint32_t)i, (uint32_t)j, TAG_GAMMA, false, &fail) / rate;
      capped += fail ? 1 : 0;
      normals4(key, (uint32_t)i, (uint32_t)j, TAG_THETA, P, z.data());
      const double den = std::sqrt(s_t[j] * lam);
      const double *Uj = U.data() + (size_t)j * P * P;
      for (int k = 0; k < P; ++k) {
        double acc = 0.0;
        for (int l = 0; l <= k; ++l) acc += Uj[l + P * k] * z[l];
        theta[((size_t)j * n + i) * P + k] = m_t[(size_t)j * P + k] + acc / den;
      }
      lambda[(size_t)j * n + i] = lam;
    }
  }
  return capped;
}

// log|det(I - Gamma_i)| of every draw with partial pivoting (getrf, SGDLM.cu:280).
void orc_logdet(int m, int P, const unsigned *sp, long n, const double *theta, double *logdet,
                int nthreads) {
#pragma omp parallel num_threads(nthreads_eff(nthreads))
  {
    std::vector<double> A((size_t)m * m);
    std::vector<int> perm(m);
#pragma omp for schedule(dynamic, 4)
    for (long i = 0; i < n; ++i) {
      build_gamma(m, P, sp, n, i, theta, A.data());
      logdet[i] = lu_pp(m, A.data(), perm.data());
    }
  }
}

// IS weights as the reference forms them: det = exp(sum log|u|), NaN/Inf -> 0
// (detFromLU, kernel_functions.cuh:905-926), serial sum (sumVector :26-39),
// w = det / sum (scale :165-184).  Returns sum.
double orc_weights(long n, const double *logdet, double *w) {
  double sum = 0.0;
  for (long i = 0; i < n; ++i) {
    double d = std::exp(logdet[i]);
    if (std::isnan(d) || std::isinf(d)) d = 0.0;
    w[i] = d;
    sum += d;
  }
  for (long i = 0; i < n; ++i) w[i] /= sum;
  return sum;
}

// The VB refit, SGDLM.cu:341-500, literally: E_w lambda, E_w log lambda,
// m_bar, theta~ = sqrt(lambda)(theta - m_bar), V, cuts, V^-1 by LU inverse,
// Q_ij = theta~' V^-1 theta~ and Q_bar = sum w Q_ij, Newton for n_bar,
// s_bar, C_bar = V s_bar.  aux (m x 3, may be NULL) = {E lambda, E log lambda, Q_bar}.
void orc_vb(int m, int P, const unsigned *p, const double *n_t, const double *s_t, long n,
            const double *w, const double *lambda, const double *theta, double *mean_m,
            double *mean_C, double *mean_n, double *mean_s, double *aux) {
  std::vector<double> tt((size_t)n * P), V((size_t)P * P), LU((size_t)P * P),
      Vinv((size_t)P * P), col(P);
  std::vector<int> perm(P);
  for (int j = 0; j < m; ++j) {
    const unsigned pj = p[j];
    const int pi = (int)std::min((unsigned)P, pj);
    double El = 0.0, Ell = 0.0;  // meanScalarAndLog (kernel_functions.cuh:929-946)
    for (long i = 0; i < n; ++i) {
      El += w[i] * lambda[(size_t)j * n + i];
      Ell += w[i] * std::log(lambda[(size_t)j * n + i]);
    }
    double *mb = mean_m + (size_t)j * P;
    for (int k = 0; k < P; ++k) {  // compute_mean_m_t (:949-967)
      double acc = 0.0;
      for (long i = 0; i < n; ++i)
        acc += w[i] * lambda[(size_t)j * n + i] * theta[((size_t)j * n + i) * P + k];
      mb[k] = acc / El;
    }
    for (long i = 0; i < n; ++i)  // compute_VB_vector1 (:971-982)
      for (int k = 0; k < P; ++k)
        tt[(size_t)i * P + k] =
            std::sqrt(lambda[(size_t)j * n + i]) * (theta[((size_t)j * n + i) * P + k] - mb[k]);
    for (int y = 0; y < P; ++y)  // meanBatchedVecVecT (:1103-1133)
      for (int x = 0; x < P; ++x) {
        double v;
        if (x < pi && y < pi) {
          v = 0.0;
          for (long i = 0; i < n; ++i) v += w[i] * tt[(size_t)i * P + x] * tt[(size_t)i * P + y];
        } else {
          v = (x == y) ? 1.0 : 0.0;
        }
        V[x + P * y] = v;
      }
    for (int k = pi; k < P; ++k) mb[k] = 0.0;  // cut m_bar (SGDLM.cu:387)
    for (int y = 0; y < P; ++y)                // cut V, AND rule (SGDLM.cu:396)
      for (int x = 0; x < P; ++x)
        if (x >= pi && y >= pi) V[x + P * y] = 0.0;
    LU = V;  // C_t_buffer = V; diagonal outside p = 1 (SGDLM.cu:407-419)
    for (int k = pi; k < P; ++k) LU[k + P * k] = 1.0;
    lu_pp(P, LU.data(), perm.data());  // getrf + getri (SGDLM.cu:427-434)
    for (int c = 0; c < P; ++c) {
      for (int r = 0; r < P; ++r) col[r] = (r == c) ? 1.0 : 0.0;
      lu_solve(P, LU.data(), perm.data(), col.data());
      for (int r = 0; r < P; ++r) Vinv[r + P * c] = col[r];
    }
    for (int y = 0; y < P; ++y)  // cut V^-1 (SGDLM.cu:441)
      for (int x = 0; x < P; ++x)
        if (x >= pi && y >= pi) Vinv[x + P * y] = 0.0;
    double Qb = 0.0;  // Q_ij (SGDLM.cu:447-457), mean (compute_mean_Q_t :1088-1100)
    for (long i = 0; i < n; ++i) {
      double q = 0.0;
      for (int y = 0; y < P; ++y) {
        double t = 0.0;
        for (int x = 0; x < P; ++x) t += tt[(size_t)i * P + x] * Vinv[x + P * y];
        q += t * tt[(size_t)i * P + y];
      }
      Qb += w[i] * q;
    }
    // compute_mean_n_t (:1025-1068)
    double mn = n_t[j], fun, dfun, step = 0.0;
    size_t iter = 0;
    const double pd = (double)pj;
    do {
      mn -= step;
      fun = std::log(mn + pd - Qb) - psi_series(mn / 2) - (pd - Qb) / mn - std::log(2 * El) + Ell;
      dfun = 1 / (mn + pd - Qb) - .5 * psi1_series(mn / 2) + (pd - Qb) / (mn * mn);
      step = fun / dfun;
      if (step > mn) step = .5 * mn;
    } while (std::fabs(fun) > 1e-6 && iter++ < 50);
    // iteration cap -> prior shape (kernel_functions.cuh:1062-1066); a non-finite
    // iterate (which the reference would return) is treated the same way
    if (iter >= 50 || !std::isfinite(mn)) mn = n_t[j];
    double sb = (mn + pd - Qb) / (mn * El);  // compute_mean_s_t (:1071-1085)
    if (sb < 0) sb = s_t[j];
    mean_n[j] = mn;
    mean_s[j] = sb;
    double *Cb = mean_C + (size_t)j * P * P;  // batchedScale inside p x p (SGDLM.cu:497-499)
    for (int y = 0; y < P; ++y)
      for (int x = 0; x < P; ++x)
        Cb[x + P * y] = (x < pi && y < pi) ? V[x + P * y] * sb : V[x + P * y];
    if (aux) {
      aux[(size_t)j * 3 + 0] = El;
      aux[(size_t)j * 3 + 1] = Ell;
      aux[(size_t)j * 3 + 2] = Qb;
    }
  }
}

// Forecast solve (SGDLM.cu:538-620): nu_ij = z/sqrt(lambda) + sum_ext x theta
// (batchedComputeNuPlusMu, kernel_functions.cuh:1156-1178), y_i = (I - Gamma_i)^-1 nu_i.
// y is draw-major (m x nsim); nu_out (optional) likewise.
void orc_forecast(int m, int P, const unsigned *sp, long n, const double *lambda,
                  const double *theta, const double *x, uint64_t seed, uint64_t epoch, double *y,
                  double *logdet, int nthreads) {
  const Key key = make_key(seed, epoch);
  const size_t mm = (size_t)m * m;
#pragma omp parallel num_threads(nthreads_eff(nthreads))
  {
    std::vector<double> A((size_t)m * m), b(m);
    std::vector<int> perm(m);
#pragma omp for schedule(dynamic, 4)
    for (long i = 0; i < n; ++i) {
      for (int j = 0; j < m; ++j) {
        const U4 g = draw_block(key, (uint32_t)i, (uint32_t)j, TAG_NU, 0);
        double z0, z1;
        box_muller(g.x, g.y, z0, z1);
        double v = z0 / std::sqrt(lambda[(size_t)j * n + i]);
        for (int k = 0; k < P; ++k)
          if ((size_t)sp[(size_t)j * P + k] >= mm)
            v += x[(size_t)j * P + k] * theta[((size_t)j * n + i) * P + k];
        b[j] = v;
      }
      build_gamma(m, P, sp, n, i, theta, A.data());
      const double ld = lu_pp(m, A.data(), perm.data());
      if (logdet) logdet[i] = ld;
      if (std::isinf(ld)) {
        for (int j = 0; j < m; ++j) y[(size_t)i * m + j] = std::nan("");
        continue;
      }
      lu_solve(m, A.data(), perm.data(), b.data());
      for (int j = 0; j < m; ++j) y[(size_t)i * m + j] = b[j];
    }
  }
}

// evolve_lambdas_and_thetas, SGDLM.cu:679-762 with r_t = forecasting n, c_t =
// forecasting s (HostWrapperImpl.cu:891-900): eta ~ Beta(beta r/2,(1-beta) r/2)/beta,
// lambda *= eta, omega ~ N(0,1) scaled (see compat flags), theta += chol(W)' omega.
// compat bit 1: only draw 0 of series 0 is scaled (reference launch geometry);
// compat bit 2: Marsaglia-Tsang without the boost for shapes below one.
// G (P x P x m, or nullptr): theta = G theta first (SGDLM.cu:729-740, the full
// max_p x max_p product).
long orc_evolve(int m, int P, const unsigned *p, const double *W_t, const double *r_t,
                const double *c_t, const double *beta, const double *G, long n, uint64_t seed,
                uint64_t epoch, unsigned compat, double *lambda, double *theta, int nthreads) {
  const Key key = make_key(seed, epoch);
  std::vector<double> UW((size_t)P * P * m);
  orc_cholesky(m, P, p, W_t, UW.data());
  const bool unscaled = (compat & 1u) != 0, no_boost = (compat & 2u) != 0;
  long capped = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads_eff(nthreads)) reduction(+ : capped)
  for (long i = 0; i < n; ++i) {
    std::vector<double> om(P + 4);
    for (int j = 0; j < m; ++j) {
      bool fail = false;
      double eta = 1.0;
      if (beta[j] != 1.0) {
        const double ga = gamma_mt(0.5 * beta[j] * r_t[j], key, (uint32_t)i, (uint32_t)j,
                                   TAG_BETA_A, no_boost, &fail);
        const double gb = gamma_mt(0.5 * (1.0 - beta[j]) * r_t[j], key, (uint32_t)i,
                                   (uint32_t)j, TAG_BETA_B, no_boost, &fail);
        eta = (ga / (ga + gb)) / beta[j];
      }
      capped += fail ? 1 : 0;
      const double lam = lambda[(size_t)j * n + i] * eta;
      lambda[(size_t)j * n + i] = lam;
      normals4(key, (uint32_t)i, (uint32_t)j, TAG_OMEGA, P, om.data());
      if (!unscaled || (i == 0 && j == 0)) {
        const double den = std::sqrt(c_t[j] * lam);
        for (int k = 0; k < P; ++k) om[k] = ((unsigned)k < p[j]) ? om[k] / den : 0.0;
      }
      double *th = theta + ((size_t)j * n + i) * P;
      if (G) {
        const double *Gj = G + (size_t)j * P * P;
        std::vector<double> old(th, th + P);
        for (int k = 0; k < P; ++k) {
          double acc = 0.0;
          for (int l = 0; l < P; ++l) acc += Gj[k + (size_t)P * l] * old[l];
          th[k] = acc;
        }
      }
      const double *U = UW.data() + (size_t)j * P * P;
      for (int k = 0; k < P; ++k) {
        double acc = 0.0;
        for (int l = 0; l <= k; ++l) acc += U[l + P * k] * om[l];
        th[k] += acc;
      }
    }
  }
  return capped;
}

}  // extern "C"
