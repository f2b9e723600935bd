// Test harness: evaluates the product's sparse pre-elimination plan
// (gpusgdlm_gb300/csrc/elimination.cu) in FP64 on the host, so that the planner
// can be checked against a dense factorisation without a GPU.
#include <cmath>
#include <vector>

#include "../gpusgdlm_gb300/csrc/elimination.cu"

extern "C" int elim_check(int m, int P, const unsigned *sp, const double *theta_e, int max_levels,
                          const double *rhs, double *sol, double *info) {
  std::vector<unsigned> spv(sp, sp + (size_t)m * P);
  const sgdlm::EliminationPlanHost pl = sgdlm::plan_elimination(m, P, spv, max_levels);
  std::vector<double> v(pl.nv, 0.0);
  for (int r = 0; r < m; ++r) v[r] = 1.0;
  for (size_t k = 0; k < pl.l0_e.size(); ++k) v[m + k] = -theta_e[pl.l0_e[k]];
  double ld = 0.0;
  std::vector<double> z(rhs, rhs + m);
  for (int lev = 0; lev < pl.nlev; ++lev) {
    for (int q = pl.lev_entry[lev]; q < pl.lev_entry[lev + 1]; ++q) {
      double x = pl.ent_base[q] >= 0 ? v[pl.ent_base[q]] : 0.0;
      for (int t = pl.ent_tptr[q]; t < pl.ent_tptr[q + 1]; ++t)
        x -= v[pl.terms[t].x] / v[pl.terms[t].z] * v[pl.terms[t].y];
      v[pl.ent_out[q]] = x;
    }
    for (int q = pl.lev_piv[lev]; q < pl.lev_piv[lev + 1]; ++q) ld += std::log(std::fabs(v[pl.piv[q]]));
    for (int g = pl.lev_fwd_nodes[lev]; g < pl.lev_fwd_nodes[lev + 1]; ++g) {
      double acc = z[pl.fwd_node[g]];
      for (int q = pl.fwd_ptr[g]; q < pl.fwd_ptr[g + 1]; ++q)
        acc -= v[pl.fwd[q].x] / v[pl.fwd[q].z] * z[pl.fwd[q].y];
      z[pl.fwd_node[g]] = acc;
    }
  }
  const int n = pl.core_n;
  std::vector<double> A((size_t)n * n, 0.0), b(n);
  for (const int3 &ce : pl.core_ent) A[ce.y + (size_t)n * ce.z] = v[ce.x];
  for (int r = 0; r < n; ++r) b[r] = z[pl.core_node[r]];
  // dense partial-pivoting LU and solve of the core
  std::vector<int> perm(n);
  for (int r = 0; r < n; ++r) perm[r] = r;
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int r = k + 1; r < n; ++r)
      if (std::fabs(A[r + (size_t)n * k]) > std::fabs(A[p + (size_t)n * k])) p = r;
    if (p != k) {
      for (int c = 0; c < n; ++c) std::swap(A[k + (size_t)n * c], A[p + (size_t)n * c]);
      std::swap(b[k], b[p]);
    }
    ld += std::log(std::fabs(A[k + (size_t)n * k]));
    for (int r = k + 1; r < n; ++r) {
      const double l = A[r + (size_t)n * k] / A[k + (size_t)n * k];
      A[r + (size_t)n * k] = l;
      for (int c = k + 1; c < n; ++c) A[r + (size_t)n * c] -= l * A[k + (size_t)n * c];
      b[r] -= l * b[k];
    }
  }
  for (int k = n - 1; k >= 0; --k) {
    for (int c = k + 1; c < n; ++c) b[k] -= A[k + (size_t)n * c] * b[c];
    b[k] /= A[k + (size_t)n * k];
  }
  std::vector<double> y(m, 0.0);
  for (int r = 0; r < n; ++r) y[pl.core_node[r]] = b[r];
  for (int lev = pl.nlev - 1; lev >= 0; --lev)
    for (int g = pl.lev_bwd_nodes[lev]; g < pl.lev_bwd_nodes[lev + 1]; ++g) {
      double acc = z[pl.bwd_node[g]];
      for (int q = pl.bwd_ptr[g]; q < pl.bwd_ptr[g + 1]; ++q) acc -= v[pl.bwd[q].x] * y[pl.bwd[q].y];
      y[pl.bwd_node[g]] = acc / v[pl.bwd_diag[g]];
    }
  for (int r = 0; r < m; ++r) sol[r] = y[r];
  info[0] = ld;
  info[1] = n;
  info[2] = pl.nlev;
  info[3] = (double)pl.terms.size();
  return 0;
}
