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
  v[sgdlm::kSlotOne] = 1.0;
  for (int r = 0; r < m; ++r) v[pl.diag_slot[r]] = 1.0;
  for (size_t k = 0; k < pl.l0_e.size(); ++k) v[pl.l0_slot[k]] = -theta_e[pl.l0_e[k]];
  auto lo = [](unsigned w) { return (int)(w & 0xFFFFu); };
  auto hi = [](unsigned w) { return (int)(w >> 16); };
  double ld = 0.0;
  std::vector<double> z(rhs, rhs + m);
  for (int lev = 0; lev < pl.nlev; ++lev) {
    for (int q = pl.lev_piv[lev]; q < pl.lev_piv[lev + 1]; ++q) ld += std::log(std::fabs(v[pl.piv[q]]));
    for (int q = pl.lev_scale[lev]; q < pl.lev_scale[lev + 1]; ++q)
      v[lo(pl.scale[q])] /= v[hi(pl.scale[q])];
    // all entries of a level read values of the previous state only
    std::vector<std::pair<int, double>> out;
    for (int c = pl.lev_chunk[lev]; c < pl.lev_chunk[lev + 1]; ++c) {
      const int K = (pl.chunk_tofs[c + 1] - pl.chunk_tofs[c]) / 32;
      for (int l = 0; l < 32; ++l) {
        const unsigned e = pl.ent[(size_t)c * 32 + l];
        double x = v[hi(e)];
        for (int k = 0; k < K; ++k) {
          const unsigned t = pl.terms[pl.chunk_tofs[c] + 32 * k + l];
          x -= v[lo(t)] * v[hi(t)];
        }
        if ((unsigned)lo(e) != sgdlm::kSlotNone) out.emplace_back(lo(e), x);
      }
    }
    for (auto &o : out) v[o.first] = o.second;
    for (int g = pl.lev_fwd_nodes[lev]; g < pl.lev_fwd_nodes[lev + 1]; ++g) {
      double acc = z[pl.fwd_node[g]];
      for (int q = pl.fwd_ptr[g]; q < pl.fwd_ptr[g + 1]; ++q) acc -= v[lo(pl.fwd[q])] * z[hi(pl.fwd[q])];
      z[pl.fwd_node[g]] = acc;
    }
  }
  const int n = pl.core_n;
  std::vector<double> A((size_t)n * n, 0.0), b(n);
  if (pl.nlev > 0) {
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) A[r + (size_t)n * c] = v[pl.core_map[r + (size_t)pl.dp * c]];
  } else {
    for (int r = 0; r < m; ++r) A[r + (size_t)n * r] = 1.0;
    for (int e = 0; e < m * P; ++e)
      if ((size_t)sp[e] < (size_t)m * m) A[sp[e] % m + (size_t)n * (sp[e] / m)] = -theta_e[e];
  }
  for (int r = 0; r < n; ++r) b[r] = z[pl.core_node[r]];
  // dense partial-pivoting LU and solve of the core
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
      for (int q = pl.bwd_ptr[g]; q < pl.bwd_ptr[g + 1]; ++q) acc -= v[lo(pl.bwd[q])] * y[hi(pl.bwd[q])];
      y[pl.bwd_node[g]] = acc / v[pl.bwd_diag[g]];
    }
  for (int r = 0; r < m; ++r) sol[r] = y[r];
  // the solve programs read only the prefix [0, n_solve) of the slots
  bool prefix_ok = true;
  for (unsigned f : pl.fwd) prefix_ok &= (int)lo(f) < pl.n_solve;
  for (unsigned b : pl.bwd) prefix_ok &= (int)lo(b) < pl.n_solve;
  for (int d : pl.bwd_diag) prefix_ok &= d < pl.n_solve;
  if (!prefix_ok) info[1] = -1;
  info[0] = ld;
  if (info[1] != -1) info[1] = n;
  info[2] = pl.nlev;
  info[3] = (double)pl.n_terms;
  return 0;
}
