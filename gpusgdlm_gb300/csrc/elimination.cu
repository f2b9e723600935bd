// Host-side planning of the sparse pre-elimination (see elimination.hpp).
#include <algorithm>
#include <map>
#include <utility>

#include "elimination.hpp"

namespace sgdlm {

namespace {
// Stop when a level would eliminate fewer than this share of the active nodes.
constexpr double kMinLevelShare = 0.05;
}  // namespace

EliminationPlanHost plan_elimination(int m, int P, const std::vector<unsigned> &sp,
                                     int max_levels) {
  EliminationPlanHost pl;
  pl.m = m;
  pl.P = P;
  const size_t mm = (size_t)m * m;
  // current pattern: row r -> (col -> vals index), col c -> (row -> vals index)
  std::vector<std::map<int, int>> rows(m), cols(m);
  std::vector<int> diag(m);
  for (int r = 0; r < m; ++r) diag[r] = r;
  int nv = m;
  for (int e = 0; e < m * P; ++e) {
    const unsigned pos = sp[e];
    if ((size_t)pos >= mm) continue;
    const int r = (int)(pos % (unsigned)m), c = (int)(pos / (unsigned)m);
    rows[r][c] = nv;
    cols[c][r] = nv;
    pl.l0_e.push_back(e);
    ++nv;
  }
  std::vector<char> active(m, 1);
  int n_active = m;
  pl.lev_entry.push_back(0);
  pl.ent_tptr.push_back(0);
  pl.lev_piv.push_back(0);
  pl.lev_fwd_nodes.push_back(0);
  pl.fwd_ptr.push_back(0);
  pl.lev_bwd_nodes.push_back(0);
  pl.bwd_ptr.push_back(0);

  for (int lev = 0; lev < max_levels; ++lev) {
    // greedy independent set, ascending degree in the symmetrised active graph
    std::vector<std::pair<int, int>> order;
    order.reserve(n_active);
    for (int r = 0; r < m; ++r) {
      if (!active[r]) continue;
      int d = 0;
      for (auto &kv : rows[r]) d += active[kv.first] ? 1 : 0;
      for (auto &kv : cols[r]) d += active[kv.first] ? 1 : 0;
      order.emplace_back(d, r);
    }
    std::sort(order.begin(), order.end());
    std::vector<char> blocked(m, 0), inS(m, 0);
    std::vector<int> S;
    for (auto &dr : order) {
      const int r = dr.second;
      if (blocked[r]) continue;
      S.push_back(r);
      inS[r] = 1;
      blocked[r] = 1;
      for (auto &kv : rows[r]) blocked[kv.first] = 1;
      for (auto &kv : cols[r]) blocked[kv.first] = 1;
    }
    if ((int)S.size() == n_active) S.pop_back();  // keep a non-empty dense core
    if (S.empty() || (double)S.size() < kMinLevelShare * n_active) break;
    std::sort(S.begin(), S.end());
    // terms of the new entries, in a deterministic order
    std::map<std::pair<int, int>, std::vector<int3>> acc;
    for (int t : S) {
      for (auto &rq : cols[t]) {
        const int r = rq.first;
        if (!active[r] || inS[r]) continue;
        for (auto &cq : rows[t]) {
          const int c = cq.first;
          if (!active[c] || inS[c]) continue;
          acc[{r, c}].push_back(make_int3(rq.second, cq.second, diag[t]));
        }
      }
    }
    // forward and backward solve programs use this level's values
    std::map<int, std::vector<int3>> fwd_by_row;
    for (int t : S)
      for (auto &rq : cols[t])
        if (active[rq.first] && !inS[rq.first])
          fwd_by_row[rq.first].push_back(make_int3(rq.second, t, diag[t]));
    for (auto &kv : fwd_by_row) {
      pl.fwd_node.push_back(kv.first);
      for (const int3 &f : kv.second) pl.fwd.push_back(f);
      pl.fwd_ptr.push_back((int)pl.fwd.size());
    }
    for (int t : S) {
      pl.piv.push_back(diag[t]);
      pl.bwd_node.push_back(t);
      pl.bwd_diag.push_back(diag[t]);
      for (auto &cq : rows[t])
        if (active[cq.first] && !inS[cq.first]) pl.bwd.push_back(make_int2(cq.second, cq.first));
      pl.bwd_ptr.push_back((int)pl.bwd.size());
    }
    for (auto &kv : acc) {
      const int r = kv.first.first, c = kv.first.second;
      int base;
      if (r == c) {
        base = diag[r];
      } else {
        auto it = rows[r].find(c);
        base = (it == rows[r].end()) ? -1 : it->second;
      }
      const int q = nv++;
      pl.ent_out.push_back(q);
      pl.ent_base.push_back(base);
      for (const int3 &tm : kv.second) pl.terms.push_back(tm);
      pl.ent_tptr.push_back((int)pl.terms.size());
      if (r == c) {
        diag[r] = q;
      } else {
        rows[r][c] = q;
        cols[c][r] = q;
      }
    }
    for (int t : S) {
      active[t] = 0;
      --n_active;
    }
    pl.lev_entry.push_back((int)pl.ent_out.size());
    pl.lev_piv.push_back((int)pl.piv.size());
    pl.lev_fwd_nodes.push_back((int)pl.fwd_node.size());
    pl.lev_bwd_nodes.push_back((int)pl.bwd_node.size());
    ++pl.nlev;
  }
  pl.nv = nv;
  pl.node_core.assign(m, -1);
  for (int r = 0; r < m; ++r)
    if (active[r]) {
      pl.node_core[r] = (int)pl.core_node.size();
      pl.core_node.push_back(r);
    }
  pl.core_n = (int)pl.core_node.size();
  for (int r : pl.core_node) {
    const int pr = pl.node_core[r];
    pl.core_ent.push_back(make_int3(diag[r], pr, pr));
    for (auto &cq : rows[r])
      if (active[cq.first]) pl.core_ent.push_back(make_int3(cq.second, pr, pl.node_core[cq.first]));
  }
  return pl;
}

}  // namespace sgdlm
