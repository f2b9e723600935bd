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
  // current pattern: row r -> (col -> slot), col c -> (row -> slot)
  std::vector<std::map<int, int>> rows(m), cols(m);
  std::vector<int> diag(m);
  for (int r = 0; r < m; ++r) diag[r] = (int)kSlotDiag0 + r;
  int nv = (int)kSlotDiag0 + m;
  for (int e = 0; e < m * P; ++e) {
    const unsigned pos = sp[e];
    if ((size_t)pos >= mm) continue;
    const int r = (int)(pos % (unsigned)m), c = (int)(pos / (unsigned)m);
    rows[r][c] = nv;
    cols[c][r] = nv;
    pl.l0_e.push_back(e);
    ++nv;
  }
  pl.lev_piv.push_back(0);
  pl.lev_scale.push_back(0);
  pl.lev_chunk.push_back(0);
  pl.chunk_tofs.push_back(0);
  pl.lev_fwd_nodes.push_back(0);
  pl.fwd_ptr.push_back(0);
  pl.lev_bwd_nodes.push_back(0);
  pl.bwd_ptr.push_back(0);
  std::vector<char> active(m, 1);
  int n_active = m;
  // slot indices and node numbers are stored in 16 bits
  if (nv > kMaxSlots || m > 0xFFFF) max_levels = 0;

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
    auto keep = [&](int v) { return active[v] && !inS[v]; };
    // terms of the updated entries, in a deterministic order
    std::map<std::pair<int, int>, std::vector<unsigned>> acc;
    for (int t : S)
      for (auto &rq : cols[t]) {
        if (!keep(rq.first)) continue;
        for (auto &cq : rows[t])
          if (keep(cq.first))
            acc[{rq.first, cq.first}].push_back(pack16((unsigned)rq.second, (unsigned)cq.second));
      }
    int fill = 0;
    for (auto &kv : acc) {
      const int r = kv.first.first, c = kv.first.second;
      if (r != c && !rows[r].count(c)) ++fill;
    }
    if (nv + fill > kMaxSlots) break;  // the slots would not fit 16 bits

    for (int t : S) pl.piv.push_back(diag[t]);
    for (int t : S)
      for (auto &rq : cols[t])
        if (keep(rq.first)) pl.scale.push_back(pack16((unsigned)rq.second, (unsigned)diag[t]));
    // forward program, grouped by the updated node
    std::map<int, std::vector<unsigned>> fwd_by_row;
    for (int t : S)
      for (auto &rq : cols[t])
        if (keep(rq.first)) fwd_by_row[rq.first].push_back(pack16((unsigned)rq.second, (unsigned)t));
    for (auto &kv : fwd_by_row) {
      pl.fwd_node.push_back(kv.first);
      for (unsigned f : kv.second) pl.fwd.push_back(f);
      pl.fwd_ptr.push_back((int)pl.fwd.size());
    }
    for (int t : S) {
      pl.bwd_node.push_back(t);
      pl.bwd_diag.push_back(diag[t]);
      for (auto &cq : rows[t])
        if (keep(cq.first)) pl.bwd.push_back(pack16((unsigned)cq.second, (unsigned)cq.first));
      pl.bwd_ptr.push_back((int)pl.bwd.size());
    }
    // entries: updated in place, or a fresh slot for fill-in (base = constant 0)
    struct Entry {
      unsigned out, base;
      const std::vector<unsigned> *terms;
    };
    std::vector<Entry> ents;
    ents.reserve(acc.size());
    for (auto &kv : acc) {
      const int r = kv.first.first, c = kv.first.second;
      int slot;
      unsigned base;
      if (r == c) {
        slot = diag[r];
        base = (unsigned)slot;
      } else {
        auto it = rows[r].find(c);
        if (it != rows[r].end()) {
          slot = it->second;
          base = (unsigned)slot;
        } else {
          slot = nv++;
          base = kSlotZero;
          rows[r][c] = slot;
          cols[c][r] = slot;
        }
      }
      ents.push_back(Entry{(unsigned)slot, base, &kv.second});
      pl.n_terms += kv.second.size();
    }
    // chunks of 32 lanes with similar term counts
    std::stable_sort(ents.begin(), ents.end(), [](const Entry &a, const Entry &b) {
      return a.terms->size() > b.terms->size();
    });
    for (size_t c0 = 0; c0 < ents.size(); c0 += 32) {
      size_t K = 0;
      for (size_t l = 0; l < 32 && c0 + l < ents.size(); ++l) K = std::max(K, ents[c0 + l].terms->size());
      const size_t tofs = pl.terms.size();
      pl.terms.resize(tofs + 32 * K, pack16(kSlotZero, kSlotZero));
      for (size_t l = 0; l < 32; ++l) {
        if (c0 + l < ents.size()) {
          const Entry &e = ents[c0 + l];
          pl.ent.push_back(pack16(e.out, e.base));
          for (size_t k = 0; k < e.terms->size(); ++k) pl.terms[tofs + 32 * k + l] = (*e.terms)[k];
        } else {
          pl.ent.push_back(pack16(kSlotNone, kSlotZero));
        }
      }
      pl.chunk_tofs.push_back((int)pl.terms.size());
    }
    for (int t : S) {
      active[t] = 0;
      --n_active;
    }
    pl.lev_piv.push_back((int)pl.piv.size());
    pl.lev_scale.push_back((int)pl.scale.size());
    pl.lev_chunk.push_back((int)pl.chunk_tofs.size() - 1);
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
  pl.dp = std::max(32, (pl.core_n + 31) / 32 * 32);
  // renumber the slots: the constants, then the values the solve programs read,
  // then the rest (so that a solve needs only a prefix of the slot array)
  std::vector<int> remap(nv, -1);
  int next = 0;
  remap[kSlotZero] = next++;
  remap[kSlotOne] = next++;
  auto take = [&](int slot) {
    if (remap[slot] < 0) remap[slot] = next++;
  };
  for (unsigned f : pl.fwd) take((int)(f & 0xFFFFu));
  for (unsigned b : pl.bwd) take((int)(b & 0xFFFFu));
  for (int d : pl.bwd_diag) take(d);
  pl.n_solve = next;
  for (int v = 0; v < nv; ++v) take(v);
  auto lo_map = [&](unsigned w) { return pack16((unsigned)remap[w & 0xFFFFu], w >> 16); };
  auto both_map = [&](unsigned w) {
    return pack16((unsigned)remap[w & 0xFFFFu], (unsigned)remap[w >> 16]);
  };
  pl.diag_slot.resize(m);
  for (int r = 0; r < m; ++r) pl.diag_slot[r] = remap[(int)kSlotDiag0 + r];
  pl.l0_slot.resize(pl.l0_e.size());
  for (size_t k = 0; k < pl.l0_e.size(); ++k) pl.l0_slot[k] = remap[(int)kSlotDiag0 + m + (int)k];
  for (int &v : pl.piv) v = remap[v];
  for (unsigned &w : pl.scale) w = both_map(w);
  for (unsigned &w : pl.ent) {
    const unsigned out = w & 0xFFFFu;
    w = pack16(out == kSlotNone ? kSlotNone : (unsigned)remap[out], (unsigned)remap[w >> 16]);
  }
  for (unsigned &w : pl.terms) w = both_map(w);
  for (unsigned &w : pl.fwd) w = lo_map(w);
  for (unsigned &w : pl.bwd) w = lo_map(w);
  for (int &v : pl.bwd_diag) v = remap[v];
  for (int &v : diag) v = remap[v];
  for (int r = 0; r < m; ++r)
    for (auto &kv : rows[r]) kv.second = remap[kv.second];
  if (pl.nlev > 0) {
    const size_t dp = (size_t)pl.dp;
    pl.core_map.assign(dp * dp, (uint16_t)kSlotZero);
    for (int r : pl.core_node) {
      const int pr = pl.node_core[r];
      pl.core_map[pr + dp * pr] = (uint16_t)diag[r];
      for (auto &cq : rows[r])
        if (active[cq.first]) pl.core_map[pr + dp * pl.node_core[cq.first]] = (uint16_t)cq.second;
    }
    for (size_t pr = pl.core_n; pr < dp; ++pr) pl.core_map[pr + dp * pr] = (uint16_t)kSlotOne;
  }
  return pl;
}

}  // namespace sgdlm
