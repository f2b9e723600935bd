// Sparse pre-elimination of (I - Gamma) before the dense LU.
//
// (I - Gamma) has a unit diagonal and at most max_p off-diagonal entries per
// row, at the same positions for every draw.  Once per parental-set change the
// host plans a sequence of elimination levels: at each level it picks a greedy
// independent set S of the current sparsity graph (no edge between two members
// of S, so the S x S block is diagonal) and eliminates it,
//   M'[r][c] = M[r][c] - sum_{t in S} M[r][t] M[t][c] / M[t][t],
//   log|det M| = sum_{t in S} log|M[t][t]| + log|det M'|.
// This is a symmetric permutation plus exact block elimination, so |det| is
// unchanged; what is left (the "core") goes to the blocked dense LU.  At m = 400
// with ~8.5 parents per series two levels shrink the dense core from 400 to
// about 260 nodes.
//
// The plan is a small program over a per-draw value array `vals`:
//   vals[0 .. m)          diagonal of (I - Gamma) = 1
//   vals[m .. m + nnz0)   off-diagonal entries, -theta[e]   (e = j*max_p + k)
//   then the entries each level creates (in level order).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace sgdlm {

struct EliminationPlanHost {
  int m = 0, P = 0;
  int nlev = 0;
  int nv = 0;                      // values per draw
  std::vector<int> l0_e;           // nnz0 theta indices of the level-0 entries
  std::vector<int> lev_entry;      // nlev+1 offsets into entries (computed entries per level)
  std::vector<int> ent_out;        // vals index written by computed entry
  std::vector<int> ent_base;       // vals index of M[r][c] at the previous level, or -1
  std::vector<int> ent_tptr;       // term ranges, size #entries + 1
  std::vector<int3> terms;         // (M[r][t], M[t][c], M[t][t]) vals indices
  std::vector<int> lev_piv;        // nlev+1 offsets into piv
  std::vector<int> piv;            // vals index of M[t][t] of eliminated nodes
  // forward (RHS) program, grouped by the updated node r:
  //   z[r] -= sum_t M[r][t] / M[t][t] * z[t]
  std::vector<int> lev_fwd_nodes;  // nlev+1 offsets into fwd_node
  std::vector<int> fwd_node;       // r
  std::vector<int> fwd_ptr;        // term ranges per node (size #nodes + 1)
  std::vector<int3> fwd;           // (vals M[r][t], t, vals M[t][t])
  // backward program: y[t] = (z[t] - sum M[t][c] y[c]) / M[t][t]
  std::vector<int> lev_bwd_nodes;  // nlev+1 offsets into bwd_node
  std::vector<int> bwd_node;       // t
  std::vector<int> bwd_diag;       // vals M[t][t]
  std::vector<int> bwd_ptr;        // term ranges per node (size #nodes + 1)
  std::vector<int2> bwd;           // (vals M[t][c], c)
  // dense core
  int core_n = 0;
  std::vector<int> core_node;      // core position -> node
  std::vector<int> node_core;      // node -> core position or -1
  std::vector<int3> core_ent;      // (vals index, core row, core col), off-diagonal + diagonal
};

// Device copy of the plan (pointers into one allocation owned by the engine).
struct EliminationPlan {
  int m, P, nlev, nv, nnz0, core_n, n_core_ent;
  const int *l0_e;
  const int *lev_entry, *ent_out, *ent_base, *ent_tptr;
  const int3 *terms;
  const int *lev_piv, *piv;
  const int *lev_fwd_nodes, *fwd_node, *fwd_ptr;
  const int3 *fwd;
  const int *lev_bwd_nodes, *bwd_node, *bwd_diag, *bwd_ptr;
  const int2 *bwd;
  const int *core_node;
  const int3 *core_ent;
};

// Builds the plan from the parental sets (sp: max_p x m, entries < m*m address
// (I - Gamma) at row + m*col).  max_levels = 0 gives the plain dense LU of the
// whole matrix.
EliminationPlanHost plan_elimination(int m, int P, const std::vector<unsigned> &sp,
                                     int max_levels);

}  // namespace sgdlm
