// Sparse pre-elimination of (I - Gamma) before the dense LU.
//
// (I - Gamma) has a unit diagonal and at most max_p off-diagonal entries per
// row, at the same positions for every draw.  Once per parental-set change the
// host plans a sequence of elimination levels: at each level it picks a greedy
// independent set S of the current sparsity graph (no edge between two members
// of S, so the S x S block is diagonal) and eliminates it,
//   L[r][t]  = M[r][t] / M[t][t]                       (t in S, r not in S)
//   M'[r][c] = M[r][c] - sum_{t in S} L[r][t] M[t][c],
//   log|det M| = sum_{t in S} log|M[t][t]| + log|det M'|.
// This is a symmetric permutation plus exact block elimination, so |det| is
// unchanged; what is left (the "core") goes to the dense LU.  At m = 400 with
// ~8.5 parents per series four levels shrink the dense core from 400 to about
// 210 nodes.
//
// The plan is a small program over a per-draw array of value slots `vals`.
// Every matrix position owns one slot for its whole life: an entry that a level
// updates is overwritten in place, a fill-in entry gets a fresh slot, and a
// multiplier L[r][t] replaces M[r][t] in its slot.  Slot indices fit 16 bits.
//   slot 0             constant 0 (padding terms read it; never written)
//   slot 1             constant 1 (identity padding of the dense core)
//   slots 2 .. n_solve the values the forward / backward solve programs read
//                      (rows, columns and pivots of the eliminated nodes)
//   then everything else.
// Initial values: vals[diag_slot[r]] = 1, vals[l0_slot[k]] = -theta[l0_e[k]].
// A level runs as: pivots and multipliers (scale), barrier, new entries,
// barrier.  Entries are grouped in chunks of 32 (one per warp lane), sorted by
// term count so that a chunk's lanes do the same number of terms; a chunk's
// terms are stored term-major (term k of lane l at chunk_tofs + 32 k + l) so
// that each load of the program is one coalesced 128-byte line.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace sgdlm {

constexpr unsigned kSlotZero = 0, kSlotOne = 1, kSlotDiag0 = 2;
constexpr unsigned kSlotNone = 0xFFFFu;  // padding lane of a chunk: no store
constexpr int kMaxSlots = 0xFFFF;        // slots 0 .. 0xFFFE

inline unsigned pack16(unsigned lo, unsigned hi) { return (lo & 0xFFFFu) | (hi << 16); }

struct EliminationPlanHost {
  int m = 0, P = 0;
  int nlev = 0;
  int nv = 0;                        // slots per draw
  int n_solve = 2;                   // slots [0, n_solve) hold what the solves read
  std::vector<int> diag_slot;        // m initial diagonal slots (value 1)
  std::vector<int> l0_e;             // theta index e (j*max_p + k) of level-0 entry
  std::vector<int> l0_slot;          // its slot (value -theta[e])
  // per level (nlev + 1 offsets each)
  std::vector<int> lev_piv;          // -> piv
  std::vector<int> piv;              // slot of M[t][t] of the eliminated nodes
  std::vector<int> lev_scale;        // -> scale
  std::vector<unsigned> scale;       // (slot M[r][t] | slot M[t][t] << 16): M[r][t] /= M[t][t]
  std::vector<int> lev_chunk;        // -> chunks
  std::vector<int> chunk_tofs;       // #chunks + 1 offsets into terms (multiples of 32)
  std::vector<unsigned> ent;         // 32 per chunk: (out slot | base slot << 16)
  std::vector<unsigned> terms;       // (slot L[r][t] | slot M[t][c] << 16)
  // forward (right-hand side) program, grouped by the updated node r:
  //   z[r] -= sum_t L[r][t] z[t]
  std::vector<int> lev_fwd_nodes;    // -> fwd_node
  std::vector<int> fwd_node;         // r
  std::vector<int> fwd_ptr;          // term ranges per node (size #nodes + 1)
  std::vector<unsigned> fwd;         // (slot L[r][t] | t << 16)
  // backward program: y[t] = (z[t] - sum_c M[t][c] y[c]) / M[t][t]
  std::vector<int> lev_bwd_nodes;    // -> bwd_node
  std::vector<int> bwd_node;         // t
  std::vector<int> bwd_diag;         // slot M[t][t]
  std::vector<int> bwd_ptr;          // term ranges per node (size #nodes + 1)
  std::vector<unsigned> bwd;         // (slot M[t][c] | c << 16)
  // dense core
  int core_n = 0;
  int dp = 0;                        // core_n rounded up to 32
  std::vector<int> core_node;        // core position -> node
  std::vector<int> node_core;        // node -> core position or -1
  std::vector<uint16_t> core_map;    // dp x dp (column-major) slot of each core cell
  size_t n_terms = 0;                // unpadded term count (for reporting)
};

// Device copy of the plan (pointers into one allocation owned by the engine).
// core_map == nullptr means "no plan": the whole matrix is the dense core.
struct EliminationPlan {
  int m, P, nlev, nv, n_solve, nnz0, core_n;
  const int *diag_slot, *l0_e, *l0_slot;
  const int *lev_piv, *piv;
  const int *lev_scale;
  const unsigned *scale;
  const int *lev_chunk, *chunk_tofs;
  const unsigned *ent, *terms;
  const int *lev_fwd_nodes, *fwd_node, *fwd_ptr;
  const unsigned *fwd;
  const int *lev_bwd_nodes, *bwd_node, *bwd_diag, *bwd_ptr;
  const unsigned *bwd;
  const int *core_node;
  const uint16_t *core_map;
  // the solve programs (lev_fwd_nodes .. bwd) are one contiguous, 16-byte aligned
  // run of prog_len ints starting at prog, so that a kernel can stage them
  const int *prog;
  int prog_len;
};

// Builds the plan from the parental sets (sp: max_p x m, entries < m*m address
// (I - Gamma) at row + m*col).  max_levels = 0, or parental sets with more than
// kMaxSlots values, give no levels (the plain dense LU of the whole matrix).
EliminationPlanHost plan_elimination(int m, int P, const std::vector<unsigned> &sp,
                                     int max_levels);

}  // namespace sgdlm
