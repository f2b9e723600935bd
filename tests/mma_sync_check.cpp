// Host model of a CTA's MMA completion waits (tests/test_mma_sync.py): the
// barrier, the issuing thread and the polling threads, run with the rules the
// tensor-core LU kernel uses (gpusgdlm_gb300/csrc/mma_sync.hpp).
//
// Time is counted in polls.  Tile c's MMAs are committed when the CTA starts the
// tile (if it still issues); the barrier completes commits in order, commit c at
// max(issue time + delay[c], completion of commit c - 1); delay < 0: never.
// Thread t starts polling jitter[t] after the issue, and the CTA passes a
// barrier when its slowest thread is done.  A wait that reports its tile's
// results valid while the tile's commit has not completed is a violation.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../gpusgdlm_gb300/csrc/mma_sync.hpp"

using namespace sgdlm;

namespace {
constexpr long kNever = -1;
}

extern "C" int mma_model_run(int tiles, const long *delay, int nthreads, const long *jitter,
                             long first_polls, long drain_polls, int legacy_rule,
                             int *status /* tiles x nthreads */, int *issued /* tiles */,
                             int *bad_out /* tiles x nthreads */) {
  std::vector<long> done_at;  // completion time of each issued commit (kNever: never)
  std::vector<uint32_t> phase(nthreads, 0u);
  int dead = 0;
  long now = 0;
  int violations = 0;
  for (int c = 0; c < tiles; ++c) {
    const bool live = dead == 0;  // thread 0 reads the flag before issuing
    issued[c] = live ? 1 : 0;
    int commit = -1;
    if (live) {
      commit = (int)done_at.size();
      long t = delay[c] < 0 ? kNever : now + delay[c];
      if (t != kNever && !done_at.empty()) {
        const long prev = done_at.back();
        t = (prev == kNever) ? kNever : std::max(t, prev);
      }
      done_at.push_back(t);
    }
    // completed phases of the barrier at time tau
    auto completed = [&](long tau) {
      uint32_t k = 0;
      for (long d : done_at) {
        if (d == kNever || d > tau) break;
        ++k;
      }
      return k;
    };
    long finish = now;
    int dead_seen = dead;  // the flag as the threads read it (visible after the last barrier)
    int dead_set = 0;
    for (int t = 0; t < nthreads; ++t) {
      bool bad = false;
      long tau = now + jitter[t];
      bool first = false, drained = false;
      if (!dead_seen) {
        for (long i = 0; i < first_polls && !first; ++i, ++tau)
          first = mbar_phase_done(completed(tau), phase[t]);
        if (!first && !legacy_rule)
          for (long i = 0; i < drain_polls && !drained; ++i, ++tau)
            drained = mbar_phase_done(completed(tau), phase[t]);
      }
      int r;
      if (legacy_rule) {
        // the rule this model guards against: flip the phase on a timeout and go on
        if (dead_seen) {
          bad = true;
          r = kMmaSkipped;
        } else {
          if (!first) bad = true;
          phase[t] ^= 1u;
          r = first ? kMmaDone : kMmaLost;
        }
      } else {
        r = mma_wait_rule(dead_seen != 0, first, drained, phase[t], bad);
        if (r == kMmaLost) dead_set = 1;
      }
      status[c * nthreads + t] = r;
      bad_out[c * nthreads + t] = bad ? 1 : 0;
      // a wait that hands out results (no bad mark) must see its own commit done
      if (!bad) {
        const bool ok = commit >= 0 && done_at[commit] != kNever && done_at[commit] <= tau;
        if (!ok) ++violations;
      }
      finish = std::max(finish, tau);
    }
    if (dead_set) dead = 1;
    now = finish + 1;  // __syncthreads
  }
  return violations;
}
