// Bookkeeping of a CTA's bounded waits for its tensor-core MMAs (k_lu's
// tensor-core instantiation).  Kept free of device intrinsics so that the host
// can run the same rules in a model of the barrier (tests/mma_sync_check.cpp).
//
// One thread issues a tile's tcgen05.mma instructions and commits them to an
// mbarrier; every thread of the CTA then polls that barrier for the phase it
// expects (its `phase` bit) with a bounded number of polls.  The rules:
//  * completion seen within the first bound: the tile's results are used and
//    the phase bit flips;
//  * otherwise the draw is marked bad (the pivoting pass redoes it) and the
//    thread keeps polling, with a second, longer bound, until the late MMAs
//    complete ("drained"): the phase bit flips, so the next wait still waits
//    for the next commit and never mistakes this late completion for it;
//  * if the drain bound runs out too, the barrier's phase is unknown from then
//    on: the thread sets the CTA's `dead` flag.  A CTA with the flag set issues
//    no more MMAs and waits on the barrier no more; every later draw of the CTA
//    is marked bad, so all of them go to the pivoting pass, whose kernel does
//    not use the tensor cores.
#pragma once
#include <cstdint>

#if defined(__CUDACC__)
#define SGDLM_HD __host__ __device__ __forceinline__
#else
#define SGDLM_HD inline
#endif

namespace sgdlm {

// Polls of the first and of the drain bound (each poll is one
// mbarrier.try_wait, which itself suspends for a hardware-chosen time).
constexpr int kMmaPolls = 1 << 22;
constexpr int kMmaDrainPolls = 1 << 26;

enum MmaWait : int {
  kMmaDone = 0,     // completed within the first bound: results valid
  kMmaDrained = 1,  // completed late: results unused, draw bad, phase in step
  kMmaLost = 2,     // never seen: draw bad, the CTA must give the barrier up
  kMmaSkipped = 3   // the CTA had given the barrier up: no wait, draw bad
};

// dead: the CTA's flag as read before the wait; first / drained: whether the
// expected phase completed within the first / the drain bound.
SGDLM_HD int mma_wait_rule(bool dead, bool first, bool drained, uint32_t &phase, bool &bad) {
  if (dead) {
    bad = true;
    return kMmaSkipped;
  }
  if (first) {
    phase ^= 1u;
    return kMmaDone;
  }
  bad = true;
  if (drained) {
    phase ^= 1u;
    return kMmaDrained;
  }
  return kMmaLost;
}

// try_wait.parity semantics: the phase with parity `parity` has completed when
// the barrier's current phase count has the other parity.
SGDLM_HD bool mbar_phase_done(uint32_t completed_phases, uint32_t parity) {
  return (completed_phases & 1u) != parity;
}

}  // namespace sgdlm
