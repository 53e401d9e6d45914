// One Jenkins-Traub solve finished by a warp whose lanes try the remaining
// shifts of a stage at the same time.
//
// Within one stage of rpoly (src/rpoly.h:211-249) the quadratic shifts are
// tried one after another: shift cnt rotates the shift point by 94 degrees,
// restores K to the polynomial left by the unshifted steps (temp) and runs
// the fixed-shift stage with 20 * cnt iterations; the first shift whose
// stage finds a zero deflates the polynomial and ends the stage, and a stage
// whose 20 shifts all fail ends the solve.  A failed shift leaves nothing
// that the next one reads: every field a shift uses is set by its own start
// (jt::begin_shift: u, v, the betas, the old values, the quotient and the
// scalars), from the stage's p, temp and root bound, and the shift point,
// which depends only on how many rotations came before.  So shift c can start
// before shifts c0 .. c-1 have failed, and its result is the one the
// sequential loop would reach if they do.
//
// Here lane L of the warp takes shift c0 + L, where c0 is the shift the
// solve is in: lane 0 goes on with the solve's own state, every other lane
// restores K from temp, rotates the shift point L times (the same operations
// as L starts of a shift) and starts its shift.  The lanes advance their
// shifts with the sequential code (ccd_jt.h) on private copies of the state.
// The stage's outcome is the lowest lane whose shift found a zero once every
// lower lane's shift has failed; when all of them fail, the last shift's
// lane holds the sequential end of the solve (20 shifts, no convergence).
// Every lane then takes that lane's state, and the next stage starts (its
// unshifted steps run on every lane alike, with identical results).  The
// values are those of the sequential solve bit for bit; the stage's latency
// becomes that of its winning shift instead of the sum of all the shifts
// before it, which is what the slowest solves of a batch spend their time
// on (near-degenerate polynomials whose stages fail shift after shift).
#pragma once

#include "ccd_jt.h"

namespace ccd {
namespace jt {
namespace shifts {

constexpr int kShifts = 20;  // shifts per stage (rpoly.h:211)

// Lane L > 0's start of shift c0 + L, from the solve's state while it is in
// shift c0: K restored from temp, the shift point rotated L - 1 times, then
// the start of a shift (which rotates it once more).
template <class S>
CCD_HD void start_later_shift(S s, int lane) {
  const int n = s.I(N);
  for (int i = 0; i < n; i++) s.D(K + i) = s.D(TEMP + i);
  for (int r = 1; r < lane; r++) rotate_shift(s);
  s.I(CNT) += lane;
  s.I(MODE) = kFixed;
  begin_shift(s);
}

// Where shift c of a stage entered with n0 unknowns stands: 0 still running,
// 1 failed (the next shift began, or the 20th failed and ended the solve), 2
// found a zero (deflated: the next stage, or the closed forms and done).
template <class S>
CCD_HD int shift_outcome(S s, int c, int n0) {
  if (s.I(N) != n0) return 2;
  if (s.I(CNT) != c || s.I(MODE) == kDone) return 1;
  return 0;
}

#if defined(__CUDACC__)
constexpr unsigned kFull = 0xffffffffu;

// This lane's whole state := lane src's.
__device__ __forceinline__ void take(LocalStorage &st, int src) {
  for (int f = 0; f < kDoubles; f++) st.d[f] = __shfl_sync(kFull, st.d[f], src);
  for (int k = 0; k < 6; k++) st.zr[k] = __shfl_sync(kFull, st.zr[k], src);
  for (int f = 0; f < kInts; f++) st.i[f] = __shfl_sync(kFull, st.i[f], src);
}

// Runs the solve held (identically) by every lane of the warp to its end;
// every lane returns with the final state.  All 32 lanes must call it.  A
// stage's first `after` shifts run one at a time, every lane stepping the
// same state (most stages end within them, and trying later shifts early
// would only add divergent work); once `after` shifts of the stage have
// failed, the remaining ones run at once.
__device__ __noinline__ inline void run(LocalStorage &st, int after) {
  const LocalState s{&st};
  const int lane = (int)(threadIdx.x & 31);
  for (;;) {
    const int mode = s.I(MODE);
    if (mode == kDone) return;
    if (mode == kInit) {
      step_init(s);
      continue;
    }
    // In the shift loop of a stage: shift c0 is under way.
    const int c0 = s.I(CNT), n0 = s.I(N);
    if (c0 < after) {
      step(s);
      continue;
    }
    const int c = c0 + lane;
    bool running = c < kShifts, won = false;
    if (lane > 0 && running) start_later_shift(s, lane);
    int w;
    for (;;) {
      if (running) {
        step(s);
        const int o = shift_outcome(s, c, n0);
        running = o == 0;
        won = o == 2;
      }
      const unsigned run_m = __ballot_sync(kFull, running);
      const unsigned won_m = __ballot_sync(kFull, won);
      if (won_m) {
        const int lo = __ffs(won_m) - 1;
        if ((run_m & ((1u << lo) - 1u)) == 0u) {  // every earlier shift has failed
          w = lo;
          break;
        }
      } else if (run_m == 0u) {
        w = kShifts - 1 - c0;  // every shift failed: the last one ended the solve
        break;
      }
    }
    take(st, w);
  }
}
#endif

}  // namespace shifts
}  // namespace jt
}  // namespace ccd
