// Staged FP64 refinement of the rows that survive the FP32 stage.
//
// One thread per row keeps a warp busy only as long as its most expensive row
// (the reference's early exits and the root finder's data-dependent iteration
// counts differ from row to row), and FP64 issue slots are scarce on this GPU
// (1/64 of the FP32 rate), so masked lanes are expensive.  The refinement is
// therefore split into kernels over a tile of survivor rows:
//
//   stage_build    thread per row: every polynomial of the row in FP64
//                  (reference expressions), normalised and degree-reduced;
//                  lists of degree <= 2 are finished here, the others are
//                  queued per polynomial slot (one queue per slot, so every
//                  queue holds polynomials of one nominal degree);
//   root solving   the queued polynomials through the Jenkins-Traub state
//                  machine (ccd_jt.h), in one of two ways:
//     wavefront    (large batches) wave_start / wave_step: every solver state
//                  lives in global memory; each launch advances every
//                  unfinished job by one step and re-bins it by (phase,
//                  degree), so a warp steps 32 jobs through the same code;
//                  after a fixed number of steps the few unfinished jobs
//                  continue in the pool kernel, and the last ones finish one
//                  per warp (wave_finish);
//     pool         stage_roots: every warp keeps 64 solver states in shared
//                  memory and, each iteration, advances up to 32 of them that
//                  are in the same phase, refilling finished slots from the
//                  queues -- lanes stay busy on equal work without any
//                  block-wide barrier;
//   stage_combine  thread per row: the interval-overlap decision.
//
// The result equals the reference's: every list the reference computes is
// computed the same way, and the extra lists computed for rows the reference
// would have abandoned early do not change the decision (it is "no hit" as
// soon as any list is empty).
#pragma once

#include "ccd_ctcd64.h"
#include "ccd_jt_shifts.h"
#include "ccd_jt_warp.h"
#include "narrow.cuh"

namespace ccd {

constexpr int kMaxSlots = 5;
constexpr int kStageThreads = 128;
// Wavefront defaults (per-context options override them): lock-step steps
// before the unfinished jobs move to the pool kernel (about 99% of the queued
// polynomials finish within 40 solver steps, 99.9% within 120), the steps the
// pool kernel then gives each before the last ones finish one per warp, and
// the batch size below which the pool kernel alone solves (the wavefront pays
// a global-memory round trip per step, which only a large batch hides).
constexpr int kWaveSteps = 48;
// 0: the pool kernel finishes every job it resumes.  Handing long solves to
// the one-per-warp finish only pays when few remain: on near-degenerate
// polynomials (coplanar edges of flat sheets) about 1% of the solves run
// through all 20 shifts, 12-15 thousand steps each, and the pool's lane
// packing beats one busy lane per warp by about 9x there.
constexpr int kPoolBudget = 0;
constexpr int64_t kWaveMinRows = (int64_t)1 << 18;
// Job lists: one per (working phase, current degree 3..6).
constexpr int kWaveBins = 16;

// Device scratch for one tile of `cap` survivor rows (layouts are slot-major,
// then coefficient / span index, then row, so warps access consecutive rows).
struct StageScratch {
  int64_t cap;
  double *coef;         // [slot][k < 7][cap]   queued polynomial coefficients
  int32_t *job_row;     // [slot][cap]          tile row of each queued polynomial
  uint8_t *job_deg;     // [slot][cap]
  double *span_l;       // [slot][k < 7][cap]
  double *span_u;       // [slot][k < 7][cap]
  uint8_t *span_n;      // [slot][cap]
  unsigned *queue;      // [slot] queued polynomials per slot; [kMaxSlots] next job to start
  uint32_t *row_status; // [cap]
  double *roots;        // [slot][k < 6][cap]   roots found by the solver
  // Wavefront solver (null when not attached: the pool kernel then solves
  // every queued polynomial).  Jobs are numbered slot by slot (queue order).
  int64_t jcap;         // kMaxSlots * cap
  double *wd;           // [field < jt::kDoubles][jcap]  solver states
  int *wi;              // [field < jt::kInts][jcap]
  uint32_t *wlist;      // [2][bin < 16][jcap]           jobs per (phase, degree)
  unsigned *wcount;     // [3][16] list lengths (rotating), then the tail and spill lengths
  uint32_t *tail;       // [jcap]                        jobs left after the wavefront steps
  int wave_steps;       // wavefront steps (0: pool kernel only)
  int64_t wave_min_rows;
  int pool_budget;      // steps the pool kernel gives a resumed job before handing it on
  int warp_finish;      // how the last solves run: 0 on one lane; 1 on all 32 lanes of their warp
                        // (ccd_jt_warp.h); 2 with a stage's remaining shifts tried at once, one per
                        // lane (ccd_jt_shifts.h), once shift_after of its shifts have failed
  int shift_after;
  int pool_slots;       // pool kernel of a batch the wavefront does not take: 32 or 64 slots per warp
  int pool_slots_min;   // pool kernel: fewest slots a warp may fill (its share of a small batch is spread)
  int pool_all;         // pool kernel: once the queue is drained, at most this many solves left step together
  int pool_phase_sync;  // pool kernel: 0, or k: prefer the phase of the SM clock's current 2^k-cycle window
};

// Bytes of the scratch for a tile of `cap` rows: three [slot][7][cap]
// double arrays (coefficients, span bounds), one [slot][6][cap] double array
// (roots), a [slot][cap] int32 array, two [slot][cap] byte arrays, the queue
// words and a [cap] status array, each rounded up to 256 bytes.
constexpr size_t kScratchAlign = 256;
constexpr size_t scratch_up(size_t x) { return (x + kScratchAlign - 1) / kScratchAlign * kScratchAlign; }
constexpr size_t stage_scratch_bytes(int64_t cap) {
  return scratch_up(kMaxSlots * 7 * (size_t)cap * sizeof(double)) * 3 +
         scratch_up(kMaxSlots * 6 * (size_t)cap * sizeof(double)) + scratch_up(kMaxSlots * (size_t)cap * sizeof(int32_t)) +
         scratch_up(kMaxSlots * (size_t)cap) * 2 + scratch_up((kMaxSlots + 1) * sizeof(unsigned)) +
         scratch_up((size_t)cap * sizeof(uint32_t));
}
// Carves the scratch arrays out of one allocation of stage_scratch_bytes(cap)
// (no wavefront solver attached).
StageScratch stage_scratch_view(void *base, int64_t cap);
// Bytes of the wavefront solver's scratch for a tile of `cap` rows, and its
// attachment to a view.
size_t wave_scratch_bytes(int64_t cap);
void attach_wave(StageScratch &sc, void *base);

// The list of every row (0 .. n-1) with counters->survivors = n: the input
// of the staged refinement when no FP32 stage runs (CCD_PATH_REFINE_ALL).
cudaError_t launch_all_rows(const PrimBatch &b, int32_t *list, cudaStream_t s);

// Enqueues build/roots/combine over every tile of the survivor list.
// Returns the number of kernels launched through *launches.
cudaError_t launch_stages(const PrimBatch &b, const int32_t *list, const StageScratch &sc, int num_sms,
                          cudaStream_t s, int *launches);

namespace stages {

__device__ __forceinline__ void store_spans(const StageScratch &sc, int slot, int64_t r, const SpanList &sl) {
  sc.span_n[slot * sc.cap + r] = (uint8_t)sl.n;
  for (int k = 0; k < sl.n; k++) {
    sc.span_l[(slot * 7 + k) * sc.cap + r] = sl.s[k].l;
    sc.span_u[(slot * 7 + k) * sc.cap + r] = sl.s[k].u;
  }
}

__device__ __forceinline__ void load_spans(const StageScratch &sc, int slot, int64_t r, SpanList &sl) {
  sl.n = sc.span_n[slot * sc.cap + r];
  for (int k = 0; k < sl.n; k++) {
    sl.s[k].l = sc.span_l[(slot * 7 + k) * sc.cap + r];
    sl.s[k].u = sc.span_u[(slot * 7 + k) * sc.cap + r];
  }
}

template <class Polys>
__global__ void __launch_bounds__(kStageThreads) stage_build(PrimBatch b, const int32_t *__restrict__ list,
                                                             int64_t tile_begin, StageScratch sc) {
  const unsigned lane = threadIdx.x & 31;
  const int64_t count = (int64_t)b.counters->survivors;
  const int64_t end = count < tile_begin + sc.cap ? count : tile_begin + sc.cap;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp_base = tile_begin + (int64_t)blockIdx.x * blockDim.x + (threadIdx.x - lane);
  for (int64_t w = warp_base; w < end; w += stride) {
    const int64_t r = w + lane;
    const bool active = r < end;
    const int64_t tr = r - tile_begin;
    double x[24];
    double eta = 0.0;
    if (active) {
      const int64_t i = list[r];
      const double *src = b.rows + i * 24;
#pragma unroll
      for (int j = 0; j < 24; j++) x[j] = __ldg(src + j);
      eta = b.eta_per_row ? __ldg(b.eta + i) : __ldg(b.eta);
      sc.row_status[tr] = 0;
    }
    for (int slot = 0; slot < Polys::kSlots; slot++) {
      double op[7];
      bool queue = false;
      int deg = 0;
      if (active) {
        const bool pos = Polys::want_pos(slot);
        Polys::coeffs(x, eta, slot, op);
        deg = reduce_poly(op, Polys::degree(slot));
        SpanList sl;
        sl.clear();
        if (deg > 2) {
          queue = sign_possible(op, deg, pos);  // otherwise the list stays empty
        } else {
          low_degree_spans(op, deg, sl, pos);
        }
        if (!queue) store_spans(sc, slot, tr, sl);
      }
      const unsigned mask = __ballot_sync(0xffffffffu, queue);
      if (mask) {
        unsigned base = 0;
        const int leader = __ffs(mask) - 1;
        if ((int)lane == leader) base = atomicAdd(&sc.queue[slot], (unsigned)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (queue) {
          const int64_t j = base + __popc(mask & ((1u << lane) - 1u));
          for (int k = 0; k <= deg; k++) sc.coef[(slot * 7 + k) * sc.cap + j] = op[k];
          sc.job_row[slot * sc.cap + j] = (int32_t)tr;
          sc.job_deg[slot * sc.cap + j] = (uint8_t)deg;
        }
      }
    }
  }
}

// Solver slots per warp (one warp per block) at most, and the shared memory
// of a block with `pool` slots.
constexpr int kWarpPool = 64;
constexpr size_t pool_smem(int pool) { return (size_t)pool * (jt::kDoubles * sizeof(double) + jt::kInts * sizeof(int)); }
constexpr size_t kPoolSmem = pool_smem(kWarpPool);

// Spans of a finished solve, written to the polynomial's row slot.
// Spans of a solve that found `roots` zeros tr[0 .. deg-1] (sorted in place).
template <class Polys>
__device__ __forceinline__ void finish_roots(const StageScratch &sc, int slot, int64_t j, double *tr, int roots,
                                             int status) {
  const int deg = sc.job_deg[slot * sc.cap + j];
  double op[7];
  for (int k = 0; k <= deg; k++) op[k] = sc.coef[(slot * 7 + k) * sc.cap + j];
  SpanList sl;
  sl.clear();
  root_spans(op, deg, tr, roots, sl, Polys::want_pos(slot));
  const int64_t row = sc.job_row[slot * sc.cap + j];
  store_spans(sc, slot, row, sl);
  if (status) atomicOr(&sc.row_status[row], (uint32_t)status);
}

template <class Polys, class S>
__device__ __forceinline__ void finish_job(const StageScratch &sc, const S &st, int slot, int64_t j) {
  const int deg = sc.job_deg[slot * sc.cap + j];
  double tr[6];
  for (int k = 0; k < deg; k++) tr[k] = st.Z(k);
  finish_roots<Polys>(sc, slot, j, tr, st.I(jt::ROOTS), st.I(jt::STATUS));
}

// The solve of state st run to its end by the whole (converged) warp
// (ccd_jt_warp.h); lane 0 writes its spans.
template <class Polys, class S>
__device__ __forceinline__ void warp_solve(const StageScratch &sc, const S &st, int slot, int64_t j) {
  jt::warp::Solve ws;
  ws.load(st);
  double tr[6];
  ws.run(tr);
  if ((threadIdx.x & 31) == 0) finish_roots<Polys>(sc, slot, j, tr, ws.roots, ws.status);
}

__device__ __forceinline__ int job_queue(const int *qbase, int nslots, int64_t g) {
  int q = 0;
  while (q + 1 < nslots && g >= qbase[q + 1]) q++;
  return q;
}

// The solve of state st run to its end by the whole warp, each lane trying
// one of the stage's remaining shifts (ccd_jt_shifts.h); lane 0 writes its
// spans.
template <class Polys, class S>
__device__ __forceinline__ void shift_solve(const StageScratch &sc, const S &st, int slot, int64_t j) {
  jt::LocalStorage ls;
  for (int f = 0; f < jt::kDoubles; f++) ls.d[f] = st.D(f);
  for (int f = 0; f < jt::kInts; f++) ls.i[f] = st.I(f);
  for (int k = 0; k < 6; k++) ls.zr[k] = st.Z(k);
  jt::shifts::run(ls, sc.shift_after);
  if ((threadIdx.x & 31) == 0) finish_job<Polys>(sc, jt::LocalState{&ls}, slot, j);
}

// Which jobs the pool kernel solves.  Default (list null): every queued job,
// from the start.  After the wavefront steps: the jobs in list, resumed from
// their field-major states; a job that takes `budget` more steps is handed on
// (state written back, index appended to spill) to the one-per-warp finish.
struct PoolJobs {
  const uint32_t *list;
  const unsigned *count;
  int budget;
  uint32_t *spill;
  unsigned *spill_count;
};

// POOL solver slots per warp (a multiple of 32; H = POOL / 32 slots per
// lane): 64 packs more solves of one phase into each iteration, 32 halves the
// shared memory a warp holds, so twice as many warps fit on an SM and hide
// each other's FP64 latency.
template <class Polys, int POOL>
__global__ void __launch_bounds__(32) stage_roots(StageScratch sc, PoolJobs pj) {
  constexpr int H = POOL / 32;
  static_assert(POOL % 32 == 0 && H >= 1 && H <= 2, "pool of 32 or 64 slots");
  extern __shared__ double pool_d[];
  int *pool_i = (int *)(pool_d + (size_t)POOL * jt::kDoubles);
  __shared__ int64_t job_of[POOL];
  __shared__ int sel[32];
  __shared__ int qbase[kMaxSlots + 1];
  __shared__ int steps[POOL];
  const int lane = threadIdx.x;
  const unsigned lt = (1u << lane) - 1u;
  if (lane == 0) {
    int acc = 0;
    for (int q = 0; q < Polys::kSlots; q++) {
      qbase[q] = acc;
      acc += (int)sc.queue[q];
    }
    qbase[Polys::kSlots] = acc;
  }
  for (int k = lane; k < POOL; k += 32) pool_i[jt::MODE * POOL + k] = jt::kEmpty;
  __syncwarp();
  const uint32_t *tail = pj.list;
  const int njobs = tail ? (int)*pj.count : qbase[Polys::kSlots];
  // Slots this warp fills at most: its fair share of the jobs, but no fewer
  // than sc.pool_slots_min.  A small batch then spreads over more warps
  // instead of filling the first warps' slots while the rest of the grid
  // idles: each warp advances fewer solves per iteration, with fewer
  // divergent paths, and so each of them more often.  The wavefront's
  // leftovers (long solves, where packing lanes of one phase pays) fill
  // every slot.
  const int share = (int)(((int64_t)njobs + gridDim.x - 1) / gridDim.x);
  const int lo = tail ? POOL : (sc.pool_slots_min < 1 ? 1 : sc.pool_slots_min);
  const int lim = share < lo ? lo : (share < POOL ? share : POOL);
  auto state = [&](int k) {
    const int64_t g = job_of[k];
    const int q = job_queue(qbase, Polys::kSlots, g);
    const int64_t j = g - qbase[q];
    return jt::PoolState<POOL>{pool_d, pool_i, k, sc.roots + (int64_t)q * 6 * sc.cap + j, sc.cap};
  };
  int *mode = pool_i + jt::MODE * POOL;
  bool exhausted = njobs == 0;
  for (;;) {
    // Write out finished solves.
    for (int k = lane; k < POOL; k += 32) {
      if (mode[k] == jt::kDone) {
        const jt::PoolState<POOL> st = state(k);
        const int64_t g = job_of[k];
        const int q = job_queue(qbase, Polys::kSlots, g);
        finish_job<Polys>(sc, st, q, g - qbase[q]);
        mode[k] = jt::kEmpty;
      }
    }
    __syncwarp();
    // Refill empty slots: one atomic per warp reserves consecutive jobs.
    if (!exhausted) {
      unsigned e[H];
#pragma unroll
      for (int h = 0; h < H; h++) {
        const int k = lane + 32 * h;
        e[h] = __ballot_sync(0xffffffffu, k < lim && mode[k] == jt::kEmpty);
      }
      int nempty = 0;
#pragma unroll
      for (int h = 0; h < H; h++) nempty += __popc(e[h]);
      if (nempty) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(&sc.queue[kMaxSlots], (unsigned)nempty);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((int64_t)base + nempty >= njobs) exhausted = true;
        int before = 0;
#pragma unroll
        for (int h = 0; h < H; h++) {
          const int ahead = before;
          before += __popc(e[h]);
          if (!((e[h] >> lane) & 1u)) continue;
          const int k = lane + 32 * h;
          const int64_t g0 = (int64_t)base + ahead + __popc(e[h] & lt);
          if (g0 >= njobs) continue;
          const int64_t g = tail ? (int64_t)tail[g0] : g0;
          job_of[k] = g;
          steps[k] = 0;
          const int q = job_queue(qbase, Polys::kSlots, g);
          const int64_t j = g - qbase[q];
          const jt::PoolState<POOL> st{pool_d, pool_i, k, sc.roots + (int64_t)q * 6 * sc.cap + j, sc.cap};
          if (tail) {
            const jt::FieldState fs{sc.wd, sc.wi, g, sc.jcap, st.zr, sc.cap};
            for (int f = 0; f < jt::kDoubles; f++) st.D(f) = fs.D(f);
            for (int f = 0; f < jt::kInts; f++) st.I(f) = fs.I(f);
          } else {
            const int deg = sc.job_deg[q * sc.cap + j];
            double op[7];
            for (int c = 0; c <= deg; c++) op[c] = sc.coef[(q * 7 + c) * sc.cap + j];
            jt::start(st, op, deg);
          }
        }
      }
    }
    __syncwarp();
    // The most populated working phase.
    int best = 0, bestc = 0, working = 0;
    bool pending = false;
    for (int m = jt::kInit; m <= jt::kDone; m++) {
      int c = 0;
#pragma unroll
      for (int h = 0; h < H; h++) c += __popc(__ballot_sync(0xffffffffu, mode[lane + 32 * h] == m));
      if (m == jt::kDone) {
        pending = c > 0;
      } else {
        working += c;
        if (c > bestc) {
          best = m;
          bestc = c;
        }
      }
    }
    if (bestc == 0) {
      if (exhausted && !pending) break;
      continue;
    }
    if (sc.pool_phase_sync && !tail) {
      // The phase of this moment (rotating every 2^k cycles of the SM's
      // clock, alike for the warps of one SM) when it holds at least half
      // as many solves as the most populated one: the SM's warps then run
      // the same phase's code at once.  Not for the wavefront's leftovers,
      // long solves whose lanes the most populated phase packs best.
      const int pref = jt::kInit + (int)((clock64() >> sc.pool_phase_sync) & 3);
      int c = 0;
#pragma unroll
      for (int h = 0; h < H; h++) c += __popc(__ballot_sync(0xffffffffu, mode[lane + 32 * h] == pref));
      if (2 * c >= bestc && c > 0) {
        best = pref;
        bestc = c;
      }
    }
    if (exhausted && working == 1 && sc.warp_finish) {
      // The warp's last unfinished solve, with no job left to take: all 32
      // lanes copy its state and advance it together to the end
      // (jt::warp::step, or one shift per lane), then lane 0 writes it out.
      int k = 0;
#pragma unroll
      for (int h = H - 1; h >= 0; h--) {
        const unsigned w = __ballot_sync(0xffffffffu, mode[lane + 32 * h] == best);
        if (w) k = 32 * h + __ffs(w) - 1;
      }
      const int64_t g = job_of[k];
      const int q = job_queue(qbase, Polys::kSlots, g);
      if (sc.warp_finish == 2)
        shift_solve<Polys>(sc, state(k), q, g - qbase[q]);
      else
        warp_solve<Polys>(sc, state(k), q, g - qbase[q]);
      __syncwarp();
      if (lane == 0) mode[k] = jt::kEmpty;
      __syncwarp();
      continue;
    }
    // Up to 32 slots, one per lane: of the most populated phase (lanes on
    // equal work), or -- once nothing is left to take and at most
    // sc.pool_all solves remain -- all of them, whatever their phases: their
    // lanes diverge, but every remaining solve advances at every iteration
    // instead of waiting for its phase to be the most populated one.
    const bool all = exhausted && working <= sc.pool_all;
    unsigned b[H];
#pragma unroll
    for (int h = 0; h < H; h++) {
      const int m = mode[lane + 32 * h];
      b[h] = __ballot_sync(0xffffffffu, all ? (m >= jt::kInit && m < jt::kDone) : m == best);
    }
    if (all) bestc = working;
    int before = 0;
#pragma unroll
    for (int h = 0; h < H; h++) {
      if ((b[h] >> lane) & 1u) {
        const int r = before + __popc(b[h] & lt);
        if (r < 32) sel[r] = lane + 32 * h;
      }
      before += __popc(b[h]);
    }
    __syncwarp();
    if (lane < bestc) {
      const int k = sel[lane];
      const jt::PoolState<POOL> st = state(k);
      jt::step(st);
      if (pj.budget > 0 && mode[k] != jt::kDone && ++steps[k] >= pj.budget) {
        // Hand the job on: its state back home, its index to the spill list.
        const jt::FieldState fs{sc.wd, sc.wi, job_of[k], sc.jcap, st.zr, sc.cap};
        for (int f = 0; f < jt::kDoubles; f++) fs.D(f) = st.D(f);
        for (int f = 0; f < jt::kInts; f++) fs.I(f) = st.I(f);
        pj.spill[atomicAdd(pj.spill_count, 1u)] = (uint32_t)job_of[k];
        mode[k] = jt::kEmpty;
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- wavefront solver
// Every queued polynomial's solver state lives in global memory (FieldState).
// wave_start starts all of them; each wave_step advances every unfinished
// one by one step and re-bins it by its next phase, so a warp steps jobs of
// one phase through the same code.  After a fixed number of steps the few
// jobs still running are gathered for the pool kernel, which solves them
// again from the start.
constexpr int kWaveThreads = 128;

__device__ __forceinline__ void queue_bases(const StageScratch &sc, int nslots, int *qbase) {
  int acc = 0;
  for (int q = 0; q < nslots; q++) {
    qbase[q] = acc;
    acc += (int)sc.queue[q];
  }
  qbase[nslots] = acc;
}

// List of a working job: (phase, current degree).
__device__ __forceinline__ int wave_bin(int mode, int n) {
  n = n < 3 ? 3 : (n > 6 ? 6 : n);
  return (mode - 1) * 4 + (n - 3);
}

// Warp-aggregated append of job g to list `bin` (lanes with equal bins share
// one atomic).
__device__ __forceinline__ void wave_append(uint32_t *lists, unsigned *counts, int64_t jcap, bool active, int bin,
                                            int64_t g) {
  const unsigned lane = threadIdx.x & 31;
  const unsigned key = active ? (unsigned)bin : 0xffffffffu;
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const int leader = __ffs(peers) - 1;
  unsigned base = 0;
  if (active && (int)lane == leader) base = atomicAdd(&counts[bin], (unsigned)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (active) lists[(int64_t)bin * jcap + base + __popc(peers & ((1u << lane) - 1u))] = (uint32_t)g;
}

template <class Polys>
__device__ __forceinline__ jt::FieldState wave_state(const StageScratch &sc, const int *qbase, int64_t g, int &q,
                                                     int64_t &j) {
  q = job_queue(qbase, Polys::kSlots, g);
  j = g - qbase[q];
  return jt::FieldState{sc.wd, sc.wi, g, sc.jcap, sc.roots + (int64_t)q * 6 * sc.cap + j, sc.cap};
}

// Offsets of the concatenated lists (off[kWaveBins] = total).
__device__ __forceinline__ void list_offsets(const unsigned *cin, int64_t *off) {
  int64_t acc = 0;
  for (int m = 0; m < kWaveBins; m++) {
    off[m] = acc;
    acc += cin[m];
  }
  off[kWaveBins] = acc;
}

__device__ __forceinline__ int64_t list_entry(const uint32_t *in, const int64_t *off, int64_t jcap, int64_t r) {
  int m = 0;
  while (m + 1 < kWaveBins && r >= off[m + 1]) m++;
  return in[(int64_t)m * jcap + (r - off[m])];
}

// Whole solver state from global (field-major) to thread-private storage.
__device__ __forceinline__ void load_state(const jt::FieldState &fs, jt::LocalStorage &st) {
  for (int f = 0; f < jt::kDoubles; f++) st.d[f] = fs.D(f);
  for (int f = 0; f < jt::kInts; f++) st.i[f] = fs.I(f);
  for (int k = 0; k < 6; k++) st.zr[k] = fs.Z(k);
}

template <class Polys>
__global__ void __launch_bounds__(kWaveThreads) wave_start(StageScratch sc) {
  __shared__ int qbase[kMaxSlots + 1];
  if (threadIdx.x == 0) queue_bases(sc, Polys::kSlots, qbase);
  __syncthreads();
  const int64_t njobs = qbase[Polys::kSlots];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp_base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  for (int64_t w = warp_base; w < njobs; w += stride) {
    const int64_t g = w + (threadIdx.x & 31);
    bool work = false;
    int bin = 0;
    if (g < njobs) {
      int q;
      int64_t j;
      const jt::FieldState s = wave_state<Polys>(sc, qbase, g, q, j);
      const int deg = sc.job_deg[q * sc.cap + j];
      double op[7];
      for (int c = 0; c <= deg; c++) op[c] = sc.coef[(q * 7 + c) * sc.cap + j];
      jt::start(s, op, deg);
      const int mode = s.I(jt::MODE);
      if (mode == jt::kDone) {
        finish_job<Polys>(sc, s, q, j);
      } else {
        work = true;
        bin = wave_bin(mode, s.I(jt::N));
      }
    }
    wave_append(sc.wlist, sc.wcount, sc.jcap, work, bin, g);
  }
}

// One step of every job in lists `in` (counts cin), re-binned into lists
// `out` (counts cout, zeroed before); also zeroes czero, the counts the step
// after next will fill.
template <class Polys>
__global__ void __launch_bounds__(kWaveThreads) wave_step(StageScratch sc, const uint32_t *in, const unsigned *cin,
                                                          uint32_t *out, unsigned *cout, unsigned *czero) {
  __shared__ int qbase[kMaxSlots + 1];
  __shared__ int64_t off[kWaveBins + 1];
  if (threadIdx.x == 0) {
    queue_bases(sc, Polys::kSlots, qbase);
    list_offsets(cin, off);
  }
  if (blockIdx.x == 0 && threadIdx.x < kWaveBins) czero[threadIdx.x] = 0;
  __syncthreads();
  const int64_t total = off[kWaveBins];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp_base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  for (int64_t w = warp_base; w < total; w += stride) {
    const int64_t r = w + (threadIdx.x & 31);
    bool work = false;
    int bin = 0;
    int64_t g = 0;
    if (r < total) {
      g = list_entry(in, off, sc.jcap, r);
      int q;
      int64_t j;
      const jt::FieldState s = wave_state<Polys>(sc, qbase, g, q, j);
      jt::step(s);
      const int mode = s.I(jt::MODE);
      if (mode == jt::kDone) {
        finish_job<Polys>(sc, s, q, j);
      } else {
        work = true;
        bin = wave_bin(mode, s.I(jt::N));
      }
    }
    wave_append(out, cout, sc.jcap, work, bin, g);
  }
}

// Concatenates the unfinished jobs' lists into sc.tail; the count goes to
// tcount.
template <class Polys>
__global__ void __launch_bounds__(kWaveThreads) wave_gather_tail(StageScratch sc, const uint32_t *in,
                                                                 const unsigned *cin, unsigned *tcount) {
  int64_t off[kWaveBins + 1];
  list_offsets(cin, off);
  const int64_t total = off[kWaveBins];
  if (blockIdx.x == 0 && threadIdx.x == 0) *tcount = (unsigned)total;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < total; r += stride)
    sc.tail[r] = (uint32_t)list_entry(in, off, sc.jcap, r);
}

// The jobs the wavefront steps left unfinished, one per warp, each run to
// its end (the solver's own iteration limits bound the loop).  Few jobs
// remain by then and each is a long sequential chain, so latency, not lane
// use, matters here.  With sc.warp_finish the warp holds the state in
// registers spread over its lanes and advances the solve together
// (jt::warp::Solve: element-wise updates and independent divisions on
// different lanes); otherwise lane 0 runs it alone from a private copy.
template <class Polys>
__global__ void __launch_bounds__(32) wave_finish(StageScratch sc, const uint32_t *tail, const unsigned *tcount) {
  __shared__ int qbase[kMaxSlots + 1];
  if (threadIdx.x == 0) queue_bases(sc, Polys::kSlots, qbase);
  __syncwarp();
  const bool whole = sc.warp_finish != 0;
  if (!whole && threadIdx.x != 0) return;
  const int64_t count = *tcount;
  for (int64_t r = blockIdx.x; r < count; r += gridDim.x) {
    const int64_t g = tail[r];
    int q;
    int64_t j;
    const jt::FieldState fs = wave_state<Polys>(sc, qbase, g, q, j);
    if (sc.warp_finish == 2) {
      shift_solve<Polys>(sc, fs, q, j);
    } else if (whole) {
      warp_solve<Polys>(sc, fs, q, j);
    } else {
      jt::LocalStorage st;
      load_state(fs, st);
      const jt::LocalState s{&st};
      while (s.I(jt::MODE) != jt::kDone) jt::step(s);
      finish_job<Polys>(sc, s, q, j);
    }
  }
}

template <class Polys>
__global__ void __launch_bounds__(kStageThreads) stage_combine(PrimBatch b, const int32_t *__restrict__ list,
                                                               int64_t tile_begin, StageScratch sc) {
  const unsigned lane = threadIdx.x & 31;
  const int64_t count = (int64_t)b.counters->survivors;
  const int64_t end = count < tile_begin + sc.cap ? count : tile_begin + sc.cap;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t warp_base = tile_begin + (int64_t)blockIdx.x * blockDim.x + (threadIdx.x - lane);
  unsigned hits = 0, flags = 0;
  for (int64_t w = warp_base; w < end; w += stride) {
    const int64_t r = w + lane;
    if (r < end) {
      const int64_t tr = r - tile_begin;
      const int64_t i = list[r];
      SpanList l[Polys::kSlots];
      for (int slot = 0; slot < Polys::kSlots; slot++) load_spans(sc, slot, tr, l[slot]);
      double t = 0.0;
      bool h;
      if constexpr (Polys::kSlots == 4) {
        h = vf_combine(l[0], l[1], l[2], l[3], t);
      } else {
        double x[24];
        const double *src = b.rows + i * 24;
#pragma unroll
        for (int j = 0; j < 24; j++) x[j] = __ldg(src + j);
        SpanList cop, par;
        ee_split_parallel(x, l[0], cop, par);
        h = ee_combine(cop, par, l[1], l[2], l[3], l[4], t);
      }
      const uint8_t st = (uint8_t)sc.row_status[tr];
      b.hit[i] = h;
      if (h) b.t[i] = t;
      if (b.status) b.status[i] = st;
      hits += h;
      flags += (st != 0);
    }
  }
  const unsigned hsum = __reduce_add_sync(0xffffffffu, hits);
  const unsigned fsum = __reduce_add_sync(0xffffffffu, flags);
  if (lane == 0) {
    if (hsum) atomicAdd(&b.counters->hits, (unsigned long long)hsum);
    if (fsum) atomicAdd(&b.counters->status_flags, (unsigned long long)fsum);
  }
}

inline int stage_grid(int64_t work, int num_sms) {
  int64_t need = (work + kStageThreads - 1) / kStageThreads;
  int64_t cap = (int64_t)num_sms * 16;
  return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

template <class Polys>
cudaError_t run(const PrimBatch &b, const int32_t *list, const StageScratch &sc, int num_sms, cudaStream_t s,
                int *launches) {
  // The pool kernel's dynamic shared memory stays under the 48 KB that any
  // launch may use without an opt-in attribute (set once per device and
  // function), so launches from any host thread or device need no setup.
  static_assert(kPoolSmem + 1024 <= 48 * 1024, "stage_roots needs an opt-in shared-memory attribute");
  cudaError_t e;
  const int64_t tiles = (b.n + sc.cap - 1) / sc.cap;
  const int grid = stage_grid(sc.cap, num_sms);
  // Five 64-slot warp pools (about 41 KB each) fit one SM's shared memory,
  // ten 32-slot ones (about 21 KB; 168 registers a lane allow 12 warps).
  const int pool_grid = num_sms * 5, pool32_grid = num_sms * 10;
  const int wave_grid = num_sms * 8;
  for (int64_t tile = 0; tile < tiles; tile++) {
    e = cudaMemsetAsync(sc.queue, 0, (kMaxSlots + 1) * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    stage_build<Polys><<<grid, kStageThreads, 0, s>>>(b, list, tile * sc.cap, sc);
    if (sc.wd && sc.wave_steps > 0 && b.n >= sc.wave_min_rows) {
      const int steps = sc.wave_steps;
      const int64_t lstride = (int64_t)kWaveBins * sc.jcap;
      // counts: 3 rotating sets, then the tail and spill lengths
      e = cudaMemsetAsync(sc.wcount, 0, (3 * kWaveBins + 2) * sizeof(unsigned), s);
      if (e != cudaSuccess) return e;
      wave_start<Polys><<<wave_grid, kWaveThreads, 0, s>>>(sc);
      for (int it = 0; it < steps; it++) {
        wave_step<Polys><<<wave_grid, kWaveThreads, 0, s>>>(
            sc, sc.wlist + (it & 1) * lstride, sc.wcount + kWaveBins * (it % 3), sc.wlist + ((it + 1) & 1) * lstride,
            sc.wcount + kWaveBins * ((it + 1) % 3), sc.wcount + kWaveBins * ((it + 2) % 3));
      }
      unsigned *tcount = sc.wcount + 3 * kWaveBins, *scount = tcount + 1;
      wave_gather_tail<Polys><<<num_sms, kWaveThreads, 0, s>>>(sc, sc.wlist + (steps & 1) * lstride,
                                                               sc.wcount + kWaveBins * (steps % 3), tcount);
      // The unfinished jobs continue in the pool kernel (many per warp); the
      // few that exceed its step budget finish one per warp, as many warps as
      // can be resident at once.  The wavefront lists are free again and hold
      // the spilled jobs.
      stage_roots<Polys, kWarpPool><<<pool_grid, 32, kPoolSmem, s>>>(
          sc, PoolJobs{sc.tail, tcount, sc.pool_budget, sc.wlist, scount});
      wave_finish<Polys><<<num_sms * 32, 32, 0, s>>>(sc, sc.wlist, scount);
      *launches += steps + 4;
    } else {
      if (sc.pool_slots == 32)
        stage_roots<Polys, 32><<<pool32_grid, 32, pool_smem(32), s>>>(sc, PoolJobs{nullptr, nullptr, 0, nullptr, nullptr});
      else
        stage_roots<Polys, kWarpPool><<<pool_grid, 32, kPoolSmem, s>>>(sc, PoolJobs{nullptr, nullptr, 0, nullptr, nullptr});
      *launches += 1;
    }
    stage_combine<Polys><<<grid, kStageThreads, 0, s>>>(b, list, tile * sc.cap, sc);
    *launches += 2;
  }
  return cudaGetLastError();
}

}  // namespace stages
}  // namespace ccd
