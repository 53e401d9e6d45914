// Host build of the device CTCD core (csrc/ccd_ctcd64.h) for the CPU tests:
// the same source the CUDA kernels compile, checked against the oracle here.
#include <cmath>
#include <cstdint>

#include "../../collisiondetection_gb300/csrc/ccd_ctcd64.h"

extern "C" void hc_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit,
                         double *t, uint8_t *status) {
  static const int width[4] = {24, 24, 18, 12};
  for (int64_t i = 0; i < n; i++) {
    const double *xi = x + i * width[kind];
    double e = eta_per_test ? eta[i] : eta[0];
    uint8_t st = 0;
    bool h;
    switch (kind) {
      case 0: h = ccd::vf_ctcd(xi, e, t[i], st); break;
      case 1: h = ccd::ee_ctcd(xi, e, t[i], st); break;
      case 2: h = ccd::ve_ctcd(xi, e, t[i], st); break;
      default: h = ccd::vv_ctcd(xi, e, t[i]); break;
    }
    hit[i] = h;
    status[i] = st;
  }
}

#include "../../collisiondetection_gb300/csrc/ccd_cull32.h"

// 1 where the FP32 stage rejects the row (kinds 0, 1 and 2).
extern "C" void hc_cull(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *rej) {
  const int w = kind == 2 ? 18 : 24;
  for (int64_t i = 0; i < n; i++) {
    const double *xi = x + i * w;
    double e = eta_per_test ? eta[i] : eta[0];
    rej[i] = kind == 0 ? ccd::vf_rejects(xi, e) : (kind == 1 ? ccd::ee_rejects(xi, e) : ccd::ve_rejects(xi, e));
  }
}

#include <queue>
#include <vector>

#include "../../collisiondetection_gb300/csrc/ccd_heap.h"

// The device event queue's heap (csrc/ccd_heap.h) against std::priority_queue
// with the active layers' comparator on the same operations: op[i] >= 0
// pushes element op[i] (its key key[op[i]], which may change between
// operations as the firing times do: newkey[i] replaces key[op_key[i]] first
// when op_key[i] >= 0), op[i] < 0 pops.  The top seen before every pop is
// written to ours[] / theirs[] (-1 when empty).
extern "C" void hc_heap_replay(int n, const int *op, const int *op_key, const double *newkey, double *key,
                               int nkeys, int *ours, int *theirs) {
  std::vector<double> k1(key, key + nkeys), k2(key, key + nkeys);
  struct Cmp {
    const std::vector<double> *k;
    bool operator()(int a, int b) const { return (*k)[b] < (*k)[a]; }
  };
  std::priority_queue<int, std::vector<int>, Cmp> pq(Cmp{&k2});
  std::vector<int> heap(n + 1);
  int size = 0;
  auto lower = [&](int a, int b) { return k1[b] < k1[a]; };
  int npop = 0;
  for (int i = 0; i < n; i++) {
    if (op_key[i] >= 0) {
      k1[op_key[i]] = newkey[i];
      k2[op_key[i]] = newkey[i];
    }
    if (op[i] >= 0) {
      ccd::heap_push(heap.data(), &size, op[i], lower);
      pq.push(op[i]);
    } else {
      ours[npop] = size ? heap[0] : -1;
      theirs[npop] = pq.empty() ? -1 : pq.top();
      npop++;
      if (size) ccd::heap_pop(heap.data(), &size, lower);
      if (!pq.empty()) pq.pop();
    }
  }
}

#include <cstring>

#include "../../collisiondetection_gb300/csrc/ccd_jt_shifts.h"

// The Jenkins-Traub solve with each stage's shifts resolved the way the
// warp-parallel finish (csrc/ccd_jt_shifts.h) resolves them: every remaining
// shift of the stage started from the stage's state (start_later_shift), run
// to its end on its own copy, and the first one in order that finds a zero
// taken (or the last one, when all of them fail).  Against the sequential
// driver on the same polynomials: zeros, root count and status, bit for bit.
// shifts_run[i] counts the shifts started ahead of time in solve i.
extern "C" void hc_shift_check(int64_t n, const double *coef, const int *deg, double *zr_seq, int *roots_seq,
                               double *zr_par, int *roots_par, int *status, int *shifts_run) {
  using namespace ccd::jt;
  for (int64_t p = 0; p < n; p++) {
    const double *op = coef + 7 * p;
    const int d = deg[p];
    {
      LocalStorage st;
      std::memset(&st, 0, sizeof(st));
      const LocalState s{&st};
      start(s, op, d);
      while (s.I(MODE) != kDone) step(s);
      for (int k = 0; k < 6; k++) zr_seq[6 * p + k] = st.zr[k];
      roots_seq[p] = s.I(ROOTS);
      status[2 * p] = s.I(STATUS);
    }
    LocalStorage st;
    std::memset(&st, 0, sizeof(st));
    const LocalState s{&st};
    start(s, op, d);
    int ahead = 0;
    while (s.I(MODE) != kDone) {
      if (s.I(MODE) == kInit) {
        step_init(s);
        continue;
      }
      const int c0 = s.I(CNT), n0 = s.I(N);
      LocalStorage win = st;
      for (int lane = 0; c0 + lane < shifts::kShifts; lane++) {
        LocalStorage ls = st;
        const LocalState t{&ls};
        if (lane > 0) {
          shifts::start_later_shift(t, lane);
          ahead++;
        }
        int o;
        while ((o = shifts::shift_outcome(t, c0 + lane, n0)) == 0) step(t);
        if (o == 2 || c0 + lane == shifts::kShifts - 1) {
          win = ls;
          break;
        }
      }
      st = win;
    }
    for (int k = 0; k < 6; k++) zr_par[6 * p + k] = st.zr[k];
    roots_par[p] = s.I(ROOTS);
    status[2 * p + 1] = s.I(STATUS);
    shifts_run[p] = ahead;
  }
}
