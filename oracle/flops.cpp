// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Floating-point operation counts of the reference's primitive tests: the
// oracle's restatement (ccd_oracle_prims.h, which follows src/CTCD.cpp and
// src/rpoly.h operation for operation) compiled over a scalar that counts
// every arithmetic operation it performs.  The counts are the algorithmic
// FP64 work of a test -- what the reference's own code computes for that
// row -- and are what the refinement's FP64 roofline divides by time.
//
// Categories: add (+, -), mul, div, sqrt, cmp (<, <=, ==, ...; not flops),
// and transcendental calls (exp, log, pow, cos, sin; once per root-finder
// start).  flops = add + mul + div + sqrt.  Negation and fabs are sign
// operations and are not counted.
//
// Results (hit, t) equal the oracle's: the counted scalar holds an IEEE
// double and rounds every operation the same way (-ffp-contract=off).
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <string.h>

namespace {

struct Counts {
  uint64_t add, mul, div, sqrt, cmp, trans;
};

thread_local Counts *g_counts = nullptr;

struct counted {
  double v;
  counted() = default;
  counted(double x) : v(x) {}  // NOLINT: literals and raw inputs convert implicitly, as doubles would
  explicit operator double() const { return v; }
};

inline counted operator+(counted a, counted b) { g_counts->add++; return counted(a.v + b.v); }
inline counted operator-(counted a, counted b) { g_counts->add++; return counted(a.v - b.v); }
inline counted operator*(counted a, counted b) { g_counts->mul++; return counted(a.v * b.v); }
inline counted operator/(counted a, counted b) { g_counts->div++; return counted(a.v / b.v); }
inline counted operator-(counted a) { return counted(-a.v); }
inline counted &operator+=(counted &a, counted b) { a = a + b; return a; }
inline counted &operator-=(counted &a, counted b) { a = a - b; return a; }
inline counted &operator*=(counted &a, counted b) { a = a * b; return a; }
inline counted &operator/=(counted &a, counted b) { a = a / b; return a; }
inline bool operator<(counted a, counted b) { g_counts->cmp++; return a.v < b.v; }
inline bool operator>(counted a, counted b) { g_counts->cmp++; return a.v > b.v; }
inline bool operator<=(counted a, counted b) { g_counts->cmp++; return a.v <= b.v; }
inline bool operator>=(counted a, counted b) { g_counts->cmp++; return a.v >= b.v; }
inline bool operator==(counted a, counted b) { g_counts->cmp++; return a.v == b.v; }
inline bool operator!=(counted a, counted b) { g_counts->cmp++; return a.v != b.v; }
inline counted fabs(counted a) { return counted(::fabs(a.v)); }
inline counted sqrt(counted a) { g_counts->sqrt++; return counted(::sqrt(a.v)); }
inline counted exp(counted a) { g_counts->trans++; return counted(::exp(a.v)); }
inline counted log(counted a) { g_counts->trans++; return counted(::log(a.v)); }
inline counted cos(counted a) { g_counts->trans++; return counted(::cos(a.v)); }
inline counted sin(counted a) { g_counts->trans++; return counted(::sin(a.v)); }
inline counted pow(counted a, int e) { g_counts->trans++; return counted(::pow(a.v, e)); }

}  // namespace

#define ORACLE_REAL counted
#define ORACLE_OUT(x) ((double)(x))
#include "ccd_oracle_prims.h"

namespace {

struct Job {
  int kind;
  int64_t begin, end;
  const double *x;
  const double *eta;
  int eta_per_test;
  uint8_t *hit;
  double *t;
  uint32_t *flops;
  Counts total;
};

void *worker(void *arg) {
  static const int width[4] = {24, 24, 18, 12};
  Job *jb = static_cast<Job *>(arg);
  memset(&jb->total, 0, sizeof(jb->total));
  for (int64_t i = jb->begin; i < jb->end; i++) {
    Counts c;
    memset(&c, 0, sizeof(c));
    g_counts = &c;
    const double *xi = jb->x + i * width[jb->kind];
    const double e = jb->eta_per_test ? jb->eta[i] : jb->eta[0];
    double t = 0.0;
    int h;
    switch (jb->kind) {
      case 0: h = prim_vf(xi, e, &t); break;
      case 1: h = prim_ee(xi, e, &t); break;
      case 2: h = prim_ve(xi, e, &t); break;
      default: h = prim_vv(xi, e, &t); break;
    }
    g_counts = nullptr;
    if (jb->hit) jb->hit[i] = (uint8_t)h;
    if (jb->t && h) jb->t[i] = t;
    if (jb->flops) {
      const uint64_t f = c.add + c.mul + c.div + c.sqrt;
      jb->flops[i] = f > 0xffffffffull ? 0xffffffffu : (uint32_t)f;
    }
    jb->total.add += c.add;
    jb->total.mul += c.mul;
    jb->total.div += c.div;
    jb->total.sqrt += c.sqrt;
    jb->total.cmp += c.cmp;
    jb->total.trans += c.trans;
  }
  return nullptr;
}

}  // namespace

extern "C" {

// n tests of one kind (0 VF, 1 EE, 2 VE, 3 VV) over rows x, as oracle_batch.
// hit / t (either may be null) receive the oracle's results, flops (may be
// null) each row's add + mul + div + sqrt count, and totals[6] the sums of
// add, mul, div, sqrt, cmp and transcendental calls over all rows.
void oracle_flops_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit,
                        double *t, uint32_t *flops, uint64_t *totals, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  static Job jobs[256];
  pthread_t th[256];
  for (int w = 0; w < nthreads; w++) {
    jobs[w].kind = kind;
    jobs[w].begin = n * w / nthreads;
    jobs[w].end = n * (w + 1) / nthreads;
    jobs[w].x = x;
    jobs[w].eta = eta;
    jobs[w].eta_per_test = eta_per_test;
    jobs[w].hit = hit;
    jobs[w].t = t;
    jobs[w].flops = flops;
  }
  for (int w = 1; w < nthreads; w++) pthread_create(&th[w], nullptr, worker, &jobs[w]);
  worker(&jobs[0]);
  for (int w = 1; w < nthreads; w++) pthread_join(th[w], nullptr);
  for (int k = 0; k < 6; k++) totals[k] = 0;
  for (int w = 0; w < nthreads; w++) {
    totals[0] += jobs[w].total.add;
    totals[1] += jobs[w].total.mul;
    totals[2] += jobs[w].total.div;
    totals[3] += jobs[w].total.sqrt;
    totals[4] += jobs[w].total.cmp;
    totals[5] += jobs[w].total.trans;
  }
}

}  // extern "C"
