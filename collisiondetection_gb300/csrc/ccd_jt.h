// Jenkins-Traub real-polynomial root finder as a resumable state machine.
//
// Same numerical steps, constants and iteration limits as the reference's
// vendored C translation of ACM TOMS 493 (src/rpoly.h), with the control flow
// re-expressed as explicit phases so that a solve can be advanced one bounded
// step at a time and its whole state kept outside the executing thread:
//
//   kInit   scale, root-modulus bound (Cauchy polynomial, chop + Newton),
//           derivative K polynomial and five unshifted steps, first shift
//           (rpoly.h:110-224);
//   kFixed  one fixed-shift iteration (rpoly.h:292-382 loop body);
//   kQuad   one variable-shift quadratic iteration (rpoly.h:405-466 body);
//   kReal   one variable-shift linear iteration (rpoly.h:487-557 body);
//   kDone   finished; roots = degree - n (or -1).
//
// Transitions between the phases follow the reference's gotos exactly
// (fixed shift -> quadratic / linear attempts -> restore -> next shift ->
// deflate -> next stage).  The state is accessed through a storage policy S
// (S::D(field) -> double&, S::I(field) -> int&), so the same code runs with
// the state in a thread's local array (sequential driver jt_solve) or in
// shared memory, where a block regroups its slots by phase between steps.
#pragma once

#include "ccd_common.h"
#include "ccd_math.h"

namespace ccd {

namespace jt {

// Double fields: arrays first (indexed at run time), then scalars (always
// indexed by constants, so a thread-private state keeps them in registers).
// The roots themselves are written through S::Z(k).
enum : int {
  P = 0,      // [7] current polynomial
  QP = 7,     // [7] quotient of p
  K = 14,     // [6] K polynomial
  QK = 20,    // [6] quotient of k
  SVK = 26,   // [6] saved K during variable-shift attempts
  TEMP = 32,  // [6] K after the unshifted steps (restored for each new shift)
  kArrays = 38,
  U = kArrays, V, A, B, C, DD, A1, A3, A7, E, F, G, H,  // quadratic factor and scalars of calcsc
  BND, XX, YY,                                          // root bound and shift rotation
  SVU, SVV, XS, BETAS, BETAV, OSS, OVV, OTS, OTV,       // fixed-shift stage
  VV, SS, TV, TS, UI, VI,                               // fixed-shift iteration values
  RELSTP, OMP, RX, RT,                                  // variable-shift iterations
  kDoubles
};
// Integer fields.
enum : int { MODE = 0, N, DEG, CNT, J, L2, TYPE, FLAGS, JQ, JR, ROOTS, STATUS, kInts };
// FLAGS bits.
enum : int { kVpass = 1, kSpass = 2, kVtried = 4, kStried = 8, kTried = 16 };
// Phases.
enum : int { kEmpty = 0, kInit = 1, kFixed = 2, kQuad = 3, kReal = 4, kDone = 5 };
constexpr int kPhases = 6;

constexpr double kEps = 2.22e-16;  // eta = are = mre in the reference
constexpr double kInfin = 3.4e38;
constexpr double kSmalno = 1.2e-38;
constexpr int kBoundLimit = 4096;  // cap on the root-bound loops (endless for non-finite input)

// State private to one thread, and the view the phase functions take.
struct LocalStorage {
  double d[kDoubles];
  double zr[6];
  int i[kInts];
};
struct LocalState {
  LocalStorage *st;
  CCD_HD double &D(int f) const { return st->d[f]; }
  CCD_HD double &Z(int k) const { return st->zr[k]; }
  CCD_HD int &I(int f) const { return st->i[f]; }
};

// State of slot `slot` in a shared pool laid out field-major: field f of all
// POOL slots is contiguous, so any thread can advance any slot.
// The roots go to zr (global memory, stride zstride).
template <int POOL>
struct PoolState {
  double *d;
  int *i;
  int slot;
  double *zr;
  int64_t zstride;
  CCD_HD double &D(int f) const { return d[f * POOL + slot]; }
  CCD_HD double &Z(int k) const { return zr[k * zstride]; }
  CCD_HD int &I(int f) const { return i[f * POOL + slot]; }
};

// State of job `g` in a field-major global array of `stride` jobs: field f of
// all jobs is contiguous, so a warp advancing neighbouring jobs touches
// neighbouring words.  The roots go to zr (stride zstride).
struct FieldState {
  double *d;
  int *i;
  int64_t g, stride;
  double *zr;
  int64_t zstride;
  CCD_HD double &D(int f) const { return d[f * stride + g]; }
  CCD_HD double &Z(int k) const { return zr[k * zstride]; }
  CCD_HD int &I(int f) const { return i[f * stride + g]; }
};

// Every division of the solver's phases calls one out-of-line copy of the
// division sequence: the pool kernel runs every phase's code in the warps of
// one SM at once, and stalls most on instruction fetch; one shared copy in
// place of 30-odd inline ones measured 10% off the two-sphere step and 3-4%
// off the headline batch.  The quotient is the IEEE one, as inline.
CCD_NOINLINE double jt_div(double a, double b) { return a / b; }
#define JT_DIV(a, b) jt_div((a), (b))

// ---------------------------------------------------------------- primitives
// Quotient and remainder of p by x^2 + u x + v  (rpoly.h:680-695).
template <class S>
CCD_NOINLINE void divide(S s, int nn, int src, int dst, double u, double v, int ra, int rb) {
  double bb = s.D(src);
  s.D(dst) = bb;
  double aa = s.D(src + 1) - bb * u;
  s.D(dst + 1) = aa;
  for (int i = 2; i <= nn; i++) {
    double cc = s.D(src + i) - aa * u - bb * v;
    s.D(dst + i) = cc;
    bb = aa;
    aa = cc;
  }
  s.D(ra) = aa;
  s.D(rb) = bb;
}

// Zeros of a z^2 + b1 z + c  (rpoly.h:702-754).
CCD_NOINLINE void quadratic(double a, double b1, double c, double &sr, double &si, double &lr, double &li) {
  if (a == 0.0) {
    sr = (b1 != 0.0) ? JT_DIV(-c, b1) : 0.0;
    lr = 0.0;
    si = 0.0;
    li = 0.0;
    return;
  }
  if (c == 0.0) {
    sr = 0.0;
    lr = JT_DIV(-b1, a);
    si = 0.0;
    li = 0.0;
    return;
  }
  double b = b1 / 2.0, d, e;
  if (fabs(b) < fabs(c)) {
    e = (c < 0.0) ? -a : a;
    e = b * JT_DIV(b, fabs(c)) - e;
    d = sqrt(fabs(e)) * sqrt(fabs(c));
  } else {
    e = 1.0 - JT_DIV(a, b) * JT_DIV(c, b);
    d = sqrt(fabs(e)) * fabs(b);
  }
  if (e < 0.0) {
    sr = JT_DIV(-b, a);
    lr = sr;
    si = fabs(JT_DIV(d, a));
    li = -si;
  } else {
    if (b >= 0.0) d = -d;
    lr = JT_DIV(-b + d, a);
    sr = 0.0;
    if (lr != 0.0) sr = JT_DIV(JT_DIV(c, lr), a);
    si = 0.0;
    li = 0.0;
  }
}

// Scalars for the next K polynomial; returns its type  (rpoly.h:566-597).
template <class S>
CCD_NOINLINE int scalars(S s) {
  const int n = s.I(N);
  const double u = s.D(U), v = s.D(V);
  divide(s, n - 1, K, QK, u, v, C, DD);
  const double a = s.D(A), b = s.D(B), c = s.D(C), d = s.D(DD);
  if (!(fabs(c) > fabs(s.D(K + n - 1) * 100.0 * kEps)) && !(fabs(d) > fabs(s.D(K + n - 2) * 100.0 * kEps))) return 3;
  if (fabs(d) < fabs(c)) {
    const double e = JT_DIV(a, c), f = JT_DIV(d, c), g = u * e, h = v * b;
    s.D(E) = e;
    s.D(F) = f;
    s.D(G) = g;
    s.D(H) = h;
    s.D(A3) = a * e + (JT_DIV(h, c) + g) * b;
    s.D(A1) = b - a * JT_DIV(d, c);
    s.D(A7) = a + g * d + h * f;
    return 1;
  }
  const double e = JT_DIV(a, d), f = JT_DIV(c, d), g = u * b, h = v * b;
  s.D(E) = e;
  s.D(F) = f;
  s.D(G) = g;
  s.D(H) = h;
  s.D(A3) = (a + g) * e + h * JT_DIV(b, d);
  s.D(A1) = b * f - a;
  s.D(A7) = (f + u) * a + h;
  return 2;
}

// Next K polynomial  (rpoly.h:601-636).
template <class S>
CCD_NOINLINE void next_k(S s, int type) {
  const int n = s.I(N);
  if (type == 3) {
    s.D(K) = 0.0;
    s.D(K + 1) = 0.0;
    for (int i = 2; i < n; i++) s.D(K + i) = s.D(QK + i - 2);
    return;
  }
  const double ref = (type == 1) ? s.D(B) : s.D(A);
  double a1 = s.D(A1), a3 = s.D(A3), a7 = s.D(A7);
  if (fabs(a1) <= fabs(ref) * kEps * 10.0) {
    s.D(K) = 0.0;
    s.D(K + 1) = -a7 * s.D(QP);
    for (int i = 2; i < n; i++) s.D(K + i) = a3 * s.D(QK + i - 2) - a7 * s.D(QP + i - 1);
    return;
  }
  a7 = JT_DIV(a7, a1);
  a3 = JT_DIV(a3, a1);
  s.D(A7) = a7;
  s.D(A3) = a3;
  s.D(K) = s.D(QP);
  s.D(K + 1) = s.D(QP + 1) - a7 * s.D(QP);
  for (int i = 2; i < n; i++) s.D(K + i) = a3 * s.D(QK + i - 2) - a7 * s.D(QP + i - 1) + s.D(QP + i);
}

// New estimate of the quadratic coefficients  (rpoly.h:640-675).
template <class S>
CCD_NOINLINE void estimate(S s, int type, double &uu, double &vv) {
  if (type == 3) {
    uu = 0.0;
    vv = 0.0;
    return;
  }
  const int n = s.I(N);
  const double u = s.D(U), v = s.D(V), a = s.D(A), b = s.D(B), c = s.D(C), d = s.D(DD);
  const double f = s.D(F), g = s.D(G), h = s.D(H), a1 = s.D(A1), a3 = s.D(A3), a7 = s.D(A7);
  double a4, a5;
  if (type == 2) {
    a4 = (a + g) * f + h;
    a5 = (f + u) * c + v * d;
  } else {
    a4 = a + u * b + h * f;
    a5 = c + (u + v * f) * d;
  }
  const double pn = s.D(P + n);
  const double b1 = JT_DIV(-s.D(K + n - 1), pn);
  const double b2 = JT_DIV(-(s.D(K + n - 2) + b1 * s.D(P + n - 1)), pn);
  const double c1 = v * b2 * a1;
  const double c2 = b1 * a7;
  const double c3 = b1 * b1 * a3;
  const double c4 = c1 - c2 - c3;
  const double den = a5 + b1 * a4 - c4;
  if (den == 0.0) {
    uu = 0.0;
    vv = 0.0;
    return;
  }
  uu = u - JT_DIV(u * (c3 + c2) + v * (b1 * a1 + b2 * a7), den);
  vv = v * (1.0 + JT_DIV(c4, den));
}

// ---------------------------------------------------------------- transitions
// The shift point rotated by 94 degrees (rpoly.h:217-220).
template <class S>
CCD_HD void rotate_shift(S s) {
  const double cosr = -0x1.1db902ec147e0p-4;  // cos(94.0 * 0.017453293)
  const double sinr = 0x1.fec0b6fc05f20p-1;   // sin(94.0 * 0.017453293)
  const double xx = s.D(XX), yy = s.D(YY);
  const double xxx = cosr * xx - sinr * yy;
  const double ny = sinr * xx + cosr * yy;
  s.D(XX) = xxx;
  s.D(YY) = ny;
}

// Shift number CNT: rotate the shift point and start the fixed-shift stage
// (rpoly.h:217-224 and 284-291).
template <class S>
CCD_NOINLINE void begin_shift(S s) {
  rotate_shift(s);
  const double bnd = s.D(BND);
  const double sr = bnd * s.D(XX);
  s.D(U) = -2.0 * sr;
  s.D(V) = bnd;
  s.D(BETAV) = 0.25;
  s.D(BETAS) = 0.25;
  s.D(OSS) = sr;
  s.D(OVV) = bnd;
  s.D(OTS) = 0.0;
  s.D(OTV) = 0.0;
  divide(s, s.I(N), P, QP, s.D(U), s.D(V), A, B);
  s.I(TYPE) = scalars(s);
  s.I(J) = 0;
  s.I(L2) = 20 * (s.I(CNT) + 1);
}

template <class S>
CCD_HD void begin_quad(S s, double uu, double vv) {
  s.D(RELSTP) = 0.0;
  s.D(OMP) = 0.0;
  s.I(FLAGS) &= ~kTried;
  s.D(U) = uu;
  s.D(V) = vv;
  s.I(JQ) = 0;
  s.I(MODE) = kQuad;
}

template <class S>
CCD_HD void begin_real(S s) {
  s.D(RX) = s.D(XS);
  s.D(OMP) = 0.0;
  s.D(RT) = 0.0;
  s.I(JR) = 0;
  s.I(MODE) = kReal;
}

// Quadratic p(z) = p0 z^2 + p1 z + p2 or linear remainder: closed forms
// (rpoly.h:97-108); finishes the solve.
template <class S>
CCD_HD void finish_low(S s) {
  const int n = s.I(N), deg = s.I(DEG);
  if (n == 1) {
    s.Z(deg - 1) = JT_DIV(-s.D(P + 1), s.D(P));
  } else {
    double si, li, sr, lr;
    quadratic(s.D(P), s.D(P + 1), s.D(P + 2), sr, si, lr, li);
    s.Z(deg - 2) = sr;
    s.Z(deg - 1) = lr;
  }
  s.I(N) = 0;
  s.I(ROOTS) = deg;
  s.I(MODE) = kDone;
}

// nz zeros found (szr, and lzr when nz == 2): store them, deflate, and
// continue with the next stage (rpoly.h:225-241).
template <class S>
CCD_HD void deflate(S s, int nz, double szr, double lzr) {
  const int deg = s.I(DEG);
  int n = s.I(N);
  const int jpos = deg - n;
  s.Z(jpos) = szr;
  n -= nz;
  s.I(N) = n;
  for (int i = 0; i <= n; i++) s.D(P + i) = s.D(QP + i);
  if (nz != 1) s.Z(jpos + 1) = lzr;
  if (n <= 2)
    finish_low(s);
  else
    s.I(MODE) = kInit;
}

// End of a fixed-shift iteration (rpoly.h:377-381), then the next iteration,
// or a new shift when this one is exhausted (rpoly.h:246-249).
template <class S>
CCD_HD void end_fixed_iteration(S s) {
  s.D(OVV) = s.D(VV);
  s.D(OSS) = s.D(SS);
  s.D(OTV) = s.D(TV);
  s.D(OTS) = s.D(TS);
  s.I(MODE) = kFixed;
  if (++s.I(J) < s.I(L2)) return;
  const int n = s.I(N);
  for (int i = 0; i < n; i++) s.D(K + i) = s.D(TEMP + i);
  if (++s.I(CNT) >= 20) {  // no convergence with 20 shifts
    s.I(ROOTS) = s.I(DEG) - n;
    s.I(MODE) = kDone;
    return;
  }
  begin_shift(s);
}

// Both variable-shift iterations have been tried or ruled out: restore the
// fixed-shift state (rpoly.h:362-376).
template <class S>
CCD_NOINLINE void after_tries(S s) {
  const int n = s.I(N);
  s.D(U) = s.D(SVU);
  s.D(V) = s.D(SVV);
  for (int i = 0; i < n; i++) s.D(K + i) = s.D(SVK + i);
  const int fl = s.I(FLAGS);
  if ((fl & kVpass) && !(fl & kVtried)) {
    begin_quad(s, s.D(UI), s.D(VI));
    return;
  }
  divide(s, n, P, QP, s.D(U), s.D(V), A, B);
  s.I(TYPE) = scalars(s);
  end_fixed_iteration(s);
}

template <class S>
CCD_HD void quad_failed(S s) {  // rpoly.h:334-345
  s.I(FLAGS) |= kVtried;
  s.D(BETAV) *= 0.25;
  const int fl = s.I(FLAGS);
  if ((fl & kStried) || !(fl & kSpass)) {
    after_tries(s);
    return;
  }
  const int n = s.I(N);
  for (int i = 0; i < n; i++) s.D(K + i) = s.D(SVK + i);
  begin_real(s);
}

template <class S>
CCD_HD void real_failed(S s, bool near_double) {  // rpoly.h:348-360
  s.I(FLAGS) |= kStried;
  s.D(BETAS) *= 0.25;
  if (!near_double) {
    after_tries(s);
    return;
  }
  const double xs = s.D(XS);
  s.D(UI) = -(xs + xs);
  s.D(VI) = xs * xs;
  begin_quad(s, s.D(UI), s.D(VI));
}

// ---------------------------------------------------------------- phases
// Start of a solve on op (degree >= 3 after the caller's degree reduction):
// zeros at the origin and the closed forms (rpoly.h:71-109).
template <class S>
CCD_HD void start(S s, const double *op, int degree) {
  s.I(DEG) = degree;
  s.I(STATUS) = 0;
  s.I(ROOTS) = -1;
  s.D(XX) = 0x1.6a09e667f3bcdp-1;  // sqrt(0.5)
  s.D(YY) = -0x1.6a09e667f3bcdp-1;
  s.I(MODE) = kDone;
  int n = degree;
  if (op[0] == 0.0) return;
  while (op[n] == 0.0) {
    s.Z(degree - n) = 0.0;
    n--;
  }
  if (n < 1) return;
  s.I(N) = n;
  for (int i = 0; i <= n; i++) s.D(P + i) = op[i];
  if (n <= 2)
    finish_low(s);
  else
    s.I(MODE) = kInit;
}

// Scaling, root bound, unshifted K steps and the first shift
// (rpoly.h:110-224).  A bound loop that hits its cap ends the solve with -1
// and kStatusRootLimit.
template <class S>
CCD_NOINLINE void step_init(S s) {
  const int n = s.I(N);
  const double lo = kSmalno / kEps;
  double maxc = 0.0, minc = kInfin, x, xm, ff, df, dx;
  for (int i = 0; i <= n; i++) {
    x = fabs(s.D(P + i));
    if (x > maxc) maxc = x;
    if (x != 0.0 && x < minc) minc = x;
  }
  double sc = JT_DIV(lo, minc);
  const bool keep = (sc > 1.0 && JT_DIV(kInfin, sc) < maxc) || (sc <= 1.0 && maxc < 10.0);
  if (!keep) {
    if (sc == 0.0) sc = kSmalno;
    const int l = (int)(cr_log(sc) / 0x1.62e42fefa39efp-1 + 0.5);  // log(sc) / log(2.0)
    const double factor = ldexp(1.0, l);                            // pow(2.0, l), exact
    if (factor != 1.0)
      for (int i = 0; i <= n; i++) s.D(P + i) = factor * s.D(P + i);
  }
  double pt[7];
  for (int i = 0; i <= n; i++) pt[i] = fabs(s.D(P + i));
  pt[n] = -pt[n];
  x = cr_exp((cr_log(-pt[n]) - cr_log(pt[0])) / (double)n);
  if (pt[n - 1] != 0.0) {
    xm = JT_DIV(-pt[n], pt[n - 1]);
    if (xm < x) x = xm;
  }
  for (int it = 0;; it++) {
    if (it >= kBoundLimit) {
      s.I(STATUS) |= kStatusRootLimit;
      s.I(ROOTS) = -1;
      s.I(MODE) = kDone;
      return;
    }
    xm = x * 0.1;
    ff = pt[0];
    for (int i = 1; i <= n; i++) ff = ff * xm + pt[i];
    if (ff <= 0.0) break;
    x = xm;
  }
  dx = x;
  for (int it = 0; fabs(JT_DIV(dx, x)) > 0.005; it++) {
    if (it >= kBoundLimit) {
      s.I(STATUS) |= kStatusRootLimit;
      s.I(ROOTS) = -1;
      s.I(MODE) = kDone;
      return;
    }
    ff = pt[0];
    df = ff;
    for (int i = 1; i < n; i++) {
      ff = ff * x + pt[i];
      df = df * x + ff;
    }
    ff = ff * x + pt[n];
    dx = JT_DIV(ff, df);
    x -= dx;
  }
  s.D(BND) = x;
  // Derivative as the first K polynomial, then five unshifted steps.
  const int nm1 = n - 1;
  for (int i = 1; i < n; i++) s.D(K + i) = JT_DIV((double)(n - i) * s.D(P + i), (double)n);
  s.D(K) = s.D(P);
  const double aa = s.D(P + n), bb = s.D(P + n - 1);
  bool zerok = (s.D(K + n - 1) == 0);
  for (int jj = 0; jj < 5; jj++) {
    const double cc = s.D(K + n - 1);
    if (!zerok) {
      const double t = JT_DIV(-aa, cc);
      for (int i = 0; i < nm1; i++) {
        const int j = n - i - 1;
        s.D(K + j) = t * s.D(K + j - 1) + s.D(P + j);
      }
      s.D(K) = s.D(P);
      zerok = (fabs(s.D(K + n - 1)) <= fabs(bb) * kEps * 10.0);
    } else {
      for (int i = 0; i < nm1; i++) {
        const int j = n - i - 1;
        s.D(K + j) = s.D(K + j - 1);
      }
      s.D(K) = 0.0;
      zerok = (s.D(K + n - 1) == 0.0);
    }
  }
  for (int i = 0; i < n; i++) s.D(TEMP + i) = s.D(K + i);
  s.I(CNT) = 0;
  s.I(MODE) = kFixed;
  begin_shift(s);
}

// One fixed-shift iteration (rpoly.h:293-382).
template <class S>
CCD_NOINLINE void step_fixed(S s) {
  const int n = s.I(N);
  int type = s.I(TYPE);
  next_k(s, type);
  type = scalars(s);
  s.I(TYPE) = type;
  double ui, vi;
  estimate(s, type, ui, vi);
  s.D(UI) = ui;
  s.D(VI) = vi;
  const double vv = vi;
  double ss = 0.0;
  const double kn1 = s.D(K + n - 1);
  if (kn1 != 0.0) ss = JT_DIV(-s.D(P + n), kn1);
  double tv = 1.0, ts = 1.0;
  s.D(VV) = vv;
  s.D(SS) = ss;
  if (s.I(J) != 0 && type != 3) {
    if (vv != 0.0) tv = fabs(JT_DIV(vv - s.D(OVV), vv));
    if (ss != 0.0) ts = fabs(JT_DIV(ss - s.D(OSS), ss));
    const double otv = s.D(OTV), ots = s.D(OTS);
    const double tvv = (tv < otv) ? tv * otv : 1.0;
    const double tss = (ts < ots) ? ts * ots : 1.0;
    const bool vpass = tvv < s.D(BETAV), spass = tss < s.D(BETAS);
    s.D(TV) = tv;
    s.D(TS) = ts;
    if (spass || vpass) {
      s.D(SVU) = s.D(U);
      s.D(SVV) = s.D(V);
      for (int i = 0; i < n; i++) s.D(SVK + i) = s.D(K + i);
      s.D(XS) = ss;
      s.I(FLAGS) = (vpass ? kVpass : 0) | (spass ? kSpass : 0);
      if ((spass && !vpass) || tss < tvv)
        begin_real(s);
      else
        begin_quad(s, ui, vi);
      return;
    }
  }
  s.D(TV) = tv;
  s.D(TS) = ts;
  end_fixed_iteration(s);
}

// One quadratic variable-shift iteration (rpoly.h:405-466).
template <class S>
CCD_NOINLINE void step_quad(S s) {
  const int n = s.I(N);
  double u = s.D(U), v = s.D(V);
  double szr, szi, lzr, lzi;
  quadratic(1.0, u, v, szr, szi, lzr, lzi);
  if (fabs(fabs(szr) - fabs(lzr)) > 0.01 * fabs(lzr)) {
    quad_failed(s);
    return;
  }
  divide(s, n, P, QP, u, v, A, B);
  const double a = s.D(A), b = s.D(B);
  const double mp = fabs(a - szr * b) + fabs(szi * b);
  const double zm = sqrt(fabs(v));
  double ee = 2.0 * fabs(s.D(QP));
  const double t = -szr * b;
  for (int i = 1; i < n; i++) ee = ee * zm + fabs(s.D(QP + i));
  ee = ee * zm + fabs(a + t);
  ee *= (5.0 * kEps + 4.0 * kEps);
  ee = ee - (5.0 * kEps + 2.0 * kEps) * (fabs(a + t) + fabs(b) * zm) + 2.0 * kEps * fabs(t);
  if (mp <= 20.0 * ee) {
    deflate(s, 2, szr, lzr);
    return;
  }
  const int j = ++s.I(JQ);
  if (j > 20) {
    quad_failed(s);
    return;
  }
  double relstp = s.D(RELSTP);
  if (j >= 2 && !(relstp > 0.01 || mp < s.D(OMP) || (s.I(FLAGS) & kTried))) {
    // A cluster stalls convergence: five fixed-shift steps near it.
    if (relstp < kEps) relstp = kEps;
    relstp = sqrt(relstp);
    u = u - u * relstp;
    v = v + v * relstp;
    s.D(U) = u;
    s.D(V) = v;
    divide(s, n, P, QP, u, v, A, B);
    for (int i = 0; i < 5; i++) next_k(s, scalars(s));
    s.I(FLAGS) |= kTried;
    s.I(JQ) = 0;
  }
  s.D(OMP) = mp;
  next_k(s, scalars(s));
  const int type = scalars(s);
  double ui, vi;
  estimate(s, type, ui, vi);
  if (vi == 0.0) {
    quad_failed(s);
    return;
  }
  s.D(RELSTP) = fabs(JT_DIV(vi - v, vi));
  s.D(U) = ui;
  s.D(V) = vi;
}

// One linear variable-shift iteration (rpoly.h:487-557).
template <class S>
CCD_NOINLINE void step_real(S s) {
  const int n = s.I(N);
  const double x = s.D(RX);
  double pv = s.D(P);
  s.D(QP) = pv;
  for (int i = 1; i <= n; i++) {
    pv = pv * x + s.D(P + i);
    s.D(QP + i) = pv;
  }
  const double mp = fabs(pv);
  const double ms = fabs(x);
  double ee = (kEps / (kEps + kEps)) * fabs(s.D(QP));
  for (int i = 1; i <= n; i++) ee = ee * ms + fabs(s.D(QP + i));
  if (mp <= 20.0 * ((kEps + kEps) * ee - kEps * mp)) {
    deflate(s, 1, x, 0.0);
    return;
  }
  const int j = ++s.I(JR);
  if (j > 10) {
    real_failed(s, false);
    return;
  }
  double t = s.D(RT);
  if (j >= 2 && !(fabs(t) > 0.001 * fabs(x - t) || mp < s.D(OMP))) {
    s.D(XS) = x;
    real_failed(s, true);
    return;
  }
  s.D(OMP) = mp;
  double kv = s.D(K);
  s.D(QK) = kv;
  for (int i = 1; i < n; i++) {
    kv = kv * x + s.D(K + i);
    s.D(QK + i) = kv;
  }
  if (fabs(kv) <= fabs(s.D(K + n - 1)) * 10.0 * kEps) {
    s.D(K) = 0.0;
    for (int i = 1; i < n; i++) s.D(K + i) = s.D(QK + i - 1);
  } else {
    t = JT_DIV(-pv, kv);
    s.D(K) = s.D(QP);
    for (int i = 1; i < n; i++) s.D(K + i) = t * s.D(QK + i - 1) + s.D(QP + i);
  }
  kv = s.D(K);
  for (int i = 1; i < n; i++) kv = kv * x + s.D(K + i);
  t = 0.0;
  if (fabs(kv) > fabs(s.D(K + n - 1) * 10.0 * kEps)) t = JT_DIV(-pv, kv);
  s.D(RT) = t;
  s.D(RX) = x + t;
}

// One bounded step of whatever phase the state is in.
template <class S>
CCD_HD void step(S s) {
  switch (s.I(MODE)) {
    case kInit: step_init(s); break;
    case kFixed: step_fixed(s); break;
    case kQuad: step_quad(s); break;
    case kReal: step_real(s); break;
    default: break;
  }
}

}  // namespace jt

// Sequential driver: the whole solve in one thread (rpoly.h:49-261).
// Returns the number of zeros found (real parts in zr), or -1.
CCD_NOINLINE int jt_solve(const double *op, int degree, double *zr, uint8_t &status) {
  jt::LocalStorage storage;
  const jt::LocalState s{&storage};
  jt::start(s, op, degree);
  while (s.I(jt::MODE) != jt::kDone) jt::step(s);
  for (int i = 0; i < degree; i++) zr[i] = s.Z(i);
  status |= (uint8_t)s.I(jt::STATUS);
  return s.I(jt::ROOTS);
}

}  // namespace ccd
