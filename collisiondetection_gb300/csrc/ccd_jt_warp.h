// One Jenkins-Traub solve advanced by a whole warp (the slowest solves of a
// batch, which otherwise run alone on one lane of a warp).
//
// The solver state lives in registers, spread over the warp: element i of
// each coefficient array (p, qp, k, qk, the saved k, the unshifted k, the
// roots) sits in lane i, and every lane holds a copy of the scalars.  A read
// of element i is a __shfl_sync from lane i, a write is a move predicated on
// lane i.  The scalar operations run redundantly on every lane -- a warp
// instruction costs the FP64 pipe the same whatever its active lanes, so the
// redundancy is free, and with identical operands every lane takes identical
// branches, so the warp stays converged -- while the operations that do not
// depend on one another run on different lanes at once: element-wise updates
// of the arrays (the next K polynomial, the unshifted K steps, deflation,
// copies) and groups of independent divisions, lane j computing the j-th
// quotient.  Every value is computed by the same operation on the same
// operands as in ccd_jt.h (and the reference, src/rpoly.h), so results are
// bit-identical; only which lane computes what changes.
//
// Division groups of one fixed-shift iteration (rpoly.h:293-382), in
// dependency order, where the sequential code issues twelve:
//   1. next K:     a7 / a1, a3 / a1                    (rpoly.h:601-636)
//   2. scalars:    a / c, d / c, h / c (or a / d, c / d, b / d), and the
//                  iteration's s = -p[n] / k[n-1]       (rpoly.h:566-597, 311)
//   3. estimate:   b1 = -k[n-1] / p[n], and ts = (s - old s) / s
//   4.             b2 = -(k[n-2] + b1 p[n-1]) / p[n]
//   5.             the new u and v corrections over den (rpoly.h:640-675)
//   6.             tv = (v - old v) / v
#pragma once

#include "ccd_jt.h"

namespace ccd {
namespace jt {
namespace warp {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int lane_id() { return (int)(threadIdx.x & 31); }
// Element i of a lane-distributed array.
__device__ __forceinline__ double at(double x, int i) { return __shfl_sync(kFull, x, i); }
// Element i := v.
__device__ __forceinline__ void put(double &x, int i, double v) {
  if (lane_id() == i) x = v;
}

// q[j] = x[j] / y[j] for j < NQ: lane j computes quotient j, every lane
// receives all of them.  Lanes past NQ repeat quotient 0.
template <int NQ>
__device__ __forceinline__ void pdiv(const double (&x)[NQ], const double (&y)[NQ], double (&q)[NQ]) {
  const int lane = lane_id();
  double xn = x[0], yn = y[0];
#pragma unroll
  for (int j = 1; j < NQ; j++)
    if (lane == j) {
      xn = x[j];
      yn = y[j];
    }
  const double r = xn / yn;
#pragma unroll
  for (int j = 0; j < NQ; j++) q[j] = __shfl_sync(kFull, r, j);
}

// The state of one solve (the fields of ccd_jt.h's state, same names).
struct Solve {
  // lane-distributed arrays (element = lane)
  double p, qp, k, qk, svk, temp, zr;
  // scalars, the same in every lane
  double u, v, a, b, c, d, a1, a3, a7, e, f, g, h;
  double bnd, xx, yy;
  double svu, svv, xs, betas, betav, oss, ovv, ots, otv;
  double vv, ss, tv, ts, ui, vi;
  double relstp, omp, rx, rt;
  int mode, n, deg, cnt, j, l2, type, flags, jq, jr, roots, status;

  // Quotient and remainder of src by x^2 + u x + v (jt::divide).
  __device__ __forceinline__ void divide(int nn, double src, double &dst, double uu, double vv_, double &ra, double &rb) const {
    double bb = at(src, 0);
    put(dst, 0, bb);
    double aa = at(src, 1) - bb * uu;
    put(dst, 1, aa);
    for (int i = 2; i <= nn; i++) {
      const double cc = at(src, i) - aa * uu - bb * vv_;
      put(dst, i, cc);
      bb = aa;
      aa = cc;
    }
    ra = aa;
    rb = bb;
  }

  // Scalars for the next K polynomial (jt::scalars); also returns ex / ey in
  // *eq (when eq is not null), a division of the caller's that is
  // independent of these.
  __device__ __forceinline__ int scalars(double ex, double ey, double *eq) {
    divide(n - 1, k, qk, u, v, c, d);
    if (!(fabs(c) > fabs(at(k, n - 1) * 100.0 * kEps)) && !(fabs(d) > fabs(at(k, n - 2) * 100.0 * kEps))) {
      if (eq) *eq = ex / ey;
      return 3;
    }
    double q[4];
    if (fabs(d) < fabs(c)) {
      const double hh = v * b;
      pdiv<4>({a, d, hh, ex}, {c, c, c, ey}, q);
      e = q[0];
      f = q[1];
      g = u * e;
      h = hh;
      if (eq) *eq = q[3];
      a3 = a * e + (q[2] + g) * b;  // q[2] = h / c
      a1 = b - a * f;               // f = d / c
      a7 = a + g * d + h * f;
      return 1;
    }
    const double gg = u * b, hh = v * b;
    pdiv<4>({a, c, b, ex}, {d, d, d, ey}, q);
    e = q[0];
    f = q[1];
    g = gg;
    h = hh;
    if (eq) *eq = q[3];
    a3 = (a + g) * e + h * q[2];  // q[2] = b / d
    a1 = b * f - a;
    a7 = (f + u) * a + h;
    return 2;
  }

  // Next K polynomial (jt::next_k): element-wise, every lane at once.
  __device__ __forceinline__ void next_k(int ty) {
    const int lane = lane_id();
    const double qk2 = __shfl_up_sync(kFull, qk, 2);
    if (ty == 3) {
      if (lane < 2)
        k = 0.0;
      else if (lane < n)
        k = qk2;
      return;
    }
    const double ref = (ty == 1) ? b : a;
    const double qp0 = at(qp, 0), qp1 = __shfl_up_sync(kFull, qp, 1);
    if (fabs(a1) <= fabs(ref) * kEps * 10.0) {
      if (lane == 0)
        k = 0.0;
      else if (lane == 1)
        k = -a7 * qp0;
      else if (lane < n)
        k = a3 * qk2 - a7 * qp1;
      return;
    }
    double q[2];
    pdiv<2>({a7, a3}, {a1, a1}, q);
    a7 = q[0];
    a3 = q[1];
    if (lane == 0)
      k = qp0;
    else if (lane == 1)
      k = qp - a7 * qp0;
    else if (lane < n)
      k = a3 * qk2 - a7 * qp1 + qp;
  }

  // New estimate of the quadratic coefficients (jt::estimate); also returns
  // ex / ey in *eq when eq is not null (unset when ty == 3).
  __device__ __forceinline__ void estimate(int ty, double &uu, double &vv_, double ex, double ey, double *eq) const {
    if (ty == 3) {
      uu = 0.0;
      vv_ = 0.0;
      return;
    }
    double a4, a5;
    if (ty == 2) {
      a4 = (a + g) * f + h;
      a5 = (f + u) * c + v * d;
    } else {
      a4 = a + u * b + h * f;
      a5 = c + (u + v * f) * d;
    }
    const double pn = at(p, n);
    double q[2];
    pdiv<2>({-at(k, n - 1), ex}, {pn, ey}, q);
    const double b1 = q[0];
    if (eq) *eq = q[1];
    const double b2 = -(at(k, n - 2) + b1 * at(p, n - 1)) / pn;
    const double c1 = v * b2 * a1;
    const double c2 = b1 * a7;
    const double c3 = b1 * b1 * a3;
    const double c4 = c1 - c2 - c3;
    const double den = a5 + b1 * a4 - c4;
    if (den == 0.0) {
      uu = 0.0;
      vv_ = 0.0;
      return;
    }
    pdiv<2>({u * (c3 + c2) + v * (b1 * a1 + b2 * a7), c4}, {den, den}, q);
    uu = u - q[0];
    vv_ = v * (1.0 + q[1]);
  }

  // Shift number cnt (jt::begin_shift).
  __device__ __forceinline__ void begin_shift() {
    const double cosr = -0x1.1db902ec147e0p-4;  // cos(94.0 * 0.017453293)
    const double sinr = 0x1.fec0b6fc05f20p-1;   // sin(94.0 * 0.017453293)
    const double xxx = cosr * xx - sinr * yy;
    const double ny = sinr * xx + cosr * yy;
    xx = xxx;
    yy = ny;
    const double sr = bnd * xxx;
    u = -2.0 * sr;
    v = bnd;
    betav = 0.25;
    betas = 0.25;
    oss = sr;
    ovv = bnd;
    ots = 0.0;
    otv = 0.0;
    divide(n, p, qp, u, v, a, b);
    type = scalars(1.0, 1.0, nullptr);
    j = 0;
    l2 = 20 * (cnt + 1);
  }

  __device__ __forceinline__ void begin_quad(double uu, double vv_) {
    relstp = 0.0;
    omp = 0.0;
    flags &= ~kTried;
    u = uu;
    v = vv_;
    jq = 0;
    mode = kQuad;
  }

  __device__ __forceinline__ void begin_real() {
    rx = xs;
    omp = 0.0;
    rt = 0.0;
    jr = 0;
    mode = kReal;
  }

  // Closed forms of the last one or two zeros (jt::finish_low).
  __device__ __forceinline__ void finish_low() {
    if (n == 1) {
      put(zr, deg - 1, -at(p, 1) / at(p, 0));
    } else {
      double si, li, sr, lr;
      quadratic(at(p, 0), at(p, 1), at(p, 2), sr, si, lr, li);
      put(zr, deg - 2, sr);
      put(zr, deg - 1, lr);
    }
    n = 0;
    roots = deg;
    mode = kDone;
  }

  // nz zeros found: store, deflate, next stage (jt::deflate).
  __device__ __forceinline__ void deflate(int nz, double szr, double lzr) {
    const int jpos = deg - n;
    put(zr, jpos, szr);
    n -= nz;
    if (lane_id() <= n) p = qp;
    if (nz != 1) put(zr, jpos + 1, lzr);
    if (n <= 2)
      finish_low();
    else
      mode = kInit;
  }

  __device__ __forceinline__ void end_fixed_iteration() {
    ovv = vv;
    oss = ss;
    otv = tv;
    ots = ts;
    mode = kFixed;
    if (++j < l2) return;
    if (lane_id() < n) k = temp;
    if (++cnt >= 20) {
      roots = deg - n;
      mode = kDone;
      return;
    }
    begin_shift();
  }

  __device__ __forceinline__ void after_tries() {
    u = svu;
    v = svv;
    if (lane_id() < n) k = svk;
    if ((flags & kVpass) && !(flags & kVtried)) {
      begin_quad(ui, vi);
      return;
    }
    divide(n, p, qp, u, v, a, b);
    type = scalars(1.0, 1.0, nullptr);
    end_fixed_iteration();
  }

  __device__ __forceinline__ void quad_failed() {
    flags |= kVtried;
    betav *= 0.25;
    if ((flags & kStried) || !(flags & kSpass)) {
      after_tries();
      return;
    }
    if (lane_id() < n) k = svk;
    begin_real();
  }

  __device__ __forceinline__ void real_failed(bool near_double) {
    flags |= kStried;
    betas *= 0.25;
    if (!near_double) {
      after_tries();
      return;
    }
    ui = -(xs + xs);
    vi = xs * xs;
    begin_quad(ui, vi);
  }

  // Scaling, root bound, unshifted K steps and the first shift
  // (jt::step_init).
  __device__ __forceinline__ void step_init() {
    const int lane = lane_id();
    const double lo = kSmalno / kEps;
    double maxc = 0.0, minc = kInfin, x, xm, ff, df, dx;
    for (int i = 0; i <= n; i++) {
      x = fabs(at(p, i));
      if (x > maxc) maxc = x;
      if (x != 0.0 && x < minc) minc = x;
    }
    double sc = lo / minc;
    const bool keep = (sc > 1.0 && kInfin / sc < maxc) || (sc <= 1.0 && maxc < 10.0);
    if (!keep) {
      if (sc == 0.0) sc = kSmalno;
      const int l = (int)(cr_log(sc) / 0x1.62e42fefa39efp-1 + 0.5);  // log(sc) / log(2.0)
      const double factor = ldexp(1.0, l);                            // pow(2.0, l), exact
      if (factor != 1.0 && lane <= n) p = factor * p;
    }
    double pt = fabs(p);
    if (lane == n) pt = -pt;
    const double pt0 = at(pt, 0), ptn = at(pt, n), ptn1 = at(pt, n - 1);
    x = cr_exp((cr_log(-ptn) - cr_log(pt0)) / (double)n);
    if (ptn1 != 0.0) {
      xm = -ptn / ptn1;
      if (xm < x) x = xm;
    }
    for (int it = 0;; it++) {
      if (it >= kBoundLimit) {
        status |= kStatusRootLimit;
        roots = -1;
        mode = kDone;
        return;
      }
      xm = x * 0.1;
      ff = pt0;
      for (int i = 1; i <= n; i++) ff = ff * xm + at(pt, i);
      if (ff <= 0.0) break;
      x = xm;
    }
    dx = x;
    for (int it = 0; fabs(dx / x) > 0.005; it++) {
      if (it >= kBoundLimit) {
        status |= kStatusRootLimit;
        roots = -1;
        mode = kDone;
        return;
      }
      ff = pt0;
      df = ff;
      for (int i = 1; i < n; i++) {
        const double pti = at(pt, i);
        ff = ff * x + pti;
        df = df * x + ff;
      }
      ff = ff * x + ptn;
      dx = ff / df;
      x -= dx;
    }
    bnd = x;
    // Derivative as the first K polynomial, then five unshifted steps; each
    // step's update k[j] = t k[j-1] + p[j] reads the previous step's k, so
    // every element is computed at once.
    if (lane >= 1 && lane < n) k = (double)(n - lane) * p / (double)n;
    const double p0 = at(p, 0);
    if (lane == 0) k = p0;
    const double aa = at(p, n), bb = at(p, n - 1);
    bool zerok = (at(k, n - 1) == 0);
    for (int jj = 0; jj < 5; jj++) {
      const double cc = at(k, n - 1);
      const double km1 = __shfl_up_sync(kFull, k, 1);
      if (!zerok) {
        const double t = -aa / cc;
        if (lane >= 1 && lane < n) k = t * km1 + p;
        if (lane == 0) k = p0;
        zerok = (fabs(at(k, n - 1)) <= fabs(bb) * kEps * 10.0);
      } else {
        if (lane >= 1 && lane < n) k = km1;
        if (lane == 0) k = 0.0;
        zerok = (at(k, n - 1) == 0.0);
      }
    }
    if (lane < n) temp = k;
    cnt = 0;
    mode = kFixed;
    begin_shift();
  }

  // One fixed-shift iteration (jt::step_fixed).
  __device__ __forceinline__ void step_fixed() {
    int ty = type;
    next_k(ty);
    const double kn1 = at(k, n - 1);
    double sq = 0.0;
    ty = scalars(-at(p, n), kn1, &sq);
    type = ty;
    const double s_ = (kn1 != 0.0) ? sq : 0.0;
    double uu, vv_, tq = 0.0;
    estimate(ty, uu, vv_, s_ - oss, s_, &tq);
    ui = uu;
    vi = vv_;
    double tv_ = 1.0, ts_ = 1.0;
    vv = vv_;
    ss = s_;
    if (j != 0 && ty != 3) {
      if (vv_ != 0.0) tv_ = fabs((vv_ - ovv) / vv_);
      if (s_ != 0.0) ts_ = fabs(tq);
      const double tvv = (tv_ < otv) ? tv_ * otv : 1.0;
      const double tss = (ts_ < ots) ? ts_ * ots : 1.0;
      const bool vpass = tvv < betav, spass = tss < betas;
      tv = tv_;
      ts = ts_;
      if (spass || vpass) {
        svu = u;
        svv = v;
        if (lane_id() < n) svk = k;
        xs = s_;
        flags = (vpass ? kVpass : 0) | (spass ? kSpass : 0);
        if ((spass && !vpass) || tss < tvv)
          begin_real();
        else
          begin_quad(uu, vv_);
        return;
      }
    }
    tv = tv_;
    ts = ts_;
    end_fixed_iteration();
  }

  // One quadratic variable-shift iteration (jt::step_quad).
  __device__ __forceinline__ void step_quad() {
    double uu = u, vv_ = v;
    double szr, szi, lzr, lzi;
    quadratic(1.0, uu, vv_, szr, szi, lzr, lzi);
    if (fabs(fabs(szr) - fabs(lzr)) > 0.01 * fabs(lzr)) {
      quad_failed();
      return;
    }
    divide(n, p, qp, uu, vv_, a, b);
    const double mp = fabs(a - szr * b) + fabs(szi * b);
    const double zm = sqrt(fabs(vv_));
    double ee = 2.0 * fabs(at(qp, 0));
    const double t = -szr * b;
    for (int i = 1; i < n; i++) ee = ee * zm + fabs(at(qp, i));
    ee = ee * zm + fabs(a + t);
    ee *= (5.0 * kEps + 4.0 * kEps);
    ee = ee - (5.0 * kEps + 2.0 * kEps) * (fabs(a + t) + fabs(b) * zm) + 2.0 * kEps * fabs(t);
    if (mp <= 20.0 * ee) {
      deflate(2, szr, lzr);
      return;
    }
    const int jj = ++jq;
    if (jj > 20) {
      quad_failed();
      return;
    }
    double rel = relstp;
    if (jj >= 2 && !(rel > 0.01 || mp < omp || (flags & kTried))) {
      // A cluster stalls convergence: five fixed-shift steps near it.
      if (rel < kEps) rel = kEps;
      rel = sqrt(rel);
      uu = uu - uu * rel;
      vv_ = vv_ + vv_ * rel;
      u = uu;
      v = vv_;
      divide(n, p, qp, uu, vv_, a, b);
      for (int i = 0; i < 5; i++) next_k(scalars(1.0, 1.0, nullptr));
      flags |= kTried;
      jq = 0;
    }
    omp = mp;
    next_k(scalars(1.0, 1.0, nullptr));
    const int ty = scalars(1.0, 1.0, nullptr);
    double un, vn;
    estimate(ty, un, vn, 1.0, 1.0, nullptr);
    if (vn == 0.0) {
      quad_failed();
      return;
    }
    relstp = fabs((vn - vv_) / vn);
    u = un;
    v = vn;
  }

  // One linear variable-shift iteration (jt::step_real).
  __device__ __forceinline__ void step_real() {
    const int lane = lane_id();
    const double x = rx;
    double pv = at(p, 0);
    put(qp, 0, pv);
    for (int i = 1; i <= n; i++) {
      pv = pv * x + at(p, i);
      put(qp, i, pv);
    }
    const double mp = fabs(pv);
    const double ms = fabs(x);
    double ee = (kEps / (kEps + kEps)) * fabs(at(qp, 0));
    for (int i = 1; i <= n; i++) ee = ee * ms + fabs(at(qp, i));
    if (mp <= 20.0 * ((kEps + kEps) * ee - kEps * mp)) {
      deflate(1, x, 0.0);
      return;
    }
    const int jj = ++jr;
    if (jj > 10) {
      real_failed(false);
      return;
    }
    double t = rt;
    if (jj >= 2 && !(fabs(t) > 0.001 * fabs(x - t) || mp < omp)) {
      xs = x;
      real_failed(true);
      return;
    }
    omp = mp;
    double kv = at(k, 0);
    put(qk, 0, kv);
    for (int i = 1; i < n; i++) {
      kv = kv * x + at(k, i);
      put(qk, i, kv);
    }
    const double qkm1 = __shfl_up_sync(kFull, qk, 1);
    if (fabs(kv) <= fabs(at(k, n - 1)) * 10.0 * kEps) {
      if (lane == 0)
        k = 0.0;
      else if (lane < n)
        k = qkm1;
    } else {
      t = -pv / kv;
      if (lane == 0)
        k = qp;
      else if (lane < n)
        k = t * qkm1 + qp;
    }
    kv = at(k, 0);
    for (int i = 1; i < n; i++) kv = kv * x + at(k, i);
    t = 0.0;
    if (fabs(kv) > fabs(at(k, n - 1) * 10.0 * kEps)) t = -pv / kv;
    rt = t;
    rx = x + t;
  }

  // One bounded step of whatever phase the state is in.
  __device__ __forceinline__ void step() {
    switch (mode) {
      case kInit: step_init(); break;
      case kFixed: step_fixed(); break;
      case kQuad: step_quad(); break;
      case kReal: step_real(); break;
      default: break;
    }
  }

  // The state of a solve from a storage policy of ccd_jt.h (every lane
  // calls it with the same state).
  template <class S>
  __device__ __forceinline__ void load(const S &s) {
    const int lane = lane_id();
    p = lane < 7 ? s.D(P + lane) : 0.0;
    qp = lane < 7 ? s.D(QP + lane) : 0.0;
    k = lane < 6 ? s.D(K + lane) : 0.0;
    qk = lane < 6 ? s.D(QK + lane) : 0.0;
    svk = lane < 6 ? s.D(SVK + lane) : 0.0;
    temp = lane < 6 ? s.D(TEMP + lane) : 0.0;
    zr = lane < 6 ? s.Z(lane) : 0.0;
    u = s.D(U), v = s.D(V), a = s.D(A), b = s.D(B), c = s.D(C), d = s.D(DD);
    a1 = s.D(A1), a3 = s.D(A3), a7 = s.D(A7), e = s.D(E), f = s.D(F), g = s.D(G), h = s.D(H);
    bnd = s.D(BND), xx = s.D(XX), yy = s.D(YY);
    svu = s.D(SVU), svv = s.D(SVV), xs = s.D(XS), betas = s.D(BETAS), betav = s.D(BETAV);
    oss = s.D(OSS), ovv = s.D(OVV), ots = s.D(OTS), otv = s.D(OTV);
    vv = s.D(VV), ss = s.D(SS), tv = s.D(TV), ts = s.D(TS), ui = s.D(UI), vi = s.D(VI);
    relstp = s.D(RELSTP), omp = s.D(OMP), rx = s.D(RX), rt = s.D(RT);
    mode = s.I(MODE), n = s.I(N), deg = s.I(DEG), cnt = s.I(CNT), j = s.I(J), l2 = s.I(L2);
    type = s.I(TYPE), flags = s.I(FLAGS), jq = s.I(JQ), jr = s.I(JR), roots = s.I(ROOTS), status = s.I(STATUS);
  }

  // Runs the solve to its end; every lane receives the roots in tr[0 .. 5].
  __device__ __forceinline__ void run(double (&tr)[6]) {
    while (mode != kDone) step();
#pragma unroll
    for (int i = 0; i < 6; i++) tr[i] = at(zr, i);
  }
};

}  // namespace warp
}  // namespace jt
}  // namespace ccd
