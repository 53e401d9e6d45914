// One Jenkins-Traub solve advanced by a whole warp (the slowest solves of a
// batch, which otherwise run alone on one lane of a warp).
//
// Every lane holds the whole solver state in its own storage and executes the
// solve's scalar operations redundantly: a warp instruction costs the FP64
// pipe the same whatever its active lanes, so the redundancy is free, and with
// identical data every lane takes identical branches, so the warp stays
// converged.  The operations that do not depend on one another are spread
// over the lanes instead: lane j computes the j-th of a group of independent
// divisions (one division sequence for the warp instead of several), and lane
// l the (l+2)-th coefficient of the next K polynomial; __shfl_sync hands the
// results to every lane.  Each value is computed by the same operation on the
// same operands as in ccd_jt.h (and the reference, src/rpoly.h), so results
// are bit-identical -- only which lane computes what changes.
//
// Division groups of one fixed-shift iteration (rpoly.h:293-382), in
// dependency order:
//   1. next K:     a7 / a1, a3 / a1                    (rpoly.h:601-636)
//   2. scalars:    a / c, d / c, h / c (or a / d, c / d, b / d), and the
//                  iteration's s = -p[n] / k[n-1]       (rpoly.h:566-597, 311)
//   3. estimate:   b1 = -k[n-1] / p[n], and ts = (s - old s) / s
//   4.             b2 = -(k[n-2] + b1 p[n-1]) / p[n]
//   5.             the new u and v corrections over den (rpoly.h:640-675)
//   6.             tv = (v - old v) / v
// where the sequential code issues twelve.
#pragma once

#include "ccd_jt.h"

namespace ccd {
namespace jt {
namespace warp {

constexpr unsigned kFull = 0xffffffffu;

// q[j] = x[j] / y[j] for j < NQ: lane j computes quotient j, every lane
// receives all of them.  Lanes past NQ repeat quotient 0.
template <int NQ>
__device__ __forceinline__ void pdiv(const double (&x)[NQ], const double (&y)[NQ], double (&q)[NQ]) {
  const int lane = threadIdx.x & 31;
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

// K[i] = a3 * QK[i-2] - a7 * QP[i-1] (+ QP[i] when plus) for 2 <= i < n, one
// coefficient per lane (rpoly.h:619-635).
template <class S>
__device__ __forceinline__ void next_k_tail(S s, int n, double a3, double a7, bool plus) {
  const int lane = threadIdx.x & 31;
  int i = lane + 2;
  if (i >= n) i = 2;  // spare lanes repeat the first coefficient
  double val = a3 * s.D(QK + i - 2) - a7 * s.D(QP + i - 1);
  if (plus) val = val + s.D(QP + i);
  for (int k = 2; k < n; k++) s.D(K + k) = __shfl_sync(kFull, val, k - 2);
}

// Next K polynomial (jt::next_k).
template <class S>
__device__ void next_k(S s, int type) {
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
    warp::next_k_tail(s, n, a3, a7, false);
    return;
  }
  double q[2];
  pdiv<2>({a7, a3}, {a1, a1}, q);
  a7 = q[0];
  a3 = q[1];
  s.D(A7) = a7;
  s.D(A3) = a3;
  s.D(K) = s.D(QP);
  s.D(K + 1) = s.D(QP + 1) - a7 * s.D(QP);
  warp::next_k_tail(s, n, a3, a7, true);
}

// Scalars for the next K polynomial (jt::scalars); also returns ex / ey in
// *eq (when eq is not null), a division of the caller's that is independent
// of these.
template <class S>
__device__ int scalars(S s, double ex, double ey, double *eq) {
  const int n = s.I(N);
  const double u = s.D(U), v = s.D(V);
  divide(s, n - 1, K, QK, u, v, C, DD);
  const double a = s.D(A), b = s.D(B), c = s.D(C), d = s.D(DD);
  if (!(fabs(c) > fabs(s.D(K + n - 1) * 100.0 * kEps)) && !(fabs(d) > fabs(s.D(K + n - 2) * 100.0 * kEps))) {
    if (eq) *eq = ex / ey;
    return 3;
  }
  double q[4];
  if (fabs(d) < fabs(c)) {
    const double h = v * b;
    pdiv<4>({a, d, h, ex}, {c, c, c, ey}, q);
    const double e = q[0], f = q[1], g = u * e;
    if (eq) *eq = q[3];
    s.D(E) = e;
    s.D(F) = f;
    s.D(G) = g;
    s.D(H) = h;
    s.D(A3) = a * e + (q[2] + g) * b;  // q[2] = h / c
    s.D(A1) = b - a * f;               // f = d / c
    s.D(A7) = a + g * d + h * f;
    return 1;
  }
  const double g = u * b, h = v * b;
  pdiv<4>({a, c, b, ex}, {d, d, d, ey}, q);
  const double e = q[0], f = q[1];
  if (eq) *eq = q[3];
  s.D(E) = e;
  s.D(F) = f;
  s.D(G) = g;
  s.D(H) = h;
  s.D(A3) = (a + g) * e + h * q[2];  // q[2] = b / d
  s.D(A1) = b * f - a;
  s.D(A7) = (f + u) * a + h;
  return 2;
}

// New estimate of the quadratic coefficients (jt::estimate); also returns
// ex / ey in *eq when eq is not null (computed with b1; unset when
// type == 3).
template <class S>
__device__ void estimate(S s, int type, double &uu, double &vv, double ex, double ey, double *eq) {
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
  double q[2];
  pdiv<2>({-s.D(K + n - 1), ex}, {pn, ey}, q);
  const double b1 = q[0];
  if (eq) *eq = q[1];
  const double b2 = -(s.D(K + n - 2) + b1 * s.D(P + n - 1)) / pn;
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
  pdiv<2>({u * (c3 + c2) + v * (b1 * a1 + b2 * a7), c4}, {den, den}, q);
  uu = u - q[0];
  vv = v * (1.0 + q[1]);
}

// One fixed-shift iteration (jt::step_fixed).
template <class S>
__device__ void step_fixed(S s) {
  const int n = s.I(N);
  int type = s.I(TYPE);
  warp::next_k(s, type);
  const double kn1 = s.D(K + n - 1);
  double sq = 0.0;
  type = warp::scalars(s, -s.D(P + n), kn1, &sq);
  s.I(TYPE) = type;
  const double ss = (kn1 != 0.0) ? sq : 0.0;
  double ui, vi, tq = 0.0;
  warp::estimate(s, type, ui, vi, ss - s.D(OSS), ss, &tq);
  s.D(UI) = ui;
  s.D(VI) = vi;
  const double vv = vi;
  double tv = 1.0, ts = 1.0;
  s.D(VV) = vv;
  s.D(SS) = ss;
  if (s.I(J) != 0 && type != 3) {
    if (vv != 0.0) tv = fabs((vv - s.D(OVV)) / vv);
    if (ss != 0.0) ts = fabs(tq);
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

// One quadratic variable-shift iteration (jt::step_quad) with the warp's
// next_k / scalars / estimate.
template <class S>
__device__ void step_quad(S s) {
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
    if (relstp < kEps) relstp = kEps;
    relstp = sqrt(relstp);
    u = u - u * relstp;
    v = v + v * relstp;
    s.D(U) = u;
    s.D(V) = v;
    divide(s, n, P, QP, u, v, A, B);
    for (int i = 0; i < 5; i++) warp::next_k(s, warp::scalars(s, 1.0, 1.0, nullptr));
    s.I(FLAGS) |= kTried;
    s.I(JQ) = 0;
  }
  s.D(OMP) = mp;
  warp::next_k(s, warp::scalars(s, 1.0, 1.0, nullptr));
  const int type = warp::scalars(s, 1.0, 1.0, nullptr);
  double ui, vi;
  warp::estimate(s, type, ui, vi, 1.0, 1.0, nullptr);
  if (vi == 0.0) {
    quad_failed(s);
    return;
  }
  s.D(RELSTP) = fabs((vi - v) / vi);
  s.D(U) = ui;
  s.D(V) = vi;
}

// One bounded step of whatever phase the state is in; every lane of the warp
// must call it with the same state.
template <class S>
__device__ void step(S s) {
  switch (s.I(MODE)) {
    case kInit: jt::step_init(s); break;
    case kFixed: warp::step_fixed(s); break;
    case kQuad: warp::step_quad(s); break;
    case kReal: jt::step_real(s); break;
    default: break;
  }
}

}  // namespace warp
}  // namespace jt
}  // namespace ccd
