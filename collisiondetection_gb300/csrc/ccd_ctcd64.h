// FP64 continuous-time collision tests, op-for-op with the reference
// (evouga/collisiondetection src/CTCD.cpp and src/rpoly.h).
//
// Every expression keeps the reference's evaluation order with one IEEE
// rounding per operation (no contraction: see ccd_common.h).  Vector algebra
// follows the Eigen contract: dot = (a0*b0 + a1*b1) + a2*b2, cross = component
// formula.  The only departures are
//  * exp/log in the root bound are correctly rounded (ccd_math.h) where the
//    reference calls the host C library;
//  * cos/sin of the constant 94-degree shift rotation are folded to constants;
//  * the two root-bound loops that never end on non-finite coefficients
//    (src/rpoly.h:151-158, 163-173) are capped; hitting the cap sets
//    kStatusRootLimit and reports the polynomial as having no roots
//    (ccd_jt.h).
#pragma once

#include "ccd_common.h"
#include "ccd_math.h"
#include "ccd_jt.h"

namespace ccd {

// ------------------------------------------------------------------ 3-vectors
struct v3d {
  double x, y, z;
};
CCD_HD v3d ld3(const double *p) { return v3d{p[0], p[1], p[2]}; }
CCD_HD v3d operator+(v3d a, v3d b) { return v3d{a.x + b.x, a.y + b.y, a.z + b.z}; }
CCD_HD v3d operator-(v3d a, v3d b) { return v3d{a.x - b.x, a.y - b.y, a.z - b.z}; }
CCD_HD v3d operator*(double s, v3d a) { return v3d{s * a.x, s * a.y, s * a.z}; }
CCD_HD double dot(v3d a, v3d b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
CCD_HD v3d cross(v3d a, v3d b) {
  return v3d{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
CCD_HD double norm(v3d a) { return sqrt(dot(a, a)); }

// ------------------------------------------------------------------ time spans
// TimeInterval (include/CTCD.h:7-26): endpoints ordered, clamped to [0,1].
struct Span {
  double l, u;
};
CCD_HD Span make_span(double a, double b) {
  if (a > b) {
    double t = a;
    a = b;
    b = t;
  }
  return Span{smax(a, 0.0), smin(b, 1.0)};
}
CCD_HD bool meet(Span a, Span b) { return !(a.l > b.u || b.l > a.u); }

// At most deg+1 <= 7 segments come out of one polynomial.
struct SpanList {
  int n;
  Span s[7];
  CCD_HD void clear() { n = 0; }
  CCD_HD void push(double a, double b) { s[n++] = make_span(a, b); }
};

// Overlap / intersection over a fixed set of spans (TimeInterval::overlap and
// ::intersect, src/CTCD.cpp:15-36).
template <int K>
CCD_HD bool all_meet(const Span (&s)[K]) {
CCD_UNROLL
  for (int i = 0; i < K; i++)
CCD_UNROLL
    for (int j = i + 1; j < K; j++)
      if (!meet(s[i], s[j])) return false;
  return true;
}
template <int K>
CCD_HD double common_lo(const Span (&s)[K]) {
  double l = 0.0;
CCD_UNROLL
  for (int i = 0; i < K; i++) l = smax(s[i].l, l);
  return l;
}

// ------------------------------------------------------------------ quadratics
// CTCD::getQuadRoots (src/CTCD.cpp:38-56).
CCD_HD int quad_roots(double a, double b, double c, double &t0, double &t1) {
  int sign = (b < 0) ? -1 : 1;
  double disc = b * b - 4 * a * c;
  if (disc >= 0) {
    double q = -0.5 * (b + sign * sqrt(disc));
    t0 = q / a;
    t1 = c / q;
    if (t0 > t1) {
      double t = t0;
      t0 = t1;
      t1 = t;
    }
    return 2;
  }
  return 0;
}

// CTCD::checkInterval (src/CTCD.cpp:59-79).
CCD_HD void keep_if_sign(double t1, double t2, const double *op, int degree, SpanList &out, bool want_pos) {
  t1 = smax(0.0, t1);
  t2 = smax(0.0, t2);
  t1 = smin(1.0, t1);
  t2 = smin(1.0, t2);
  double tm = (t2 + t1) / 2;
  double f = op[0];
  for (int i = 1; i <= degree; i++) {
    f *= tm;
    f += op[i];
  }
  if (want_pos ? (f >= 0) : (f <= 0)) out.push(t1, t2);
}

// CTCD::couldHaveRoots (src/CTCD.cpp:81-94).
CCD_HD bool sign_possible(const double *op, int degree, bool want_pos) {
  double acc = 0;
  if (want_pos ? (op[0] > 0) : (op[0] < 0)) acc = op[0];
  for (int i = 1; i < degree; i++) {
    acc *= 1.0;
    if (want_pos ? (op[i] > 0) : (op[i] < 0)) acc += op[i];
  }
  acc *= 1.0;
  acc += op[degree];
  return !(want_pos ? (acc < 0) : (acc > 0));
}

// std::sort on <= 16 doubles in libstdc++ is an insertion sort; the same
// permutation is reproduced for root lists that contain NaN.
CCD_HD void sort_roots(double *a, int n) {
  for (int i = 1; i < n; i++) {
    double v = a[i];
    if (v < a[0]) {
      for (int j = i; j > 0; j--) a[j] = a[j - 1];
      a[0] = v;
    } else {
      int j = i;
      while (v < a[j - 1]) {
        a[j] = a[j - 1];
        j--;
      }
      a[j] = v;
    }
  }
}

// ------------------------------------------------------------------ Jenkins-Traub
// The root finder (src/rpoly.h) lives in ccd_jt.h as a resumable state
// machine; jt_solve runs it to completion in one thread.

// ------------------------------------------------------------------ sign intervals
// CTCD::findIntervals (src/CTCD.cpp:98-177), in three pieces so that the
// staged kernels can run the root finder as a separate job:
//   reduce_poly   normalise by max|c| and drop exactly-zero leading terms;
//   low_degree_spans / root_spans   the two ways the spans are produced.

// Normalises op (degree n) in place and returns the reduced degree.
CCD_HD int reduce_poly(double *op, int n) {
  int deg = n;
  double maxval = 0;
  for (int i = 0; i <= n; i++) maxval = smax(maxval, fabs(op[i]));
  if (maxval != 0)
    for (int i = 0; i <= n; i++) op[i] /= maxval;
  for (int i = 0; i < n; i++) {
    if (op[i] == 0)
      deg--;
    else
      break;
  }
  if (deg < n)
    for (int i = 0; i <= deg; i++) op[i] = op[i + n - deg];
  return deg;
}

// Spans from `roots` real root parts tr (unsorted; roots <= 0: none found).
CCD_HD void root_spans(const double *op, int deg, double *tr, int roots, SpanList &out, bool want_pos) {
  if (roots > 0) {
    sort_roots(tr, roots);
    if (tr[0] >= 0) keep_if_sign(0, tr[0], op, deg, out, want_pos);
    for (int i = 0; i < roots - 1; i++)
      if (!((tr[i] < 0 && tr[i + 1] < 0) || (tr[i] > 1.0 && tr[i + 1] > 1.0)))
        keep_if_sign(tr[i], tr[i + 1], op, deg, out, want_pos);
    if (tr[roots - 1] <= 1.0) keep_if_sign(tr[roots - 1], 1.0, op, deg, out, want_pos);
  } else {
    keep_if_sign(0.0, 1.0, op, deg, out, want_pos);
  }
}

// Spans of a reduced polynomial of degree <= 2.
CCD_HD void low_degree_spans(const double *op, int deg, SpanList &out, bool want_pos) {
  double tr[2];
  int roots;
  if (deg == 2) {
    roots = quad_roots(op[0], op[1], op[2], tr[0], tr[1]);
  } else if (deg == 1) {
    tr[0] = -op[1] / op[0];
    roots = 1;
  } else {
    if (want_pos ? (op[0] >= 0) : (op[0] <= 0)) out.push(0, 1.0);
    return;
  }
  root_spans(op, deg, tr, roots, out, want_pos);
}

// Full findIntervals on op (degree n <= 6), normalised in place.
CCD_NOINLINE void sign_spans(double *op, int n, SpanList &out, bool want_pos, uint8_t &status) {
  int deg = reduce_poly(op, n);
  if (deg > 2) {
    if (!sign_possible(op, deg, want_pos)) return;
    double tr[6];
    int roots = jt_solve(op, deg, tr, status);
    root_spans(op, deg, tr, roots, out, want_pos);
  } else {
    low_degree_spans(op, deg, out, want_pos);
  }
}

// ------------------------------------------------------------------ polynomials
// Coefficients (descending powers) exactly as the reference forms them.

// CTCD::barycentricPoly3D (src/CTCD.cpp:179-213), quartic, want_pos.
CCD_HD void bary_coeffs(v3d x10, v3d x20, v3d x30, v3d v10, v3d v20, v3d v30, double *op) {
  double A = dot(x10, x10);
  double B = 2 * dot(x10, v10);
  double C = dot(v10, v10);
  double D = dot(x20, x10);
  double E = dot(x20, v10) + dot(v20, x10);
  double F = dot(v20, v10);
  double G = dot(x30, x20);
  double H = dot(x30, v20) + dot(v30, x20);
  double I = dot(v30, v20);
  double J = dot(x30, x10);
  double K = dot(x30, v10) + dot(v30, x10);
  double L = dot(v30, v10);
  op[0] = F * L - C * I;
  op[1] = F * K + E * L - C * H - B * I;
  op[2] = F * J + D * L + E * K - C * G - A * I - B * H;
  op[3] = D * K + E * J - A * H - B * G;
  op[4] = D * J - A * G;
}

// CTCD::planePoly3D (src/CTCD.cpp:215-229), cubic, want_pos.
CCD_HD void plane_coeffs(v3d x10, v3d x20, v3d x30, v3d v10, v3d v20, v3d v30, double *op) {
  v3d vv = cross(v20, v30);
  op[0] = dot(v10, vv);
  op[1] = dot(x10, vv) + dot(v10, cross(x20, v30)) + dot(v10, cross(v20, x30));
  op[2] = dot(x10, cross(x20, v30)) + dot(x10, cross(v20, x30)) + dot(v10, cross(x20, x30));
  op[3] = dot(x10, cross(x20, x30));
}

// CTCD::distancePoly3D (src/CTCD.cpp:231-257), sextic, want_neg.
CCD_HD void dist_coeffs(v3d x10, v3d x20, v3d x30, v3d v10, v3d v20, v3d v30, double minD, double *op) {
  v3d G = cross(v20, v30);
  v3d xv = cross(x20, v30), vx = cross(v20, x30);
  v3d E = cross(x20, x30);
  double A = dot(v10, G);
  double B = dot(x10, G) + dot(v10, xv) + dot(v10, vx);
  double C = dot(x10, xv) + dot(x10, vx) + dot(v10, E);
  double D = dot(x10, E);
  v3d F = xv + vx;
  op[0] = A * A;
  op[1] = 2 * A * B;
  op[2] = B * B + 2 * A * C - dot(G, G) * minD;
  op[3] = 2 * A * D + 2 * B * C - 2 * dot(G, F) * minD;
  op[4] = 2 * B * D + C * C - (2 * dot(G, E) + dot(F, F)) * minD;
  op[5] = 2 * C * D - 2 * dot(F, E) * minD;
  op[6] = D * D - dot(E, E) * minD;
}

// The polynomials of one vertex-face row (src/CTCD.cpp:423-472): slots 0-2 are
// the three edge-side cubics (want >= 0), slot 3 the distance sextic (want <= 0).
// x: q0s..q3s q0e..q3e.
struct VFPolys {
  static constexpr int kSlots = 4;
  static CCD_HD int degree(int slot) { return slot < 3 ? 3 : 6; }
  static CCD_HD bool want_pos(int slot) { return slot < 3; }
  static CCD_HD void coeffs(const double *x, double eta, int slot, double *op) {
    v3d q0s = ld3(x), q1s = ld3(x + 3), q2s = ld3(x + 6), q3s = ld3(x + 9);
    v3d v0 = ld3(x + 12) - q0s, v1 = ld3(x + 15) - q1s, v2 = ld3(x + 18) - q2s, v3 = ld3(x + 21) - q3s;
    if (slot == 0)
      plane_coeffs(q0s - q1s, cross(q3s - q1s, q2s - q1s), q3s - q1s, v0 - v1, cross(v3 - v1, v2 - v1), v3 - v1, op);
    else if (slot == 1)
      plane_coeffs(q0s - q2s, cross(q1s - q2s, q3s - q2s), q1s - q2s, v0 - v2, cross(v1 - v2, v3 - v2), v1 - v2, op);
    else if (slot == 2)
      plane_coeffs(q0s - q3s, cross(q2s - q3s, q1s - q3s), q2s - q3s, v0 - v3, cross(v2 - v3, v1 - v3), v2 - v3, op);
    else
      dist_coeffs(q0s - q1s, q2s - q1s, q3s - q1s, v0 - v1, v2 - v1, v3 - v1, eta * eta, op);
  }
};

// The polynomials of one edge-edge row (src/CTCD.cpp:270-350): slot 0 the
// distance sextic (want <= 0), slots 1-4 the barycentric quartics a0 a1 b0 b1.
// x: q0s p0s q1s p1s q0e p0e q1e p1e.
struct EEPolys {
  static constexpr int kSlots = 5;
  static CCD_HD int degree(int slot) { return slot == 0 ? 6 : 4; }
  static CCD_HD bool want_pos(int slot) { return slot != 0; }
  static CCD_HD void coeffs(const double *x, double eta, int slot, double *op) {
    v3d q0s = ld3(x), p0s = ld3(x + 3), q1s = ld3(x + 6), p1s = ld3(x + 9);
    v3d vp0 = ld3(x + 15) - p0s, vp1 = ld3(x + 21) - p1s, vq0 = ld3(x + 12) - q0s, vq1 = ld3(x + 18) - q1s;
    if (slot == 0)
      dist_coeffs(p0s - p1s, p0s - q0s, p1s - q1s, vp0 - vp1, vp0 - vq0, vp1 - vq1, eta * eta, op);
    else if (slot == 1)
      bary_coeffs(p1s - q1s, p0s - q0s, q0s - q1s, vp1 - vq1, vp0 - vq0, vq0 - vq1, op);
    else if (slot == 2)
      bary_coeffs(p1s - q1s, q0s - p0s, p0s - q1s, vp1 - vq1, vq0 - vp0, vp0 - vq1, op);
    else if (slot == 3)
      bary_coeffs(p0s - q0s, p1s - q1s, q1s - q0s, vp0 - vq0, vp1 - vq1, vq1 - vq0, op);
    else
      bary_coeffs(p0s - q0s, q1s - p1s, p1s - q0s, vp0 - vq0, vq1 - vp1, vp1 - vq0, op);
  }
};

// ------------------------------------------------------------------ interval logic
// Final decision of vertexFaceCTCD from its four lists (src/CTCD.cpp:477-507).
CCD_HD bool vf_combine(const SpanList &e1, const SpanList &e2, const SpanList &e3, const SpanList &cop,
                       double &tout) {
  if (e1.n == 0 || e2.n == 0 || e3.n == 0 || cop.n == 0) return false;
  bool hit = false;
  double mint = 1.0;
  for (int i = 0; i < cop.n; i++)
    for (int j = 0; j < e1.n; j++)
      for (int k = 0; k < e2.n; k++)
        for (int l = 0; l < e3.n; l++) {
          Span set[4] = {cop.s[i], e1.s[j], e2.s[k], e3.s[l]};
          if (all_meet(set)) {
            mint = smin(common_lo(set), mint);
            hit = true;
          }
        }
  if (hit) tout = mint;
  return hit;
}

// Splits the distance spans of an edge-edge row into non-parallel (cop) and
// parallel ones (src/CTCD.cpp:291-308).
CCD_HD void ee_split_parallel(const double *x, const SpanList &raw, SpanList &cop, SpanList &par) {
  v3d q0s = ld3(x), p0s = ld3(x + 3), q1s = ld3(x + 6), p1s = ld3(x + 9);
  v3d vp0 = ld3(x + 15) - p0s, vp1 = ld3(x + 21) - p1s, vq0 = ld3(x + 12) - q0s, vq1 = ld3(x + 18) - q1s;
  cop.clear();
  par.clear();
  for (int i = 0; i < raw.n; i++) {
    double midt = (raw.s[i].u + raw.s[i].l) / 2;
    v3d e0 = (q0s - p0s) + midt * (vq0 - vp0);
    v3d e1 = (q1s - p1s) + midt * (vq1 - vp1);
    if (norm(cross(e0, e1)) < 1e-8)
      par.s[par.n++] = raw.s[i];
    else
      cop.s[cop.n++] = raw.s[i];
  }
}

// Final decision of edgeEdgeCTCD (src/CTCD.cpp:310-410).
CCD_HD bool ee_combine(const SpanList &cop, const SpanList &par, const SpanList &a0, const SpanList &a1,
                       const SpanList &b0, const SpanList &b1, double &tout) {
  if (cop.n == 0 || a0.n == 0 || a1.n == 0 || b0.n == 0 || b1.n == 0) return false;
  bool hit = false;
  double mint = 1.0;
  for (int i = 0; i < cop.n; i++)
    for (int j = 0; j < a0.n; j++)
      for (int k = 0; k < a1.n; k++)
        for (int l = 0; l < b0.n; l++)
          for (int m = 0; m < b1.n; m++) {
            Span set[5] = {cop.s[i], a0.s[j], a1.s[k], b0.s[l], b1.s[m]};
            if (!all_meet(set)) continue;
            Span isect{common_lo(set), 1.0};
            double u = 1.0;
            for (int q = 0; q < 5; q++) u = smin(set[q].u, u);
            isect.u = u;
            bool skip = false;
            for (int q = 0; q < par.n; q++)
              if (meet(isect, par.s[q])) {
                skip = true;
                break;
              }
            if (!skip) {
              mint = smin(mint, isect.l);
              hit = true;
            }
          }
  if (hit) tout = mint;
  return hit;
}

// ------------------------------------------------------------------ primitive tests
// One thread per row, with the reference's early exits.

// CTCD::edgeEdgeCTCD (src/CTCD.cpp:259-411).  x: q0s p0s q1s p1s q0e p0e q1e p1e.
CCD_HDI inline bool ee_ctcd(const double *x, double eta, double &tout, uint8_t &status) {
  SpanList raw, cop, par, l[4];
  double op[7];
  EEPolys::coeffs(x, eta, 0, op);
  raw.clear();
  sign_spans(op, 6, raw, false, status);
  ee_split_parallel(x, raw, cop, par);
  if (cop.n == 0) return false;
  for (int s = 0; s < 4; s++) {
    EEPolys::coeffs(x, eta, s + 1, op);
    l[s].clear();
    sign_spans(op, 4, l[s], true, status);
    if (l[s].n == 0) return false;
  }
  return ee_combine(cop, par, l[0], l[1], l[2], l[3], tout);
}

// CTCD::vertexFaceCTCD (src/CTCD.cpp:413-508).  x: q0s..q3s q0e..q3e.
CCD_HDI inline bool vf_ctcd(const double *x, double eta, double &tout, uint8_t &status) {
  SpanList l[4];
  double op[7];
  for (int s = 0; s < 4; s++) {
    VFPolys::coeffs(x, eta, s, op);
    l[s].clear();
    sign_spans(op, VFPolys::degree(s), l[s], VFPolys::want_pos(s), status);
    if (l[s].n == 0) return false;
  }
  return vf_combine(l[0], l[1], l[2], l[3], tout);
}

// CTCD::vertexEdgeCTCD (src/CTCD.cpp:511-602).  x: q0s q1s q2s q0e q1e q2e.
CCD_HDI inline bool ve_ctcd(const double *x, double eta, double &tout, uint8_t &status) {
  v3d q0s = ld3(x), q1s = ld3(x + 3), q2s = ld3(x + 6);
  double minD = eta * eta;
  v3d v0 = ld3(x + 9) - q0s, v1 = ld3(x + 12) - q1s, v2 = ld3(x + 15) - q2s;
  v3d ab = q2s - q1s, ac = q0s - q1s, cb = q2s - q0s;
  v3d vab = v2 - v1, vac = v0 - v1, vcb = v2 - v0;
  SpanList colin, e1, e2;
  double op[5];
  op[0] = dot(vab, vac);
  op[1] = dot(ac, vab) + dot(ab, vac);
  op[2] = dot(ab, ac);
  e1.clear();
  sign_spans(op, 2, e1, true, status);
  if (e1.n == 0) return false;
  op[0] = dot(vab, vcb);
  op[1] = dot(cb, vab) + dot(ab, vcb);
  op[2] = dot(ab, cb);
  e2.clear();
  sign_spans(op, 2, e2, true, status);
  if (e2.n == 0) return false;
  double A = dot(ab, ab);
  double B = 2 * dot(ab, vab);
  double C = dot(vab, vab);
  double D = dot(ac, ac);
  double E = 2 * dot(ac, vac);
  double F = dot(vac, vac);
  double G = dot(ac, ab);
  double H = dot(vab, ac) + dot(vac, ab);
  double I = dot(vab, vac);
  op[4] = A * D - G * G - minD * A;
  op[3] = B * D + A * E - 2 * G * H - minD * B;
  op[2] = B * E + A * F + C * D - H * H - 2 * G * I - minD * C;
  op[1] = B * F + C * E - 2 * H * I;
  op[0] = C * F - I * I;
  colin.clear();
  sign_spans(op, 4, colin, false, status);
  if (colin.n == 0) return false;
  bool hit = false;
  double mint = 1.0;
  for (int i = 0; i < colin.n; i++)
    for (int j = 0; j < e1.n; j++)
      for (int k = 0; k < e2.n; k++) {
        Span set[3] = {colin.s[i], e1.s[j], e2.s[k]};
        if (all_meet(set)) {
          mint = smin(common_lo(set), mint);
          hit = true;
        }
      }
  if (hit) tout = mint;
  return hit;
}

// CTCD::vertexVertexCTCD (src/CTCD.cpp:604-692).  x: q1s q2s q1e q2e.  The
// reported time is the raw root and may lie outside [0,1].
CCD_HDI inline bool vv_ctcd(const double *x, double eta, double &tout) {
  v3d q1s = ld3(x), q2s = ld3(x + 3);
  v3d v1 = ld3(x + 6) - q1s, v2 = ld3(x + 9) - q2s;
  double min_d = eta * eta;
  double t1 = 0, t2 = 0;
  int roots;
  double a = dot(v1, v1) + dot(v2, v2) - 2 * dot(v1, v2);
  double b = 2 * (dot(v1, q1s) - dot(v2, q1s) - dot(v1, q2s) + dot(v2, q2s));
  double c = dot(q1s, q1s) + dot(q2s, q2s) - 2 * dot(q1s, q2s) - min_d;
  if (a != 0) {
    roots = quad_roots(a, b, c, t1, t2);
  } else if (b != 0) {
    t1 = -c / b;
    roots = 1;
  } else {
    if (c <= 0) {
      tout = 0;
      return true;
    }
    return false;
  }
  double op[3] = {a, b, c};
  SpanList iv;
  iv.clear();
  if (roots == 2) {
    keep_if_sign(0, t1, op, 2, iv, false);
    if (iv.n) { tout = 0; return true; }
    keep_if_sign(t1, t2, op, 2, iv, false);
    if (iv.n) { tout = t1; return true; }
    keep_if_sign(t2, 1.0, op, 2, iv, false);
    if (iv.n) { tout = t2; return true; }
    return false;
  }
  if (roots == 1) {
    keep_if_sign(0, t1, op, 2, iv, false);
    if (iv.n) { tout = 0; return true; }
    keep_if_sign(t1, 1.0, op, 2, iv, false);
    if (iv.n) { tout = t1; return true; }
    return false;
  }
  keep_if_sign(0, 1.0, op, 2, iv, false);
  if (iv.n) { tout = 0; return true; }
  return false;
}

}  // namespace ccd
