// Conservative FP32 rejection for the vertex-face, edge-edge and vertex-edge
// tests.
//
// The reference returns "no collision" as soon as one of its interval lists
// is empty (src/CTCD.cpp:441-475 for vertex-face, 310-350 for edge-edge).  A
// list is empty when the reference's FP64 evaluation of its polynomial has
// the wrong sign at every sample point in [0,1] (checkInterval samples
// segment midpoints; couldHaveRoots only removes segments).  This stage
// proves that in FP32:
//
//  * each polynomial coefficient is computed in FP32 along the reference's own
//    expression tree, together with m = the same tree over absolute values
//    (subtractions become additions).  With k <= 14 roundings on any path,
//    |fl32(c) - c| <= gamma_14 * m < 1.0e-6 * m (standard running-error bound);
//  * the reference's own FP64 coefficient and Horner errors are below
//    4e-15 * sum(m) for t in [0,1] -- folded into the margin;
//  * the sign over [0,1] is bounded by the Bernstein coefficients of the
//    polynomial: min_j b_j <= p(t) <= max_j b_j.
//
// Degree-6 distance test: the reference's sextic is D(t)^2 - eta^2 |N(t)|^2
// with D the exact coplanarity cubic and N the moving normal.  If D is bounded
// away from zero, |D| >= L > 0 on [0,1], and L^2 exceeds eta^2 max|N|^2 plus
// the FP64 error bound, the sextic is positive everywhere and its (<= 0)
// interval list is empty.
//
// Every rejection test is a strict comparison that is false for NaN, and all
// bounds are checked for finiteness, so non-finite input is never rejected.
#pragma once

#include "ccd_common.h"

namespace ccd {

// FP32 value with the absolute-value expression bound alongside it.
struct fb {
  float v, m;
};
CCD_HD fb fb_in(double x) {
  float f = (float)x;
  return fb{f, fabsf(f)};
}
CCD_HD fb operator+(fb a, fb b) { return fb{a.v + b.v, a.m + b.m}; }
CCD_HD fb operator-(fb a, fb b) { return fb{a.v - b.v, a.m + b.m}; }
CCD_HD fb operator*(fb a, fb b) { return fb{a.v * b.v, a.m * b.m}; }
CCD_HD fb scale(float s, fb a) { return fb{s * a.v, fabsf(s) * a.m}; }  // exact for s = 2

struct v3f {
  fb x, y, z;
};

// The reference's difference vectors are formed in FP64 (positions minus
// positions, velocities minus velocities) before any product.  The stage
// forms the same FP64 differences, operation for operation, and rounds them
// to FP32 only then: its error bounds are relative to the differences
// themselves, not to the absolute coordinates (with coordinates near 1 and
// edges near 0.01, bounds built from rounded coordinates would exceed the
// quantities they bound).
struct d3 {
  double x, y, z;
};
CCD_HD d3 ld3d(const double *p) { return d3{p[0], p[1], p[2]}; }
CCD_HD d3 operator-(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
CCD_HD v3f f3(d3 a) { return v3f{fb_in(a.x), fb_in(a.y), fb_in(a.z)}; }
CCD_HD v3f operator-(v3f a, v3f b) { return v3f{a.x - b.x, a.y - b.y, a.z - b.z}; }
CCD_HD v3f operator+(v3f a, v3f b) { return v3f{a.x + b.x, a.y + b.y, a.z + b.z}; }
CCD_HD fb dotf(v3f a, v3f b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
CCD_HD v3f crossf(v3f a, v3f b) {
  return v3f{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Relative margin on sum(m): FP32 coefficient error (gamma_14 < 8.4e-7), the
// Bernstein combination's own rounding (< 6 * 2^-24 * sum|a|) and the
// reference's FP64 error (< 4e-15), with headroom.
constexpr float kRelSlack = 1.5e-6f;
constexpr float kAbsSlack = 1e-35f;  // covers FP32 gradual underflow
constexpr float kFinite = 3.0e38f;

// Bernstein extrema over [0,1] of a polynomial given by FP32 coefficients in
// the reference's order (op[0] = highest power).  Returns false when the
// slack-widened bounds are not finite.
template <int N>
CCD_HD bool bern_range(const fb (&op)[N + 1], float &lo, float &hi, float &slack) {
  float a[N + 1];  // ascending powers
  float s = 0.0f;
CCD_UNROLL
  for (int i = 0; i <= N; i++) {
    a[i] = op[N - i].v;
    s += op[N - i].m;
  }
  float b[N + 1];
  if (N == 2) {
    b[0] = a[0];
    b[1] = a[0] + a[1] * 0.5f;
    b[N] = a[0] + a[1] + a[N];
  } else if (N == 3) {
    b[0] = a[0];
    b[1] = a[0] + a[1] * (1.0f / 3.0f);
    b[2] = a[0] + a[1] * (2.0f / 3.0f) + a[2] * (1.0f / 3.0f);
    b[3] = a[0] + a[1] + a[2] + a[3];
  } else {  // N == 4
    b[0] = a[0];
    b[1] = a[0] + a[1] * 0.25f;
    b[2] = a[0] + a[1] * 0.5f + a[2] * (1.0f / 6.0f);
    b[3] = a[0] + a[1] * 0.75f + a[2] * 0.5f + a[3] * 0.25f;
    b[N] = a[0] + a[1] + a[2] + a[3] + a[N];
  }
  lo = b[0];
  hi = b[0];
CCD_UNROLL
  for (int j = 1; j <= N; j++) {
    lo = fminf(lo, b[j]);
    hi = fmaxf(hi, b[j]);
  }
  slack = kRelSlack * s + kAbsSlack;
  return fabsf(lo) < kFinite && fabsf(hi) < kFinite && slack < kFinite && s == s && lo == lo && hi == hi;
}

// True when the polynomial is provably < 0 at every point of [0,1] in the
// reference's own FP64 evaluation ("want >= 0" list is empty).
template <int N>
CCD_HD bool surely_negative(const fb (&op)[N + 1]) {
  float lo, hi, slack;
  if (!bern_range<N>(op, lo, hi, slack)) return false;
  return hi + slack < 0.0f;
}

// True when the reference's distance sextic D^2 - minD |N|^2 is provably > 0
// on [0,1] ("want <= 0" list is empty).  D: coplanarity cubic (reference
// order), N(t) = G t^2 + F t + E.
CCD_HD bool surely_apart(const fb (&D)[4], v3f E, v3f F, v3f G, double minD) {
  float lo, hi, slack;
  if (!bern_range<3>(D, lo, hi, slack)) return false;
  float L;
  if (lo - slack > 0.0f)
    L = lo - slack;
  else if (hi + slack < 0.0f)
    L = -(hi + slack);
  else
    return false;
  float sD = D[0].m + D[1].m + D[2].m + D[3].m;
  float nb = (E.x.m + E.y.m + E.z.m) + (F.x.m + F.y.m + F.z.m) + (G.x.m + G.y.m + G.z.m);
  float md = (float)(minD > 1e-30 ? minD : 1e-30) * 1.00001f;
  float lhs = (L * L) * 0.99999f;
  float rhs = (md * (nb * nb)) * 1.00001f + 1e-14f * (sD * sD) + 1e-37f;
  if (!(fabsf(rhs) < kFinite) || !(fabsf(lhs) < kFinite)) return false;
  return lhs > rhs;
}

// Coplanarity cubic of the reference's distancePoly3D (src/CTCD.cpp:240-246)
// plus the normal polynomial N(t) = E + F t + G t^2.
CCD_HD void dist_terms(v3f x10, v3f x20, v3f x30, v3f v10, v3f v20, v3f v30, fb (&D)[4], v3f &E, v3f &F,
                       v3f &G) {
  G = crossf(v20, v30);
  v3f xv = crossf(x20, v30), vx = crossf(v20, x30);
  E = crossf(x20, x30);
  D[0] = dotf(v10, G);
  D[1] = dotf(x10, G) + dotf(v10, xv) + dotf(v10, vx);
  D[2] = dotf(x10, xv) + dotf(x10, vx) + dotf(v10, E);
  D[3] = dotf(x10, E);
  F = xv + vx;
}

// planePoly3D cubic (src/CTCD.cpp:215-229).
CCD_HD void plane_terms(v3f x10, v3f x20, v3f x30, v3f v10, v3f v20, v3f v30, fb (&op)[4]) {
  v3f vv = crossf(v20, v30);
  op[0] = dotf(v10, vv);
  op[1] = dotf(x10, vv) + dotf(v10, crossf(x20, v30)) + dotf(v10, crossf(v20, x30));
  op[2] = dotf(x10, crossf(x20, v30)) + dotf(x10, crossf(v20, x30)) + dotf(v10, crossf(x20, x30));
  op[3] = dotf(x10, crossf(x20, x30));
}

// barycentricPoly3D quartic (src/CTCD.cpp:179-213).
CCD_HD void bary_terms(v3f x10, v3f x20, v3f x30, v3f v10, v3f v20, v3f v30, fb (&op)[5]) {
  fb A = dotf(x10, x10);
  fb B = scale(2.0f, dotf(x10, v10));
  fb C = dotf(v10, v10);
  fb D = dotf(x20, x10);
  fb E = dotf(x20, v10) + dotf(v20, x10);
  fb F = dotf(v20, v10);
  fb G = dotf(x30, x20);
  fb H = dotf(x30, v20) + dotf(v30, x20);
  fb I = dotf(v30, v20);
  fb J = dotf(x30, x10);
  fb K = dotf(x30, v10) + dotf(v30, x10);
  fb L = dotf(v30, v10);
  op[0] = F * L - C * I;
  op[1] = F * K + E * L - C * H - B * I;
  op[2] = F * J + D * L + E * K - C * G - A * I - B * H;
  op[3] = D * K + E * J - A * H - B * G;
  op[4] = D * J - A * G;
}

// True when vertexFaceCTCD(x, eta) is provably false.  x: as vf_ctcd.
CCD_HD bool vf_rejects(const double *x, double eta) {
  if (!(fabs(eta) < 1e300)) return false;
  const d3 q0s = ld3d(x), q1s = ld3d(x + 3), q2s = ld3d(x + 6), q3s = ld3d(x + 9);
  const d3 v0 = ld3d(x + 12) - q0s, v1 = ld3d(x + 15) - q1s, v2 = ld3d(x + 18) - q2s, v3 = ld3d(x + 21) - q3s;
  fb op[4];
  // src/CTCD.cpp:428-435, 443-449, 455-461
  plane_terms(f3(q0s - q1s), crossf(f3(q3s - q1s), f3(q2s - q1s)), f3(q3s - q1s), f3(v0 - v1),
              crossf(f3(v3 - v1), f3(v2 - v1)), f3(v3 - v1), op);
  if (surely_negative<3>(op)) return true;
  plane_terms(f3(q0s - q2s), crossf(f3(q1s - q2s), f3(q3s - q2s)), f3(q1s - q2s), f3(v0 - v2),
              crossf(f3(v1 - v2), f3(v3 - v2)), f3(v1 - v2), op);
  if (surely_negative<3>(op)) return true;
  plane_terms(f3(q0s - q3s), crossf(f3(q2s - q3s), f3(q1s - q3s)), f3(q2s - q3s), f3(v0 - v3),
              crossf(f3(v2 - v3), f3(v1 - v3)), f3(v2 - v3), op);
  if (surely_negative<3>(op)) return true;
  fb D[4];
  v3f E, F, G;
  // src/CTCD.cpp:466-472
  dist_terms(f3(q0s - q1s), f3(q2s - q1s), f3(q3s - q1s), f3(v0 - v1), f3(v2 - v1), f3(v3 - v1), D, E, F, G);
  return surely_apart(D, E, F, G, eta * eta);
}

// True when edgeEdgeCTCD(x, eta) is provably false.  x: as ee_ctcd.
CCD_HD bool ee_rejects(const double *x, double eta) {
  if (!(fabs(eta) < 1e300)) return false;
  const d3 q0s = ld3d(x), p0s = ld3d(x + 3), q1s = ld3d(x + 6), p1s = ld3d(x + 9);
  const d3 vq0 = ld3d(x + 12) - q0s, vp0 = ld3d(x + 15) - p0s, vq1 = ld3d(x + 18) - q1s, vp1 = ld3d(x + 21) - p1s;
  fb D[4];
  v3f E, F, G;
  // src/CTCD.cpp:274-286
  dist_terms(f3(p0s - p1s), f3(p0s - q0s), f3(p1s - q1s), f3(vp0 - vp1), f3(vp0 - vq0), f3(vp1 - vq1), D, E, F, G);
  if (surely_apart(D, E, F, G, eta * eta)) return true;
  fb op[5];
  // src/CTCD.cpp:313-346
  v3f x10 = f3(p1s - q1s), v10 = f3(vp1 - vq1);
  bary_terms(x10, f3(p0s - q0s), f3(q0s - q1s), v10, f3(vp0 - vq0), f3(vq0 - vq1), op);
  if (surely_negative<4>(op)) return true;
  bary_terms(x10, f3(q0s - p0s), f3(p0s - q1s), v10, f3(vq0 - vp0), f3(vp0 - vq1), op);
  if (surely_negative<4>(op)) return true;
  x10 = f3(p0s - q0s);
  v10 = f3(vp0 - vq0);
  bary_terms(x10, f3(p1s - q1s), f3(q1s - q0s), v10, f3(vp1 - vq1), f3(vq1 - vq0), op);
  if (surely_negative<4>(op)) return true;
  bary_terms(x10, f3(q1s - p1s), f3(p1s - q0s), v10, f3(vq1 - vp1), f3(vp1 - vq0), op);
  return surely_negative<4>(op);
}

// Lower bound of |X(t)|^2 over t in [a, a + h] for the vector quadratic
// X(t) = X0 + X1 t + X2 t^2, or -1 when none is found.  For n = X(mid),
// |X(t)| >= |n.X(t)| / |n|; n.X(t) is a scalar quadratic, re-expanded in
// s = (t - a) / h in FP32 with running error bounds and bounded by its
// Bernstein coefficients.  a and h are exact binary fractions.
CCD_HD float cross_lower_sq(v3f X0, v3f X1, v3f X2, float a, float h) {
  const float mid = a + 0.5f * h;
  const float nx = X0.x.v + mid * (X1.x.v + mid * X2.x.v);
  const float ny = X0.y.v + mid * (X1.y.v + mid * X2.y.v);
  const float nz = X0.z.v + mid * (X1.z.v + mid * X2.z.v);
  const v3f n{fb{nx, fabsf(nx)}, fb{ny, fabsf(ny)}, fb{nz, fabsf(nz)}};
  const fb c0 = dotf(n, X0), c1 = dotf(n, X1), c2 = dotf(n, X2);
  const fb A{a, a}, H{h, h}, H2{h * h, h * h};
  const fb d0 = c0 + (c1 + c2 * A) * A;       // q(a)
  const fb d1 = (c1 + scale(2.0f, c2 * A)) * H;  // h q'(a)
  const fb d2 = c2 * H2;                       // h^2 q''/2
  const float b0 = d0.v, b1 = d0.v + 0.5f * d1.v, b2 = (d0.v + d1.v) + d2.v;
  const float lo = fminf(b0, fminf(b1, b2)), hi = fmaxf(b0, fmaxf(b1, b2));
  // At most 20 roundings on any path (gamma_20 < 1.2e-6) plus the Bernstein
  // combination's own (< 3 * 2^-24 of the magnitudes), with headroom.
  const float slack = 3e-6f * ((d0.m + d1.m) + d2.m) + kAbsSlack;
  float L;
  if (lo - slack > 0.0f)
    L = lo - slack;
  else if (hi + slack < 0.0f)
    L = -(hi + slack);
  else
    return -1.0f;
  const float nn = ((nx * nx + ny * ny) + nz * nz) * 1.00001f;  // >= |n|^2
  if (!(nn > 0.0f) || !(nn < kFinite) || !(slack < kFinite) || !(L < kFinite)) return -1.0f;
  return ((L * L) / nn) * 0.99999f;
}

// True when vertexEdgeCTCD(x, eta) is provably false (src/CTCD.cpp:511-602).
// x: q0s q1s q2s q0e q1e q2e (q0 = vertex, edge q1-q2).
//
// The two "between the endpoints" quadratics are tested like the other
// sign lists.  The quartic is the reference's expansion of
// A(t) D(t) - G(t)^2 - eta^2 A(t) with A = |ab|^2, D = |ac|^2, G = ab.ac, which
// equals |X(t)|^2 - eta^2 |ab(t)|^2 with X(t) = ab(t) x ac(t) (Lagrange's
// identity).  |X(t)|^2 is bounded from below on each quarter of [0,1]
// (cross_lower_sq); the row is rejected when every bound exceeds
// eta^2 max|ab(t)|^2 plus the reference's own FP64 error bound on the quartic
// (its "<= 0" list is then empty).
CCD_HD bool ve_rejects(const double *x, double eta) {
  if (!(fabs(eta) < 1e300)) return false;
  const d3 q0s = ld3d(x), q1s = ld3d(x + 3), q2s = ld3d(x + 6);
  const d3 v0 = ld3d(x + 9) - q0s, v1 = ld3d(x + 12) - q1s, v2 = ld3d(x + 15) - q2s;
  // src/CTCD.cpp:521-534
  const v3f ab = f3(q2s - q1s), ac = f3(q0s - q1s), cb = f3(q2s - q0s);
  const v3f vab = f3(v2 - v1), vac = f3(v0 - v1), vcb = f3(v2 - v0);
  fb op[3];
  op[0] = dotf(vab, vac);  // e1: src/CTCD.cpp:536-543
  op[1] = dotf(ac, vab) + dotf(ab, vac);
  op[2] = dotf(ab, ac);
  if (surely_negative<2>(op)) return true;
  op[0] = dotf(vab, vcb);  // e2: src/CTCD.cpp:547-555
  op[1] = dotf(cb, vab) + dotf(ab, vcb);
  op[2] = dotf(ab, cb);
  if (surely_negative<2>(op)) return true;
  // Distance from the vertex to the edge's line (src/CTCD.cpp:557-573).
  const v3f X0 = crossf(ab, ac), X1 = crossf(ab, vac) + crossf(vab, ac), X2 = crossf(vab, vac);
  // Upper bounds of |ab| + |vab| and |ac| + |vac| (1-norms of the values
  // plus their FP32 error bounds).
  auto norm1 = [](v3f a) { return (fabsf(a.x.v) + fabsf(a.y.v)) + fabsf(a.z.v); };
  auto err1 = [](v3f a) { return (a.x.m + a.y.m) + a.z.m; };
  const float pa = (norm1(ab) + norm1(vab) + 1e-6f * (err1(ab) + err1(vab))) * 1.00001f;
  const float pc = (norm1(ac) + norm1(vac) + 1e-6f * (err1(ac) + err1(vac))) * 1.00001f;
  const float P = pa * pa, Q = pc * pc;
  const float md = (float)(eta * eta > 1e-30 ? eta * eta : 1e-30) * 1.00001f;
  const float rhs = (md * P) * 1.00001f + 1e-14f * (2.0f * P * Q + md * P) + 1e-37f;
  if (!(fabsf(rhs) < kFinite)) return false;
  for (int k = 0; k < 4; k++) {
    const float lower = cross_lower_sq(X0, X1, X2, 0.25f * (float)k, 0.25f);
    if (!(lower > rhs)) return false;
  }
  return true;
}

}  // namespace ccd
