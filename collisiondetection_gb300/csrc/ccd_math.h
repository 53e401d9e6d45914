// Correctly rounded double exp() and log() for the root finder.
//
// The reference's root finder seeds its root-modulus bound with
//   exp((log(a) - log(b)) / n)                         (src/rpoly.h:144)
// evaluated by the host C library.  The device code computes the correctly
// rounded value; glibc agrees with it on all but ~0.1% of inputs (where glibc
// itself is off by one ulp), and a one-ulp change of the seed moves the roots
// found by at most a few ulps.
//
// Method (written from the mathematics, not from any library):
//  * arithmetic in double-double (a value is hi + lo, |lo| <= ulp(hi)/2), with
//    exact products from fma() (Dekker / Knuth error-free transformations);
//  * fast path, table-driven argument reduction after P. T. P. Tang
//    ("Table-driven implementation of the exponential / logarithm function in
//    IEEE floating-point arithmetic", ACM TOMS 1989/1990), evaluated to about
//    2^-64 relative error, followed by a rounding test: when the error interval
//    around the approximation rounds to a single double, that double is the
//    correctly rounded result;
//  * otherwise (about 0.4% of inputs) the slow path, series in double-double:
//    log(m) = 2 atanh((m-1)/(m+1)) for m in [sqrt(1/2), sqrt(2)),
//    exp(r) from expm1(r/256) and eight squarings, about 2^-96 relative error.
#pragma once

#include "ccd_common.h"
#include "ccd_math_tables.h"

namespace ccd {

struct dd {
  double hi, lo;
};

CCD_HD dd dd_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return dd{s, e};
}
CCD_HD dd dd_fast_two_sum(double a, double b) {  // requires |a| >= |b| or a == 0
  double s = a + b;
  double e = b - (s - a);
  return dd{s, e};
}
CCD_HD dd dd_two_prod(double a, double b) {
  double p = a * b;
  double e = fma(a, b, -p);
  return dd{p, e};
}
CCD_HD dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_fast_two_sum(s.hi, s.lo);
}
CCD_HD dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }
CCD_HD dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
CCD_HD dd dd_mul(dd a, dd b) {
  dd p = dd_two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return dd_fast_two_sum(p.hi, p.lo);
}
CCD_HD dd dd_mul_d(dd a, double b) {
  dd p = dd_two_prod(a.hi, b);
  p.lo += a.lo * b;
  return dd_fast_two_sum(p.hi, p.lo);
}
CCD_HD dd dd_div(dd a, dd b) {
  double q1 = a.hi / b.hi;
  dd r = dd_sub(a, dd_mul_d(b, q1));
  double q2 = r.hi / b.hi;
  r = dd_sub(r, dd_mul_d(b, q2));
  double q3 = r.hi / b.hi;
  dd q = dd_fast_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}

// ln 2 = kLn2Hi + kLn2Lo (double-double, |error| < 2^-108).
#define CCD_LN2_HI 0x1.62e42fefa39efp-1
#define CCD_LN2_LO 0x1.abc9e3b39803fp-56

// 1/(2k+1) as double-doubles, k = 0..22.
CCD_HD dd inv_odd(int k) {
  switch (k) {
    case 0: return dd{0x1p+0, 0.0};
    case 1: return dd{0x1.5555555555555p-2, 0x1.5555555555555p-56};
    case 2: return dd{0x1.999999999999ap-3, -0x1.999999999999ap-57};
    case 3: return dd{0x1.2492492492492p-3, 0x1.2492492492492p-57};
    case 4: return dd{0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58};
    case 5: return dd{0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59};
    case 6: return dd{0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58};
    case 7: return dd{0x1.1111111111111p-4, 0x1.1111111111111p-60};
    case 8: return dd{0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61};
    case 9: return dd{0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59};
    case 10: return dd{0x1.8618618618618p-5, 0x1.8618618618618p-59};
    case 11: return dd{0x1.642c8590b2164p-5, 0x1.642c8590b2164p-60};
    case 12: return dd{0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61};
    case 13: return dd{0x1.2f684bda12f68p-5, 0x1.2f684bda12f68p-59};
    case 14: return dd{0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61};
    case 15: return dd{0x1.0842108421084p-5, 0x1.0842108421084p-60};
    case 16: return dd{0x1.f07c1f07c1f08p-6, -0x1.f07c1f07c1f08p-61};
    case 17: return dd{0x1.d41d41d41d41dp-6, 0x1.0750750750750p-60};
    case 18: return dd{0x1.bacf914c1bad0p-6, -0x1.bacf914c1bad0p-60};
    case 19: return dd{0x1.a41a41a41a41ap-6, 0x1.0690690690690p-60};
    case 20: return dd{0x1.8f9c18f9c18fap-6, -0x1.f3831f3831f38p-61};
    case 21: return dd{0x1.7d05f417d05f4p-6, 0x1.7d05f417d05f4p-62};
    default: return dd{0x1.6c16c16c16c17p-6, -0x1.f49f49f49f49fp-61};
  }
}

// 1/n! as double-doubles, n = 0..12.
CCD_HD dd inv_fact(int n) {
  switch (n) {
    case 0:
    case 1: return dd{0x1p+0, 0.0};
    case 2: return dd{0x1p-1, 0.0};
    case 3: return dd{0x1.5555555555555p-3, 0x1.5555555555555p-57};
    case 4: return dd{0x1.5555555555555p-5, 0x1.5555555555555p-59};
    case 5: return dd{0x1.1111111111111p-7, 0x1.1111111111111p-63};
    case 6: return dd{0x1.6c16c16c16c17p-10, -0x1.f49f49f49f49fp-65};
    case 7: return dd{0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-73};
    case 8: return dd{0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76};
    case 9: return dd{0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73};
    case 10: return dd{0x1.27e4fb7789f5cp-22, 0x1.cbbc05b4fa99ap-76};
    case 11: return dd{0x1.ae64567f544e4p-26, -0x1.c062e06d1f209p-80};
    default: return dd{0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83};
  }
}

CCD_NOINLINE double cr_log_slow(double x) {
  if (!(x > 0.0)) return (x == 0.0) ? -HUGE_VAL : (x - x) / (x - x);  // log(0) = -inf; x<0 or NaN -> NaN
  if (x == HUGE_VAL) return x;
  int e;
  double m = frexp(x, &e);  // x = m 2^e, m in [0.5, 1)
  if (m < 0x1.6a09e667f3bcdp-1) {  // sqrt(1/2): move m into [sqrt(1/2), sqrt(2))
    m *= 2.0;
    e -= 1;
  }
  dd num = dd{m - 1.0, 0.0};  // exact (Sterbenz)
  dd den = dd_two_sum(m, 1.0);
  dd s = dd_div(num, den);
  dd z = dd_mul(s, s);
  dd q = inv_odd(22);
  for (int k = 21; k >= 0; k--) q = dd_add(dd_mul(q, z), inv_odd(k));
  dd lm = dd_mul(dd{2.0 * s.hi, 2.0 * s.lo}, q);
  dd le = dd_mul_d(dd{CCD_LN2_HI, CCD_LN2_LO}, (double)e);
  dd r = dd_add(le, lm);
  return r.hi + r.lo;
}

CCD_NOINLINE double cr_exp_slow(double x) {
  if (x != x) return x + x;
  if (x > 710.0) return HUGE_VAL;
  if (x < -746.0) return 0.0;
  double kd = nearbyint(x * 0x1.71547652b82fep+0);  // x / ln2, any nearby integer
  int k = (int)kd;
  dd p = dd_two_prod(kd, CCD_LN2_HI);  // exact
  double rh = x - p.hi;                // exact (Sterbenz) for k != 0; trivially for k == 0
  dd r = dd_two_sum(rh, -p.lo);
  r = dd_sub(r, dd_two_prod(kd, CCD_LN2_LO));
  r.hi *= 0x1p-8;  // exact scalings
  r.lo *= 0x1p-8;
  dd poly = inv_fact(12);
  for (int n = 11; n >= 1; n--) poly = dd_add(dd_mul(poly, r), inv_fact(n));
  dd em = dd_mul(poly, r);  // expm1(r/256)
  for (int i = 0; i < 8; i++) em = dd_mul(em, dd_add(dd{2.0, 0.0}, em));
  dd y = dd_add(dd{1.0, 0.0}, em);
  if (k >= -1021) return ldexp(y.hi + y.lo, k);
  // Subnormal result: round y * 2^(k+1074) to an integer once (ties to even).
  double shi = ldexp(y.hi, k + 1074), slo = ldexp(y.lo, k + 1074);
  double n = nearbyint(shi);
  double d = (shi - n) + slo;
  if (d > 0.5 || (d == 0.5 && fmod(n, 2.0) != 0.0)) n += 1.0;
  if (d < -0.5 || (d == -0.5 && fmod(n, 2.0) != 0.0)) n -= 1.0;
  return ldexp(n, -1074);
}

#if defined(__CUDACC__)
__device__ const double kLogTable[384] = CCD_LOG_TABLE_DATA;
__device__ const double kExpTable[64] = CCD_EXP_TABLE_DATA;
#endif
static const double kLogTableHost[384] = CCD_LOG_TABLE_DATA;
static const double kExpTableHost[64] = CCD_EXP_TABLE_DATA;
#if defined(__CUDA_ARCH__)
#define CCD_LOG_TAB kLogTable
#define CCD_EXP_TAB kExpTable
#else
#define CCD_LOG_TAB kLogTableHost
#define CCD_EXP_TAB kExpTableHost
#endif

// Rounds hi + lo to double when every value within eps of it rounds the same
// way; returns false when the test is inconclusive.
CCD_HD bool round_if_certain(dd s, double eps, double &out) {
  double y1 = s.hi + (s.lo + eps);
  double y2 = s.hi + (s.lo - eps);
  out = y1;
  return y1 == y2;
}

// log(x), correctly rounded.
CCD_NOINLINE double cr_log(double x) {
  if (!(x > 0.0) || x == HUGE_VAL) return cr_log_slow(x);
  int e;
  double m = frexp(x, &e) * 2.0;  // x = m 2^(e-1), m in [1, 2); exact
  e -= 1;
  int j = (int)((m - 1.0) * 128.0);  // top 7 fraction bits, exact
  if (j >= 64) {                     // reduce [1.5, 2) as m/2 in [0.75, 1)
    m *= 0.5;
    e += 1;
  }
  const double *t = CCD_LOG_TAB + 3 * j;
  dd p = dd_two_prod(m, t[0]);      // m * inv_j, exact
  dd r = dd_two_sum(p.hi - 1.0, p.lo);  // exact, |r| <= 2^-7
  double rh = r.hi;
  // log1p(r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - ... + r^8/11)
  double q = 1.0 / 11.0;
  q = q * rh - 0.1;
  q = q * rh + 1.0 / 9.0;
  q = q * rh - 0.125;
  q = q * rh + 1.0 / 7.0;
  q = q * rh - 1.0 / 6.0;
  q = q * rh + 0.2;
  q = q * rh - 0.25;
  q = q * rh + 1.0 / 3.0;
  double tail = ((rh * rh) * rh) * q;
  dd r2 = dd_mul(r, r);
  dd lp = dd_add(r, dd{-0.5 * r2.hi, -0.5 * r2.lo});
  lp = dd_add(lp, dd{tail, 0.0});
  dd s = dd_add(dd_mul_d(dd{CCD_LN2_HI, CCD_LN2_LO}, (double)e), dd{t[1], t[2]});
  s = dd_add(s, lp);
  double y;
  if (round_if_certain(s, fabs(s.hi) * 0x1p-61, y)) return y;
  return cr_log_slow(x);
}

// exp(x), correctly rounded.
CCD_NOINLINE double cr_exp(double x) {
  if (!(fabs(x) < 700.0)) return cr_exp_slow(x);  // NaN, inf, near over/underflow
  double nd = nearbyint(x * CCD_32_OVER_LN2);
  int n = (int)nd;
  int j = n & 31;
  int k = (n - j) / 32;
  double a = x - nd * CCD_LN2_32_L1;  // exact (Sterbenz; nd * L1 exact)
  dd r = dd_two_sum(a, -(nd * CCD_LN2_32_L2));
  r = dd_add(r, dd{-(nd * CCD_LN2_32_L3), 0.0});  // |r| <= ln2/64
  double rh = r.hi;
  // expm1(r) = r + r^2/2 + r^3 (1/6 + r/24 + ... + r^5/8!)
  double q = 1.0 / 40320.0;
  q = q * rh + 1.0 / 5040.0;
  q = q * rh + 1.0 / 720.0;
  q = q * rh + 1.0 / 120.0;
  q = q * rh + 1.0 / 24.0;
  q = q * rh + 1.0 / 6.0;
  double tail = ((rh * rh) * rh) * q;
  dd r2 = dd_mul(r, r);
  dd em = dd_add(r, dd{0.5 * r2.hi, 0.5 * r2.lo});
  em = dd_add(em, dd{tail, 0.0});
  const double *t = CCD_EXP_TAB + 2 * j;
  dd tj = dd{t[0], t[1]};
  dd y = dd_add(tj, dd_mul(tj, em));
  double out;
  if (round_if_certain(y, fabs(y.hi) * 0x1p-61, out)) return ldexp(out, k);  // |k| <= 1010: exact
  return cr_exp_slow(x);
}

}  // namespace ccd
