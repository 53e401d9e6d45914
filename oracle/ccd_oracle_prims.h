/* ORACLE / TEST INFRASTRUCTURE ONLY -- the primitive CTCD tests of the
 * oracle (src/CTCD.cpp, src/rpoly.h), included by ccd_oracle.c.
 *
 * Written once over the scalar type `real`: ccd_oracle.c compiles it as C
 * with real = double; flops.cpp compiles the same text as C++ with a scalar
 * that counts each floating-point operation, which gives the FP64 operation
 * count of the reference's op sequence per test (the algorithmic work behind
 * the refinement's roofline).  Both builds use -ffp-contract=off.
 *
 * Raw inputs (rows of points) are read as double and converted on load;
 * contact times leave through ORACLE_OUT.
 */
#ifndef CCD_ORACLE_PRIMS_H
#define CCD_ORACLE_PRIMS_H

#ifndef ORACLE_REAL
#define ORACLE_REAL double
#endif
#ifndef ORACLE_OUT
#define ORACLE_OUT(x) ((double)(x))
#endif
typedef ORACLE_REAL real;

/* ------------------------------------------------------------ scalar helpers */
static real smin(real a, real b) { return (b < a) ? b : a; }
static real smax(real a, real b) { return (a < b) ? b : a; }

typedef struct { real x, y, z; } vec3;

static vec3 v3(const double *p) { vec3 r = {p[0], p[1], p[2]}; return r; }
static vec3 vsub(vec3 a, vec3 b) { vec3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static vec3 vadd(vec3 a, vec3 b) { vec3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static vec3 vscale(real s, vec3 a) { vec3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static real vdot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static vec3 vcross(vec3 a, vec3 b) {
  vec3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static real vnorm(vec3 a) { return sqrt(vdot(a, a)); }

/* --------------------------------------------- time intervals (include/CTCD.h:7-26, src/CTCD.cpp:10-36) */
typedef struct { real l, u; } span;
typedef struct { int n; span s[8]; } span_list; /* at most deg+1 <= 7 segments per polynomial */

static span span_make(real a, real b) {
  span r;
  if (a > b) { real tmp = a; a = b; b = tmp; }
  r.l = smax(a, 0.0);
  r.u = smin(b, 1.0);
  return r;
}
static int span_meet(span a, span b) { return !(a.l > b.u || b.l > a.u); }
static void span_push(span_list *L, real a, real b) { L->s[L->n++] = span_make(a, b); }

/* Pairwise-overlap test over k spans (TimeInterval::overlap(vector)). */
static int spans_all_meet(const span *s, int k) {
  for (int i = 0; i < k; i++)
    for (int j = i + 1; j < k; j++)
      if (!span_meet(s[i], s[j])) return 0;
  return 1;
}
/* TimeInterval::intersect: starts from [0,1]. */
static span spans_common(const span *s, int k) {
  span r = {0.0, 1.0};
  for (int i = 0; i < k; i++) {
    r.l = smax(s[i].l, r.l);
    r.u = smin(s[i].u, r.u);
  }
  return r;
}

/* ------------------------------------------------------------ polynomial sign intervals */
/* src/CTCD.cpp:38-56 */
static int quad_roots(real a, real b, real c, real *t0, real *t1) {
  int sign = 1;
  if (b < 0) sign = -1;
  real disc = b * b - 4 * a * c;
  if (disc >= 0) {
    real q = -0.5 * (b + sign * sqrt(disc));
    *t0 = q / a;
    *t1 = c / q;
    if (*t0 > *t1) { real tmp = *t0; *t0 = *t1; *t1 = tmp; }
    return 2;
  }
  return 0;
}

/* src/CTCD.cpp:59-79: sign of the polynomial at the middle of the clamped
 * segment decides whether the segment is kept. */
static void sign_segment(real t1, real t2, const real *op, int degree, span_list *out, int want_pos) {
  t1 = smax(0.0, t1);
  t2 = smax(0.0, t2);
  t1 = smin(1.0, t1);
  t2 = smin(1.0, t2);
  real tmid = (t2 + t1) / 2;
  real f = op[0];
  for (int i = 1; i <= degree; i++) {
    f *= tmid;
    f += op[i];
  }
  if (want_pos && f >= 0)
    span_push(out, t1, t2);
  else if (!want_pos && f <= 0)
    span_push(out, t1, t2);
}

/* src/CTCD.cpp:81-94 */
static int may_change_sign(const real *op, int degree, int want_pos) {
  real acc = 0;
  if ((want_pos && op[0] > 0) || (!want_pos && op[0] < 0)) acc = op[0];
  for (int i = 1; i < degree; i++) {
    acc *= 1.0;
    if ((want_pos && op[i] > 0) || (!want_pos && op[i] < 0)) acc += op[i];
  }
  acc *= 1.0;
  acc += op[degree];
  return !((want_pos && acc < 0) || (!want_pos && acc > 0));
}

/* libstdc++'s std::sort on <= 16 elements is a plain insertion sort
 * (__final_insertion_sort -> __insertion_sort); restated so that root lists
 * holding NaN are permuted exactly as the reference permutes them. */
static void small_sort(real *a, int n) {
  for (int i = 1; i < n; i++) {
    real val = a[i];
    if (val < a[0]) {
      for (int j = i; j > 0; j--) a[j] = a[j - 1];
      a[0] = val;
    } else {
      int j = i;
      while (val < a[j - 1]) {
        a[j] = a[j - 1];
        j--;
      }
      a[j] = val;
    }
  }
}

static int jt_roots(real *op, int degree, real *zr, real *zi);

/* src/CTCD.cpp:98-177 */
static void sign_intervals(real *op, int n, span_list *out, int want_pos) {
  int roots = 0;
  int deg = n;
  real tr[6], ti[6];

  real maxval = 0;
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

  if (deg > 2) {
    if (!may_change_sign(op, deg, want_pos)) return;
    roots = jt_roots(op, deg, tr, ti);
  } else if (deg == 2) {
    roots = quad_roots(op[0], op[1], op[2], &tr[0], &tr[1]);
  } else if (deg == 1) {
    tr[0] = -op[1] / op[0];
    roots = 1;
  } else {
    if ((!want_pos && op[0] <= 0) || (want_pos && op[0] >= 0)) span_push(out, 0, 1.0);
    return;
  }

  if (roots > 0) {
    small_sort(tr, roots);
    if (tr[0] >= 0) sign_segment(0, tr[0], op, deg, out, want_pos);
    for (int i = 0; i < roots - 1; i++) {
      if (!((tr[i] < 0 && tr[i + 1] < 0) || (tr[i] > 1.0 && tr[i + 1] > 1.0)))
        sign_segment(tr[i], tr[i + 1], op, deg, out, want_pos);
    }
    if (tr[roots - 1] <= 1.0) sign_segment(tr[roots - 1], 1.0, op, deg, out, want_pos);
  } else {
    sign_segment(0.0, 1.0, op, deg, out, want_pos);
  }
}

/* ------------------------------------------------------------ Jenkins-Traub (src/rpoly.h)
 * The reference vendors C. Bond's C translation of ACM TOMS 493 (the
 * Jenkins-Traub three-stage real-polynomial root finder).  The restatement
 * below follows the same numerical steps in the same order -- fixed-shift,
 * variable-shift quadratic and linear iterations, the same convergence tests,
 * constants and iteration limits -- with the goto-based control flow written
 * as explicit loops and state. */
typedef struct {
  real p[7], qp[7], k[7], qk[7], svk[7];
  real sr, si, u, v, a, b, c, d, a1, a3, a7, e, f, g, h;
  real szr, szi, lzr, lzi;
  real eps, are, mre;
  int n;
} jt;

/* Quotient q and remainder (a, b) of p by x^2 + u x + v (rpoly.h:680-695). */
static void jt_divide(int nn, real u, real v, const real *p, real *q, real *ra, real *rb) {
  real b = p[0];
  q[0] = b;
  real a = p[1] - b * u;
  q[1] = a;
  for (int i = 2; i <= nn; i++) {
    real c = p[i] - a * u - b * v;
    q[i] = c;
    b = a;
    a = c;
  }
  *ra = a;
  *rb = b;
}

/* Zeros of a z^2 + b1 z + c (rpoly.h:702-754). */
static void jt_quadratic(real a, real b1, real c, real *sr, real *si, real *lr, real *li) {
  real b, d, e;
  if (a == 0.0) {
    if (b1 != 0.0)
      *sr = -c / b1;
    else
      *sr = 0.0;
    *lr = 0.0;
    *si = 0.0;
    *li = 0.0;
    return;
  }
  if (c == 0.0) {
    *sr = 0.0;
    *lr = -b1 / a;
    *si = 0.0;
    *li = 0.0;
    return;
  }
  b = b1 / 2.0;
  if (fabs(b) < fabs(c)) {
    if (c < 0.0)
      e = -a;
    else
      e = a;
    e = b * (b / fabs(c)) - e;
    d = sqrt(fabs(e)) * sqrt(fabs(c));
  } else {
    e = 1.0 - (a / b) * (c / b);
    d = sqrt(fabs(e)) * fabs(b);
  }
  if (e < 0.0) {
    *sr = -b / a;
    *lr = *sr;
    *si = fabs(d / a);
    *li = -(*si);
  } else {
    if (b >= 0.0) d = -d;
    *lr = (-b + d) / a;
    *sr = 0.0;
    if (*lr != 0.0) *sr = (c / *lr) / a;
    *si = 0.0;
    *li = 0.0;
  }
}

/* Scalars for the next K polynomial (rpoly.h:566-597); returns the type. */
static int jt_scalars(jt *s) {
  jt_divide(s->n - 1, s->u, s->v, s->k, s->qk, &s->c, &s->d);
  if (!(fabs(s->c) > fabs(s->k[s->n - 1] * 100.0 * s->eps)) && !(fabs(s->d) > fabs(s->k[s->n - 2] * 100.0 * s->eps)))
    return 3;
  if (fabs(s->d) < fabs(s->c)) {
    s->e = s->a / s->c;
    s->f = s->d / s->c;
    s->g = s->u * s->e;
    s->h = s->v * s->b;
    s->a3 = s->a * s->e + (s->h / s->c + s->g) * s->b;
    s->a1 = s->b - s->a * (s->d / s->c);
    s->a7 = s->a + s->g * s->d + s->h * s->f;
    return 1;
  }
  s->e = s->a / s->d;
  s->f = s->c / s->d;
  s->g = s->u * s->b;
  s->h = s->v * s->b;
  s->a3 = (s->a + s->g) * s->e + s->h * (s->b / s->d);
  s->a1 = s->b * s->f - s->a;
  s->a7 = (s->f + s->u) * s->a + s->h;
  return 2;
}

/* Next K polynomial (rpoly.h:601-636). */
static void jt_next_k(jt *s, int type) {
  int n = s->n;
  if (type == 3) {
    s->k[0] = 0.0;
    s->k[1] = 0.0;
    for (int i = 2; i < n; i++) s->k[i] = s->qk[i - 2];
    return;
  }
  real ref = (type == 1) ? s->b : s->a;
  if (fabs(s->a1) <= fabs(ref) * s->eps * 10.0) {
    s->k[0] = 0.0;
    s->k[1] = -s->a7 * s->qp[0];
    for (int i = 2; i < n; i++) s->k[i] = s->a3 * s->qk[i - 2] - s->a7 * s->qp[i - 1];
    return;
  }
  s->a7 /= s->a1;
  s->a3 /= s->a1;
  s->k[0] = s->qp[0];
  s->k[1] = s->qp[1] - s->a7 * s->qp[0];
  for (int i = 2; i < n; i++) s->k[i] = s->a3 * s->qk[i - 2] - s->a7 * s->qp[i - 1] + s->qp[i];
}


/* New quadratic estimate (rpoly.h:640-675). */
static void jt_estimate(const jt *s, int type, real *uu, real *vv) {
  real a4, a5, b1, b2, c1, c2, c3, c4, den;
  int n = s->n;
  if (type == 3) {
    *uu = 0.0;
    *vv = 0.0;
    return;
  }
  if (type == 2) {
    a4 = (s->a + s->g) * s->f + s->h;
    a5 = (s->f + s->u) * s->c + s->v * s->d;
  } else {
    a4 = s->a + s->u * s->b + s->h * s->f;
    a5 = s->c + (s->u + s->v * s->f) * s->d;
  }
  b1 = -s->k[n - 1] / s->p[n];
  b2 = -(s->k[n - 2] + b1 * s->p[n - 1]) / s->p[n];
  c1 = s->v * b2 * s->a1;
  c2 = b1 * s->a7;
  c3 = b1 * b1 * s->a3;
  c4 = c1 - c2 - c3;
  den = a5 + b1 * a4 - c4;
  if (den == 0.0) {
    *uu = 0.0;
    *vv = 0.0;
    return;
  }
  *uu = s->u - (s->u * (c3 + c2) + s->v * (b1 * s->a1 + b2 * s->a7)) / den;
  *vv = s->v * (1.0 + c4 / den);
}

/* Variable-shift iteration for one real zero (rpoly.h:473-558).  Returns the
 * number of zeros found (0/1); *near_double is set when a cluster near the
 * real axis suggests a quadratic iteration from *s. */
static int jt_real_iter(jt *s, real *sp, int *near_double) {
  real pv, kv, t = 0, x = *sp, ms, mp, omp = 0, ee;
  int n = s->n;
  *near_double = 0;
  for (int j = 1;; j++) {
    pv = s->p[0];
    s->qp[0] = pv;
    for (int i = 1; i <= n; i++) {
      pv = pv * x + s->p[i];
      s->qp[i] = pv;
    }
    mp = fabs(pv);
    ms = fabs(x);
    ee = (s->mre / (s->are + s->mre)) * fabs(s->qp[0]);
    for (int i = 1; i <= n; i++) ee = ee * ms + fabs(s->qp[i]);
    if (mp <= 20.0 * ((s->are + s->mre) * ee - s->mre * mp)) {
      s->szr = x;
      s->szi = 0.0;
      return 1;
    }
    if (j > 10) return 0;
    if (j >= 2 && !(fabs(t) > 0.001 * fabs(x - t) || mp < omp)) {
      *near_double = 1;
      *sp = x;
      return 0;
    }
    omp = mp;
    kv = s->k[0];
    s->qk[0] = kv;
    for (int i = 1; i < n; i++) {
      kv = kv * x + s->k[i];
      s->qk[i] = kv;
    }
    if (fabs(kv) <= fabs(s->k[n - 1]) * 10.0 * s->eps) {
      s->k[0] = 0.0;
      for (int i = 1; i < n; i++) s->k[i] = s->qk[i - 1];
    } else {
      t = -pv / kv;
      s->k[0] = s->qp[0];
      for (int i = 1; i < n; i++) s->k[i] = t * s->qk[i - 1] + s->qp[i];
    }
    kv = s->k[0];
    for (int i = 1; i < n; i++) kv = kv * x + s->k[i];
    t = 0.0;
    if (fabs(kv) > fabs(s->k[n - 1] * 10.0 * s->eps)) t = -pv / kv;
    x += t;
  }
}

/* Variable-shift iteration for a quadratic factor (rpoly.h:390-467).
 * Returns the number of zeros found (0/2). */
static int jt_quad_iter(jt *s, real uu, real vv) {
  real ui, vi, mp, omp = 0, ee, relstp = 0, t, zm;
  int type, tried = 0, j = 0, n = s->n;
  s->u = uu;
  s->v = vv;
  for (;;) {
    jt_quadratic(1.0, s->u, s->v, &s->szr, &s->szi, &s->lzr, &s->lzi);
    if (fabs(fabs(s->szr) - fabs(s->lzr)) > 0.01 * fabs(s->lzr)) return 0;
    jt_divide(n, s->u, s->v, s->p, s->qp, &s->a, &s->b);
    mp = fabs(s->a - s->szr * s->b) + fabs(s->szi * s->b);
    zm = sqrt(fabs(s->v));
    ee = 2.0 * fabs(s->qp[0]);
    t = -s->szr * s->b;
    for (int i = 1; i < n; i++) ee = ee * zm + fabs(s->qp[i]);
    ee = ee * zm + fabs(s->a + t);
    ee *= (5.0 * s->mre + 4.0 * s->are);
    ee = ee - (5.0 * s->mre + 2.0 * s->are) * (fabs(s->a + t) + fabs(s->b) * zm) + 2.0 * s->are * fabs(t);
    if (mp <= 20.0 * ee) return 2;
    j++;
    if (j > 20) return 0;
    if (j >= 2 && !(relstp > 0.01 || mp < omp || tried)) {
      /* A cluster stalls convergence: five fixed-shift steps near it. */
      if (relstp < s->eps) relstp = s->eps;
      relstp = sqrt(relstp);
      s->u = s->u - s->u * relstp;
      s->v = s->v + s->v * relstp;
      jt_divide(n, s->u, s->v, s->p, s->qp, &s->a, &s->b);
      for (int i = 0; i < 5; i++) {
        type = jt_scalars(s);
        jt_next_k(s, type);
      }
      tried = 1;
      j = 0;
    }
    omp = mp;
    type = jt_scalars(s);
    jt_next_k(s, type);
    type = jt_scalars(s);
    jt_estimate(s, type, &ui, &vi);
    if (vi == 0.0) return 0;
    relstp = fabs((vi - s->v) / vi);
    s->u = ui;
    s->v = vi;
  }
}

/* Second stage: up to l2 fixed-shift K polynomials, then the variable-shift
 * iterations (rpoly.h:277-383).  Returns the number of zeros found. */
static int jt_fixed_shift(jt *s, int l2) {
  real svu = 0, svv = 0, ui, vi, xs = 0;
  real betas = 0.25, betav = 0.25, oss = s->sr, ovv = s->v, ss, vv, ts, tv;
  real ots = 0, otv = 0, tvv, tss;
  int type, n = s->n;

  jt_divide(n, s->u, s->v, s->p, s->qp, &s->a, &s->b);
  type = jt_scalars(s);
  for (int j = 0; j < l2; j++) {
    jt_next_k(s, type);
    type = jt_scalars(s);
    jt_estimate(s, type, &ui, &vi);
    vv = vi;
    ss = 0.0;
    if (s->k[n - 1] != 0.0) ss = -s->p[n] / s->k[n - 1];
    tv = 1.0;
    ts = 1.0;
    if (j != 0 && type != 3) {
      if (vv != 0.0) tv = fabs((vv - ovv) / vv);
      if (ss != 0.0) ts = fabs((ss - oss) / ss);
      tvv = 1.0;
      if (tv < otv) tvv = tv * otv;
      tss = 1.0;
      if (ts < ots) tss = ts * ots;
      int vpass = (tvv < betav), spass = (tss < betas);
      if (spass || vpass) {
        svu = s->u;
        svv = s->v;
        for (int i = 0; i < n; i++) s->svk[i] = s->k[i];
        xs = ss;
        int vtried = 0, stried = 0;
        /* 0: quadratic iteration, 1: linear iteration, 2: restore and resume */
        int step = ((spass && !vpass) || tss < tvv) ? 1 : 0;
        for (;;) {
          if (step == 0) {
            int nz = jt_quad_iter(s, ui, vi);
            if (nz > 0) return nz;
            vtried = 1;
            betav *= 0.25;
            if (stried || !spass) {
              step = 2;
              continue;
            }
            for (int i = 0; i < n; i++) s->k[i] = s->svk[i];
            step = 1;
          } else if (step == 1) {
            int near_double;
            int nz = jt_real_iter(s, &xs, &near_double);
            if (nz > 0) return nz;
            stried = 1;
            betas *= 0.25;
            if (!near_double) {
              step = 2;
              continue;
            }
            ui = -(xs + xs);
            vi = xs * xs;
            step = 0;
          } else {
            s->u = svu;
            s->v = svv;
            for (int i = 0; i < n; i++) s->k[i] = s->svk[i];
            if (vpass && !vtried) {
              step = 0;
              continue;
            }
            jt_divide(n, s->u, s->v, s->p, s->qp, &s->a, &s->b);
            type = jt_scalars(s);
            break;
          }
        }
      }
    }
    ovv = vv;
    oss = ss;
    otv = tv;
    ots = ts;
  }
  return 0;
}

/* Number of chop steps after which a non-finite root bound is declared (the
 * reference loops forever there; finite inputs never come close). */
#define JT_CHOP_LIMIT 4096
#define JT_NEWTON_LIMIT 4096

/* Driver (rpoly.h:49-261).  Returns the number of zeros found, or -1. */
static int jt_roots(real *op, int degree, real *zr, real *zi) {
  jt s;
  real t, aa, bb, cc, factor, rot, lo, maxc, minc, xx, yy, cosr, sinr, xxx, x, sc, bnd, xm, ff, df, dx;
  real temp[7], pt[7];
  const real infin = 3.4e38, smalno = 1.2e-38, base = 2.0;
  int nm1, zerok;

  s.eps = 2.22e-16;
  s.are = s.eps;
  s.mre = s.eps;
  lo = smalno / s.eps;
  xx = sqrt(0.5);
  yy = -xx;
  rot = 94.0;
  rot *= 0.017453293;
  cosr = cos(rot);
  sinr = sin(rot);
  s.n = degree;
  if (op[0] == 0.0) return -1;
  while (op[s.n] == 0.0) {
    zr[degree - s.n] = 0.0;
    zi[degree - s.n] = 0.0;
    s.n--;
  }
  if (s.n < 1) return -1;
  for (int i = 0; i <= s.n; i++) s.p[i] = op[i];

  while (s.n > 0) {
    int n = s.n;
    if (n == 1) {
      zr[degree - 1] = -s.p[1] / s.p[0];
      zi[degree - 1] = 0.0;
      s.n = 0;
      break;
    }
    if (n == 2) {
      jt_quadratic(s.p[0], s.p[1], s.p[2], &zr[degree - 2], &zi[degree - 2], &zr[degree - 1], &zi[degree - 1]);
      s.n = 0;
      break;
    }
    /* Scale by a power of the base when coefficients are extreme. */
    maxc = 0.0;
    minc = infin;
    for (int i = 0; i <= n; i++) {
      x = fabs(s.p[i]);
      if (x > maxc) maxc = x;
      if (x != 0.0 && x < minc) minc = x;
    }
    sc = lo / minc;
    int keep = (sc > 1.0 && infin / sc < maxc) || (sc <= 1.0 && maxc < 10.0);
    if (!keep) {
      if (sc == 0.0) sc = smalno;
      int l = (int)ORACLE_OUT(log(sc) / log(base) + 0.5);
      factor = pow(base * 1.0, l);
      if (factor != 1.0)
        for (int i = 0; i <= n; i++) s.p[i] = factor * s.p[i];
    }
    /* Lower bound on the root moduli: Cauchy polynomial, chopped, then Newton. */
    for (int i = 0; i <= n; i++) pt[i] = fabs(s.p[i]);
    pt[n] = -pt[n];
    x = exp((log(-pt[n]) - log(pt[0])) / (real)n);
    if (pt[n - 1] != 0.0) {
      xm = -pt[n] / pt[n - 1];
      if (xm < x) x = xm;
    }
    for (int it = 0;; it++) {
      if (it >= JT_CHOP_LIMIT) return -1;
      xm = x * 0.1;
      ff = pt[0];
      for (int i = 1; i <= n; i++) ff = ff * xm + pt[i];
      if (ff <= 0.0) break;
      x = xm;
    }
    dx = x;
    for (int it = 0; fabs(dx / x) > 0.005; it++) {
      if (it >= JT_NEWTON_LIMIT) return -1;
      ff = pt[0];
      df = ff;
      for (int i = 1; i < n; i++) {
        ff = ff * x + pt[i];
        df = df * x + ff;
      }
      ff = ff * x + pt[n];
      dx = ff / df;
      x -= dx;
    }
    bnd = x;
    /* Derivative as the first K polynomial, then five unshifted steps. */
    nm1 = n - 1;
    for (int i = 1; i < n; i++) s.k[i] = (real)(n - i) * s.p[i] / (real)n;
    s.k[0] = s.p[0];
    aa = s.p[n];
    bb = s.p[n - 1];
    zerok = (s.k[n - 1] == 0);
    for (int jj = 0; jj < 5; jj++) {
      cc = s.k[n - 1];
      if (!zerok) {
        t = -aa / cc;
        for (int i = 0; i < nm1; i++) {
          int j = n - i - 1;
          s.k[j] = t * s.k[j - 1] + s.p[j];
        }
        s.k[0] = s.p[0];
        zerok = (fabs(s.k[n - 1]) <= fabs(bb) * s.eps * 10.0);
      } else {
        for (int i = 0; i < nm1; i++) {
          int j = n - i - 1;
          s.k[j] = s.k[j - 1];
        }
        s.k[0] = 0.0;
        zerok = (s.k[n - 1] == 0.0);
      }
    }
    for (int i = 0; i < n; i++) temp[i] = s.k[i];
    /* Up to 20 shifts, each rotated by 94 degrees from the last. */
    int found = 0;
    for (int cnt = 0; cnt < 20; cnt++) {
      xxx = cosr * xx - sinr * yy;
      yy = sinr * xx + cosr * yy;
      xx = xxx;
      s.sr = bnd * xx;
      s.si = bnd * yy;
      s.u = -2.0 * s.sr;
      s.v = bnd;
      int nz = jt_fixed_shift(&s, 20 * (cnt + 1));
      if (nz != 0) {
        int j = degree - s.n;
        zr[j] = s.szr;
        zi[j] = s.szi;
        s.n -= nz;
        for (int i = 0; i <= s.n; i++) s.p[i] = s.qp[i];
        if (nz != 1) {
          zr[j + 1] = s.lzr;
          zi[j + 1] = s.lzi;
        }
        found = 1;
        break;
      }
      for (int i = 0; i < s.n; i++) s.k[i] = temp[i];
    }
    if (!found) break;
  }
  return degree - s.n;
}

/* ------------------------------------------------------------ polynomial builders */
/* src/CTCD.cpp:179-213 -- quartic side test for edge-edge. */
static void bary_poly(vec3 x10, vec3 x20, vec3 x30, vec3 v10, vec3 v20, vec3 v30, span_list *out) {
  real A = vdot(x10, x10);
  real B = 2 * vdot(x10, v10);
  real C = vdot(v10, v10);
  real D = vdot(x20, x10);
  real E = vdot(x20, v10) + vdot(v20, x10);
  real F = vdot(v20, v10);
  real G = vdot(x30, x20);
  real H = vdot(x30, v20) + vdot(v30, x20);
  real I = vdot(v30, v20);
  real J = vdot(x30, x10);
  real K = vdot(x30, v10) + vdot(v30, x10);
  real L = vdot(v30, v10);
  real op[5];
  op[0] = F * L - C * I;
  op[1] = F * K + E * L - C * H - B * I;
  op[2] = F * J + D * L + E * K - C * G - A * I - B * H;
  op[3] = D * K + E * J - A * H - B * G;
  op[4] = D * J - A * G;
  sign_intervals(op, 4, out, 1);
}

/* src/CTCD.cpp:215-229 -- cubic side test for vertex-face; the "normal" is
 * x20 + t v20 as given by the caller. */
static void plane_poly(vec3 x10, vec3 x20, vec3 x30, vec3 v10, vec3 v20, vec3 v30, span_list *out) {
  real op[4];
  op[0] = vdot(v10, vcross(v20, v30));
  op[1] = vdot(x10, vcross(v20, v30)) + vdot(v10, vcross(x20, v30)) + vdot(v10, vcross(v20, x30));
  op[2] = vdot(x10, vcross(x20, v30)) + vdot(x10, vcross(v20, x30)) + vdot(v10, vcross(x20, x30));
  op[3] = vdot(x10, vcross(x20, x30));
  sign_intervals(op, 3, out, 1);
}

/* src/CTCD.cpp:231-257 -- squared distance to the moving plane minus eta^2 |n|^2. */
static void dist_poly(vec3 x10, vec3 x20, vec3 x30, vec3 v10, vec3 v20, vec3 v30, real minD, span_list *out) {
  real A = vdot(v10, vcross(v20, v30));
  real B = vdot(x10, vcross(v20, v30)) + vdot(v10, vcross(x20, v30)) + vdot(v10, vcross(v20, x30));
  real C = vdot(x10, vcross(x20, v30)) + vdot(x10, vcross(v20, x30)) + vdot(v10, vcross(x20, x30));
  real D = vdot(x10, vcross(x20, x30));
  vec3 E = vcross(x20, x30);
  vec3 F = vadd(vcross(x20, v30), vcross(v20, x30));
  vec3 G = vcross(v20, v30);
  real op[7];
  op[0] = A * A;
  op[1] = 2 * A * B;
  op[2] = B * B + 2 * A * C - vdot(G, G) * minD;
  op[3] = 2 * A * D + 2 * B * C - 2 * vdot(G, F) * minD;
  op[4] = 2 * B * D + C * C - (2 * vdot(G, E) + vdot(F, F)) * minD;
  op[5] = 2 * C * D - 2 * vdot(F, E) * minD;
  op[6] = D * D - vdot(E, E) * minD;
  sign_intervals(op, 6, out, 0);
}

/* ------------------------------------------------------------ primitive tests */
/* src/CTCD.cpp:259-411 -- argument order q0s,p0s,q1s,p1s,q0e,p0e,q1e,p1e. */
static int prim_ee(const double *x, real eta, double *tout) {
  vec3 q0s = v3(x), p0s = v3(x + 3), q1s = v3(x + 6), p1s = v3(x + 9);
  vec3 q0e = v3(x + 12), p0e = v3(x + 15), q1e = v3(x + 18), p1e = v3(x + 21);
  real minD = eta * eta;
  span_list raw = {0}, cop = {0}, par = {0}, a0 = {0}, a1 = {0}, b0 = {0}, b1 = {0};

  vec3 x10 = vsub(p0s, p1s), x20 = vsub(p0s, q0s), x30 = vsub(p1s, q1s);
  vec3 vp0 = vsub(p0e, p0s), vp1 = vsub(p1e, p1s), vq0 = vsub(q0e, q0s), vq1 = vsub(q1e, q1s);
  vec3 v10 = vsub(vp0, vp1), v20 = vsub(vp0, vq0), v30 = vsub(vp1, vq1);
  dist_poly(x10, x20, x30, v10, v20, v30, minD, &raw);

  /* Split off segments where the edges are (nearly) parallel. */
  for (int i = 0; i < raw.n; i++) {
    real midt = (raw.s[i].u + raw.s[i].l) / 2;
    vec3 e0 = vadd(vsub(q0s, p0s), vscale(midt, vsub(vq0, vp0)));
    vec3 e1 = vadd(vsub(q1s, p1s), vscale(midt, vsub(vq1, vp1)));
    if (vnorm(vcross(e0, e1)) < 1e-8)
      par.s[par.n++] = raw.s[i];
    else
      cop.s[cop.n++] = raw.s[i];
  }
  if (cop.n == 0) return 0;

  x10 = vsub(p1s, q1s);
  v10 = vsub(vp1, vq1);
  x20 = vsub(p0s, q0s);
  v20 = vsub(vp0, vq0);
  x30 = vsub(q0s, q1s);
  v30 = vsub(vq0, vq1);
  bary_poly(x10, x20, x30, v10, v20, v30, &a0);
  if (a0.n == 0) return 0;

  x20 = vsub(q0s, p0s);
  v20 = vsub(vq0, vp0);
  x30 = vsub(p0s, q1s);
  v30 = vsub(vp0, vq1);
  bary_poly(x10, x20, x30, v10, v20, v30, &a1);
  if (a1.n == 0) return 0;

  x10 = vsub(p0s, q0s);
  v10 = vsub(vp0, vq0);
  x20 = vsub(p1s, q1s);
  v20 = vsub(vp1, vq1);
  x30 = vsub(q1s, q0s);
  v30 = vsub(vq1, vq0);
  bary_poly(x10, x20, x30, v10, v20, v30, &b0);
  if (b0.n == 0) return 0;

  x20 = vsub(q1s, p1s);
  v20 = vsub(vq1, vp1);
  x30 = vsub(p1s, q0s);
  v30 = vsub(vp1, vq0);
  bary_poly(x10, x20, x30, v10, v20, v30, &b1);
  if (b1.n == 0) return 0;

  int hit = 0;
  real mint = 1.0;
  span set[5];
  for (int i = 0; i < cop.n; i++)
    for (int j = 0; j < a0.n; j++)
      for (int k = 0; k < a1.n; k++)
        for (int l = 0; l < b0.n; l++)
          for (int m = 0; m < b1.n; m++) {
            set[0] = cop.s[i];
            set[1] = a0.s[j];
            set[2] = a1.s[k];
            set[3] = b0.s[l];
            set[4] = b1.s[m];
            if (!spans_all_meet(set, 5)) continue;
            span isect = spans_common(set, 5);
            int skip = 0;
            for (int p = 0; p < par.n; p++)
              if (span_meet(isect, par.s[p])) {
                skip = 1;
                break;
              }
            if (!skip) {
              mint = smin(mint, isect.l);
              hit = 1;
            }
          }
  if (hit) *tout = ORACLE_OUT(mint);
  return hit;
}

/* src/CTCD.cpp:413-508 -- argument order q0s..q3s, q0e..q3e (q0 = vertex). */
static int prim_vf(const double *x, real eta, double *tout) {
  vec3 q0s = v3(x), q1s = v3(x + 3), q2s = v3(x + 6), q3s = v3(x + 9);
  vec3 q0e = v3(x + 12), q1e = v3(x + 15), q2e = v3(x + 18), q3e = v3(x + 21);
  real minD = eta * eta;
  vec3 v0 = vsub(q0e, q0s), v1 = vsub(q1e, q1s), v2 = vsub(q2e, q2s), v3_ = vsub(q3e, q3s);
  span_list cop = {0}, e1 = {0}, e2 = {0}, e3 = {0};
  vec3 x10, x20, x30, v10, v20, v30;

  x10 = vsub(q0s, q1s);
  v10 = vsub(v0, v1);
  x20 = vcross(vsub(q3s, q1s), vsub(q2s, q1s));
  v20 = vcross(vsub(v3_, v1), vsub(v2, v1));
  x30 = vsub(q3s, q1s);
  v30 = vsub(v3_, v1);
  plane_poly(x10, x20, x30, v10, v20, v30, &e1);
  if (e1.n == 0) return 0;

  x10 = vsub(q0s, q2s);
  v10 = vsub(v0, v2);
  x20 = vcross(vsub(q1s, q2s), vsub(q3s, q2s));
  v20 = vcross(vsub(v1, v2), vsub(v3_, v2));
  x30 = vsub(q1s, q2s);
  v30 = vsub(v1, v2);
  plane_poly(x10, x20, x30, v10, v20, v30, &e2);
  if (e2.n == 0) return 0;

  x10 = vsub(q0s, q3s);
  v10 = vsub(v0, v3_);
  x20 = vcross(vsub(q2s, q3s), vsub(q1s, q3s));
  v20 = vcross(vsub(v2, v3_), vsub(v1, v3_));
  x30 = vsub(q2s, q3s);
  v30 = vsub(v2, v3_);
  plane_poly(x10, x20, x30, v10, v20, v30, &e3);
  if (e3.n == 0) return 0;

  x10 = vsub(q0s, q1s);
  x20 = vsub(q2s, q1s);
  x30 = vsub(q3s, q1s);
  v10 = vsub(v0, v1);
  v20 = vsub(v2, v1);
  v30 = vsub(v3_, v1);
  dist_poly(x10, x20, x30, v10, v20, v30, minD, &cop);
  if (cop.n == 0) return 0;

  int hit = 0;
  real mint = 1.0;
  span set[4];
  for (int i = 0; i < cop.n; i++)
    for (int j = 0; j < e1.n; j++)
      for (int k = 0; k < e2.n; k++)
        for (int l = 0; l < e3.n; l++) {
          set[0] = cop.s[i];
          set[1] = e1.s[j];
          set[2] = e2.s[k];
          set[3] = e3.s[l];
          if (spans_all_meet(set, 4)) {
            mint = smin(spans_common(set, 4).l, mint);
            hit = 1;
          }
        }
  if (hit) *tout = ORACLE_OUT(mint);
  return hit;
}

/* src/CTCD.cpp:511-602 -- argument order q0s,q1s,q2s,q0e,q1e,q2e (q0 = vertex). */
static int prim_ve(const double *x, real eta, double *tout) {
  vec3 q0s = v3(x), q1s = v3(x + 3), q2s = v3(x + 6), q0e = v3(x + 9), q1e = v3(x + 12), q2e = v3(x + 15);
  real op[5];
  real minD = eta * eta;
  vec3 v0 = vsub(q0e, q0s), v1 = vsub(q1e, q1s), v2 = vsub(q2e, q2s);
  span_list colin = {0}, e1 = {0}, e2 = {0};
  vec3 ab = vsub(q2s, q1s), ac = vsub(q0s, q1s), cb = vsub(q2s, q0s);
  vec3 vab = vsub(v2, v1), vac = vsub(v0, v1), vcb = vsub(v2, v0);

  real c = vdot(ab, ac);
  real b = vdot(ac, vab) + vdot(ab, vac);
  real a = vdot(vab, vac);
  op[0] = a;
  op[1] = b;
  op[2] = c;
  sign_intervals(op, 2, &e1, 1);
  if (e1.n == 0) return 0;

  c = vdot(ab, cb);
  b = vdot(cb, vab) + vdot(ab, vcb);
  a = vdot(vab, vcb);
  op[0] = a;
  op[1] = b;
  op[2] = c;
  sign_intervals(op, 2, &e2, 1);
  if (e2.n == 0) return 0;

  real A = vdot(ab, ab);
  real B = 2 * vdot(ab, vab);
  real C = vdot(vab, vab);
  real D = vdot(ac, ac);
  real E = 2 * vdot(ac, vac);
  real F = vdot(vac, vac);
  real G = vdot(ac, ab);
  real H = vdot(vab, ac) + vdot(vac, ab);
  real I = vdot(vab, vac);
  op[4] = A * D - G * G - minD * A;
  op[3] = B * D + A * E - 2 * G * H - minD * B;
  op[2] = B * E + A * F + C * D - H * H - 2 * G * I - minD * C;
  op[1] = B * F + C * E - 2 * H * I;
  op[0] = C * F - I * I;
  sign_intervals(op, 4, &colin, 0);
  if (colin.n == 0) return 0;

  real mint = 1.0;
  int hit = 0;
  span set[3];
  for (int i = 0; i < colin.n; i++)
    for (int j = 0; j < e1.n; j++)
      for (int k = 0; k < e2.n; k++) {
        set[0] = colin.s[i];
        set[1] = e1.s[j];
        set[2] = e2.s[k];
        if (spans_all_meet(set, 3)) {
          mint = smin(spans_common(set, 3).l, mint);
          hit = 1;
        }
      }
  if (hit) *tout = ORACLE_OUT(mint);
  return hit;
}

/* src/CTCD.cpp:604-692 -- argument order q1s,q2s,q1e,q2e.  The reported time
 * is the raw root, which may lie outside [0,1]. */
static int prim_vv(const double *x, real eta, double *tout) {
  vec3 q1s = v3(x), q2s = v3(x + 3), q1e = v3(x + 6), q2e = v3(x + 9);
  int roots = 0;
  real min_d = eta * eta;
  real t1 = 0, t2 = 0;
  vec3 v1 = vsub(q1e, q1s), v2 = vsub(q2e, q2s);
  real a = vdot(v1, v1) + vdot(v2, v2) - 2 * vdot(v1, v2);
  real b = 2 * (vdot(v1, q1s) - vdot(v2, q1s) - vdot(v1, q2s) + vdot(v2, q2s));
  real c = vdot(q1s, q1s) + vdot(q2s, q2s) - 2 * vdot(q1s, q2s) - min_d;
  if (a != 0) {
    roots = quad_roots(a, b, c, &t1, &t2);
  } else if (b != 0) {
    t1 = -c / b;
    roots = 1;
  } else {
    if (c <= 0) {
      *tout = 0.0;
      return 1;
    }
    return 0;
  }
  real op[3] = {a, b, c};
  span_list iv = {0};
  if (roots == 2) {
    sign_segment(0, t1, op, 2, &iv, 0);
    if (iv.n) { *tout = 0.0; return 1; }
    sign_segment(t1, t2, op, 2, &iv, 0);
    if (iv.n) { *tout = ORACLE_OUT(t1); return 1; }
    sign_segment(t2, 1.0, op, 2, &iv, 0);
    if (iv.n) { *tout = ORACLE_OUT(t2); return 1; }
    return 0;
  } else if (roots == 1) {
    sign_segment(0, t1, op, 2, &iv, 0);
    if (iv.n) { *tout = 0.0; return 1; }
    sign_segment(t1, 1.0, op, 2, &iv, 0);
    if (iv.n) { *tout = ORACLE_OUT(t1); return 1; }
    return 0;
  }
  sign_segment(0, 1.0, op, 2, &iv, 0);
  if (iv.n) { *tout = 0.0; return 1; }
  return 0;
}

#endif /* CCD_ORACLE_PRIMS_H */
