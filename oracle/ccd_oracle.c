/* ORACLE / TEST INFRASTRUCTURE ONLY -- see ccd_oracle.h.
 *
 * Every floating-point expression below is evaluated in the same order, with
 * one IEEE rounding per operation, as the reference source it cites, and the
 * file must be compiled with -ffp-contract=off (oracle/Makefile does).
 * Vector algebra follows the Eigen contract of the project's Eigen-API subset:
 * dot = (a0*b0 + a1*b1) + a2*b2, cross = component formula.
 *
 * std::min / std::max are restated as smin/smax with their exact argument
 * semantics ((b < a) ? b : a and (a < b) ? b : a), which matters for NaN.
 */
#include "ccd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ccd_oracle_prims.h"

/* ------------------------------------------------------------ primitive tests (public) */
int oracle_ee(const double *x, double eta, double *t) { return prim_ee(x, eta, t); }
int oracle_vf(const double *x, double eta, double *t) { return prim_vf(x, eta, t); }
int oracle_ve(const double *x, double eta, double *t) { return prim_ve(x, eta, t); }
int oracle_vv(const double *x, double eta, double *t) { return prim_vv(x, eta, t); }

/* ------------------------------------------------------------ threaded batch */
typedef struct {
  int kind;
  int64_t begin, end;
  const double *x;
  const double *eta;
  int eta_per_test;
  uint8_t *hit;
  double *t;
} batch_job;

static void *batch_worker(void *arg) {
  static const int width[4] = {24, 24, 18, 12};
  batch_job *jb = (batch_job *)arg;
  for (int64_t i = jb->begin; i < jb->end; i++) {
    const double *xi = jb->x + i * width[jb->kind];
    double e = jb->eta_per_test ? jb->eta[i] : jb->eta[0];
    int h;
    switch (jb->kind) {
      case 0: h = oracle_vf(xi, e, &jb->t[i]); break;
      case 1: h = oracle_ee(xi, e, &jb->t[i]); break;
      case 2: h = oracle_ve(xi, e, &jb->t[i]); break;
      default: h = oracle_vv(xi, e, &jb->t[i]); break;
    }
    jb->hit[i] = (uint8_t)h;
  }
  return NULL;
}

void oracle_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit, double *t,
                  int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  batch_job jobs[256];
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
  }
  for (int w = 1; w < nthreads; w++) pthread_create(&th[w], NULL, batch_worker, &jobs[w]);
  batch_worker(&jobs[0]);
  for (int w = 1; w < nthreads; w++) pthread_join(th[w], NULL);
}

/* ------------------------------------------------------------ stencils (src/Stencils.h) */
void oracle_vf_canon(int p, int q0, int q1, int q2, int32_t *out) {
  /* VertexFaceStencil: the face's three vertices ascending. */
  int a = q0, b = q1, c = q2, tmp;
  if (a > b) { tmp = a; a = b; b = tmp; }
  if (b > c) { tmp = b; b = c; c = tmp; }
  if (a > b) { tmp = a; a = b; b = tmp; }
  out[0] = p; out[1] = a; out[2] = b; out[3] = c;
}

void oracle_ee_canon(int p0, int p1, int q0, int q1, int32_t *out) {
  /* EdgeEdgeStencil: each edge ascending, then edges ordered by first vertex. */
  int a0 = p0 <= p1 ? p0 : p1, a1 = p0 <= p1 ? p1 : p0;
  int b0 = q0 <= q1 ? q0 : q1, b1 = q0 <= q1 ? q1 : q0;
  if (a0 > b0) {
    int t0 = a0, t1 = a1;
    a0 = b0; a1 = b1; b0 = t0; b1 = t1;
  }
  out[0] = a0; out[1] = a1; out[2] = b0; out[3] = b1;
}

/* ------------------------------------------------------------ swept-volume candidates */
typedef struct { int64_t n, cap; int32_t *v; } i4_vec;

static int i4_push(i4_vec *vec, const int32_t *r) {
  if (vec->n == vec->cap) {
    int64_t nc = vec->cap ? 2 * vec->cap : 1024;
    int32_t *nv = (int32_t *)realloc(vec->v, (size_t)nc * 4 * sizeof(int32_t));
    if (!nv) return -1;
    vec->v = nv;
    vec->cap = nc;
  }
  memcpy(vec->v + 4 * vec->n, r, 4 * sizeof(int32_t));
  vec->n++;
  return 0;
}

static int cmp_i4(const void *a, const void *b) {
  const int32_t *x = (const int32_t *)a, *y = (const int32_t *)b;
  for (int i = 0; i < 4; i++) {
    if (x[i] < y[i]) return -1;
    if (x[i] > y[i]) return 1;
  }
  return 0;
}

static void i4_sort_unique(i4_vec *vec) {
  if (vec->n == 0) return;
  qsort(vec->v, (size_t)vec->n, 4 * sizeof(int32_t), cmp_i4);
  int64_t w = 1;
  for (int64_t r = 1; r < vec->n; r++)
    if (cmp_i4(vec->v + 4 * r, vec->v + 4 * (w - 1)) != 0) {
      if (w != r) memcpy(vec->v + 4 * w, vec->v + 4 * r, 4 * sizeof(int32_t));
      w++;
    }
  vec->n = w;
}

static i4_vec g_vf, g_ee;
static int64_t g_pairs;

typedef struct { double lo; int face; } sweep_key;
static int cmp_sweep(const void *a, const void *b) {
  double x = ((const sweep_key *)a)->lo, y = ((const sweep_key *)b)->lo;
  if (x < y) return -1;
  if (x > y) return 1;
  return ((const sweep_key *)a)->face - ((const sweep_key *)b)->face;
}

/* TrivialBroadPhase::findCollisionCandidates (src/TrivialBroadPhase.cpp:4-53):
 * every vertex with every face that does not contain it, every pair of face
 * edges without a common vertex, minus all-fixed stencils.  Positions and
 * padding are not used. */
static int trivial_candidates(int nverts, int nfaces, const int32_t *faces, const uint8_t *fixed) {
#define FIXED(v) (fixed && fixed[(v)])
  int rc = 0;
  int32_t r[4];
  for (int i = 0; i < nverts && !rc; i++) {
    for (int j = 0; j < nfaces && !rc; j++) {
      const int32_t *F = faces + 3 * (size_t)j;
      if (F[0] == i || F[1] == i || F[2] == i) continue;
      if (FIXED(i) && FIXED(F[0]) && FIXED(F[1]) && FIXED(F[2])) continue;
      oracle_vf_canon(i, F[0], F[1], F[2], r);
      rc |= i4_push(&g_vf, r);
    }
  }
  for (int64_t e1 = 0; e1 < 3 * (int64_t)nfaces && !rc; e1++) {
    for (int64_t e2 = e1 + 1; e2 < 3 * (int64_t)nfaces && !rc; e2++) {
      const int64_t f1 = e1 / 3, f2 = e2 / 3;
      const int a = faces[3 * f1 + e1 % 3], b = faces[3 * f1 + (e1 + 1) % 3];
      const int c = faces[3 * f2 + e2 % 3], d = faces[3 * f2 + (e2 + 1) % 3];
      if (a == c || a == d || b == c || b == d) continue;
      if (FIXED(a) && FIXED(b) && FIXED(c) && FIXED(d)) continue;
      oracle_ee_canon(a, b, c, d, r);
      rc |= i4_push(&g_ee, r);
    }
  }
#undef FIXED
  return rc;
}

static int broadphase_impl(int kind, int nverts, const double *qstart, const double *qend, const int32_t *hoff,
                           const double *hpos, int nfaces, const int32_t *faces, double eta, const uint8_t *fixed,
                           int64_t *n_vf, int64_t *n_ee);

int oracle_broadphase(int kind, int nverts, const double *qstart, const double *qend, int nfaces,
                      const int32_t *faces, double eta, const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee) {
  return broadphase_impl(kind, nverts, qstart, qend, NULL, NULL, nfaces, faces, eta, fixed, n_vf, n_ee);
}

int oracle_broadphase_history(int kind, int nverts, const int32_t *offsets, const double *positions, int nfaces,
                              const int32_t *faces, double eta, const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee) {
  return broadphase_impl(kind, nverts, NULL, NULL, offsets, positions, nfaces, faces, eta, fixed, n_vf, n_ee);
}

static int broadphase_impl(int kind, int nverts, const double *qstart, const double *qend, const int32_t *hoff,
                           const double *hpos, int nfaces, const int32_t *faces, double eta, const uint8_t *fixed,
                           int64_t *n_vf, int64_t *n_ee) {
  if (kind == 2) {
    g_vf.n = g_ee.n = 0;
    g_pairs = 0;
    if (trivial_candidates(nverts, nfaces, faces, fixed)) return -1;
    i4_sort_unique(&g_vf);
    i4_sort_unique(&g_ee);
    *n_vf = g_vf.n;
    *n_ee = g_ee.n;
    return 0;
  }
  int K = (kind == 0) ? 13 : 3;
  /* The 13 k-DOP directions, normalised as the reference does (KDOPBroadPhase.cpp:12-31). */
  static const double dirs[13][3] = {{1, 0, 0},  {0, 1, 0},  {0, 0, 1},  {1, 1, 0},  {1, -1, 0},
                                     {0, 1, 1},  {0, 1, -1}, {1, 0, 1},  {1, 0, -1}, {1, 1, 1},
                                     {1, 1, -1}, {1, -1, 1}, {1, -1, -1}};
  vec3 axis[13];
  for (int k = 0; k < 13; k++) {
    vec3 a = {dirs[k][0], dirs[k][1], dirs[k][2]};
    double nrm = vnorm(a);
    axis[k].x = a.x / nrm;
    axis[k].y = a.y / nrm;
    axis[k].z = a.z / nrm;
  }
  g_vf.n = g_ee.n = 0;
  g_pairs = 0;
  double *lo = (double *)malloc((size_t)nfaces * K * sizeof(double));
  double *hi = (double *)malloc((size_t)nfaces * K * sizeof(double));
  sweep_key *order = (sweep_key *)malloc((size_t)nfaces * sizeof(sweep_key));
  if ((nfaces && (!lo || !hi || !order))) {
    free(lo); free(hi); free(order);
    return -1;
  }
  /* Leaf slabs (KDOPBroadPhase.cpp:43-74 / AABBBroadPhase.cpp:18-46). */
  for (int f = 0; f < nfaces; f++) {
    double *L = lo + (size_t)f * K, *H = hi + (size_t)f * K;
    for (int k = 0; k < K; k++) {
      L[k] = INFINITY;
      H[k] = -INFINITY;
    }
    for (int j = 0; j < 3; j++) {
      int vtx = faces[3 * f + j];
      /* every History entry of the vertex (KDOPBroadPhase.cpp:60-70) */
      int e0 = hoff ? hoff[vtx] : 0, e1 = hoff ? hoff[vtx + 1] : 2;
      for (int e = e0; e < e1; e++) {
        vec3 pos = hoff ? v3(hpos + 3 * (size_t)e) : v3((e == 0 ? qstart : qend) + 3 * (size_t)vtx);
        for (int k = 0; k < K; k++) {
          double s = (kind == 0) ? vdot(pos, axis[k]) : (k == 0 ? pos.x : (k == 1 ? pos.y : pos.z));
          L[k] = smin(s - eta, L[k]);
          H[k] = smax(s + eta, H[k]);
        }
      }
    }
    order[f].lo = L[0];
    order[f].face = f;
  }
  /* Every pair of leaves whose slabs overlap on all axes is reached by the
   * reference's self-traversal (a parent's slab contains its children's), so
   * the candidate set is a function of the leaf slabs alone; a sweep along
   * axis 0 enumerates exactly those pairs. */
  qsort(order, (size_t)nfaces, sizeof(sweep_key), cmp_sweep);
  int rc = 0;
  for (int ia = 0; ia < nfaces && !rc; ia++) {
    int fa = order[ia].face;
    const double *La = lo + (size_t)fa * K, *Ha = hi + (size_t)fa * K;
    for (int ib = ia + 1; ib < nfaces && !rc; ib++) {
      int fb = order[ib].face;
      const double *Lb = lo + (size_t)fb * K, *Hb = hi + (size_t)fb * K;
      if (Ha[0] < Lb[0]) break;
      int sep = 0;
      for (int k = 0; k < K; k++)
        if (Ha[k] < Lb[k] || Hb[k] < La[k]) {
          sep = 1;
          break;
        }
      if (sep) continue;
      const int32_t *A = faces + 3 * (size_t)fa, *B = faces + 3 * (size_t)fb;
      int nb = 0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
          if (A[i] == B[j]) nb = 1;
      if (nb) continue;
      g_pairs++;
      /* Emission (KDOPBroadPhase.cpp:150-183), from one visiting order; the
       * other order emits the same canonical stencils. */
#define FIXED(v) (fixed && fixed[(v)])
      int32_t r[4];
      for (int i = 0; i < 3; i++) {
        int allA = FIXED(A[i]) && FIXED(B[0]) && FIXED(B[1]) && FIXED(B[2]);
        int allB = FIXED(B[i]) && FIXED(A[0]) && FIXED(A[1]) && FIXED(A[2]);
        if (!allA) {
          oracle_vf_canon(A[i], B[0], B[1], B[2], r);
          rc |= i4_push(&g_vf, r);
        }
        if (!allB) {
          oracle_vf_canon(B[i], A[0], A[1], A[2], r);
          rc |= i4_push(&g_vf, r);
        }
        for (int j = 0; j < 3; j++) {
          int allE = FIXED(A[i]) && FIXED(A[(i + 1) % 3]) && FIXED(B[j]) && FIXED(B[(j + 1) % 3]);
          if (!allE) {
            oracle_ee_canon(A[i], A[(i + 1) % 3], B[j], B[(j + 1) % 3], r);
            rc |= i4_push(&g_ee, r);
          }
        }
      }
#undef FIXED
    }
  }
  free(lo);
  free(hi);
  free(order);
  if (rc) return -1;
  i4_sort_unique(&g_vf);
  i4_sort_unique(&g_ee);
  *n_vf = g_vf.n;
  *n_ee = g_ee.n;
  return 0;
}

void oracle_broadphase_get(int32_t *vf, int32_t *ee) {
  if (g_vf.n) memcpy(vf, g_vf.v, (size_t)g_vf.n * 4 * sizeof(int32_t));
  if (g_ee.n) memcpy(ee, g_ee.v, (size_t)g_ee.n * 4 * sizeof(int32_t));
}

int64_t oracle_broadphase_face_pairs(void) { return g_pairs; }

/* ------------------------------------------------------------ narrow phase over stencils */
/* History::stitchCommonHistory (src/History.cpp:98-140) on a two-entry
 * history yields one segment whose start point is (1*start + 0*end)/1 and
 * whose end point is the end position itself. */
static void stitched_start(const double *qs, const double *qe, int v, double *out) {
  for (int c = 0; c < 3; c++) out[c] = (1.0 * qs[3 * (size_t)v + c] + 0.0 * qe[3 * (size_t)v + c]) / 1.0;
}

/* CTCDNarrowPhase::checkVFS (src/CTCDNarrowPhase.cpp:24-72). */
static int chain_vf(const double *P0, const double *P1, double eta, double *t);
static int chain_ee(const double *P0, const double *P1, double eta, double *t);

static int check_vf_stencil(const double *qs, const double *qe, const int32_t *st, double eta, double *t) {
  double P0[12], P1[12];
  for (int i = 0; i < 4; i++) {
    stitched_start(qs, qe, st[i], P0 + 3 * i);
    memcpy(P1 + 3 * i, qe + 3 * (size_t)st[i], 3 * sizeof(double));
  }
  return chain_vf(P0, P1, eta, t);
}

/* The chain of CTCDNarrowPhase::checkVFS (src/CTCDNarrowPhase.cpp:33-69) on
 * one segment: 0 vertex-face, 1 vertex-edge, 2 vertex-vertex hit, -1 none. */
static int chain_vf(const double *P0, const double *P1, double eta, double *t) {
  double x[24];
  memcpy(x, P0, 12 * sizeof(double));
  memcpy(x + 12, P1, 12 * sizeof(double));
  if (oracle_vf(x, eta, t)) return 0;
  for (int edge = 0; edge < 3; edge++) {
    int i1 = 1 + (edge % 3), i2 = 1 + ((edge + 1) % 3);
    memcpy(x + 0, P0, 3 * sizeof(double));
    memcpy(x + 3, P0 + 3 * i1, 3 * sizeof(double));
    memcpy(x + 6, P0 + 3 * i2, 3 * sizeof(double));
    memcpy(x + 9, P1, 3 * sizeof(double));
    memcpy(x + 12, P1 + 3 * i1, 3 * sizeof(double));
    memcpy(x + 15, P1 + 3 * i2, 3 * sizeof(double));
    if (oracle_ve(x, eta, t)) return 1;
  }
  for (int vert = 0; vert < 3; vert++) {
    memcpy(x + 0, P0, 3 * sizeof(double));
    memcpy(x + 3, P0 + 3 * (1 + vert), 3 * sizeof(double));
    memcpy(x + 6, P1, 3 * sizeof(double));
    memcpy(x + 9, P1 + 3 * (1 + vert), 3 * sizeof(double));
    if (oracle_vv(x, eta, t)) return 2;
  }
  return -1;
}

/* CTCDNarrowPhase::checkEES (src/CTCDNarrowPhase.cpp:74-135). */
static int check_ee_stencil(const double *qs, const double *qe, const int32_t *st, double eta, double *t) {
  double P0[12], P1[12];
  for (int i = 0; i < 4; i++) {
    stitched_start(qs, qe, st[i], P0 + 3 * i);
    memcpy(P1 + 3 * i, qe + 3 * (size_t)st[i], 3 * sizeof(double));
  }
  return chain_ee(P0, P1, eta, t);
}

/* The chain of CTCDNarrowPhase::checkEES (src/CTCDNarrowPhase.cpp:84-129) on
 * one segment. */
static int chain_ee(const double *P0, const double *P1, double eta, double *t) {
  static const int ve[4][3] = {{0, 2, 3}, {1, 2, 3}, {2, 0, 1}, {3, 0, 1}};
  static const int vv[4][2] = {{0, 2}, {0, 3}, {1, 2}, {1, 3}};
  double x[24];
  memcpy(x, P0, 12 * sizeof(double));
  memcpy(x + 12, P1, 12 * sizeof(double));
  if (oracle_ee(x, eta, t)) return 0;
  for (int c = 0; c < 4; c++) {
    for (int j = 0; j < 3; j++) {
      memcpy(x + 3 * j, P0 + 3 * ve[c][j], 3 * sizeof(double));
      memcpy(x + 9 + 3 * j, P1 + 3 * ve[c][j], 3 * sizeof(double));
    }
    if (oracle_ve(x, eta, t)) return 1;
  }
  for (int c = 0; c < 4; c++) {
    memcpy(x + 0, P0 + 3 * vv[c][0], 3 * sizeof(double));
    memcpy(x + 3, P0 + 3 * vv[c][1], 3 * sizeof(double));
    memcpy(x + 6, P1 + 3 * vv[c][0], 3 * sizeof(double));
    memcpy(x + 9, P1 + 3 * vv[c][1], 3 * sizeof(double));
    if (oracle_vv(x, eta, t)) return 2;
  }
  return -1;
}

typedef struct {
  const double *qs, *qe;
  int64_t n_vf, n_ee, begin, end;
  const int32_t *vf, *ee;
  const double *vf_eta, *ee_eta;
  uint8_t *vf_hit, *ee_hit;
  double *vf_t, *ee_t;
  int8_t *vf_which, *ee_which;
} np_job;

static void *np_worker(void *arg) {
  np_job *jb = (np_job *)arg;
  for (int64_t g = jb->begin; g < jb->end; g++) {
    double t = 0;
    if (g < jb->n_vf) {
      int w = check_vf_stencil(jb->qs, jb->qe, jb->vf + 4 * g, jb->vf_eta[g], &t);
      jb->vf_hit[g] = (uint8_t)(w >= 0);
      if (w >= 0 && jb->vf_t) jb->vf_t[g] = t;
      if (jb->vf_which) jb->vf_which[g] = (int8_t)w;
    } else {
      int64_t i = g - jb->n_vf;
      int w = check_ee_stencil(jb->qs, jb->qe, jb->ee + 4 * i, jb->ee_eta[i], &t);
      jb->ee_hit[i] = (uint8_t)(w >= 0);
      if (w >= 0 && jb->ee_t) jb->ee_t[i] = t;
      if (jb->ee_which) jb->ee_which[i] = (int8_t)w;
    }
  }
  return NULL;
}

void oracle_narrowphase(int nverts, const double *qstart, const double *qend, int64_t n_vf, const int32_t *vf,
                        const double *vf_eta, int64_t n_ee, const int32_t *ee, const double *ee_eta, uint8_t *vf_hit,
                        uint8_t *ee_hit, double *vf_t, double *ee_t, int8_t *vf_which, int8_t *ee_which,
                        int nthreads) {
  (void)nverts;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  np_job jobs[256];
  pthread_t th[256];
  int64_t total = n_vf + n_ee;
  for (int w = 0; w < nthreads; w++) {
    np_job j = {qstart, qend, n_vf, n_ee, total * w / nthreads, total * (w + 1) / nthreads, vf, ee, vf_eta, ee_eta,
                vf_hit, ee_hit, vf_t, ee_t, vf_which, ee_which};
    jobs[w] = j;
  }
  for (int w = 1; w < nthreads; w++) pthread_create(&th[w], NULL, np_worker, &jobs[w]);
  np_worker(&jobs[0]);
  for (int w = 1; w < nthreads; w++) pthread_join(th[w], NULL);
}

/* ------------------------------------------------------------ Distance (include/Distance.h, src/Distance.cpp) */
/* Distance::clamp (include/Distance.h:182-185). */
static double dclamp(double u) { return smin(1.0, smax(u, 0.0)); }

/* Distance::vertexFaceDistance (include/Distance.h:31-113). */
static vec3 vf_distance(vec3 p, vec3 q0, vec3 q1, vec3 q2, double *b) {
  vec3 ab = vsub(q1, q0), ac = vsub(q2, q0), ap = vsub(p, q0);
  double d1 = vdot(ab, ap), d2 = vdot(ac, ap);
  if (d1 <= 0 && d2 <= 0) {
    b[0] = 1.0; b[1] = 0.0; b[2] = 0.0;
    return vsub(q0, p);
  }
  vec3 bp = vsub(p, q1);
  double d3 = vdot(ab, bp), d4 = vdot(ac, bp);
  if (d3 >= 0 && d4 <= d3) {
    b[0] = 0.0; b[1] = 1.0; b[2] = 0.0;
    return vsub(q1, p);
  }
  double vc = d1 * d4 - d3 * d2;
  if ((vc <= 0) && (d1 >= 0) && (d3 <= 0)) {
    double v = d1 / (d1 - d3);
    b[0] = 1.0 - v; b[1] = v; b[2] = 0;
    return vsub(vadd(q0, vscale(v, ab)), p);
  }
  vec3 cp = vsub(p, q2);
  double d5 = vdot(ab, cp), d6 = vdot(ac, cp);
  if (d6 >= 0 && d5 <= d6) {
    b[0] = 0; b[1] = 0; b[2] = 1.0;
    return vsub(q2, p);
  }
  double vb = d5 * d2 - d1 * d6;
  if ((vb <= 0) && (d2 >= 0) && (d6 <= 0)) {
    double w = d2 / (d2 - d6);
    b[0] = 1 - w; b[1] = 0; b[2] = w;
    return vsub(vadd(q0, vscale(w, ac)), p);
  }
  double va = d3 * d6 - d5 * d4;
  if ((va <= 0) && (d4 - d3 >= 0) && (d5 - d6 >= 0)) {
    double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    b[0] = 0; b[1] = 1.0 - w; b[2] = w;
    return vsub(vadd(q1, vscale(w, vsub(q2, q1))), p);
  }
  double denom = 1.0 / (va + vb + vc);
  double v = vb * denom, w = vc * denom;
  double u = 1.0 - v - w;
  b[0] = u; b[1] = v; b[2] = w;
  return vsub(vadd(vadd(vscale(u, q0), vscale(v, q1)), vscale(w, q2)), p);
}

/* Distance::edgeEdgeDistance (include/Distance.h:117-170). */
static vec3 ee_distance(vec3 p0, vec3 p1, vec3 q0, vec3 q1, double *bary) {
  vec3 d1 = vsub(p1, p0), d2 = vsub(q1, q0), r = vsub(p0, q0);
  double a = vdot(d1, d1), e = vdot(d2, d2), f = vdot(d2, r);
  double s, t;
  double c = vdot(d1, r), b = vdot(d1, d2);
  double denom = a * e - b * b;
  if (denom != 0.0)
    s = dclamp((b * f - c * e) / denom);
  else
    s = 0;
  double tnom = b * s + f;
  if (tnom < 0 || e == 0) {
    t = 0;
    if (a == 0) s = 0;
    else s = dclamp(-c / a);
  } else if (tnom > e) {
    t = 1.0;
    if (a == 0) s = 0;
    else s = dclamp((b - c) / a);
  } else {
    t = tnom / e;
  }
  vec3 c1 = vadd(p0, vscale(s, d1)), c2 = vadd(q0, vscale(t, d2));
  bary[0] = 1.0 - s; bary[1] = s; bary[2] = 1.0 - t; bary[3] = t;
  return vsub(c2, c1);
}

void oracle_distance_batch(int kind, int64_t n, const double *rows, double *vec, double *bary) {
  for (int64_t i = 0; i < n; i++) {
    const double *x = rows + 12 * i;
    double b[4];
    vec3 r = kind == 0 ? vf_distance(v3(x), v3(x + 3), v3(x + 6), v3(x + 9), b)
                       : ee_distance(v3(x), v3(x + 3), v3(x + 6), v3(x + 9), b);
    vec[3 * i] = r.x; vec[3 * i + 1] = r.y; vec[3 * i + 2] = r.z;
    if (bary)
      for (int k = 0; k < (kind == 0 ? 3 : 4); k++) bary[(kind == 0 ? 3 : 4) * i + k] = b[k];
  }
}

/* Distance::vertexPlaneDistanceLessThan / lineLineDistanceLessThan
 * (include/Distance.h:13-27). */
void oracle_distance_less_than(int kind, int64_t n, const double *rows, const double *eta, int eta_per_row,
                               uint8_t *out) {
  for (int64_t i = 0; i < n; i++) {
    const double *x = rows + 12 * i;
    double e = eta[eta_per_row ? i : 0];
    vec3 a = v3(x), b = v3(x + 3), c = v3(x + 6), d = v3(x + 9);
    vec3 cr;
    double s;
    if (kind == 0) {
      cr = vcross(vsub(c, b), vsub(d, b));
      s = vdot(cr, vsub(a, b));
    } else {
      cr = vcross(vsub(b, a), vsub(d, c));
      s = vdot(cr, vsub(c, a));
    }
    out[i] = (uint8_t)(s * s < e * e * vdot(cr, cr));
  }
}

/* Distance::meshSelfDistance (src/Distance.cpp:12-66). */
double oracle_mesh_self_distance(int nverts, const double *verts, int nfaces, const int32_t *faces,
                                 const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee) {
  double closest = INFINITY;
  for (int i = 0; i < nverts; i++) {
    for (int j = 0; j < nfaces; j++) {
      const int32_t *fj = faces + 3 * (int64_t)j;
      if (fj[0] == i || fj[1] == i || fj[2] == i) continue; /* Mesh::vertexOfFace (src/Mesh.cpp:5-11) */
      for (int k = 0; k < 3; k++) {
        vec3 d = vsub(v3(verts + 3 * (int64_t)i), v3(verts + 3 * (int64_t)fj[k]));
        double dist = vdot(d, d);
        if (dist < closest) closest = dist;
      }
    }
  }
  closest = sqrt(closest);
  int64_t nvf = 0, nee = 0;
  if (oracle_broadphase(1, nverts, verts, verts, nfaces, faces, closest, fixed, &nvf, &nee) != 0) return NAN;
  int32_t *vf = (int32_t *)malloc((size_t)(4 * nvf + 1) * sizeof(int32_t));
  int32_t *ee = (int32_t *)malloc((size_t)(4 * nee + 1) * sizeof(int32_t));
  if (!vf || !ee) {
    free(vf);
    free(ee);
    return NAN;
  }
  oracle_broadphase_get(vf, ee);
  closest = INFINITY;
  for (int64_t i = 0; i < nvf; i++) {
    const int32_t *s = vf + 4 * i;
    double b[3];
    double dist = vnorm(vf_distance(v3(verts + 3 * (int64_t)s[0]), v3(verts + 3 * (int64_t)s[1]),
                                    v3(verts + 3 * (int64_t)s[2]), v3(verts + 3 * (int64_t)s[3]), b));
    if (dist < closest) closest = dist;
  }
  for (int64_t i = 0; i < nee; i++) {
    const int32_t *s = ee + 4 * i;
    double b[4];
    double dist = vnorm(ee_distance(v3(verts + 3 * (int64_t)s[0]), v3(verts + 3 * (int64_t)s[1]),
                                    v3(verts + 3 * (int64_t)s[2]), v3(verts + 3 * (int64_t)s[3]), b));
    if (dist < closest) closest = dist;
  }
  free(vf);
  free(ee);
  if (n_vf) *n_vf = nvf;
  if (n_ee) *n_ee = nee;
  return closest;
}

/* The vertex scan of Distance::meshSelfDistance (src/Distance.cpp:21-34)
 * restricted to vertices i in [i0, i1): the least squared distance found
 * there (the CPU baseline times it on a bounded sample of vertices). */
double oracle_vertex_scan(int nverts, const double *verts, int nfaces, const int32_t *faces, int i0, int i1) {
  double closest = INFINITY;
  if (i0 < 0) i0 = 0;
  if (i1 > nverts) i1 = nverts;
  for (int i = i0; i < i1; i++) {
    for (int j = 0; j < nfaces; j++) {
      const int32_t *fj = faces + 3 * (int64_t)j;
      if (fj[0] == i || fj[1] == i || fj[2] == i) continue;
      for (int k = 0; k < 3; k++) {
        vec3 d = vsub(v3(verts + 3 * (int64_t)i), v3(verts + 3 * (int64_t)fj[k]));
        double dist = vdot(d, d);
        if (dist < closest) closest = dist;
      }
    }
  }
  return closest;
}

/* ------------------------------------------------------------ penalty forces (src/PenaltyPotential.cpp, src/PenaltyGroup.cpp) */
static void add3(double *g, vec3 a) { g[0] = g[0] + a.x; g[1] = g[1] + a.y; g[2] = g[2] + a.z; }
static void sub3(double *g, vec3 a) { g[0] = g[0] - a.x; g[1] = g[1] - a.y; g[2] = g[2] - a.z; }

/* VertexFacePenaltyPotential::addForce (src/PenaltyPotential.cpp:7-34). */
static int vf_penalty(const double *q, const double *v, double *G, const int32_t *st, double oe, double ie,
                      double stiffness, double cor) {
  int32_t s[4];
  oracle_vf_canon(st[0], st[1], st[2], st[3], s);
  vec3 p = v3(q + 3 * (size_t)s[0]), q0 = v3(q + 3 * (size_t)s[1]), q1 = v3(q + 3 * (size_t)s[2]),
       q2 = v3(q + 3 * (size_t)s[3]);
  vec3 c = vcross(vsub(q1, q0), vsub(q2, q0));
  if (!(vdot(c, vsub(p, q0)) * vdot(c, vsub(p, q0)) < oe * oe * vdot(c, c))) return 0;
  double b[3];
  vec3 cv = vf_distance(p, q0, q1, q2, b);
  double dist = vnorm(cv);
  if (dist >= oe || dist < ie) return 0;
  vec3 vp = v3(v + 3 * (size_t)s[0]);
  vec3 nvp = {-vp.x, -vp.y, -vp.z};
  vec3 relvel = vadd(vadd(vadd(nvp, vscale(b[0], v3(v + 3 * (size_t)s[1]))), vscale(b[1], v3(v + 3 * (size_t)s[2]))),
                     vscale(b[2], v3(v + 3 * (size_t)s[3])));
  if (vdot(relvel, cv) > 0) stiffness *= cor;
  double k = stiffness * (oe - dist) / (oe - ie);
  vec3 sc = vscale(k, cv);
  vec3 lf = {sc.x / dist, sc.y / dist, sc.z / dist};
  sub3(G + 3 * (size_t)s[0], lf);
  add3(G + 3 * (size_t)s[1], vscale(b[0], lf));
  add3(G + 3 * (size_t)s[2], vscale(b[1], lf));
  add3(G + 3 * (size_t)s[3], vscale(b[2], lf));
  return 1;
}

/* EdgeEdgePenaltyPotential::addForce (src/PenaltyPotential.cpp:36-64). */
static int ee_penalty(const double *q, const double *v, double *G, const int32_t *st, double oe, double ie,
                      double stiffness, double cor) {
  int32_t s[4];
  oracle_ee_canon(st[0], st[1], st[2], st[3], s);
  vec3 p0 = v3(q + 3 * (size_t)s[0]), p1 = v3(q + 3 * (size_t)s[1]), q0 = v3(q + 3 * (size_t)s[2]),
       q1 = v3(q + 3 * (size_t)s[3]);
  vec3 c = vcross(vsub(p1, p0), vsub(q1, q0));
  if (!(vdot(c, vsub(q0, p0)) * vdot(c, vsub(q0, p0)) < oe * oe * vdot(c, c))) return 0;
  double b[4];
  vec3 cv = ee_distance(p0, p1, q0, q1, b);
  double dist = vnorm(cv);
  if (dist >= oe || dist < ie) return 0;
  vec3 relvel = vadd(vadd(vsub(vscale(-b[0], v3(v + 3 * (size_t)s[0])), vscale(b[1], v3(v + 3 * (size_t)s[1]))),
                          vscale(b[2], v3(v + 3 * (size_t)s[2]))),
                     vscale(b[3], v3(v + 3 * (size_t)s[3])));
  if (vdot(relvel, cv) > 0) stiffness *= cor;
  double k = stiffness * (oe - dist) / (oe - ie);
  vec3 sc = vscale(k, cv);
  vec3 lf = {sc.x / dist, sc.y / dist, sc.z / dist};
  sub3(G + 3 * (size_t)s[0], vscale(b[0], lf));
  sub3(G + 3 * (size_t)s[1], vscale(b[1], lf));
  add3(G + 3 * (size_t)s[2], vscale(b[2], lf));
  add3(G + 3 * (size_t)s[3], vscale(b[3], lf));
  return 1;
}

/* PenaltyGroup::addForce (src/PenaltyGroup.cpp:34-52). */
int oracle_penalty_group_force(int nverts, const double *q, const double *v, int64_t n_vf, const int32_t *vf,
                               const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee, const uint8_t *ee_isnew,
                               double outer_eta, double inner_eta, double stiffness, double cor, double dt,
                               double *F, uint8_t *vf_fired, uint8_t *ee_fired) {
  double *G = (double *)calloc((size_t)3 * (nverts > 0 ? nverts : 1), sizeof(double));
  if (!G) return -1;
  int newused = 0;
  for (int64_t i = 0; i < n_vf; i++) {
    int fired = vf_penalty(q, v, G, vf + 4 * i, outer_eta, inner_eta, stiffness, cor);
    if (vf_fired) vf_fired[i] = (uint8_t)fired;
    newused |= fired && vf_isnew && vf_isnew[i];
  }
  for (int64_t i = 0; i < n_ee; i++) {
    int fired = ee_penalty(q, v, G, ee + 4 * i, outer_eta, inner_eta, stiffness, cor);
    if (ee_fired) ee_fired[i] = (uint8_t)fired;
    newused |= fired && ee_isnew && ee_isnew[i];
  }
  for (int64_t i = 0; i < 3 * (int64_t)nverts; i++) F[i] = F[i] + G[i] * dt;
  free(G);
  return newused;
}


/* ------------------------------------------------------------ multi-entry history */
/* History::stitchCommonHistory (src/History.cpp:98-140) over the four
 * vertices v of a history given as offsets / times / positions: writes the
 * stitched entries' positions (12 doubles each) into out (room for cap) and
 * returns their number. */
static int stitch4(const int32_t *off, const double *times, const double *pos, const int32_t *v, double *out,
                   int cap) {
  int it[4], end[4], n = 0;
  for (int i = 0; i < 4; i++) {
    it[i] = off[v[i]];
    end[i] = off[v[i] + 1];
  }
  double curtime = 0;
  while (curtime <= 1.0 && n < cap) {
    double newtime = INFINITY;
    double *e = out + 12 * (size_t)n;
    for (int i = 0; i < 4; i++) {
      int next = it[i] + 1;
      while (next != end[i] && times[next] <= curtime) {
        ++next;
        ++it[i];
      }
      const double *oldpos = pos + 3 * (size_t)it[i];
      if (next == end[i]) {
        for (int k = 0; k < 3; k++) e[3 * i + k] = oldpos[k];
      } else {
        const double *newpos = pos + 3 * (size_t)next;
        double dt = times[next] - times[it[i]];
        double a = curtime - times[it[i]];
        double b = times[next] - curtime;
        for (int k = 0; k < 3; k++) e[3 * i + k] = (b * oldpos[k] + a * newpos[k]) / dt;
        newtime = smin(newtime, times[next]);
      }
    }
    n++;
    curtime = newtime;
  }
  return n;
}

/* CTCDNarrowPhase::findCollisions (src/CTCDNarrowPhase.cpp:9-135) on a
 * multi-entry history: each stencil's chain on every segment of its stitched
 * common history; hit / t / which of the first segment that hits. */
int oracle_narrowphase_history(int nverts, const int32_t *offsets, const double *times, const double *positions,
                               int64_t n_vf, const int32_t *vf, const double *vf_eta, int64_t n_ee, const int32_t *ee,
                               const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit, double *vf_t, double *ee_t,
                               int8_t *vf_which, int8_t *ee_which) {
  int maxe = 0;
  for (int v = 0; v < nverts; v++)
    if (offsets[v + 1] - offsets[v] > maxe) maxe = offsets[v + 1] - offsets[v];
  const int cap = 4 * maxe + 2;
  double *buf = (double *)malloc((size_t)cap * 12 * sizeof(double));
  if (!buf) return -1;
  for (int kind = 0; kind < 2; kind++) {
    const int64_t n = kind == 0 ? n_vf : n_ee;
    for (int64_t i = 0; i < n; i++) {
      const int32_t *raw = (kind == 0 ? vf : ee) + 4 * i;
      int32_t st[4];
      if (kind == 0)
        oracle_vf_canon(raw[0], raw[1], raw[2], raw[3], st);
      else
        oracle_ee_canon(raw[0], raw[1], raw[2], raw[3], st);
      const int ne = stitch4(offsets, times, positions, st, buf, cap);
      const double eta = (kind == 0 ? vf_eta : ee_eta)[i];
      int w = -1;
      double t = 0;
      for (int sgm = 0; sgm + 1 < ne && w < 0; sgm++)
        w = kind == 0 ? chain_vf(buf + 12 * (size_t)sgm, buf + 12 * (size_t)(sgm + 1), eta, &t)
                      : chain_ee(buf + 12 * (size_t)sgm, buf + 12 * (size_t)(sgm + 1), eta, &t);
      uint8_t *hit = kind == 0 ? vf_hit : ee_hit;
      double *tt = kind == 0 ? vf_t : ee_t;
      int8_t *wh = kind == 0 ? vf_which : ee_which;
      hit[i] = (uint8_t)(w >= 0);
      if (w >= 0 && tt) tt[i] = t;
      if (wh) wh[i] = (int8_t)w;
    }
  }
  free(buf);
  return 0;
}

/* ------------------------------------------------------------ separating-plane narrow phase
 * SeparatingPlaneNarrowPhase (src/SeparatingPlaneNarrowPhase.cpp) on a
 * multi-entry history given as offsets / times / positions. */
typedef struct {
  const int32_t *off;
  const double *t, *p;
} hist_view;

/* History::getPosAtTime (src/History.cpp:54-80): binary halving while the
 * range holds 10 or more entries, then a forward scan. */
static void pos_at_time(hist_view h, int v, double time, vec3 *pos, int *idx) {
  const int base = h.off[v], size = h.off[v + 1] - h.off[v];
  int start = 0, end = size - 1;
  while (end - start >= 10) {
    int mid = (start + end) / 2;
    if (h.t[base + mid] < time)
      start = mid;
    else
      end = mid;
  }
  int next = start;
  while (next < size && h.t[base + next] <= time) next++;
  int prev = next - 1;
  if (prev < 0) prev = 0; /* the reference reads before the first entry here; not reached from [0, 1] */
  if (next == size) {
    *pos = v3(h.p + 3 * (size_t)(base + prev));
    *idx = prev;
    return;
  }
  double dt = h.t[base + next] - h.t[base + prev];
  double alpha = (time - h.t[base + prev]) / dt;
  *pos = vadd(vscale(1.0 - alpha, v3(h.p + 3 * (size_t)(base + prev))), vscale(alpha, v3(h.p + 3 * (size_t)(base + next))));
  *idx = prev;
}

/* History::computeMinimumGap (src/History.cpp:82-96). */
static double minimum_gap(hist_view h, int nverts) {
  double result = 1.0;
  for (int i = 0; i < nverts; i++)
    for (int j = h.off[i] + 1; j < h.off[i + 1]; j++) {
      double gap = h.t[j] - h.t[j - 1];
      result = smin(gap, result);
    }
  return result;
}

/* SeparatingPlaneNarrowPhase::planeIntersect (:264-277). */
static double plane_intersect(vec3 planePos, vec3 planeVel, vec3 planeNormal, vec3 ptOld, vec3 ptNew, double ptdt,
                              double eta) {
  double numerator = 0.5 * eta - vdot(vsub(ptOld, planePos), planeNormal);
  double denom = -vdot(planeVel, planeNormal);
  if (ptdt != 0.0) denom += vdot(vsub(ptNew, ptOld), planeNormal) / ptdt;
  return numerator / denom;
}

/* SeparatingPlaneNarrowPhase::planeTrajectoryIntersect (:217-262); startidx
 * relative to the vertex's entries. */
static double plane_trajectory(hist_view h, int v, int startidx, int forward, vec3 planePos, vec3 planeVel,
                               vec3 planeNormal, vec3 ptstart, double timestart, double eta) {
  const int base = h.off[v], size = h.off[v + 1] - h.off[v];
  const double *T = h.t + base;
  const double *P = h.p + 3 * (size_t)base;
  double dt = forward ? T[startidx] - timestart : timestart - T[startidx];
  vec3 newpos = v3(P + 3 * startidx);
  double t = plane_intersect(planePos, vscale(forward ? 1.0 : -1.0, planeVel), planeNormal, ptstart, newpos, dt, eta);
  if (t >= 0 && t <= dt) return t;
  if (forward) {
    for (int i = startidx; i < size; i++) {
      if (i == size - 1) return INFINITY;
      int next = i + 1;
      vec3 newplanepos = vadd(planePos, vscale(T[i] - timestart, planeVel));
      double dti = T[next] - T[i];
      double ti = plane_intersect(newplanepos, planeVel, planeNormal, v3(P + 3 * i), v3(P + 3 * next), dti, eta);
      if (ti >= 0 && ti <= dti) return T[i] + ti - timestart;
    }
  } else {
    for (int i = startidx; i >= 0; i--) {
      if (i == 0) return INFINITY;
      int prev = i - 1;
      vec3 newplanepos = vsub(planePos, vscale(timestart - T[i], planeVel));
      vec3 nvel = {-planeVel.x, -planeVel.y, -planeVel.z};
      double dti = T[i] - T[prev];
      double ti = plane_intersect(newplanepos, nvel, planeNormal, v3(P + 3 * i), v3(P + 3 * prev), dti, eta);
      if (ti >= 0 && ti <= dti) return timestart - (T[i] - ti);
    }
  }
  return INFINITY;
}

/* SeparatingPlaneNarrowPhase::checkInterval (:47-215); type 0 vertex-face,
 * 1 edge-edge; v the canonical stencil.
 *
 * Every child interval is at most half its parent, so a recursion that
 * terminates is at most about 1,076 levels deep (halving 1.0 that often
 * reaches 0, and an empty interval is a leaf).  Deeper means a stall: an
 * interval that ends exactly at a history entry time never passes the leaf
 * test (its two ends lie in different entries), and once halving stops
 * shrinking it (adjacent doubles) the upper child equals its parent.  The
 * reference then recurses until its stack overflows.  Here depth 1,100 (or
 * 2^20 calls) stops the stencil and reports it through *capped. */
static int check_interval(int type, hist_view h, const int32_t *v, double eta, double mint, double maxt, double eps,
                          int64_t *frames, int *capped, int depth) {
  if (*capped) return 0;
  if (++*frames > (1 << 20) || depth > 1100) {
    *capped = 1;
    return 0;
  }
  if (maxt < mint) return 0;
  if (maxt - mint < 3 * eps) {
    int ok = 1;
    vec3 oldpos[4], newpos[4];
    for (int i = 0; i < 4; i++) {
      int oldidx, newidx;
      pos_at_time(h, v[i], mint, &oldpos[i], &oldidx);
      pos_at_time(h, v[i], maxt, &newpos[i], &newidx);
      if (oldidx != newidx) {
        ok = 0;
        break;
      }
    }
    if (ok) {
      double P0[12], P1[12], t;
      for (int i = 0; i < 4; i++) {
        P0[3 * i] = oldpos[i].x; P0[3 * i + 1] = oldpos[i].y; P0[3 * i + 2] = oldpos[i].z;
        P1[3 * i] = newpos[i].x; P1[3 * i + 1] = newpos[i].y; P1[3 * i + 2] = newpos[i].z;
      }
      return (type == 0 ? chain_vf(P0, P1, eta, &t) : chain_ee(P0, P1, eta, &t)) >= 0;
    }
  }
  double midt = 0.5 * (mint + maxt);
  vec3 midpos[4];
  int mididx[4];
  for (int i = 0; i < 4; i++) pos_at_time(h, v[i], midt, &midpos[i], &mididx[i]);
  double b[4] = {0, 0, 0, 0};
  vec3 closest = type == 0 ? vf_distance(midpos[0], midpos[1], midpos[2], midpos[3], b)
                           : ee_distance(midpos[0], midpos[1], midpos[2], midpos[3], b);
  double distsq = vdot(closest, closest);
  if (distsq < eta * eta) return 1;
  vec3 prevpos[4], nextpos[4];
  double dts[4];
  for (int i = 0; i < 4; i++) {
    const int base = h.off[v[i]];
    prevpos[i] = v3(h.p + 3 * (size_t)(base + mididx[i]));
    nextpos[i] = v3(h.p + 3 * (size_t)(base + mididx[i] + 1));
    dts[i] = h.t[base + mididx[i] + 1] - h.t[base + mididx[i]];
  }
  vec3 planepos, planevel;
  if (type == 0) {
    planepos = vscale(0.5, vadd(vadd(vadd(midpos[0], vscale(b[0], midpos[1])), vscale(b[1], midpos[2])),
                                vscale(b[2], midpos[3])));
    vec3 d0 = vsub(nextpos[0], prevpos[0]), s0 = {d0.x / dts[0], d0.y / dts[0], d0.z / dts[0]};
    vec3 acc = s0;
    for (int i = 1; i < 4; i++) {
      vec3 d = vscale(b[i - 1], vsub(nextpos[i], prevpos[i]));
      vec3 q = {d.x / dts[i], d.y / dts[i], d.z / dts[i]};
      acc = vadd(acc, q);
    }
    planevel = vscale(0.5, acc);
  } else {
    planepos = vscale(0.5, vadd(vadd(vadd(vscale(b[0], midpos[0]), vscale(b[1], midpos[1])), vscale(b[2], midpos[2])),
                                vscale(b[3], midpos[3])));
    vec3 acc = {0, 0, 0};
    for (int i = 0; i < 4; i++) {
      vec3 d = vscale(b[i], vsub(nextpos[i], prevpos[i]));
      vec3 q = {d.x / dts[i], d.y / dts[i], d.z / dts[i]};
      acc = i == 0 ? q : vadd(acc, q);
    }
    planevel = vscale(0.5, acc);
  }
  double nrm = vnorm(closest);
  closest.x = closest.x / nrm;
  closest.y = closest.y / nrm;
  closest.z = closest.z / nrm;
  double t = INFINITY;
  for (int vert = 0; vert < 4; vert++) {
    double sign = (vert == 0 || (vert == 1 && type == 1)) ? -1.0 : 1.0;
    t = smin(t, plane_trajectory(h, v[vert], mididx[vert], 0, planepos, planevel, vscale(sign, closest),
                                 midpos[vert], midt, eta));
  }
  if (t < 1.0) {
    double newmaxt = midt - smax(0.0, t - eps);
    if (check_interval(type, h, v, eta, mint, newmaxt, eps, frames, capped, depth + 1)) return 1;
  }
  t = INFINITY;
  for (int vert = 0; vert < 4; vert++) {
    double sign = (vert == 0 || (vert == 1 && type == 1)) ? -1.0 : 1.0;
    t = smin(t, plane_trajectory(h, v[vert], mididx[vert] + 1, 1, planepos, planevel, vscale(sign, closest),
                                 midpos[vert], midt, eta));
  }
  if (t < 1.0) {
    double newmint = midt + smax(0.0, t - eps);
    if (check_interval(type, h, v, eta, newmint, maxt, eps, frames, capped, depth + 1)) return 1;
  }
  return 0;
}

/* SeparatingPlaneNarrowPhase::findCollisions (:11-25): hit flags per
 * stencil; returns the number of stencils whose recursion hit the cap. */
int64_t oracle_separating_plane(int nverts, const int32_t *offsets, const double *times, const double *positions,
                                int64_t n_vf, const int32_t *vf, const double *vf_eta, int64_t n_ee,
                                const int32_t *ee, const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit,
                                uint8_t *vf_status, uint8_t *ee_status) {
  hist_view h = {offsets, times, positions};
  const double eps = minimum_gap(h, nverts) / 4.0;
  int64_t capped_total = 0;
  for (int kind = 0; kind < 2; kind++) {
    const int64_t n = kind == 0 ? n_vf : n_ee;
    for (int64_t i = 0; i < n; i++) {
      const int32_t *raw = (kind == 0 ? vf : ee) + 4 * i;
      int32_t st[4];
      if (kind == 0)
        oracle_vf_canon(raw[0], raw[1], raw[2], raw[3], st);
      else
        oracle_ee_canon(raw[0], raw[1], raw[2], raw[3], st);
      int64_t frames = 0;
      int capped = 0;
      const int hit =
          check_interval(kind, h, st, (kind == 0 ? vf_eta : ee_eta)[i], 0.0, 1.0, eps, &frames, &capped, 0);
      (kind == 0 ? vf_hit : ee_hit)[i] = (uint8_t)(hit && !capped);
      uint8_t *status = kind == 0 ? vf_status : ee_status;
      if (status) status[i] = (uint8_t)capped;
      capped_total += capped;
    }
  }
  return capped_total;
}

/* ------------------------------------------------------------ velocity filter
 * VelocityFilter::velocityFilter (src/VelocityFilter.cpp:15-87) and the
 * ActiveLayers it runs (src/ActiveLayers.cpp), on the restated pieces above. */
typedef struct { int32_t v[4]; } vf_st4;

static int st4_cmp(const vf_st4 *x, const vf_st4 *y) {
  for (int i = 0; i < 4; i++) {
    if (x->v[i] < y->v[i]) return -1;
    if (x->v[i] > y->v[i]) return 1;
  }
  return 0;
}

/* std::map<Stencil, int> as a sorted array (insertions keep it sorted). */
typedef struct { vf_st4 *key; int *val; int n, cap; } depth_map;

static int *depth_ref(depth_map *m, vf_st4 k) { /* operator[]: inserts 0 when absent */
  int lo = 0, hi = m->n;
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (st4_cmp(&m->key[mid], &k) < 0) lo = mid + 1; else hi = mid;
  }
  if (lo < m->n && st4_cmp(&m->key[lo], &k) == 0) return &m->val[lo];
  if (m->n == m->cap) {
    m->cap = m->cap ? 2 * m->cap : 64;
    m->key = (vf_st4 *)realloc(m->key, (size_t)m->cap * sizeof(vf_st4));
    m->val = (int *)realloc(m->val, (size_t)m->cap * sizeof(int));
  }
  memmove(m->key + lo + 1, m->key + lo, (size_t)(m->n - lo) * sizeof(vf_st4));
  memmove(m->val + lo + 1, m->val + lo, (size_t)(m->n - lo) * sizeof(int));
  m->key[lo] = k;
  m->val[lo] = 0;
  m->n++;
  return &m->val[lo];
}

static const int *depth_find(const depth_map *m, vf_st4 k) {
  int lo = 0, hi = m->n;
  while (lo < hi) {
    int mid = (lo + hi) / 2;
    if (st4_cmp(&m->key[mid], &k) < 0) lo = mid + 1; else hi = mid;
  }
  return (lo < m->n && st4_cmp(&m->key[lo], &k) == 0) ? &m->val[lo] : NULL;
}

typedef struct {
  double dt, eta, inner, k, cor;
  int nextstep;
  vf_st4 *st; /* vertex-face stencils first (nvf), then edge-edge (nee); kept apart until a firing */
  int nvf, nee, cvf, cee;
  vf_st4 *ee;
  int *verts; /* ascending, unique */
  int nverts, cverts;
} pgroup;

typedef struct {
  double outer, inner, base_dt, base_k, term, cor;
  int deepest;
  pgroup *g;
  int ng, cg;
  int *heap;
  int heap_size, heap_cap;
  depth_map vfdepth, eedepth;
} layers_t;

static int fires_later(const layers_t *L, int a, int b) {
  return (double)L->g[b].nextstep * L->g[b].dt < (double)L->g[a].nextstep * L->g[a].dt;
}

/* The standard library's binary heap (priority_queue over a vector). */
static void lheap_up(const layers_t *L, int *h, int hole, int value) {
  int parent = (hole - 1) / 2;
  while (hole > 0 && fires_later(L, h[parent], value)) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = value;
}
static void lheap_push(layers_t *L, int **h, int *size, int *cap, int value) {
  if (*size == *cap) {
    *cap = *cap ? 2 * *cap : 16;
    *h = (int *)realloc(*h, (size_t)*cap * sizeof(int));
  }
  lheap_up(L, *h, (*size)++, value);
}
static void lheap_pop(const layers_t *L, int *h, int *size) {
  int len = *size - 1;
  if (len > 0) {
    int value = h[len], hole = 0, child = 0;
    h[len] = h[0];
    while (child < (len - 1) / 2) {
      child = 2 * (child + 1);
      if (fires_later(L, h[child], h[child - 1])) child--;
      h[hole] = h[child];
      hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
      child = 2 * (child + 1);
      h[hole] = h[child - 1];
      hole = child - 1;
    }
    lheap_up(L, h, hole, value);
  }
  *size = len;
}

static double layer_depth(const layers_t *L, int layer) { return L->inner + (L->outer - L->inner) / (double)layer; }

static void add_groups(layers_t *L, int maxdepth) {
  while (L->deepest < maxdepth) {
    int depth = L->deepest + 1;
    double fudge = 1e-4;
    double ki = L->base_k * depth * depth * depth;
    double etai = layer_depth(L, depth);
    double dti = L->base_dt / (double)depth / sqrt((double)depth + fudge);
    if (L->ng == L->cg) {
      L->cg = L->cg ? 2 * L->cg : 16;
      L->g = (pgroup *)realloc(L->g, (size_t)L->cg * sizeof(pgroup));
    }
    pgroup z;
    memset(&z, 0, sizeof z);
    z.dt = dti; z.eta = etai; z.inner = L->inner; z.k = ki; z.cor = L->cor; z.nextstep = 1;
    L->g[L->ng++] = z;
    lheap_push(L, &L->heap, &L->heap_size, &L->heap_cap, L->ng - 1);
    L->deepest++;
  }
}

static void group_add(pgroup *g, int kind, vf_st4 s) {
  if (kind == 0) {
    if (g->nvf == g->cvf) { g->cvf = g->cvf ? 2 * g->cvf : 8; g->st = (vf_st4 *)realloc(g->st, (size_t)g->cvf * sizeof(vf_st4)); }
    g->st[g->nvf++] = s;
  } else {
    if (g->nee == g->cee) { g->cee = g->cee ? 2 * g->cee : 8; g->ee = (vf_st4 *)realloc(g->ee, (size_t)g->cee * sizeof(vf_st4)); }
    g->ee[g->nee++] = s;
  }
  for (int i = 0; i < 4; i++) { /* groupStencil_.insert */
    int v = s.v[i], lo = 0, hi = g->nverts;
    while (lo < hi) { int mid = (lo + hi) / 2; if (g->verts[mid] < v) lo = mid + 1; else hi = mid; }
    if (lo < g->nverts && g->verts[lo] == v) continue;
    if (g->nverts == g->cverts) { g->cverts = g->cverts ? 2 * g->cverts : 16; g->verts = (int *)realloc(g->verts, (size_t)g->cverts * sizeof(int)); }
    memmove(g->verts + lo + 1, g->verts + lo, (size_t)(g->nverts - lo) * sizeof(int));
    g->verts[lo] = v;
    g->nverts++;
  }
}

/* ActiveLayers::addVFStencil / addEEStencil (:43-67). */
static void layers_add(layers_t *L, int kind, vf_st4 s) {
  depth_map *dm = kind == 0 ? &L->vfdepth : &L->eedepth;
  int olddepth = *depth_ref(dm, s);
  for (int i = 0; i < 5; i++) {
    add_groups(L, olddepth + i + 1);
    group_add(&L->g[olddepth + i], kind, s);
    (*depth_ref(dm, s))++;
  }
}

/* ActiveLayers::rollback (:158-167). */
static void layers_rollback(layers_t *L) {
  for (int i = 0; i < L->ng; i++) L->g[i].nextstep = 1;
  int *fresh = NULL, fs = 0, fc = 0;
  while (L->heap_size > 0) {
    lheap_push(L, &fresh, &fs, &fc, L->heap[0]);
    lheap_pop(L, L->heap, &L->heap_size);
  }
  free(L->heap);
  L->heap = fresh; L->heap_size = fs; L->heap_cap = fc;
}

typedef struct { int n, cap; double *t, *p; } vhist;
static void vhist_add(vhist *h, double t, const double *p) {
  if (h->n == h->cap) {
    h->cap = h->cap ? 2 * h->cap : 4;
    h->t = (double *)realloc(h->t, (size_t)h->cap * sizeof(double));
    h->p = (double *)realloc(h->p, (size_t)h->cap * 3 * sizeof(double));
  }
  h->t[h->n] = t;
  memcpy(h->p + 3 * (size_t)h->n, p, 3 * sizeof(double));
  h->n++;
}

int oracle_velocity_filter(int nverts, const double *qstart, double *qend, int nfaces, const int32_t *faces,
                           const double *invmasses, double outer_eta, double inner_eta, double base_stiffness,
                           double base_substep, double cor, int max_rollbacks, int64_t *events_out) {
  if (nverts < 0 || nfaces < 0) return -1;
  if (nverts == 0) return 0; /* nothing to move; the first iteration finds nothing */
  const int64_t n3 = 3 * (int64_t)nverts;
  /* :22-39 dangling vertices */
  uint8_t *used = (uint8_t *)calloc((size_t)nverts + 1, 1);
  for (int64_t i = 0; i < 3 * (int64_t)nfaces; i++) used[faces[i]] = 1;
  for (int v = 0; v < nverts; v++)
    if (!used[v]) { free(used); return -1; }
  free(used);
  double maxmass = 0;
  for (int64_t i = 0; i < n3; i++) maxmass = smax(maxmass, invmasses[i]);
  double dt = base_substep;
  double k = base_stiffness / dt * sqrt(maxmass);
  layers_t L;
  memset(&L, 0, sizeof L);
  L.outer = outer_eta; L.inner = inner_eta; L.base_dt = dt; L.base_k = k; L.term = 1.0; L.cor = cor;
  uint8_t *fixed = (uint8_t *)calloc((size_t)nverts, 1);
  int any_fixed = 0;
  for (int64_t i = 0; i < n3; i++)
    if (invmasses[i] == 0.0) fixed[i / 3] = 1, any_fixed = 1;
  double closest = oracle_mesh_self_distance(nverts, qstart, nfaces, faces, any_fixed ? fixed : NULL, NULL, NULL);
  int result = -3;
  int64_t events = 0;
  double *q = (double *)malloc((size_t)n3 * 8), *v = (double *)malloc((size_t)n3 * 8), *lu = (double *)malloc((size_t)n3 * 8);
  double *newq = (double *)malloc((size_t)n3 * 8), *newv = (double *)malloc((size_t)n3 * 8), *G = (double *)calloc((size_t)n3, 8);
  vhist *hist = (vhist *)calloc((size_t)nverts, sizeof(vhist));
  if (closest < inner_eta) { result = -2; goto done; }
  for (int iter = 0; iter < max_rollbacks; iter++) {
    memcpy(q, qstart, (size_t)n3 * 8);
    for (int64_t i = 0; i < n3; i++) v[i] = qend[i] - qstart[i];
    memset(lu, 0, (size_t)n3 * 8);
    for (int vv = 0; vv < nverts; vv++) { hist[vv].n = 0; vhist_add(&hist[vv], 0.0, q + 3 * (size_t)vv); }
    /* ActiveLayers::step (:91-156) until the end of the step */
    for (;;) {
      if (L.heap_size > 0) {
        int gi = L.heap[0];
        pgroup *g = &L.g[gi];
        double newtime = (double)g->nextstep * g->dt;
        if (newtime < L.term) {
          lheap_pop(&L, L.heap, &L.heap_size);
          for (int j = 0; j < g->nverts; j++) {
            int vert = g->verts[j];
            for (int c = 0; c < 3; c++) {
              int64_t i = 3 * (int64_t)vert + c;
              double dtt = newtime - lu[i];
              newq[i] = q[i] + (newtime - lu[i]) * v[i];
              newv[i] = (newq[i] - q[i]) / dtt;
            }
          }
          /* PenaltyGroup::addForce into G (zero on the group's vertices) */
          for (int j = 0; j < g->nverts; j++)
            for (int c = 0; c < 3; c++) G[3 * (int64_t)g->verts[j] + c] = 0.0;
          for (int s = 0; s < g->nvf; s++) vf_penalty(newq, newv, G, g->st[s].v, g->eta, g->inner, g->k, g->cor);
          for (int s = 0; s < g->nee; s++) ee_penalty(newq, newv, G, g->ee[s].v, g->eta, g->inner, g->k, g->cor);
          for (int j = 0; j < g->nverts; j++) {
            int vert = g->verts[j];
            double F[3];
            int touched = 0;
            for (int c = 0; c < 3; c++) {
              F[c] = 0.0 + G[3 * (int64_t)vert + c] * g->dt;
              if (F[c] != 0.0) touched = 1;
            }
            if (touched) {
              for (int c = 0; c < 3; c++) {
                int64_t i = 3 * (int64_t)vert + c;
                v[i] += invmasses[i] * F[c];
                q[i] = newq[i];
                lu[i] = newtime;
              }
              vhist_add(&hist[vert], newtime, q + 3 * (size_t)vert);
            }
          }
          g->nextstep++;
          lheap_push(&L, &L.heap, &L.heap_size, &L.heap_cap, gi);
          events++;
          continue;
        }
      }
      for (int64_t i = 0; i < n3; i++) {
        q[i] += (L.term - lu[i]) * v[i];
        lu[i] = L.term;
      }
      for (int vv = 0; vv < nverts; vv++) vhist_add(&hist[vv], 1.0, q + 3 * (size_t)vv);
      break;
    }
    /* the history as arrays */
    int32_t *off = (int32_t *)malloc(((size_t)nverts + 1) * sizeof(int32_t));
    off[0] = 0;
    for (int vv = 0; vv < nverts; vv++) off[vv + 1] = off[vv] + hist[vv].n;
    double *ht = (double *)malloc((size_t)off[nverts] * 8), *hp = (double *)malloc((size_t)off[nverts] * 24);
    for (int vv = 0; vv < nverts; vv++) {
      memcpy(ht + off[vv], hist[vv].t, (size_t)hist[vv].n * 8);
      memcpy(hp + 3 * (size_t)off[vv], hist[vv].p, (size_t)hist[vv].n * 24);
    }
    /* ActiveLayers::collisionDetection (:190-226) */
    int64_t nvf = 0, nee = 0;
    oracle_broadphase_history(0, nverts, off, hp, nfaces, faces, outer_eta, any_fixed ? fixed : NULL, &nvf, &nee);
    int32_t *cvf = (int32_t *)malloc((size_t)(4 * nvf + 4) * sizeof(int32_t));
    int32_t *cee = (int32_t *)malloc((size_t)(4 * nee + 4) * sizeof(int32_t));
    oracle_broadphase_get(cvf, cee);
    double *evf = (double *)malloc((size_t)(nvf + 1) * 8), *eee = (double *)malloc((size_t)(nee + 1) * 8);
    for (int64_t i = 0; i < nvf; i++) {
      vf_st4 s; memcpy(s.v, cvf + 4 * i, 16);
      const int *d = depth_find(&L.vfdepth, s);
      evf[i] = d ? layer_depth(&L, *d + 1) : layer_depth(&L, 1);
    }
    for (int64_t i = 0; i < nee; i++) {
      vf_st4 s; memcpy(s.v, cee + 4 * i, 16);
      const int *d = depth_find(&L.eedepth, s);
      eee[i] = d ? layer_depth(&L, *d + 1) : layer_depth(&L, 1);
    }
    uint8_t *hvf = (uint8_t *)calloc((size_t)nvf + 1, 1), *hee = (uint8_t *)calloc((size_t)nee + 1, 1);
    uint8_t *svf = (uint8_t *)calloc((size_t)nvf + 1, 1), *see = (uint8_t *)calloc((size_t)nee + 1, 1);
    int64_t stalled = oracle_separating_plane(nverts, off, ht, hp, nvf, cvf, evf, nee, cee, eee, hvf, hee, svf, see);
    /* ActiveLayers::runOneIteration (:244-255) */
    layers_rollback(&L);
    int64_t found = 0;
    for (int64_t i = 0; i < nvf; i++)
      if (hvf[i]) { vf_st4 s; memcpy(s.v, cvf + 4 * i, 16); layers_add(&L, 0, s); found++; }
    for (int64_t i = 0; i < nee; i++)
      if (hee[i]) { vf_st4 s; memcpy(s.v, cee + 4 * i, 16); layers_add(&L, 1, s); found++; }
    free(off); free(ht); free(hp); free(cvf); free(cee); free(evf); free(eee); free(hvf); free(hee); free(svf); free(see);
    if (stalled) { result = -4; break; } /* the reference overflows its stack here */
    if (found == 0) {
      memcpy(qend, q, (size_t)n3 * 8);
      result = iter;
      break;
    }
  }
done:
  for (int vv = 0; vv < nverts; vv++) { free(hist[vv].t); free(hist[vv].p); }
  free(hist); free(q); free(v); free(lu); free(newq); free(newv); free(G); free(fixed);
  for (int i = 0; i < L.ng; i++) { free(L.g[i].st); free(L.g[i].ee); free(L.g[i].verts); }
  free(L.g); free(L.heap);
  free(L.vfdepth.key); free(L.vfdepth.val); free(L.eedepth.key); free(L.eedepth.val);
  if (events_out) *events_out = events;
  return result;
}
