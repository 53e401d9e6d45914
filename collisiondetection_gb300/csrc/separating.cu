// SeparatingPlaneNarrowPhase (src/SeparatingPlaneNarrowPhase.cpp) on the
// device: one thread per stencil runs the reference's interval search over a
// multi-entry history, op-for-op in FP64.
//
// The reference recurses: an interval shorter than 3 eps whose ends lie in
// the same history entries of all four vertices runs the CTCD chain
// (checkInterval's leaf); otherwise the stencil's closest points at the
// midpoint define a separating plane, and the first times before and after
// the midpoint at which a vertex trajectory can reach it bound a lower and an
// upper sub-interval, searched in that order.  Neither sub-interval's bounds
// depend on the other's outcome, so an explicit stack that pushes the upper
// child before the lower one visits the intervals in the reference's order.
//
// Termination: every child is at most half its parent, so a search that ends
// is at most about 1,076 levels deep.  Deeper means the reference's stall (an
// interval ending exactly at an entry time never passes the leaf test, and
// once halving stops shrinking it the upper child equals its parent; the
// reference then overflows its stack).  Depth 1,100, 2^20 intervals or a full
// stack stop the stencil with status 1 and no hit.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "ccd_distance.h"
#include "separating.cuh"

namespace ccd {

namespace {

constexpr int kThreads = 128;
constexpr int kStack = 256;
constexpr int kMaxDepth = 1100;
constexpr int64_t kMaxFrames = (int64_t)1 << 20;

__device__ __forceinline__ void swap_i(int &a, int &b) {
  const int t = a;
  a = b;
  b = t;
}

// src/Stencils.h:13-57 / 86-117
__device__ __forceinline__ void canonical(int kind, int *v) {
  if (kind == 0) {
    if (v[1] > v[2]) swap_i(v[1], v[2]);
    if (v[2] > v[3]) swap_i(v[2], v[3]);
    if (v[1] > v[2]) swap_i(v[1], v[2]);
  } else {
    if (v[0] > v[1]) swap_i(v[0], v[1]);
    if (v[2] > v[3]) swap_i(v[2], v[3]);
    if (v[0] > v[2]) {
      swap_i(v[0], v[2]);
      swap_i(v[1], v[3]);
    }
  }
}

// History::getPosAtTime (src/History.cpp:54-80): binary halving while the
// range holds 10 or more entries, then a forward scan; idx relative to the
// vertex's entries.  A time before the first entry (the reference reads
// before its array there; not reached from [0, 1]) takes the first entry.
__device__ void pos_at_time(const HistoryView &h, int v, double time, v3d &pos, int &idx) {
  const int base = h.off[v], size = h.off[v + 1] - base;
  int start = 0, end = size - 1;
  while (end - start >= 10) {
    const int mid = (start + end) / 2;
    if (h.t[base + mid] < time)
      start = mid;
    else
      end = mid;
  }
  int next = start;
  while (next < size && h.t[base + next] <= time) next++;
  int prev = next - 1;
  if (prev < 0) prev = 0;
  idx = prev;
  const v3d a = ld3(h.p + 3 * (int64_t)(base + prev));
  if (next == size) {
    pos = a;
    return;
  }
  const double dt = h.t[base + next] - h.t[base + prev];
  const double alpha = (time - h.t[base + prev]) / dt;
  pos = (1.0 - alpha) * a + alpha * ld3(h.p + 3 * (int64_t)(base + next));
}

// SeparatingPlaneNarrowPhase::planeIntersect (:264-277)
__device__ __forceinline__ double plane_intersect(v3d plane_pos, v3d plane_vel, v3d normal, v3d pt_old, v3d pt_new,
                                                  double ptdt, double eta) {
  const double numerator = 0.5 * eta - dot(pt_old - plane_pos, normal);
  double denom = -dot(plane_vel, normal);
  if (ptdt != 0.0) denom += dot(pt_new - pt_old, normal) / ptdt;
  return numerator / denom;
}

// SeparatingPlaneNarrowPhase::planeTrajectoryIntersect (:217-262)
__device__ double plane_trajectory(const HistoryView &h, int v, int startidx, bool forward, v3d plane_pos,
                                   v3d plane_vel, v3d normal, v3d ptstart, double timestart, double eta) {
  const int base = h.off[v], size = h.off[v + 1] - base;
  const double *T = h.t + base;
  const double *P = h.p + 3 * (int64_t)base;
  if (startidx >= size) return INFINITY;  // past the last entry (not reached from midpoints inside [0, 1))
  const double dt = forward ? T[startidx] - timestart : timestart - T[startidx];
  const double t = plane_intersect(plane_pos, (forward ? 1.0 : -1.0) * plane_vel, normal, ptstart,
                                   ld3(P + 3 * startidx), dt, eta);
  if (t >= 0 && t <= dt) return t;
  if (forward) {
    for (int i = startidx; i < size; i++) {
      if (i == size - 1) return INFINITY;
      const int next = i + 1;
      const v3d newplanepos = plane_pos + (T[i] - timestart) * plane_vel;
      const double dti = T[next] - T[i];
      const double ti = plane_intersect(newplanepos, plane_vel, normal, ld3(P + 3 * i), ld3(P + 3 * next), dti, eta);
      if (ti >= 0 && ti <= dti) return T[i] + ti - timestart;
    }
  } else {
    const v3d nvel = v3d{-plane_vel.x, -plane_vel.y, -plane_vel.z};
    for (int i = startidx; i >= 0; i--) {
      if (i == 0) return INFINITY;
      const int prev = i - 1;
      const v3d newplanepos = plane_pos - (timestart - T[i]) * plane_vel;
      const double dti = T[i] - T[prev];
      const double ti = plane_intersect(newplanepos, nvel, normal, ld3(P + 3 * i), ld3(P + 3 * prev), dti, eta);
      if (ti >= 0 && ti <= dti) return timestart - (T[i] - ti);
    }
  }
  return INFINITY;
}

__device__ __forceinline__ void put3(double *x, v3d a) {
  x[0] = a.x;
  x[1] = a.y;
  x[2] = a.z;
}

// The CTCD chain on one leaf interval (src/SeparatingPlaneNarrowPhase.cpp:
// 80-145; the chain of CTCDNarrowPhase).
template <int KIND>
__device__ bool leaf_chain(const v3d (&o)[4], const v3d (&e)[4], double eta) {
  double x[24], t;
  uint8_t st = 0;
  for (int i = 0; i < 4; i++) {
    put3(x + 3 * i, o[i]);
    put3(x + 12 + 3 * i, e[i]);
  }
  if (KIND == 0) {
    if (vf_ctcd(x, eta, t, st)) return true;
    for (int edge = 0; edge < 3; edge++) {
      const int a = 1 + (edge % 3), b = 1 + ((edge + 1) % 3);
      put3(x, o[0]), put3(x + 3, o[a]), put3(x + 6, o[b]);
      put3(x + 9, e[0]), put3(x + 12, e[a]), put3(x + 15, e[b]);
      if (ve_ctcd(x, eta, t, st)) return true;
    }
    for (int vert = 0; vert < 3; vert++) {
      put3(x, o[0]), put3(x + 3, o[1 + vert]), put3(x + 6, e[0]), put3(x + 9, e[1 + vert]);
      if (vv_ctcd(x, eta, t)) return true;
    }
  } else {
    if (ee_ctcd(x, eta, t, st)) return true;
    const int ves[4][3] = {{0, 2, 3}, {1, 2, 3}, {2, 0, 1}, {3, 0, 1}};
    for (int c = 0; c < 4; c++) {
      for (int k = 0; k < 3; k++) {
        put3(x + 3 * k, o[ves[c][k]]);
        put3(x + 9 + 3 * k, e[ves[c][k]]);
      }
      if (ve_ctcd(x, eta, t, st)) return true;
    }
    const int vvs[4][2] = {{0, 2}, {0, 3}, {1, 2}, {1, 3}};
    for (int c = 0; c < 4; c++) {
      put3(x, o[vvs[c][0]]), put3(x + 3, o[vvs[c][1]]), put3(x + 6, e[vvs[c][0]]), put3(x + 9, e[vvs[c][1]]);
      if (vv_ctcd(x, eta, t)) return true;
    }
  }
  return false;
}

struct Frame {
  double lo, hi;
  int depth;
};

template <int KIND>
__global__ void __launch_bounds__(kThreads) separating_plane(HistoryView h, const int32_t *st, int64_t n,
                                                             const double *eta, int eta_per_row, double eps,
                                                             uint8_t *hit, uint8_t *status) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int v[4] = {st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]};
  canonical(KIND, v);
  const double et = eta_per_row ? eta[i] : eta[0];
  Frame stack[kStack];
  int sp = 0;
  stack[sp++] = Frame{0.0, 1.0, 0};
  int64_t frames = 0;
  bool found = false;
  uint8_t stat = 0;
  while (sp > 0 && !found && !stat) {
    const Frame f = stack[--sp];
    if (++frames > kMaxFrames || f.depth > kMaxDepth) {
      stat = 1;
      break;
    }
    const double mint = f.lo, maxt = f.hi;
    if (maxt < mint) continue;
    if (maxt - mint < 3 * eps) {
      bool ok = true;
      v3d oldpos[4], newpos[4];
      for (int k = 0; k < 4 && ok; k++) {
        int oi, ni;
        pos_at_time(h, v[k], mint, oldpos[k], oi);
        pos_at_time(h, v[k], maxt, newpos[k], ni);
        ok = oi == ni;
      }
      if (ok) {
        if (leaf_chain<KIND>(oldpos, newpos, et)) found = true;
        continue;
      }
    }
    const double midt = 0.5 * (mint + maxt);
    v3d mid[4];
    int midx[4];
    for (int k = 0; k < 4; k++) pos_at_time(h, v[k], midt, mid[k], midx[k]);
    double b[4] = {0, 0, 0, 0};
    v3d closest;
    if (KIND == 0) {
      double w[3];
      closest = vertex_face_closest(mid[0], mid[1], mid[2], mid[3], w);
      b[0] = w[0], b[1] = w[1], b[2] = w[2];
    } else {
      closest = edge_edge_closest(mid[0], mid[1], mid[2], mid[3], b);
    }
    if (dot(closest, closest) < et * et) {
      found = true;
      break;
    }
    v3d vel[4];
    for (int k = 0; k < 4; k++) {
      const int base = h.off[v[k]], size = h.off[v[k] + 1] - base;
      const int a = midx[k], c = midx[k] + 1 < size ? midx[k] + 1 : midx[k];  // c == a only past the last entry
      const v3d d = ld3(h.p + 3 * (int64_t)(base + c)) - ld3(h.p + 3 * (int64_t)(base + a));
      const double dts = h.t[base + c] - h.t[base + a];
      const v3d s = KIND == 0 ? (k == 0 ? d : b[k - 1] * d) : b[k] * d;
      vel[k] = v3d{s.x / dts, s.y / dts, s.z / dts};
    }
    v3d plane_pos, plane_vel;
    if (KIND == 0) {
      plane_pos = 0.5 * (((mid[0] + b[0] * mid[1]) + b[1] * mid[2]) + b[2] * mid[3]);
    } else {
      plane_pos = 0.5 * (((b[0] * mid[0] + b[1] * mid[1]) + b[2] * mid[2]) + b[3] * mid[3]);
    }
    plane_vel = 0.5 * (((vel[0] + vel[1]) + vel[2]) + vel[3]);
    const double nrm = norm(closest);
    closest = v3d{closest.x / nrm, closest.y / nrm, closest.z / nrm};
    double tlo = INFINITY, thi = INFINITY;
    for (int k = 0; k < 4; k++) {
      const double sign = (k == 0 || (k == 1 && KIND == 1)) ? -1.0 : 1.0;
      tlo = smin(tlo, plane_trajectory(h, v[k], midx[k], false, plane_pos, plane_vel, sign * closest, mid[k], midt,
                                       et));
    }
    for (int k = 0; k < 4; k++) {
      const double sign = (k == 0 || (k == 1 && KIND == 1)) ? -1.0 : 1.0;
      thi = smin(thi, plane_trajectory(h, v[k], midx[k] + 1, true, plane_pos, plane_vel, sign * closest, mid[k],
                                       midt, et));
    }
    // the lower interval is searched first: push it last
    if (thi < 1.0) {
      if (sp >= kStack) {
        stat = 1;
        break;
      }
      stack[sp++] = Frame{midt + smax(0.0, thi - eps), maxt, f.depth + 1};
    }
    if (tlo < 1.0) {
      if (sp >= kStack) {
        stat = 1;
        break;
      }
      stack[sp++] = Frame{mint, midt - smax(0.0, tlo - eps), f.depth + 1};
    }
  }
  hit[i] = (found && !stat) ? 1 : 0;
  status[i] = stat;
}

__global__ void __launch_bounds__(256) two_entry_view(int nv, const double *qs, const double *qe, int32_t *off,
                                                      double *t, double *p) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v > nv) return;
  off[v] = 2 * v;
  if (v == nv) return;
  t[2 * v] = 0.0;
  t[2 * v + 1] = 1.0;
  for (int k = 0; k < 3; k++) {
    p[6 * (int64_t)v + k] = qs[3 * (int64_t)v + k];
    p[6 * (int64_t)v + 3 + k] = qe[3 * (int64_t)v + k];
  }
}

}  // namespace

cudaError_t launch_separating_plane(int kind, const HistoryView &h, const int32_t *stencils, int64_t n,
                                    const double *eta, int eta_per_row, double eps, uint8_t *hit, uint8_t *status,
                                    cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
  if (kind == 0)
    separating_plane<0><<<grid, kThreads, 0, s>>>(h, stencils, n, eta, eta_per_row, eps, hit, status);
  else
    separating_plane<1><<<grid, kThreads, 0, s>>>(h, stencils, n, eta, eta_per_row, eps, hit, status);
  return cudaGetLastError();
}

cudaError_t launch_two_entry_view(int nv, const double *qs, const double *qe, int32_t *off, double *t, double *p,
                                  cudaStream_t s) {
  two_entry_view<<<(unsigned)((nv + 1 + 255) / 256), 256, 0, s>>>(nv, qs, qe, off, t, p);
  return cudaGetLastError();
}

}  // namespace ccd
