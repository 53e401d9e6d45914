// Mesh-level pieces (mesh.cuh).
#include <algorithm>
#include <numeric>

#include "ccd_common.h"
#include "mesh.cuh"
#include "radix_sort.cuh"

namespace ccd {

bool build_topology(int32_t nverts, int32_t nfaces, const int32_t *faces, HostTopology &out) {
  for (int64_t i = 0; i < 3 * (int64_t)nfaces; i++)
    if (faces[i] < 0 || faces[i] >= nverts) return false;
  struct Tri {
    int32_t a, b, c;
  };
  std::vector<Tri> tri(nfaces);
  for (int32_t f = 0; f < nfaces; f++) {
    int32_t v[3] = {faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]};
    std::sort(v, v + 3);
    tri[f] = Tri{v[0], v[1], v[2]};
  }
  auto less = [](const Tri &x, const Tri &y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    return x.c < y.c;
  };
  std::vector<int32_t> order(nfaces);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return less(tri[x], tri[y]); });
  out.face_rank.assign(nfaces, 0);
  out.rank_triple.clear();
  for (int32_t i = 0; i < nfaces; i++) {
    const Tri &t = tri[order[i]];
    if (i == 0 || less(tri[order[i - 1]], t)) {
      out.rank_triple.push_back(t.a);
      out.rank_triple.push_back(t.b);
      out.rank_triple.push_back(t.c);
    }
    out.face_rank[order[i]] = (int32_t)(out.rank_triple.size() / 3 - 1);
  }
  std::vector<uint64_t> edges(3 * (size_t)nfaces);
  for (int32_t f = 0; f < nfaces; f++)
    for (int i = 0; i < 3; i++) {
      const uint32_t a = (uint32_t)faces[3 * f + i], b = (uint32_t)faces[3 * f + (i + 1) % 3];
      edges[3 * (size_t)f + i] = a <= b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
    }
  std::vector<uint64_t> uniq(edges);
  std::sort(uniq.begin(), uniq.end());
  uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
  out.rank_edge.resize(2 * uniq.size());
  for (size_t r = 0; r < uniq.size(); r++) {
    out.rank_edge[2 * r] = (int32_t)(uniq[r] >> 32);
    out.rank_edge[2 * r + 1] = (int32_t)(uint32_t)uniq[r];
  }
  out.face_edges.resize(edges.size());
  for (size_t i = 0; i < edges.size(); i++)
    out.face_edges[i] = (int32_t)(std::lower_bound(uniq.begin(), uniq.end(), edges[i]) - uniq.begin());
  return true;
}

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void swap_i(int &a, int &b) {
  int t = a;
  a = b;
  b = t;
}

// src/Stencils.h:13-57 (vertex-face: face vertices ascending) and 86-117
// (edge-edge: each edge ascending, edges ordered by first vertex).
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

// The rows of one segment's chain (start points P0, end points P1 of the
// four stencil vertices, 12 doubles each) at row index i: the primitive row,
// then the vertex-edge triples and vertex-vertex pairs in chain order.
__device__ __forceinline__ void write_rows(int kind, const double *P0, const double *P1, double et, int64_t i,
                                           double *prim, double *ve, double *vv, double *eta_prim, double *eta_ve,
                                           double *eta_vv) {
  double *r = prim + 24 * i;
  for (int k = 0; k < 12; k++) {
    r[k] = P0[k];
    r[12 + k] = P1[k];
  }
  eta_prim[i] = et;
  const int nsub = kind == 0 ? 3 : 4;
  for (int c = 0; c < nsub; c++) {
    int a, b0, b1, w0, w1;
    if (kind == 0) {  // CTCDNarrowPhase.cpp:51-69
      a = 0;
      b0 = 1 + c;
      b1 = 1 + (c + 1) % 3;
      w0 = 0;
      w1 = 1 + c;
    } else {  // CTCDNarrowPhase.cpp:92-129
      const int ves[4][3] = {{0, 2, 3}, {1, 2, 3}, {2, 0, 1}, {3, 0, 1}};
      const int vvs[4][2] = {{0, 2}, {0, 3}, {1, 2}, {1, 3}};
      a = ves[c][0];
      b0 = ves[c][1];
      b1 = ves[c][2];
      w0 = vvs[c][0];
      w1 = vvs[c][1];
    }
    double *x = ve + 18 * (nsub * i + c);
    const int ids[3] = {a, b0, b1};
    for (int k = 0; k < 3; k++)
      for (int q = 0; q < 3; q++) {
        x[3 * k + q] = P0[3 * ids[k] + q];
        x[9 + 3 * k + q] = P1[3 * ids[k] + q];
      }
    double *y = vv + 12 * (nsub * i + c);
    for (int q = 0; q < 3; q++) {
      y[q] = P0[3 * w0 + q];
      y[3 + q] = P0[3 * w1 + q];
      y[6 + q] = P1[3 * w0 + q];
      y[9 + q] = P1[3 * w1 + q];
    }
    eta_ve[nsub * i + c] = et;
    eta_vv[nsub * i + c] = et;
  }
}

__global__ void __launch_bounds__(kThreads) gather_rows(int kind, const int32_t *st, int64_t n, const double *qs,
                                                        const double *qe, const double *eta, int eta_per_row,
                                                        double *prim, double *ve, double *vv, double *eta_prim,
                                                        double *eta_ve, double *eta_vv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int v[4] = {st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]};
  canonical(kind, v);
  double P0[12], P1[12];
  for (int a = 0; a < 4; a++)
    for (int c = 0; c < 3; c++) {
      const double s = qs[3 * (int64_t)v[a] + c], e = qe[3 * (int64_t)v[a] + c];
      P0[3 * a + c] = (1.0 * s + 0.0 * e) / 1.0;  // History::stitchCommonHistory, two entries
      P1[3 * a + c] = e;
    }
  write_rows(kind, P0, P1, eta_per_row ? eta[i] : eta[0], i, prim, ve, vv, eta_prim, eta_ve, eta_vv);
}

// History::stitchCommonHistory (src/History.cpp:98-140) over the four stencil
// vertices of a multi-entry history: one call of next() per stitched entry,
// in the reference's loop order and arithmetic.  The loop is capped at the
// total number of entries (each stitched entry passes at least one of them).
struct Stitcher {
  const double *t, *p;
  int it[4], end[4];
  double cur;
  int budget;

  __device__ Stitcher(const int *v, const int32_t *off, const double *times, const double *pos) : t(times), p(pos) {
    budget = 1;
    for (int i = 0; i < 4; i++) {
      it[i] = off[v[i]];
      end[i] = off[v[i] + 1];
      budget += end[i] - it[i];
    }
    cur = 0.0;
  }

  // Writes the entry at the current time (12 doubles) and advances; false
  // once the reference's loop would have ended.
  __device__ bool next(double *pos) {
    if (!(cur <= 1.0) || budget-- <= 0) return false;
    double newtime = INFINITY;
    for (int i = 0; i < 4; i++) {
      int nx = it[i] + 1;
      while (nx < end[i] && t[nx] <= cur) {
        nx++;
        it[i]++;
      }
      const double *o = p + 3 * (int64_t)it[i];
      if (nx == end[i]) {
        for (int k = 0; k < 3; k++) pos[3 * i + k] = o[k];
      } else {
        const double *nw = p + 3 * (int64_t)nx;
        const double dt = t[nx] - t[it[i]];
        const double a = cur - t[it[i]];
        const double b = t[nx] - cur;
        for (int k = 0; k < 3; k++) pos[3 * i + k] = (b * o[k] + a * nw[k]) / dt;
        newtime = smin(newtime, t[nx]);
      }
    }
    cur = newtime;
    return true;
  }
};

// Segments (stitched entries - 1) of each stencil's common history.
__global__ void __launch_bounds__(kThreads) segment_counts(int kind, const int32_t *st, int64_t n,
                                                           const int32_t *off, const double *times,
                                                           const double *pos, uint32_t *count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int v[4] = {st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]};
  canonical(kind, v);
  Stitcher sh(v, off, times, pos);
  double P[12];
  uint32_t entries = 0;
  while (sh.next(P)) entries++;
  count[i] = entries > 0 ? entries - 1 : 0;
}

// The chain rows of every segment of stencils [0, n): stencil i's segments
// are rows seg_off[i] - base .. seg_off[i+1] - base - 1.
__global__ void __launch_bounds__(kThreads) gather_segment_rows(int kind, const int32_t *st, int64_t n,
                                                                const uint32_t *seg_off, uint32_t base,
                                                                const int32_t *off, const double *times,
                                                                const double *pos, const double *eta,
                                                                int eta_per_row, double *prim, double *ve, double *vv,
                                                                double *eta_prim, double *eta_ve, double *eta_vv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int v[4] = {st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]};
  canonical(kind, v);
  const double et = eta_per_row ? eta[i] : eta[0];
  Stitcher sh(v, off, times, pos);
  double P[2][12];
  int cur = 0;
  int64_t row = (int64_t)seg_off[i] - base;
  const int64_t last = (int64_t)seg_off[i + 1] - base;
  if (!sh.next(P[0])) return;
  while (row < last && sh.next(P[cur ^ 1])) {
    write_rows(kind, P[cur], P[cur ^ 1], et, row, prim, ve, vv, eta_prim, eta_ve, eta_vv);
    cur ^= 1;
    row++;
  }
}

// A stencil collides when the chain of one of its segments does; its t and
// sub-test are those of the first such segment (CTCDNarrowPhase.cpp:33-36).
__global__ void __launch_bounds__(kThreads) reduce_segments(int64_t n, const uint32_t *seg_off, uint32_t base,
                                                            const uint8_t *seg_hit, const double *seg_t,
                                                            const int8_t *seg_which, uint8_t *hit, double *t,
                                                            int8_t *which) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int8_t w = -1;
  double tt = 0.0;
  for (int64_t s = (int64_t)seg_off[i] - base; s < (int64_t)seg_off[i + 1] - base; s++)
    if (seg_hit[s]) {
      w = seg_which[s];
      tt = seg_t[s];
      break;
    }
  hit[i] = w >= 0;
  if (w >= 0 && t) t[i] = tt;
  if (which) which[i] = w;
}

__global__ void __launch_bounds__(kThreads) combine(int nsub, int64_t n, const uint8_t *h_prim, const double *t_prim,
                                                    const uint8_t *h_ve, const double *t_ve, const uint8_t *h_vv,
                                                    const double *t_vv, uint8_t *hit, double *t, int8_t *which) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int w = -1;
  double tt = 0.0;
  if (h_prim[i]) {
    w = 0;
    tt = t_prim[i];
  }
  for (int c = 0; c < nsub && w < 0; c++)
    if (h_ve[nsub * i + c]) {
      w = 1;
      tt = t_ve[nsub * i + c];
    }
  for (int c = 0; c < nsub && w < 0; c++)
    if (h_vv[nsub * i + c]) {
      w = 2;
      tt = t_vv[nsub * i + c];
    }
  hit[i] = w >= 0;
  if (w >= 0 && t) t[i] = tt;
  if (which) which[i] = (int8_t)w;
}

__global__ void __launch_bounds__(kThreads) hit_flags(const uint8_t *hit, int64_t n, uint32_t *flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[i] = hit[i] ? 1u : 0u;
}

__global__ void __launch_bounds__(kThreads) scatter_hits(const int32_t *st, const uint32_t *flags, const uint32_t *pos,
                                                         const double *t, int64_t n, int32_t *out, double *out_t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flags[i]) return;
  const int64_t o = pos[i];
  const int4 v = reinterpret_cast<const int4 *>(st)[i];
  if (out) reinterpret_cast<int4 *>(out)[o] = v;
  if (out_t) out_t[o] = t[i];
}

}  // namespace

cudaError_t compact_hits(const int32_t *stencils, const uint8_t *hit, const double *t, int64_t n, uint32_t *flags,
                         uint32_t *pos, uint32_t *count, void *temp, size_t temp_bytes, int32_t *out, double *out_t,
                         cudaStream_t s) {
  if (n <= 0) return cudaMemsetAsync(count, 0, sizeof(uint32_t), s);
  const unsigned grid = (unsigned)((n + kThreads - 1) / kThreads);
  hit_flags<<<grid, kThreads, 0, s>>>(hit, n, flags);
  cudaError_t e = exclusive_scan_u32(flags, pos, n, count, temp, temp_bytes, s);
  if (e != cudaSuccess) return e;
  scatter_hits<<<grid, kThreads, 0, s>>>(stencils, flags, pos, t, n, out, out_t);
  return cudaGetLastError();
}

cudaError_t gather_stencil_rows(int kind, const int32_t *stencils, int64_t n, const double *qs, const double *qe,
                                const double *eta, int eta_per_row, double *prim, double *ve, double *vv,
                                double *eta_prim, double *eta_ve, double *eta_vv, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  gather_rows<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      kind, stencils, n, qs, qe, eta, eta_per_row, prim, ve, vv, eta_prim, eta_ve, eta_vv);
  return cudaGetLastError();
}

cudaError_t history_segment_counts(int kind, const int32_t *stencils, int64_t n, const int32_t *off,
                                   const double *times, const double *pos, uint32_t *count, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  segment_counts<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(kind, stencils, n, off, times, pos,
                                                                                count);
  return cudaGetLastError();
}

cudaError_t gather_history_rows(int kind, const int32_t *stencils, int64_t n, const uint32_t *seg_off,
                                uint32_t base, const int32_t *off, const double *times, const double *pos,
                                const double *eta, int eta_per_row, double *prim, double *ve, double *vv,
                                double *eta_prim, double *eta_ve, double *eta_vv, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  gather_segment_rows<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(
      kind, stencils, n, seg_off, base, off, times, pos, eta, eta_per_row, prim, ve, vv, eta_prim, eta_ve, eta_vv);
  return cudaGetLastError();
}

cudaError_t reduce_history_segments(int64_t n, const uint32_t *seg_off, uint32_t base, const uint8_t *seg_hit,
                                    const double *seg_t, const int8_t *seg_which, uint8_t *hit, double *t,
                                    int8_t *which, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  reduce_segments<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(n, seg_off, base, seg_hit, seg_t,
                                                                                 seg_which, hit, t, which);
  return cudaGetLastError();
}

cudaError_t combine_chain(int kind, int64_t n, const uint8_t *h_prim, const double *t_prim, const uint8_t *h_ve,
                          const double *t_ve, const uint8_t *h_vv, const double *t_vv, uint8_t *hit, double *t,
                          int8_t *which, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  combine<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(kind == 0 ? 3 : 4, n, h_prim, t_prim, h_ve,
                                                                         t_ve, h_vv, t_vv, hit, t, which);
  return cudaGetLastError();
}

}  // namespace ccd
