// C ABI (include/ccd_gb300.h): meshes, broad phase, narrow phase over stencils.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "broadphase.cuh"
#include "ccd_common.h"
#include "context.cuh"
#include "distance.cuh"
#include "mesh.cuh"
#include "radix_sort.cuh"
#include "separating.cuh"

using namespace ccd_capi;

namespace {

// Stencils per chunk of the narrow phase (bounds its row scratch to about
// 1.2 GB).
constexpr int64_t kNarrowChunk = 1 << 20;

// Per-chunk rows and results of the narrow-phase chain.
struct NarrowScratch {
  int64_t cap = 0;  // stencils
  double *prim = nullptr, *ve = nullptr, *vv = nullptr;
  double *eta_prim = nullptr, *eta_ve = nullptr, *eta_vv = nullptr;
  uint8_t *h_prim = nullptr, *h_ve = nullptr, *h_vv = nullptr;
  double *t_prim = nullptr, *t_ve = nullptr, *t_vv = nullptr;
  int32_t *surv = nullptr;
  ccd::BatchCounters *counters = nullptr;
  // per-segment results of a multi-entry history
  uint8_t *seg_hit = nullptr;
  double *seg_t = nullptr;
  int8_t *seg_which = nullptr;
  StageBuf stage;
};

template <class T>
int grow(ccd_context *ctx, T **p, int64_t *cap, int64_t need) {
  if (*cap >= need && *p) return CCD_OK;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const int64_t c = std::max<int64_t>(need, 1);
  CCD_CUDA(cudaMalloc(p, (size_t)c * sizeof(T)));
  *cap = c;
  return CCD_OK;
}

// Per-kind narrow-phase buffers and stream.
struct Lane {
  NarrowScratch ns;
  cudaStream_t stream = nullptr;  // not owned
  uint8_t *hit = nullptr;
  int64_t hit_cap = 0;
  double *t = nullptr;
  int64_t t_cap = 0;
  uint32_t *flags = nullptr, *pos = nullptr;
  int64_t flags_cap = 0, pos_cap = 0;
  char *scan_temp = nullptr;
  int64_t scan_temp_cap = 0;
  uint32_t *d_count = nullptr;
  // segments per stencil and their offsets (multi-entry history)
  uint32_t *seg_cnt = nullptr, *seg_off = nullptr;
  int64_t seg_cnt_cap = 0, seg_off_cap = 0;
  std::vector<uint32_t> h_seg_off;
};

}  // namespace

struct ccd_mesh {
  ccd_context *ctx = nullptr;
  int32_t nv = 0, nf = 0;
  int32_t nranks = 0, nedges = 0;
  int32_t *faces = nullptr, *face_rank = nullptr, *rank_triple = nullptr, *face_edges = nullptr,
          *rank_edge = nullptr;
  int32_t *face_inst = nullptr;  // instance of each face (meshes made of independent instances)
  int32_t ninst = 1;
  double *qs = nullptr, *qe = nullptr;
  // A multi-entry History (ccd_mesh_set_history), used instead of qs / qe
  // while has_history is set: vertex v's entries are hist_off[v] ..
  // hist_off[v+1]-1 of hist_time / hist_pos.
  int32_t *hist_off = nullptr;
  double *hist_time = nullptr, *hist_pos = nullptr;
  int64_t hist_cap = 0;
  bool has_history = false;
  double hist_min_gap = 1.0;  // History::computeMinimumGap of the history set
  // the two-entry step as a history, for the separating-plane narrow phase
  int32_t *step_off = nullptr;
  double *step_time = nullptr, *step_pos = nullptr;
  uint8_t *fixed = nullptr;
  bool has_fixed = false;
  ccd::BroadphaseBuffers bp;
  ccd::PointTreeBuffers pt;  // closest-vertex-pair search (self distance)
  // candidates of the last broad phase: [0] vertex-face, [1] edge-edge
  int32_t *cand[2] = {nullptr, nullptr};
  int64_t cand_cap[2] = {0, 0};
  int64_t n_cand[2] = {0, 0};
  bool have_cand = false;
  // One narrow-phase lane per stencil kind: vertex-face on the context's
  // stream, edge-edge on the mesh's second stream, so that the two chains
  // (and their latency-bound root-solver tails) overlap.
  Lane lane[2];
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaEvent_t bp_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // broad-phase timing (profiling)
  // narrow-phase inputs of the host entry point
  int32_t *in_st = nullptr;
  int64_t in_st_cap = 0;
  double *in_eta = nullptr;
  int64_t in_eta_cap = 0;
  int8_t *which = nullptr;
  int64_t which_cap = 0;
  double *d_eta = nullptr;
  // collisions of the last detect
  int32_t *col[2] = {nullptr, nullptr};
  int64_t col_cap[2] = {0, 0};
  double *col_t[2] = {nullptr, nullptr};
  int64_t col_t_cap[2] = {0, 0};
  int64_t n_col[2] = {0, 0};
  bool have_col = false;
  ccd_mesh_stats stats{};
};

namespace {

int mesh_fail(ccd_mesh *m, int code, const std::string &msg) { return fail(m ? m->ctx : nullptr, code, msg); }

int ensure_narrow(ccd_mesh *m, Lane &L, int64_t chunk) {
  ccd_context *ctx = m->ctx;
  NarrowScratch &n = L.ns;
  if (n.cap >= chunk) return CCD_OK;
  CCD_CUDA(cudaStreamSynchronize(L.stream));
  void *ptrs[] = {n.prim, n.ve, n.vv, n.eta_prim, n.eta_ve, n.eta_vv, n.h_prim, n.h_ve, n.h_vv,
                  n.t_prim, n.t_ve, n.t_vv, n.surv, n.counters, n.stage.mem, n.seg_hit, n.seg_t, n.seg_which};
  for (void *p : ptrs) cudaFree(p);
  n = NarrowScratch{};
  const size_t c = (size_t)chunk, c4 = 4 * (size_t)chunk;
  CCD_CUDA(cudaMalloc(&n.prim, c * 24 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.ve, c4 * 18 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.vv, c4 * 12 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.eta_prim, c * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.eta_ve, c4 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.eta_vv, c4 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.h_prim, c));
  CCD_CUDA(cudaMalloc(&n.h_ve, c4));
  CCD_CUDA(cudaMalloc(&n.h_vv, c4));
  CCD_CUDA(cudaMalloc(&n.t_prim, c * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.t_ve, c4 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.t_vv, c4 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.surv, c4 * sizeof(int32_t)));
  CCD_CUDA(cudaMalloc(&n.counters, sizeof(ccd::BatchCounters)));
  CCD_CUDA(cudaMalloc(&n.seg_hit, c));
  CCD_CUDA(cudaMalloc(&n.seg_t, c * sizeof(double)));
  CCD_CUDA(cudaMalloc(&n.seg_which, c));
  n.cap = chunk;
  return CCD_OK;
}

// The chain three batches (primitive, vertex-edge, vertex-vertex) over c rows
// already gathered in L.ns, then the per-row first hit.
int run_chain(ccd_mesh *m, Lane &L, int kind, int path, int64_t c, uint8_t *hit, double *t, int8_t *which) {
  ccd_context *ctx = m->ctx;
  NarrowScratch &ns = L.ns;
  const int nsub = kind == CCD_VERTEX_FACE ? 3 : 4;
  cudaStream_t s = L.stream;
  const ccd::PrimBatch bp{kind, c, ns.prim, ns.eta_prim, true, ns.h_prim, ns.t_prim, nullptr, ns.counters};
  int rc = enqueue_batch(ctx, bp, path, ns.surv, ns.stage, s, nullptr);
  if (rc) return rc;
  const ccd::PrimBatch bve{CCD_VERTEX_EDGE, nsub * c, ns.ve, ns.eta_ve, true, ns.h_ve, ns.t_ve, nullptr,
                           ns.counters};
  rc = enqueue_batch(ctx, bve, path, ns.surv, ns.stage, s, nullptr);
  if (rc) return rc;
  const ccd::PrimBatch bvv{CCD_VERTEX_VERTEX, nsub * c, ns.vv, ns.eta_vv, true, ns.h_vv, ns.t_vv, nullptr,
                           ns.counters};
  rc = enqueue_batch(ctx, bvv, CCD_PATH_FP64, ns.surv, ns.stage, s, nullptr);
  if (rc) return rc;
  CCD_CUDA(ccd::combine_chain(kind, c, ns.h_prim, ns.t_prim, ns.h_ve, ns.t_ve, ns.h_vv, ns.t_vv, hit, t, which, s));
  return CCD_OK;
}

// The narrow phase over a multi-entry history: every segment of each
// stencil's stitched common history runs the chain; stencils are taken in
// chunks of at most kNarrowChunk segments.
int narrow_device_history(ccd_mesh *m, Lane &L, int kind, int path, int64_t n, const int32_t *st, const double *eta,
                          bool eta_per_row, uint8_t *hit, double *t, int8_t *which) {
  ccd_context *ctx = m->ctx;
  cudaStream_t s = L.stream;
  int rc = grow(ctx, &L.seg_cnt, &L.seg_cnt_cap, n);
  if (!rc) rc = grow(ctx, &L.seg_off, &L.seg_off_cap, n + 1);
  if (!rc) rc = grow(ctx, &L.scan_temp, &L.scan_temp_cap, (int64_t)ccd::scan_temp_bytes(n));
  if (rc) return rc;
  CCD_CUDA(ccd::history_segment_counts(kind, st, n, m->hist_off, m->hist_time, m->hist_pos, L.seg_cnt, s));
  CCD_CUDA(ccd::exclusive_scan_u32(L.seg_cnt, L.seg_off, n, L.seg_off + n, L.scan_temp, (size_t)L.scan_temp_cap, s));
  L.h_seg_off.resize((size_t)n + 1);
  CCD_CUDA(cudaMemcpyAsync(L.h_seg_off.data(), L.seg_off, ((size_t)n + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                           s));
  CCD_CUDA(cudaStreamSynchronize(s));
  const uint32_t *so = L.h_seg_off.data();
  for (int64_t i = 0; i < n; i++) {
    if (so[i + 1] < so[i]) return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT, "2^32 or more history segments");
    if ((int64_t)(so[i + 1] - so[i]) > kNarrowChunk)
      return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT, "a stencil's stitched history has more than 2^20 segments");
  }
  int64_t i0 = 0;
  while (i0 < n) {
    // the longest run of stencils whose segments fit one chunk
    int64_t i1 = i0;
    while (i1 < n && (int64_t)(so[i1 + 1] - so[i0]) <= kNarrowChunk) i1++;
    const int64_t segs = (int64_t)(so[i1] - so[i0]);
    if (segs > 0) {
      rc = ensure_narrow(m, L, std::min<int64_t>(kNarrowChunk, std::max<int64_t>(segs, 1)));
      if (rc) return rc;
      NarrowScratch &ns = L.ns;
      CCD_CUDA(ccd::gather_history_rows(kind, st + 4 * i0, i1 - i0, L.seg_off + i0, so[i0], m->hist_off,
                                        m->hist_time, m->hist_pos, eta_per_row ? eta + i0 : eta, eta_per_row ? 1 : 0,
                                        ns.prim, ns.ve, ns.vv, ns.eta_prim, ns.eta_ve, ns.eta_vv, s));
      rc = run_chain(m, L, kind, path, segs, ns.seg_hit, ns.seg_t, ns.seg_which);
      if (rc) return rc;
    }
    CCD_CUDA(ccd::reduce_history_segments(i1 - i0, L.seg_off + i0, so[i0], L.ns.seg_hit, L.ns.seg_t, L.ns.seg_which,
                                          hit + i0, t ? t + i0 : nullptr, which ? which + i0 : nullptr, s));
    // the next chunk reuses the row buffers: wait for this one's kernels
    CCD_CUDA(cudaStreamSynchronize(s));
    i0 = i1;
  }
  return CCD_OK;
}

// The narrow-phase chain over n device stencils of one kind, on lane L's
// stream; results into device arrays hit[n], t[n] (optional), which[n]
// (optional).
int narrow_device(ccd_mesh *m, Lane &L, int kind, int path, int64_t n, const int32_t *st, const double *eta,
                  bool eta_per_row, uint8_t *hit, double *t, int8_t *which) {
  ccd_context *ctx = m->ctx;
  if (n == 0) return CCD_OK;
  if (m->has_history) return narrow_device_history(m, L, kind, path, n, st, eta, eta_per_row, hit, t, which);
  const int64_t chunk = std::min<int64_t>(n, kNarrowChunk);
  int rc = ensure_narrow(m, L, chunk);
  if (rc) return rc;
  NarrowScratch &ns = L.ns;
  cudaStream_t s = L.stream;
  for (int64_t off = 0; off < n; off += chunk) {
    const int64_t c = std::min<int64_t>(chunk, n - off);
    CCD_CUDA(ccd::gather_stencil_rows(kind, st + 4 * off, c, m->qs, m->qe, eta_per_row ? eta + off : eta,
                                      eta_per_row ? 1 : 0, ns.prim, ns.ve, ns.vv, ns.eta_prim, ns.eta_ve, ns.eta_vv,
                                      s));
    rc = run_chain(m, L, kind, path, c, hit + off, t ? t + off : nullptr, which ? which + off : nullptr);
    if (rc) return rc;
  }
  return CCD_OK;
}

// whole: one mesh even when it is made of instances (faces of different
// instances are paired too).
int run_broadphase(ccd_mesh *m, int kind, double outer_eta, bool whole = false) {
  ccd_context *ctx = m->ctx;
  m->have_cand = false;
  m->have_col = false;
  m->stats = ccd_mesh_stats{};
  const ccd::MeshTopology topo{m->nv,         m->nf,         m->nranks,   m->nedges,
                               m->faces,      m->face_rank,  m->rank_triple, m->face_edges,
                               m->rank_edge,  whole ? nullptr : m->face_inst,  whole ? 1 : m->ninst};
  ccd::BroadphaseParams p{kind,
                          outer_eta,
                          m->qs,
                          m->qe,
                          m->has_history ? m->hist_off : nullptr,
                          m->has_history ? m->hist_pos : nullptr,
                          m->has_fixed ? m->fixed : nullptr,
                          ctx->opt_count_tests != 0,
                          {nullptr, nullptr, nullptr, nullptr}};
  const bool timed = ctx->profiling && m->nf >= 2;
  if (timed) {
    for (int k = 0; k < 4; k++) {
      if (!m->bp_ev[k]) CCD_CUDA(cudaEventCreate(&m->bp_ev[k]));
      p.ev[k] = m->bp_ev[k];
    }
  }
  cudaError_t err = cudaSuccess;
  int64_t npairs = 0, tests = 0;
  if (kind == CCD_BROADPHASE_TRIVIAL) {
    if (topo.ninst > 1) return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT, "the trivial broad phase takes single meshes");
    const int trc = ccd::trivial_candidates(topo, p.fixed, &m->cand[0], &m->cand_cap[0], &m->cand[1],
                                            &m->cand_cap[1], &m->n_cand[0], &m->n_cand[1], ctx->stream, &err);
    if (trc == 2) return cuda_fail(ctx, err, "trivial broadphase");
    if (trc == 4) return mesh_fail(m, CCD_ERR_OUT_OF_MEMORY, "trivial broadphase: 2^31 or more stencils");
    m->stats.slab_tests = -1;
    m->stats.n_vf = m->n_cand[0];
    m->stats.n_ee = m->n_cand[1];
    m->have_cand = true;
    return CCD_OK;
  }
  const int rc = ccd::broadphase_run(topo, p, m->bp, &m->cand[0], &m->cand_cap[0], &m->cand[1], &m->cand_cap[1],
                                     &m->n_cand[0], &m->n_cand[1], &npairs, &tests, ctx->num_sms, ctx->stream, &err);
  if (rc == 2) return cuda_fail(ctx, err, "broadphase");
  if (rc == 3) return mesh_fail(m, CCD_ERR_CUDA, "broadphase: malformed tree (traversal beyond its size)");
  if (rc == 4) return mesh_fail(m, CCD_ERR_OUT_OF_MEMORY, "broadphase: more than 2^27 overlapping face pairs");
  m->stats.face_pairs = npairs;
  m->stats.slab_tests = p.count_tests ? tests : -1;
  if (timed) {
    CCD_CUDA(cudaEventElapsedTime(&m->stats.broadphase_ms, p.ev[0], p.ev[3]));
    CCD_CUDA(cudaEventElapsedTime(&m->stats.traversal_ms, p.ev[1], p.ev[2]));
  }
  m->stats.n_vf = m->n_cand[0];
  m->stats.n_ee = m->n_cand[1];
  m->have_cand = true;
  return CCD_OK;
}

int check_eta(ccd_mesh *m, int64_t n, const double *eta, int64_t eta_count) {
  if (n == 0) return CCD_OK;
  if (!eta || (eta_count != 1 && eta_count != n))
    return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT, "eta must hold 1 or n values");
  return CCD_OK;
}

void free_mesh_buffers(ccd_mesh *m) {
  void *ptrs[] = {m->faces, m->face_rank, m->rank_triple, m->face_edges, m->rank_edge, m->face_inst, m->qs, m->qe,
                  m->hist_off, m->hist_time, m->hist_pos, m->step_off, m->step_time, m->step_pos, m->fixed,
                  m->cand[0], m->cand[1], m->in_st, m->in_eta, m->which, m->d_eta,
                  m->col[0], m->col[1], m->col_t[0], m->col_t[1]};
  for (void *p : ptrs) cudaFree(p);
  for (Lane &L : m->lane) {
    NarrowScratch &n = L.ns;
    void *lp[] = {L.hit, L.t, L.flags, L.pos, L.scan_temp, L.d_count, L.seg_cnt, L.seg_off, n.seg_hit, n.seg_t,
                  n.seg_which, n.prim, n.ve, n.vv, n.eta_prim, n.eta_ve,
                  n.eta_vv, n.h_prim, n.h_ve, n.h_vv, n.t_prim, n.t_ve, n.t_vv, n.surv, n.counters, n.stage.mem};
    for (void *p : lp) cudaFree(p);
  }
  ccd::broadphase_free(m->bp);
  ccd::point_tree_free(m->pt);
  for (cudaEvent_t e : m->bp_ev)
    if (e) cudaEventDestroy(e);
  if (m->fork) cudaEventDestroy(m->fork);
  if (m->join) cudaEventDestroy(m->join);
  if (m->side) cudaStreamDestroy(m->side);
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// Shared by ccd_mesh_create and ccd_mesh_create_instances (face_inst: null, or
// the instance of each face with ninst > 1 instances).
int create_mesh(ccd_context *ctx, int32_t nverts, int32_t nfaces, const int32_t *faces,
                const std::vector<int32_t> *face_inst, int32_t ninst, ccd_mesh **out) {
  if (!ctx || !out) return CCD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (nverts <= 0 || nfaces < 0 || (nfaces > 0 && !faces))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "mesh needs nverts > 0, nfaces >= 0 and a face array");
  if ((int64_t)nverts > ((int64_t)1 << 30) || (int64_t)nfaces > ((int64_t)1 << 30))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "mesh larger than 2^30 vertices or faces");
  ccd::HostTopology topo;
  if (!ccd::build_topology(nverts, nfaces, faces, topo))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "face vertex index out of range");
  CCD_CUDA(cudaSetDevice(ctx->device));
  ccd_mesh *m = new (std::nothrow) ccd_mesh();
  if (!m) return fail(ctx, CCD_ERR_OUT_OF_MEMORY, "host allocation");
  m->ctx = ctx;
  m->nv = nverts;
  m->nf = nfaces;
  m->nranks = (int32_t)(topo.rank_triple.size() / 3);
  m->nedges = (int32_t)(topo.rank_edge.size() / 2);
  auto upload = [&](int32_t **dst, const int32_t *src, size_t count) -> int {
    CCD_CUDA(cudaMalloc(dst, std::max<size_t>(count, 1) * sizeof(int32_t)));
    if (count) CCD_CUDA(cudaMemcpyAsync(*dst, src, count * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    return CCD_OK;
  };
  int rc = upload(&m->faces, faces, 3 * (size_t)nfaces);
  if (!rc) rc = upload(&m->face_rank, topo.face_rank.data(), topo.face_rank.size());
  if (!rc) rc = upload(&m->rank_triple, topo.rank_triple.data(), topo.rank_triple.size());
  if (!rc) rc = upload(&m->face_edges, topo.face_edges.data(), topo.face_edges.size());
  if (!rc) rc = upload(&m->rank_edge, topo.rank_edge.data(), topo.rank_edge.size());
  if (!rc && face_inst && ninst > 1) {
    rc = upload(&m->face_inst, face_inst->data(), face_inst->size());
    m->ninst = ninst;
  }
  auto alloc = [&]() -> int {
    CCD_CUDA(cudaMalloc(&m->qs, 3 * (size_t)nverts * sizeof(double)));
    CCD_CUDA(cudaMalloc(&m->qe, 3 * (size_t)nverts * sizeof(double)));
    CCD_CUDA(cudaMemsetAsync(m->qs, 0, 3 * (size_t)nverts * sizeof(double), ctx->stream));
    CCD_CUDA(cudaMemsetAsync(m->qe, 0, 3 * (size_t)nverts * sizeof(double), ctx->stream));
    CCD_CUDA(cudaMalloc(&m->fixed, (size_t)nverts));
    CCD_CUDA(cudaMalloc(&m->d_eta, sizeof(double)));
    CCD_CUDA(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
    CCD_CUDA(cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming));
    CCD_CUDA(cudaEventCreateWithFlags(&m->join, cudaEventDisableTiming));
    for (Lane &L : m->lane) CCD_CUDA(cudaMalloc(&L.d_count, sizeof(uint32_t)));
    return CCD_OK;
  };
  if (!rc) rc = alloc();
  if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = cuda_fail(ctx, cudaGetLastError(), "upload");
  if (rc) {
    free_mesh_buffers(m);
    delete m;
    return rc;
  }
  *out = m;
  return CCD_OK;
}

}  // namespace

extern "C" {

int ccd_mesh_create(ccd_context *ctx, int32_t nverts, int32_t nfaces, const int32_t *faces, ccd_mesh **out) {
  return create_mesh(ctx, nverts, nfaces, faces, nullptr, 1, out);
}

int ccd_mesh_create_instances(ccd_context *ctx, int32_t ninst, const int32_t *vertex_offsets,
                              const int32_t *face_offsets, const int32_t *faces, ccd_mesh **out) {
  if (!ctx || !out) return CCD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (ninst < 1 || !vertex_offsets || !face_offsets)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "instances need ninst >= 1 and offset arrays");
  if (vertex_offsets[0] != 0 || face_offsets[0] != 0)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "offsets must start at 0");
  if (face_offsets[ninst] > 0 && !faces) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null face array");
  std::vector<int32_t> inst((size_t)std::max(face_offsets[ninst], 0));
  for (int32_t i = 0; i < ninst; i++) {
    if (vertex_offsets[i + 1] <= vertex_offsets[i] || face_offsets[i + 1] < face_offsets[i])
      return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "offsets must increase (every instance needs a vertex)");
    for (int32_t f = face_offsets[i]; f < face_offsets[i + 1]; f++) {
      for (int j = 0; j < 3; j++) {
        const int32_t v = faces[3 * (int64_t)f + j];
        if (v < vertex_offsets[i] || v >= vertex_offsets[i + 1])
          return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "a face uses a vertex outside its instance");
      }
      inst[(size_t)f] = i;
    }
  }
  const int32_t nverts = vertex_offsets[ninst], nfaces = face_offsets[ninst];
  // The broad phase's sort key holds the instance, a Morton code of at least
  // 12 bits and the face index in 63 bits.
  int fbits = 1, ibits = 0;
  while (fbits < 62 && ((int64_t)1 << fbits) <= (int64_t)std::max(nfaces - 1, 0)) fbits++;
  while (ninst > 1 && ((int64_t)1 << ibits) <= (int64_t)(ninst - 1)) ibits++;
  if (12 + fbits + ibits > 63) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "too many faces and instances for the sort key");
  return create_mesh(ctx, nverts, nfaces, faces, &inst, ninst, out);
}

int ccd_mesh_destroy(ccd_mesh *m) {
  if (!m) return CCD_OK;
  cudaSetDevice(m->ctx->device);
  cudaStreamSynchronize(m->ctx->stream);
  free_mesh_buffers(m);
  delete m;
  return CCD_OK;
}

int ccd_mesh_set_positions(ccd_mesh *m, const double *qstart, const double *qend) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!qstart || !qend) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null positions");
  CCD_CUDA(cudaSetDevice(ctx->device));
  const size_t bytes = 3 * (size_t)m->nv * sizeof(double);
  CCD_CUDA(cudaMemcpyAsync(m->qs, qstart, bytes, cudaMemcpyHostToDevice, ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->qe, qend, bytes, cudaMemcpyHostToDevice, ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  m->has_history = false;
  m->have_cand = m->have_col = false;
  return CCD_OK;
}

int ccd_mesh_set_positions_device(ccd_mesh *m, const double *qstart, const double *qend) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!qstart || !qend) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null positions");
  CCD_CUDA(cudaSetDevice(ctx->device));
  const size_t bytes = 3 * (size_t)m->nv * sizeof(double);
  CCD_CUDA(cudaMemcpyAsync(m->qs, qstart, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->qe, qend, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  m->has_history = false;
  m->have_cand = m->have_col = false;
  return CCD_OK;
}

int ccd_mesh_set_history(ccd_mesh *m, const int32_t *offsets, const double *times, const double *positions) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!offsets || !times || !positions) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null history");
  if (offsets[0] != 0) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "history offsets must start at 0");
  for (int32_t v = 0; v < m->nv; v++)
    if (offsets[v + 1] <= offsets[v])
      return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "every vertex needs at least one history entry");
  const int64_t ne = offsets[m->nv];
  for (int32_t v = 0; v < m->nv; v++)
    for (int32_t e = offsets[v] + 1; e < offsets[v + 1]; e++)
      if (!(times[e - 1] <= times[e]))
        return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "history times must be non-decreasing per vertex");
  CCD_CUDA(cudaSetDevice(ctx->device));
  if (m->hist_cap < ne || !m->hist_off) {
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(m->hist_time);
    cudaFree(m->hist_pos);
    m->hist_time = m->hist_pos = nullptr;
    m->hist_cap = 0;
    CCD_CUDA(cudaMalloc(&m->hist_time, (size_t)ne * sizeof(double)));
    CCD_CUDA(cudaMalloc(&m->hist_pos, (size_t)ne * 3 * sizeof(double)));
    m->hist_cap = ne;
    if (!m->hist_off) CCD_CUDA(cudaMalloc(&m->hist_off, ((size_t)m->nv + 1) * sizeof(int32_t)));
  }
  CCD_CUDA(cudaMemcpyAsync(m->hist_off, offsets, ((size_t)m->nv + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                           ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->hist_time, times, (size_t)ne * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->hist_pos, positions, (size_t)ne * 3 * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  // History::computeMinimumGap (src/History.cpp:82-96), in its loop order
  double gap_min = 1.0;
  for (int32_t v = 0; v < m->nv; v++)
    for (int32_t e = offsets[v] + 1; e < offsets[v + 1]; e++) gap_min = ccd::smin(times[e] - times[e - 1], gap_min);
  m->hist_min_gap = gap_min;
  m->has_history = true;
  m->have_cand = m->have_col = false;
  return CCD_OK;
}

int ccd_mesh_set_fixed(ccd_mesh *m, const uint8_t *fixed) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  CCD_CUDA(cudaSetDevice(ctx->device));
  if (fixed) {
    // Normalise to 0/1 on the host.
    std::vector<uint8_t> f(fixed, fixed + m->nv);
    for (auto &x : f) x = x ? 1 : 0;
    CCD_CUDA(cudaMemcpyAsync(m->fixed, f.data(), (size_t)m->nv, cudaMemcpyHostToDevice, ctx->stream));
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));  // f is about to go away
  }
  m->has_fixed = fixed != nullptr;
  m->have_cand = m->have_col = false;
  return CCD_OK;
}

int ccd_broadphase(ccd_mesh *m, int kind, double outer_eta, int64_t *n_vf, int64_t *n_ee) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (kind != CCD_BROADPHASE_KDOP13 && kind != CCD_BROADPHASE_AABB && kind != CCD_BROADPHASE_TRIVIAL)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown broadphase kind");
  CCD_CUDA(cudaSetDevice(ctx->device));
  int rc = run_broadphase(m, kind, outer_eta);
  if (rc) return rc;
  if (n_vf) *n_vf = m->n_cand[0];
  if (n_ee) *n_ee = m->n_cand[1];
  return CCD_OK;
}

int ccd_broadphase_get(ccd_mesh *m, int32_t *vf, int32_t *ee) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!m->have_cand) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "no broad phase result on this mesh");
  CCD_CUDA(cudaSetDevice(ctx->device));
  if (vf && m->n_cand[0])
    CCD_CUDA(cudaMemcpyAsync(vf, m->cand[0], (size_t)m->n_cand[0] * 4 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                             ctx->stream));
  if (ee && m->n_cand[1])
    CCD_CUDA(cudaMemcpyAsync(ee, m->cand[1], (size_t)m->n_cand[1] * 4 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                             ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  return CCD_OK;
}

int ccd_narrowphase(ccd_mesh *m, int path, int64_t n_vf, const int32_t *vf, const double *vf_eta,
                    int64_t vf_eta_count, int64_t n_ee, const int32_t *ee, const double *ee_eta, int64_t ee_eta_count,
                    uint8_t *vf_hit, uint8_t *ee_hit, double *vf_t, double *ee_t, int8_t *vf_which,
                    int8_t *ee_which) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (path != CCD_PATH_FP64 && path != CCD_PATH_CULL_REFINE)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown path");
  if (n_vf < 0 || n_ee < 0 || n_vf > INT32_MAX / 4 || n_ee > INT32_MAX / 4)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "stencil counts must be in [0, 2^29)");
  if ((n_vf && (!vf || !vf_hit)) || (n_ee && (!ee || !ee_hit)))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null stencil or hit array");
  int rc = check_eta(m, n_vf, vf_eta, vf_eta_count);
  if (!rc) rc = check_eta(m, n_ee, ee_eta, ee_eta_count);
  if (rc) return rc;
  // Reject out-of-range vertex indices before anything touches the device.
  for (int k = 0; k < 2; k++) {
    const int32_t *st = k ? ee : vf;
    const int64_t n = k ? n_ee : n_vf;
    for (int64_t i = 0; i < 4 * n; i++)
      if (st[i] < 0 || st[i] >= m->nv) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "stencil vertex out of range");
  }
  CCD_CUDA(cudaSetDevice(ctx->device));
  m->stats = ccd_mesh_stats{};
  m->stats.n_vf = n_vf;
  m->stats.n_ee = n_ee;
  m->stats.slab_tests = -1;
  std::vector<double> tbuf;
  for (int k = 0; k < 2; k++) {
    const int64_t n = k ? n_ee : n_vf;
    if (n == 0) continue;
    const int32_t *st = k ? ee : vf;
    const double *eta = k ? ee_eta : vf_eta;
    const int64_t eta_count = k ? ee_eta_count : vf_eta_count;
    uint8_t *hit = k ? ee_hit : vf_hit;
    double *t = k ? ee_t : vf_t;
    int8_t *which = k ? ee_which : vf_which;
    rc = grow(ctx, &m->in_st, &m->in_st_cap, 4 * n);
    if (!rc) rc = grow(ctx, &m->in_eta, &m->in_eta_cap, eta_count);
    Lane &L = m->lane[0];
    L.stream = ctx->stream;
    if (!rc) rc = grow(ctx, &L.hit, &L.hit_cap, n);
    if (!rc) rc = grow(ctx, &L.t, &L.t_cap, n);
    if (!rc) rc = grow(ctx, &m->which, &m->which_cap, n);
    if (rc) return rc;
    CCD_CUDA(cudaMemcpyAsync(m->in_st, st, (size_t)n * 4 * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(m->in_eta, eta, (size_t)eta_count * sizeof(double), cudaMemcpyHostToDevice,
                             ctx->stream));
    rc = narrow_device(m, L, k ? CCD_EDGE_EDGE : CCD_VERTEX_FACE, path, n, m->in_st, m->in_eta,
                       eta_count == n && n != 1, L.hit, L.t, m->which);
    if (rc) return rc;
    CCD_CUDA(cudaMemcpyAsync(hit, L.hit, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    if (which) CCD_CUDA(cudaMemcpyAsync(which, m->which, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    if (t) {
      tbuf.resize((size_t)n);
      CCD_CUDA(cudaMemcpyAsync(tbuf.data(), L.t, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
    int64_t hits = 0;
    for (int64_t i = 0; i < n; i++) {
      hits += hit[i] != 0;
      if (t && hit[i]) t[i] = tbuf[(size_t)i];
    }
    (k ? m->stats.ee_hits : m->stats.vf_hits) = hits;
  }
  return CCD_OK;
}

int ccd_narrowphase_separating_plane(ccd_mesh *m, int64_t n_vf, const int32_t *vf, const double *vf_eta,
                                     int64_t vf_eta_count, int64_t n_ee, const int32_t *ee, const double *ee_eta,
                                     int64_t ee_eta_count, uint8_t *vf_hit, uint8_t *ee_hit, uint8_t *vf_status,
                                     uint8_t *ee_status) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (n_vf < 0 || n_ee < 0 || (n_vf && (!vf || !vf_hit)) || (n_ee && (!ee || !ee_hit)))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer or negative size");
  int rc = check_eta(m, n_vf, vf_eta, vf_eta_count);
  if (!rc) rc = check_eta(m, n_ee, ee_eta, ee_eta_count);
  if (rc) return rc;
  for (int k = 0; k < 2; k++) {
    const int32_t *st = k == 0 ? vf : ee;
    const int64_t n = k == 0 ? n_vf : n_ee;
    for (int64_t i = 0; i < 4 * n; i++)
      if (st[i] < 0 || st[i] >= m->nv) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "stencil vertex out of range");
  }
  CCD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  ccd::HistoryView hv{m->hist_off, m->hist_time, m->hist_pos};
  double gap = m->hist_min_gap;
  if (!m->has_history) {
    // the two-entry step: entries at 0 and 1, so the minimum gap is 1
    if (!m->step_off) {
      CCD_CUDA(cudaMalloc(&m->step_off, ((size_t)m->nv + 1) * sizeof(int32_t)));
      CCD_CUDA(cudaMalloc(&m->step_time, 2 * (size_t)m->nv * sizeof(double)));
      CCD_CUDA(cudaMalloc(&m->step_pos, 6 * (size_t)m->nv * sizeof(double)));
    }
    CCD_CUDA(ccd::launch_two_entry_view(m->nv, m->qs, m->qe, m->step_off, m->step_time, m->step_pos, s));
    hv = ccd::HistoryView{m->step_off, m->step_time, m->step_pos};
    gap = ccd::smin(1.0 - 0.0, 1.0);
  }
  const double eps = gap / 4.0;
  for (int k = 0; k < 2; k++) {
    const int64_t n = k == 0 ? n_vf : n_ee;
    if (n == 0) continue;
    const int32_t *st = k == 0 ? vf : ee;
    const double *eta = k == 0 ? vf_eta : ee_eta;
    const int64_t ec = k == 0 ? vf_eta_count : ee_eta_count;
    Lane &L = m->lane[0];
    rc = grow(ctx, &m->in_st, &m->in_st_cap, 4 * n);
    if (!rc) rc = grow(ctx, &m->in_eta, &m->in_eta_cap, ec);
    if (!rc) rc = grow(ctx, &L.hit, &L.hit_cap, 2 * n);
    if (rc) return rc;
    CCD_CUDA(cudaMemcpyAsync(m->in_st, st, (size_t)n * 16, cudaMemcpyHostToDevice, s));
    CCD_CUDA(cudaMemcpyAsync(m->in_eta, eta, (size_t)ec * sizeof(double), cudaMemcpyHostToDevice, s));
    CCD_CUDA(ccd::launch_separating_plane(k, hv, m->in_st, n, m->in_eta, ec == n && n != 1 ? 1 : 0, eps, L.hit,
                                          L.hit + n, s));
    CCD_CUDA(cudaMemcpyAsync(k == 0 ? vf_hit : ee_hit, L.hit, (size_t)n, cudaMemcpyDeviceToHost, s));
    uint8_t *status = k == 0 ? vf_status : ee_status;
    if (status) CCD_CUDA(cudaMemcpyAsync(status, L.hit + n, (size_t)n, cudaMemcpyDeviceToHost, s));
    CCD_CUDA(cudaStreamSynchronize(s));
  }
  return CCD_OK;
}

int ccd_mesh_detect(ccd_mesh *m, int broadphase_kind, double outer_eta, double eta, int path, int64_t *vf_hits,
                    int64_t *ee_hits) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (broadphase_kind != CCD_BROADPHASE_KDOP13 && broadphase_kind != CCD_BROADPHASE_AABB &&
      broadphase_kind != CCD_BROADPHASE_TRIVIAL)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown broadphase kind");
  if (path != CCD_PATH_FP64 && path != CCD_PATH_CULL_REFINE)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown path");
  CCD_CUDA(cudaSetDevice(ctx->device));
  int rc = run_broadphase(m, broadphase_kind, outer_eta);
  if (rc) return rc;
  CCD_CUDA(cudaMemcpyAsync(m->d_eta, &eta, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  m->lane[0].stream = ctx->stream;
  m->lane[1].stream = m->side;
  for (int k = 0; k < 2; k++) {
    Lane &L = m->lane[k];
    const int64_t n = m->n_cand[k];
    rc = grow(ctx, &L.hit, &L.hit_cap, n);
    if (!rc) rc = grow(ctx, &L.t, &L.t_cap, n);
    if (!rc) rc = grow(ctx, &L.flags, &L.flags_cap, n);
    if (!rc) rc = grow(ctx, &L.pos, &L.pos_cap, n);
    if (!rc) rc = grow(ctx, &L.scan_temp, &L.scan_temp_cap, (int64_t)ccd::scan_temp_bytes(n));
    if (!rc) rc = grow(ctx, &m->col[k], &m->col_cap[k], 4 * n);
    if (!rc) rc = grow(ctx, &m->col_t[k], &m->col_t_cap[k], n);
    if (rc) return rc;
  }
  // Fork: the edge-edge chain runs on the side stream once the broad phase
  // and eta are in place; join before the counts are read.
  CCD_CUDA(cudaEventRecord(m->fork, ctx->stream));
  CCD_CUDA(cudaStreamWaitEvent(m->side, m->fork, 0));
  for (int k = 0; k < 2; k++) {
    Lane &L = m->lane[k];
    const int64_t n = m->n_cand[k];
    rc = narrow_device(m, L, k ? CCD_EDGE_EDGE : CCD_VERTEX_FACE, path, n, m->cand[k], m->d_eta, false, L.hit, L.t,
                       nullptr);
    if (rc) return rc;
    CCD_CUDA(ccd::compact_hits(m->cand[k], L.hit, L.t, n, L.flags, L.pos, L.d_count, L.scan_temp,
                               (size_t)L.scan_temp_cap, m->col[k], m->col_t[k], L.stream));
  }
  CCD_CUDA(cudaEventRecord(m->join, m->side));
  CCD_CUDA(cudaStreamWaitEvent(ctx->stream, m->join, 0));
  uint32_t counts[2] = {0, 0};
  for (int k = 0; k < 2; k++)
    CCD_CUDA(cudaMemcpyAsync(&counts[k], m->lane[k].d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  m->n_col[0] = counts[0];
  m->n_col[1] = counts[1];
  m->stats.vf_hits = m->n_col[0];
  m->stats.ee_hits = m->n_col[1];
  m->have_col = true;
  if (vf_hits) *vf_hits = m->n_col[0];
  if (ee_hits) *ee_hits = m->n_col[1];
  return CCD_OK;
}

int ccd_mesh_get_collisions(ccd_mesh *m, int32_t *vf, double *vf_t, int32_t *ee, double *ee_t) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!m->have_col) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "no detection result on this mesh");
  CCD_CUDA(cudaSetDevice(ctx->device));
  int32_t *st[2] = {vf, ee};
  double *tt[2] = {vf_t, ee_t};
  for (int k = 0; k < 2; k++) {
    const int64_t n = m->n_col[k];
    if (!n) continue;
    if (st[k])
      CCD_CUDA(cudaMemcpyAsync(st[k], m->col[k], (size_t)n * 4 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               ctx->stream));
    if (tt[k])
      CCD_CUDA(cudaMemcpyAsync(tt[k], m->col_t[k], (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  }
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  return CCD_OK;
}

int ccd_mesh_self_distance(ccd_mesh *m, const double *verts, double *distance, int64_t *n_vf, int64_t *n_ee) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  if (!distance) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null distance");
  int rc = ccd_mesh_set_positions(m, verts, verts);  // the motionless step of src/Distance.cpp:38-39
  if (rc) return rc;
  // 1. the vertex scan (src/Distance.cpp:21-35)
  cudaError_t err = cudaSuccess;
  double d2 = INFINITY;
  rc = ccd::closest_vertex_pair(m->nv, m->nf, m->faces, m->qs, m->pt, &d2, ctx->stream, &err);
  if (rc == 2) return cuda_fail(ctx, err, "closest vertex pair");
  if (rc == 3) return mesh_fail(m, CCD_ERR_CUDA, "closest vertex pair: malformed tree");
  const double closest = std::sqrt(d2);
  // 2. candidates of the AABB broad phase padded by that distance
  //    (src/Distance.cpp:41-46).  With no qualifying vertex pair every face
  //    holds every vertex, so every face pair shares a vertex and there is
  //    no candidate; the broad phase is skipped then.
  int64_t nvf = 0, nee = 0;
  if (std::isfinite(closest)) {
    rc = run_broadphase(m, CCD_BROADPHASE_AABB, closest, /*whole=*/true);
    if (rc) return rc;
    nvf = m->n_cand[0];
    nee = m->n_cand[1];
  } else {
    m->stats = ccd_mesh_stats{};
    m->n_cand[0] = m->n_cand[1] = 0;
    m->have_cand = true;
  }
  m->stats.self_distance_eta = closest;
  // 3. the least stencil distance (src/Distance.cpp:48-64)
  unsigned long long *best = m->pt.counters ? m->pt.counters + 2 : nullptr;
  double result = INFINITY;
  if (nvf + nee > 0 && best) {
    const unsigned long long inf = 0x7ff0000000000000ull;
    CCD_CUDA(cudaMemcpyAsync(best, &inf, sizeof(inf), cudaMemcpyHostToDevice, ctx->stream));
    CCD_CUDA(ccd::launch_stencil_distance_min(m->qs, m->cand[0], nvf, m->cand[1], nee, best, ctx->num_sms,
                                              ctx->stream));
    unsigned long long bits = inf;
    CCD_CUDA(cudaMemcpyAsync(&bits, best, sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
    memcpy(&result, &bits, sizeof(result));
  }
  *distance = result;
  if (n_vf) *n_vf = nvf;
  if (n_ee) *n_ee = nee;
  return CCD_OK;
}

int ccd_self_distance(ccd_context *ctx, int32_t nverts, const double *verts, int32_t nfaces, const int32_t *faces,
                      const uint8_t *fixed, double *distance) {
  if (!ctx || !distance) return CCD_ERR_INVALID_ARGUMENT;
  if (nverts == 0 && nfaces == 0) {  // no vertex pair and no stencil, as in the reference
    *distance = INFINITY;
    return CCD_OK;
  }
  ccd_mesh *m = nullptr;
  int rc = ccd_mesh_create(ctx, nverts, nfaces, faces, &m);
  if (rc) return rc;
  if (fixed) rc = ccd_mesh_set_fixed(m, fixed);
  if (!rc) rc = ccd_mesh_self_distance(m, verts, distance, nullptr, nullptr);
  ccd_mesh_destroy(m);
  return rc;
}

int ccd_mesh_last_stats(const ccd_mesh *m, ccd_mesh_stats *out) {
  if (!m || !out) return CCD_ERR_INVALID_ARGUMENT;
  *out = m->stats;
  return CCD_OK;
}

}  // extern "C"
