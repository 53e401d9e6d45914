// C ABI (include/ccd_gb300.h): meshes, broad phase, narrow phase over stencils.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <functional>
#include <map>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "broadphase.cuh"
#include "ccd_common.h"
#include "context.cuh"
#include "distance.cuh"
#include "mesh.cuh"
#include "radix_sort.cuh"
#include "separating.cuh"
#include "ccd_heap.h"
#include "velocity.cuh"

using namespace ccd_capi;

namespace {

// Segments per chunk of the narrow phase over a multi-entry history (bounds
// its row scratch to about 1.3 GB); two-entry steps take chunks of the
// context's "narrow_chunk" stencils.
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
  // A captured refit-only detect step (ccd_mesh_detect_graph): its key, the
  // buffers it was captured with, its capacities and the pinned words its
  // counts come back in.
  cudaGraphExec_t graph = nullptr;
  std::vector<uintptr_t> graph_sig;
  int graph_kind = -1, graph_path = -1;
  double graph_outer = 0.0, graph_eta = 0.0;
  int64_t gcap_pairs = 0, gcap[2] = {0, 0};
  unsigned long long *h_graph = nullptr;  // [8] broad-phase counters, [8 + k] collisions of kind k
};

namespace {

// Padding vertices after a mesh's own (indices nv .. nv + 3): pairwise at
// least 1,000 apart and not moving, so that a vertex-face or edge-edge
// stencil of them, and each sub-test of its chain, is rejected by the FP32
// stage (or misses in FP64) for any eta below about 100.
constexpr int kPadVerts = 4;
const double kPadPositions[3 * kPadVerts] = {1e3, 0.0, 0.0, 0.0, 1e3, 0.0, 0.0, 0.0, 1e3, -1e3, -1e3, -1e3};

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
  const int64_t chunk = std::min<int64_t>(n, ctx->opt_narrow_chunk);
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
ccd::MeshTopology mesh_topology(const ccd_mesh *m, bool whole) {
  return ccd::MeshTopology{m->nv,        m->nf,        m->nranks,      m->nedges,
                           m->faces,     m->face_rank, m->rank_triple, m->face_edges,
                           m->rank_edge, whole ? nullptr : m->face_inst, whole ? 1 : m->ninst};
}

ccd::BroadphaseParams mesh_params(const ccd_mesh *m, int kind, double outer_eta) {
  const ccd_context *ctx = m->ctx;
  return ccd::BroadphaseParams{kind,
                               outer_eta,
                               m->qs,
                               m->qe,
                               m->has_history ? m->hist_off : nullptr,
                               m->has_history ? m->hist_pos : nullptr,
                               m->has_fixed ? m->fixed : nullptr,
                               ctx->opt_count_tests != 0,
                               (int)ctx->opt_traversal,
                               ctx->opt_tree_refit != 0,
                               (float)ctx->opt_tree_rebuild_pct / 100.0f,
                               ctx->opt_tree_max_refits,
                               {nullptr, nullptr, nullptr, nullptr}};
}

int run_broadphase(ccd_mesh *m, int kind, double outer_eta, bool whole = false) {
  ccd_context *ctx = m->ctx;
  m->have_cand = false;
  m->have_col = false;
  m->stats = ccd_mesh_stats{};
  const ccd::MeshTopology topo = mesh_topology(m, whole);
  ccd::BroadphaseParams p = mesh_params(m, kind, outer_eta);
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
  bool built = true;
  const int rc = ccd::broadphase_run(topo, p, m->bp, &m->cand[0], &m->cand_cap[0], &m->cand[1], &m->cand_cap[1],
                                     &m->n_cand[0], &m->n_cand[1], &npairs, &tests, ctx->num_sms, ctx->stream, &err,
                                     &built);
  m->stats.tree_built = built ? 1 : 0;
  m->stats.tree_refits = m->bp.refits;
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
  if (m->graph) cudaGraphExecDestroy(m->graph);
  if (m->h_graph) cudaFreeHost(m->h_graph);
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
    // Positions, then the four padding vertices of the graph step's
    // candidate lists (far apart and still: a stencil of them never hits).
    const size_t room = 3 * ((size_t)nverts + kPadVerts);
    CCD_CUDA(cudaMalloc(&m->qs, room * sizeof(double)));
    CCD_CUDA(cudaMalloc(&m->qe, room * sizeof(double)));
    CCD_CUDA(cudaMemsetAsync(m->qs, 0, 3 * (size_t)nverts * sizeof(double), ctx->stream));
    CCD_CUDA(cudaMemsetAsync(m->qe, 0, 3 * (size_t)nverts * sizeof(double), ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(m->qs + 3 * (size_t)nverts, kPadPositions, sizeof(kPadPositions), cudaMemcpyHostToDevice,
                             ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(m->qe + 3 * (size_t)nverts, kPadPositions, sizeof(kPadPositions), cudaMemcpyHostToDevice,
                             ctx->stream));
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
  if (!valid_path(path))
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
  if (!valid_path(path))
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

}  // extern "C"

namespace {

void drop_graph(ccd_mesh *m) {
  if (m->graph) cudaGraphExecDestroy(m->graph);
  m->graph = nullptr;
  m->graph_sig.clear();
}

// Every device buffer, capacity and option a captured step depends on: a
// replay is valid only while all of them are unchanged.
std::vector<uintptr_t> graph_signature(const ccd_mesh *m) {
  const ccd_context *ctx = m->ctx;
  const ccd::BroadphaseBuffers &b = m->bp;
  std::vector<uintptr_t> v = {
      (uintptr_t)m->qs, (uintptr_t)m->qe, (uintptr_t)m->fixed, (uintptr_t)m->has_fixed, (uintptr_t)m->d_eta,
      (uintptr_t)m->cand[0], (uintptr_t)m->cand[1], (uintptr_t)m->col[0], (uintptr_t)m->col[1],
      (uintptr_t)m->col_t[0], (uintptr_t)m->col_t[1], (uintptr_t)m->side,
      (uintptr_t)b.lo64, (uintptr_t)b.hi64, (uintptr_t)b.face_lo, (uintptr_t)b.face_hi, (uintptr_t)b.leaf_box,
      (uintptr_t)b.node_box, (uintptr_t)b.node_child, (uintptr_t)b.node_links, (uintptr_t)b.leaf_links,
      (uintptr_t)b.leaf_end, (uintptr_t)b.parent, (uintptr_t)b.arrive, (uintptr_t)b.keys, (uintptr_t)b.counters,
      (uintptr_t)b.pairs, (uintptr_t)b.vf_keys, (uintptr_t)b.ee_keys, (uintptr_t)b.keys_alt, (uintptr_t)b.flags,
      (uintptr_t)b.scan, (uintptr_t)b.temp, (uintptr_t)b.temp_bytes, (uintptr_t)b.cap_pairs,
      (uintptr_t)b.cap_faces, (uintptr_t)ctx->opt_wave_steps, (uintptr_t)ctx->opt_pool_budget,
      (uintptr_t)ctx->opt_wave_min_rows, (uintptr_t)ctx->opt_warp_finish, (uintptr_t)ctx->opt_traversal,
      (uintptr_t)ctx->opt_shift_after, (uintptr_t)ctx->opt_pool_slots_min, (uintptr_t)ctx->opt_pool_slots, (uintptr_t)ctx->opt_pool_all, (uintptr_t)ctx->opt_pool_phase_sync,
      (uintptr_t)ctx->opt_narrow_chunk};
  for (const Lane &L : m->lane) {
    const NarrowScratch &n = L.ns;
    const uintptr_t lp[] = {(uintptr_t)L.hit,    (uintptr_t)L.t,         (uintptr_t)L.flags,   (uintptr_t)L.pos,
                            (uintptr_t)L.scan_temp, (uintptr_t)L.scan_temp_cap, (uintptr_t)L.d_count,
                            (uintptr_t)n.prim,   (uintptr_t)n.ve,        (uintptr_t)n.vv,      (uintptr_t)n.eta_prim,
                            (uintptr_t)n.eta_ve, (uintptr_t)n.eta_vv,    (uintptr_t)n.h_prim,  (uintptr_t)n.h_ve,
                            (uintptr_t)n.h_vv,   (uintptr_t)n.t_prim,    (uintptr_t)n.t_ve,    (uintptr_t)n.t_vv,
                            (uintptr_t)n.surv,   (uintptr_t)n.counters,  (uintptr_t)n.cap,     (uintptr_t)n.stage.mem,
                            (uintptr_t)n.stage.cap, (uintptr_t)n.stage.view.wd};
    v.insert(v.end(), lp, lp + sizeof(lp) / sizeof(lp[0]));
  }
  return v;
}

// The kernels of one refit-only step, enqueued with no host
// synchronisation: the broad phase on the kept tree into candidate lists
// padded to their capacities, then both narrow-phase chains and the
// compaction of their hits, and the counts copied to m->h_graph.
int enqueue_graph_step(ccd_mesh *m, int kind, double outer_eta, int path) {
  ccd_context *ctx = m->ctx;
  const ccd::MeshTopology topo = mesh_topology(m, false);
  ccd::BroadphaseParams p = mesh_params(m, kind, outer_eta);
  p.count_tests = false;
  cudaError_t err = cudaSuccess;
  const int4 pad = make_int4(m->nv, m->nv + 1, m->nv + 2, m->nv + 3);
  const int brc = ccd::broadphase_enqueue_refit(topo, p, m->bp, m->gcap_pairs, m->cand[0], m->gcap[0], m->cand[1],
                                                m->gcap[1], pad, ctx->stream, &err);
  if (brc == 2) return cuda_fail(ctx, err, "broadphase (graph step)");
  if (brc) return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT, "graph step without a kept tree");
  CCD_CUDA(cudaEventRecord(m->fork, ctx->stream));
  CCD_CUDA(cudaStreamWaitEvent(m->side, m->fork, 0));
  for (int k = 0; k < 2; k++) {
    Lane &L = m->lane[k];
    const int64_t n = m->gcap[k];
    int rc = narrow_device(m, L, k ? CCD_EDGE_EDGE : CCD_VERTEX_FACE, path, n, m->cand[k], m->d_eta, false, L.hit,
                           L.t, nullptr);
    if (rc) return rc;
    CCD_CUDA(ccd::compact_hits(m->cand[k], L.hit, L.t, n, L.flags, L.pos, L.d_count, L.scan_temp,
                               (size_t)L.scan_temp_cap, m->col[k], m->col_t[k], L.stream));
  }
  CCD_CUDA(cudaEventRecord(m->join, m->side));
  CCD_CUDA(cudaStreamWaitEvent(ctx->stream, m->join, 0));
  CCD_CUDA(cudaMemcpyAsync(m->h_graph, m->bp.counters, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                           ctx->stream));
  for (int k = 0; k < 2; k++)
    CCD_CUDA(cudaMemcpyAsync(m->h_graph + 8 + k, m->lane[k].d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             ctx->stream));
  return CCD_OK;
}

// Captures the step after a direct detect of the same kind (which built or
// refitted the tree and sized every buffer for its counts): capacities are
// twice the direct step's counts, and every buffer is grown to them before
// the capture, so that the capture allocates nothing.
int capture_graph_step(ccd_mesh *m, int kind, double outer_eta, double eta, int path) {
  ccd_context *ctx = m->ctx;
  drop_graph(m);
  // Twice the direct step's counts: a growing contact then outgrows a
  // capture only every doubling, and each recapture (a direct step, the
  // capture and its instantiation) costs several steps' host time.
  const int64_t pairs = m->stats.face_pairs;
  m->gcap_pairs = std::min<int64_t>(m->bp.cap_pairs, std::max<int64_t>(2 * pairs, 4096));
  for (int k = 0; k < 2; k++) {
    const int64_t n = m->n_cand[k];
    m->gcap[k] = std::min<int64_t>((k ? 9 : 6) * m->gcap_pairs, std::max<int64_t>(2 * n, 4096));
  }
  if (!m->h_graph) CCD_CUDA(cudaMallocHost(&m->h_graph, 10 * sizeof(unsigned long long)));
  m->lane[0].stream = ctx->stream;
  m->lane[1].stream = m->side;
  for (int k = 0; k < 2; k++) {
    Lane &L = m->lane[k];
    const int64_t n = m->gcap[k];
    int rc = grow(ctx, &m->cand[k], &m->cand_cap[k], 4 * n);
    if (!rc) rc = grow(ctx, &L.hit, &L.hit_cap, n);
    if (!rc) rc = grow(ctx, &L.t, &L.t_cap, n);
    if (!rc) rc = grow(ctx, &L.flags, &L.flags_cap, n);
    if (!rc) rc = grow(ctx, &L.pos, &L.pos_cap, n);
    if (!rc) rc = grow(ctx, &L.scan_temp, &L.scan_temp_cap, (int64_t)ccd::scan_temp_bytes(n));
    if (!rc) rc = grow(ctx, &m->col[k], &m->col_cap[k], 4 * n);
    if (!rc) rc = grow(ctx, &m->col_t[k], &m->col_t_cap[k], n);
    const int64_t chunk = std::min<int64_t>(n, ctx->opt_narrow_chunk);
    if (!rc) rc = ensure_narrow(m, L, chunk);
    if (!rc) rc = ensure_stage(ctx, L.ns.stage, chunk, L.stream);
    if (rc) return rc;
  }
  CCD_CUDA(cudaMemcpyAsync(m->d_eta, &eta, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(m->side));
  CCD_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue_graph_step(m, kind, outer_eta, path);
  cudaGraph_t g = nullptr;
  const cudaError_t end = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (end != cudaSuccess) return cuda_fail(ctx, end, "cudaStreamEndCapture");
  const cudaError_t inst = cudaGraphInstantiate(&m->graph, g, 0);
  cudaGraphDestroy(g);
  if (inst != cudaSuccess) {
    m->graph = nullptr;
    return cuda_fail(ctx, inst, "cudaGraphInstantiate");
  }
  m->graph_sig = graph_signature(m);
  m->graph_kind = kind;
  m->graph_path = path;
  m->graph_outer = outer_eta;
  m->graph_eta = eta;
  return CCD_OK;
}

// Replays the captured step.  Returns 1 (results not usable: a capacity was
// exceeded or the traversal reported an error; the caller runs the direct
// step) or 0 with the mesh's counts, stats and tree bookkeeping updated.
int replay_graph_step(ccd_mesh *m, int *usable) {
  ccd_context *ctx = m->ctx;
  *usable = 0;
  memset(m->h_graph, 0, 10 * sizeof(unsigned long long));
  CCD_CUDA(cudaGraphLaunch(m->graph, ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  const unsigned long long *h = m->h_graph;
  const int64_t pairs = (int64_t)h[0];
  const int64_t nvf = (int64_t)(uint32_t)h[1], nee = (int64_t)(uint32_t)h[2];
  if (h[3] || pairs > m->gcap_pairs || nvf > m->gcap[0] || nee > m->gcap[1]) return CCD_OK;
  // tree quality, as a direct refit step judges it
  ccd::BroadphaseBuffers &b = m->bp;
  float area;
  const uint32_t bits = (uint32_t)h[5];
  memcpy(&area, &bits, sizeof(area));
  if (b.build_area < 0.0f)
    b.build_area = area;
  else if (!(area <= (float)ctx->opt_tree_rebuild_pct / 100.0f * b.build_area))
    b.rebuild_next = true;
  b.refits++;
  m->n_cand[0] = nvf;
  m->n_cand[1] = nee;
  m->n_col[0] = (int64_t)(uint32_t)h[8];
  m->n_col[1] = (int64_t)(uint32_t)h[9];
  m->stats = ccd_mesh_stats{};
  m->stats.face_pairs = pairs;
  m->stats.n_vf = nvf;
  m->stats.n_ee = nee;
  m->stats.vf_hits = m->n_col[0];
  m->stats.ee_hits = m->n_col[1];
  m->stats.slab_tests = -1;
  m->stats.tree_built = 0;
  m->stats.tree_refits = b.refits;
  m->stats.graph_replay = 1;
  m->have_cand = m->have_col = true;
  *usable = 1;
  return CCD_OK;
}

}  // namespace

extern "C" {

int ccd_mesh_detect_graph(ccd_mesh *m, int broadphase_kind, double outer_eta, double eta, int path,
                          int64_t *vf_hits, int64_t *ee_hits) {
  if (!m) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = m->ctx;
  const bool eligible = broadphase_kind != CCD_BROADPHASE_TRIVIAL && !m->has_history && ctx->opt_tree_refit &&
                        !ctx->profiling && !ctx->opt_count_tests && m->nf >= 2 && m->ninst >= 1;
  if (eligible && m->graph && m->graph_kind == broadphase_kind && m->graph_path == path &&
      m->graph_outer == outer_eta && m->graph_eta == eta && !m->bp.rebuild_next &&
      m->bp.refits < ctx->opt_tree_max_refits && m->bp.tree_kind == broadphase_kind &&
      graph_signature(m) == m->graph_sig) {
    CCD_CUDA(cudaSetDevice(ctx->device));
    int usable = 0;
    const int rc = replay_graph_step(m, &usable);
    if (rc) return rc;
    if (usable) {
      if (vf_hits) *vf_hits = m->n_col[0];
      if (ee_hits) *ee_hits = m->n_col[1];
      return CCD_OK;
    }
    drop_graph(m);  // counts outgrew the capture: the direct step below sizes a new one
  }
  int rc = ccd_mesh_detect(m, broadphase_kind, outer_eta, eta, path, vf_hits, ee_hits);
  if (rc || !eligible || m->bp.tree_kind != broadphase_kind) return rc;
  if (m->graph && graph_signature(m) == m->graph_sig && m->graph_kind == broadphase_kind &&
      m->graph_path == path && m->graph_outer == outer_eta && m->graph_eta == eta)
    return CCD_OK;
  // Capture the step, then replay it once for this step's results: growing
  // the buffers to the capture's capacities may have replaced the direct
  // step's output arrays.  The step's results do not depend on the tree, so
  // the replay's equal the direct step's.
  rc = capture_graph_step(m, broadphase_kind, outer_eta, eta, path);
  int usable = 0;
  if (!rc) rc = replay_graph_step(m, &usable);
  if (!rc && usable) {
    if (vf_hits) *vf_hits = m->n_col[0];
    if (ee_hits) *ee_hits = m->n_col[1];
    return CCD_OK;
  }
  drop_graph(m);
  return ccd_mesh_detect(m, broadphase_kind, outer_eta, eta, path, vf_hits, ee_hits);
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

// ------------------------------------------------------------------ velocity filter
namespace {

// A canonical stencil as a map key, ordered like the reference's stencils
// (lexicographic; src/Stencils.h).
struct StencilKey {
  int32_t a, b, c, d;
  bool operator<(const StencilKey &o) const {
    if (a != o.a) return a < o.a;
    if (b != o.b) return b < o.b;
    if (c != o.c) return c < o.c;
    return d < o.d;
  }
};

// PenaltyGroup (src/PenaltyGroup.h): its parameters, firing step and stencils.
struct HostGroup {
  double dt, eta, inner, k, cor;
  int nextstep;
  std::vector<StencilKey> vf, ee;  // insertion order
  std::set<int32_t> verts;         // getGroupStencil
};

// ActiveLayers (src/ActiveLayers.cpp) without its time stepping, which runs
// on the device: groups, the event queue, and the stencils' depths.
struct Layers {
  double outer, inner, base_dt, base_k, term, cor;
  int deepest = 0;
  std::vector<HostGroup> groups;
  std::vector<int> heap;
  int heap_size = 0;
  std::map<StencilKey, int> vfdepth, eedepth;

  bool later(int a, int b) const {
    return (double)groups[b].nextstep * groups[b].dt < (double)groups[a].nextstep * groups[a].dt;
  }
  void push(std::vector<int> &h, int &size, int g) {
    if ((int)h.size() < size + 1) h.resize(size + 1);
    ccd::heap_push(h.data(), &size, g, [this](int a, int b) { return later(a, b); });
  }
  // ActiveLayers::layerDepth (:169-172)
  double layer_depth(int layer) const { return inner + (outer - inner) / double(layer); }
  // ActiveLayers::addGroups (:69-89)
  void add_groups(int maxdepth) {
    while (deepest < maxdepth) {
      const int depth = deepest + 1;
      const double fudge = 1e-4;
      const double ki = base_k * depth * depth * depth;
      const double etai = layer_depth(depth);
      const double dti = base_dt / double(depth) / std::sqrt(double(depth) + fudge);
      groups.push_back(HostGroup{dti, etai, inner, ki, cor, 1, {}, {}, {}});
      push(heap, heap_size, (int)groups.size() - 1);
      deepest++;
    }
  }
  // ActiveLayers::addVFStencil / addEEStencil (:43-67)
  void add(int kind, const StencilKey &st) {
    std::map<StencilKey, int> &depth = kind == 0 ? vfdepth : eedepth;
    const int olddepth = depth[st];
    for (int i = 0; i < 5; i++) {
      add_groups(olddepth + i + 1);
      HostGroup &g = groups[(size_t)(olddepth + i)];
      (kind == 0 ? g.vf : g.ee).push_back(st);
      g.verts.insert(st.a);
      g.verts.insert(st.b);
      g.verts.insert(st.c);
      g.verts.insert(st.d);
      depth[st]++;
    }
  }
  // ActiveLayers::VFStencilThickness / EEStencilThickness (:174-188)
  double thickness(int kind, const StencilKey &st) const {
    const std::map<StencilKey, int> &depth = kind == 0 ? vfdepth : eedepth;
    auto it = depth.find(st);
    return it != depth.end() ? layer_depth(it->second + 1) : layer_depth(1);
  }
  // ActiveLayers::rollback (:158-167): firing steps reset, then the queue
  // re-built by popping the old one (whose keys just changed) into a new one.
  void rollback() {
    for (HostGroup &g : groups) g.nextstep = 1;
    std::vector<int> fresh;
    int fresh_size = 0;
    while (heap_size > 0) {
      push(fresh, fresh_size, heap[0]);
      ccd::heap_pop(heap.data(), &heap_size, [this](int a, int b) { return later(a, b); });
    }
    heap = fresh;
    heap_size = fresh_size;
  }
};

// Device buffers of one velocity-filter call.
struct FilterBuffers {
  std::vector<void *> owned;
  template <class T>
  int alloc(ccd_context *ctx, T **p, size_t count) {
    CCD_CUDA(cudaMalloc(p, std::max<size_t>(count, 1) * sizeof(T)));
    owned.push_back(*p);
    return CCD_OK;
  }
  ~FilterBuffers() {
    for (void *p : owned) cudaFree(p);
  }
};

// Makes device history arrays (off [nv+1], times, pos) the mesh's history.
int adopt_history(ccd_mesh *m, const int32_t *off, const double *times, const double *pos, int64_t ne,
                  double gap) {
  ccd_context *ctx = m->ctx;
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
  CCD_CUDA(cudaMemcpyAsync(m->hist_off, off, ((size_t)m->nv + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                           ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->hist_time, times, (size_t)ne * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(m->hist_pos, pos, (size_t)ne * 3 * sizeof(double), cudaMemcpyDeviceToDevice,
                           ctx->stream));
  m->hist_min_gap = gap;
  m->has_history = true;
  m->have_cand = m->have_col = false;
  return CCD_OK;
}

}  // namespace

extern "C" int ccd_velocity_filter(ccd_context *ctx, int32_t nverts, const double *qstart, double *qend,
                                   int32_t nfaces, const int32_t *faces, const double *invmasses, double outer_eta,
                                   double inner_eta, double base_stiffness, double base_substep, double cor,
                                   int32_t max_rollbacks, int32_t *result, ccd_velocity_filter_stats *stats) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (!result || nverts <= 0 || nfaces < 0 || !qstart || !qend || !invmasses || (nfaces && !faces))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer or empty mesh");
  ccd_velocity_filter_stats st{};
  // VelocityFilter.cpp:22-39: every vertex in some face
  {
    std::vector<uint8_t> used((size_t)nverts, 0);
    for (int64_t i = 0; i < 3 * (int64_t)nfaces; i++) {
      if (faces[i] < 0 || faces[i] >= nverts) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "face vertex out of range");
      used[(size_t)faces[i]] = 1;
    }
    for (uint8_t u : used)
      if (!u) {
        *result = -1;  // DANGLING_VERTICES
        if (stats) *stats = st;
        return CCD_OK;
      }
  }
  double maxmass = 0;
  for (int64_t i = 0; i < 3 * (int64_t)nverts; i++) maxmass = ccd::smax(maxmass, invmasses[i]);
  const double dt = base_substep;
  const double k = base_stiffness / dt * std::sqrt(maxmass);
  Layers al{outer_eta, inner_eta, dt, k, 1.0, cor};
  ccd_mesh *m = nullptr;
  int rc = ccd_mesh_create(ctx, nverts, nfaces, faces, &m);
  if (rc) return rc;
  struct MeshGuard {
    ccd_mesh *m;
    ~MeshGuard() { ccd_mesh_destroy(m); }
  } guard{m};
  std::vector<uint8_t> fixed((size_t)nverts, 0);
  bool any_fixed = false;
  for (int64_t i = 0; i < 3 * (int64_t)nverts; i++)
    if (invmasses[i] == 0.0) fixed[(size_t)(i / 3)] = 1, any_fixed = true;
  rc = ccd_mesh_set_fixed(m, any_fixed ? fixed.data() : nullptr);
  if (rc) return rc;
  // VelocityFilter.cpp:60-67
  double closest = 0;
  rc = ccd_mesh_self_distance(m, qstart, &closest, nullptr, nullptr);
  if (rc) return rc;
  st.start_distance = closest;
  if (closest < inner_eta) {
    *result = -2;  // STARTING_STATE_INTERSECTS
    if (stats) *stats = st;
    return CCD_OK;
  }
  CCD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int64_t n3 = 3 * (int64_t)nverts;
  FilterBuffers fb;
  double *d_q0 = nullptr, *d_q = nullptr, *d_v = nullptr, *d_lu = nullptr, *d_minv = nullptr, *d_newq = nullptr,
         *d_newv = nullptr, *d_qend = nullptr;
  rc = fb.alloc(ctx, &d_q0, n3);
  if (!rc) rc = fb.alloc(ctx, &d_q, n3);
  if (!rc) rc = fb.alloc(ctx, &d_v, n3);
  if (!rc) rc = fb.alloc(ctx, &d_lu, n3);
  if (!rc) rc = fb.alloc(ctx, &d_minv, n3);
  if (!rc) rc = fb.alloc(ctx, &d_newq, n3);
  if (!rc) rc = fb.alloc(ctx, &d_newv, n3);
  if (!rc) rc = fb.alloc(ctx, &d_qend, n3);
  int64_t *d_counts = nullptr;  // [0] log_n, [1] events
  ccd::GridStep *d_step = nullptr;
  int *d_status = nullptr;
  unsigned long long *d_gap = nullptr;
  uint32_t *d_count = nullptr, *d_scan = nullptr;
  int32_t *d_off = nullptr;
  if (!rc) rc = fb.alloc(ctx, &d_counts, 2);
  if (!rc) rc = fb.alloc(ctx, &d_step, 1);
  if (!rc) rc = fb.alloc(ctx, &d_status, 1);
  if (!rc) rc = fb.alloc(ctx, &d_gap, 1);
  if (!rc) rc = fb.alloc(ctx, &d_count, (size_t)nverts + 1);
  if (!rc) rc = fb.alloc(ctx, &d_scan, (size_t)nverts + 1);
  if (!rc) rc = fb.alloc(ctx, &d_off, (size_t)nverts + 1);
  if (rc) return rc;
  CCD_CUDA(cudaMemcpyAsync(d_q0, qstart, n3 * 8, cudaMemcpyHostToDevice, s));
  CCD_CUDA(cudaMemcpyAsync(d_qend, qend, n3 * 8, cudaMemcpyHostToDevice, s));
  CCD_CUDA(cudaMemcpyAsync(d_minv, invmasses, n3 * 8, cudaMemcpyHostToDevice, s));
  std::vector<double> hv((size_t)n3);
  for (int64_t i = 0; i < n3; i++) hv[(size_t)i] = qend[i] - qstart[i];  // s.v = qend - qstart
  // growable per-iteration buffers
  int64_t log_cap = 0, grp_cap[4] = {0, 0, 0, 0};
  int32_t *log_v = nullptr;
  double *log_t = nullptr, *log_p = nullptr;
  double *h_times = nullptr, *h_pos = nullptr;
  uint64_t *keys = nullptr, *keys_alt = nullptr;
  void *temp = nullptr;
  size_t temp_bytes = 0;
  std::vector<void *> grow_owned;
  auto release_growable = [&]() {
    for (void *p : grow_owned) cudaFree(p);
    grow_owned.clear();
  };
  struct Release {
    std::function<void()> f;
    ~Release() { f(); }
  } release{release_growable};
  auto dev = [&](auto **p, size_t count) -> int {
    CCD_CUDA(cudaMalloc(p, std::max<size_t>(count, 1) * sizeof(**p)));
    grow_owned.push_back(*p);
    return CCD_OK;
  };
  (void)grp_cap;
  for (int iter = 0; iter < max_rollbacks; iter++) {
    // ---- the groups of this iteration, flattened
    const int G = (int)al.groups.size();
    std::vector<double> g_dt, g_eta, g_inner, g_k, g_cor;
    std::vector<int> g_next;
    std::vector<int64_t> st_off(1, 0), gv_off(1, 0), co_off(1, 0);
    std::vector<int32_t> n_vf, stv, gvv, cov;
    int64_t max_st = 1, max_gv = 1;
    for (const HostGroup &g : al.groups) {
      max_gv = std::max<int64_t>(max_gv, (int64_t)g.verts.size());
      g_dt.push_back(g.dt), g_eta.push_back(g.eta), g_inner.push_back(g.inner), g_k.push_back(g.k);
      g_cor.push_back(g.cor), g_next.push_back(g.nextstep);
      n_vf.push_back((int32_t)g.vf.size());
      std::vector<const StencilKey *> all;
      for (const StencilKey &x : g.vf) all.push_back(&x);
      for (const StencilKey &x : g.ee) all.push_back(&x);
      for (const StencilKey *x : all) stv.insert(stv.end(), {x->a, x->b, x->c, x->d});
      st_off.push_back(st_off.back() + (int64_t)all.size());
      max_st = std::max<int64_t>(max_st, (int64_t)all.size());
      std::vector<int32_t> verts(g.verts.begin(), g.verts.end());
      std::vector<std::vector<int32_t>> lists(verts.size());
      for (size_t i = 0; i < all.size(); i++) {
        const int32_t vs[4] = {all[i]->a, all[i]->b, all[i]->c, all[i]->d};
        for (int slot = 0; slot < 4; slot++) {
          const size_t at = (size_t)(std::lower_bound(verts.begin(), verts.end(), vs[slot]) - verts.begin());
          lists[at].push_back((int32_t)((i << 2) | (size_t)slot));
        }
      }
      for (size_t j = 0; j < verts.size(); j++) {
        gvv.push_back(verts[j]);
        cov.insert(cov.end(), lists[j].begin(), lists[j].end());
        co_off.push_back((int64_t)cov.size());
      }
      gv_off.push_back((int64_t)gvv.size());
    }
    release_growable();
    double *d_gdt = nullptr, *d_geta = nullptr, *d_ginner = nullptr, *d_gk = nullptr, *d_gcor = nullptr,
           *d_contrib = nullptr;
    int *d_next = nullptr, *d_heap = nullptr, *d_heap_size = nullptr;
    int64_t *d_st_off = nullptr, *d_gv_off = nullptr, *d_co_off = nullptr;
    int32_t *d_nvf = nullptr, *d_st = nullptr, *d_gv = nullptr, *d_co = nullptr;
    uint8_t *d_fired = nullptr;
    rc = dev(&d_gdt, G);
    if (!rc) rc = dev(&d_geta, G);
    if (!rc) rc = dev(&d_ginner, G);
    if (!rc) rc = dev(&d_gk, G);
    if (!rc) rc = dev(&d_gcor, G);
    if (!rc) rc = dev(&d_next, G);
    if (!rc) rc = dev(&d_heap, G + 1);
    if (!rc) rc = dev(&d_heap_size, 1);
    if (!rc) rc = dev(&d_st_off, st_off.size());
    if (!rc) rc = dev(&d_gv_off, gv_off.size());
    if (!rc) rc = dev(&d_co_off, co_off.size());
    if (!rc) rc = dev(&d_nvf, G);
    if (!rc) rc = dev(&d_st, stv.size());
    if (!rc) rc = dev(&d_gv, gvv.size());
    if (!rc) rc = dev(&d_co, cov.size());
    if (!rc) rc = dev(&d_contrib, 12 * (size_t)max_st);
    if (!rc) rc = dev(&d_fired, (size_t)max_st);
    if (!rc && log_cap == 0) log_cap = std::max<int64_t>(1 << 20, 4 * (int64_t)nverts);
    if (!rc) rc = dev(&log_v, (size_t)log_cap);
    if (!rc) rc = dev(&log_t, (size_t)log_cap);
    if (!rc) rc = dev(&log_p, 3 * (size_t)log_cap);
    if (rc) return rc;
    auto up = [&](void *d, const void *h, size_t bytes) -> int {
      if (bytes) CCD_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
      return CCD_OK;
    };
    rc = up(d_gdt, g_dt.data(), G * 8);
    if (!rc) rc = up(d_geta, g_eta.data(), G * 8);
    if (!rc) rc = up(d_ginner, g_inner.data(), G * 8);
    if (!rc) rc = up(d_gk, g_k.data(), G * 8);
    if (!rc) rc = up(d_gcor, g_cor.data(), G * 8);
    if (!rc) rc = up(d_next, g_next.data(), G * 4);
    if (!rc) rc = up(d_heap, al.heap.data(), (size_t)al.heap_size * 4);
    if (!rc) rc = up(d_heap_size, &al.heap_size, 4);
    if (!rc) rc = up(d_st_off, st_off.data(), st_off.size() * 8);
    if (!rc) rc = up(d_gv_off, gv_off.data(), gv_off.size() * 8);
    if (!rc) rc = up(d_co_off, co_off.data(), co_off.size() * 8);
    if (!rc) rc = up(d_nvf, n_vf.data(), n_vf.size() * 4);
    if (!rc) rc = up(d_st, stv.data(), stv.size() * 4);
    if (!rc) rc = up(d_gv, gvv.data(), gvv.size() * 4);
    if (!rc) rc = up(d_co, cov.data(), cov.size() * 4);
    if (rc) return rc;
    // ---- the state (VelocityFilter.cpp:75-80) and the event loop (ActiveLayers::step)
    CCD_CUDA(cudaMemcpyAsync(d_q, d_q0, n3 * 8, cudaMemcpyDeviceToDevice, s));
    CCD_CUDA(cudaMemcpyAsync(d_v, hv.data(), n3 * 8, cudaMemcpyHostToDevice, s));
    CCD_CUDA(cudaMemsetAsync(d_lu, 0, n3 * 8, s));
    CCD_CUDA(cudaMemsetAsync(d_counts, 0, 16, s));
    ccd::LayerGroups lg{G, d_gdt, d_geta, d_ginner, d_gk, d_gcor, d_next, d_st_off, d_nvf, d_st,
                        d_gv_off, d_gv, d_co_off, d_co, d_heap, d_heap_size};
    for (;;) {
      ccd::LayerState ls{nverts, d_q, d_v, d_lu, d_minv, d_newq, d_newv, d_contrib, d_fired,
                         log_v, log_t, log_p, log_cap, d_counts, 1.0, d_status, d_counts + 1, d_step};
      CCD_CUDA(ccd::launch_layer_events(lg, ls, ctx->opt_layer_events, std::max<int64_t>(max_st, max_gv),
                                        ctx->opt_layer_grid_min, s));
      int status = 0;
      int64_t counts[2] = {0, 0};
      CCD_CUDA(cudaMemcpyAsync(&status, d_status, 4, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaMemcpyAsync(counts, d_counts, 16, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      if (status == 1) {
        st.events += counts[1];
        break;
      }
      if (counts[0] + (gv_off.back() + 1) > log_cap) {
        // the log is full: double it, keeping what it holds
        const int64_t ncap = 2 * log_cap;
        int32_t *nv_ = nullptr;
        double *nt = nullptr, *np = nullptr;
        rc = dev(&nv_, (size_t)ncap);
        if (!rc) rc = dev(&nt, (size_t)ncap);
        if (!rc) rc = dev(&np, 3 * (size_t)ncap);
        if (rc) return rc;
        CCD_CUDA(cudaMemcpyAsync(nv_, log_v, (size_t)counts[0] * 4, cudaMemcpyDeviceToDevice, s));
        CCD_CUDA(cudaMemcpyAsync(nt, log_t, (size_t)counts[0] * 8, cudaMemcpyDeviceToDevice, s));
        CCD_CUDA(cudaMemcpyAsync(np, log_p, (size_t)counts[0] * 24, cudaMemcpyDeviceToDevice, s));
        log_v = nv_, log_t = nt, log_p = np, log_cap = ncap;
      }
    }
    ccd::LayerState ls{nverts, d_q, d_v, d_lu, d_minv, d_newq, d_newv, d_contrib, d_fired,
                       log_v, log_t, log_p, log_cap, d_counts, 1.0, d_status, d_counts + 1, d_step};
    CCD_CUDA(ccd::launch_layer_finish(ls, s));
    int64_t nlog = 0;
    CCD_CUDA(cudaMemcpyAsync(&nlog, d_counts, 8, cudaMemcpyDeviceToHost, s));
    CCD_CUDA(cudaStreamSynchronize(s));
    // the nextstep values advanced on the device: the host's groups follow
    {
      std::vector<int> nx((size_t)G);
      std::vector<int> hp((size_t)G + 1);
      int hs = 0;
      if (G) CCD_CUDA(cudaMemcpyAsync(nx.data(), d_next, (size_t)G * 4, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaMemcpyAsync(&hs, d_heap_size, 4, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      if (hs) CCD_CUDA(cudaMemcpyAsync(hp.data(), d_heap, (size_t)hs * 4, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      for (int g = 0; g < G; g++) al.groups[(size_t)g].nextstep = nx[(size_t)g];
      al.heap.assign(hp.begin(), hp.begin() + hs);
      al.heap_size = hs;
    }
    // ---- the iteration's History
    const int64_t ne = 2 * (int64_t)nverts + nlog;
    rc = dev(&h_times, (size_t)ne);
    if (!rc) rc = dev(&h_pos, 3 * (size_t)ne);
    if (!rc) rc = dev(&keys, (size_t)std::max<int64_t>(nlog, 1));
    if (!rc) rc = dev(&keys_alt, (size_t)std::max<int64_t>(nlog, 1));
    if (rc) return rc;
    temp_bytes = std::max(ccd::radix_sort_temp_bytes(std::max<int64_t>(nlog, 1)), ccd::scan_temp_bytes(nverts));
    rc = dev((char **)&temp, temp_bytes);
    if (rc) return rc;
    const unsigned long long one = 0x3ff0000000000000ull;
    CCD_CUDA(cudaMemcpyAsync(d_gap, &one, 8, cudaMemcpyHostToDevice, s));
    CCD_CUDA(ccd::build_layer_history(nverts, d_q0, d_q, log_v, log_t, log_p, nlog, keys, keys_alt, temp, temp_bytes,
                                      d_count, d_scan, d_off, h_times, h_pos, d_gap, s));
    unsigned long long gap_bits = one;
    CCD_CUDA(cudaMemcpyAsync(&gap_bits, d_gap, 8, cudaMemcpyDeviceToHost, s));
    CCD_CUDA(cudaStreamSynchronize(s));
    double gap = 1.0;
    memcpy(&gap, &gap_bits, 8);
    st.history_entries = ne;
    rc = adopt_history(m, d_off, h_times, h_pos, ne, gap);
    if (rc) return rc;
    // ---- ActiveLayers::collisionDetection (:190-226)
    rc = run_broadphase(m, CCD_BROADPHASE_KDOP13, outer_eta);
    if (rc) return rc;
    const int64_t nc[2] = {m->n_cand[0], m->n_cand[1]};
    std::vector<int32_t> cand[2];
    std::vector<uint8_t> hit[2], stat[2];
    for (int kind = 0; kind < 2; kind++) {
      const int64_t n = nc[kind];
      cand[kind].resize(4 * (size_t)n);
      hit[kind].assign((size_t)n, 0);
      stat[kind].assign((size_t)n, 0);
      if (!n) continue;
      CCD_CUDA(cudaMemcpyAsync(cand[kind].data(), m->cand[kind], (size_t)n * 16, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      std::vector<double> eta((size_t)n);
      for (int64_t i = 0; i < n; i++) {
        const int32_t *c = cand[kind].data() + 4 * i;
        eta[(size_t)i] = al.thickness(kind, StencilKey{c[0], c[1], c[2], c[3]});
      }
      Lane &L = m->lane[0];
      rc = grow(ctx, &m->in_eta, &m->in_eta_cap, n);
      if (!rc) rc = grow(ctx, &L.hit, &L.hit_cap, 2 * n);
      if (rc) return rc;
      CCD_CUDA(cudaMemcpyAsync(m->in_eta, eta.data(), (size_t)n * 8, cudaMemcpyHostToDevice, s));
      const ccd::HistoryView hv2{m->hist_off, m->hist_time, m->hist_pos};
      CCD_CUDA(ccd::launch_separating_plane(kind, hv2, m->cand[kind], n, m->in_eta, 1, gap / 4.0, L.hit, L.hit + n,
                                            s));
      CCD_CUDA(cudaMemcpyAsync(hit[kind].data(), L.hit, (size_t)n, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaMemcpyAsync(stat[kind].data(), L.hit + n, (size_t)n, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      for (uint8_t x : stat[kind])
        if (x)
          return mesh_fail(m, CCD_ERR_INVALID_ARGUMENT,
                           "separating-plane search stalled (the reference's recursion does not end on this input)");
    }
    std::vector<StencilKey> found[2];
    for (int kind = 0; kind < 2; kind++)
      for (int64_t i = 0; i < nc[kind]; i++)
        if (hit[kind][(size_t)i]) {
          const int32_t *c = cand[kind].data() + 4 * i;
          found[kind].push_back(StencilKey{c[0], c[1], c[2], c[3]});
        }
    st.iterations = iter + 1;
    st.collisions += (int64_t)(found[0].size() + found[1].size());
    // ActiveLayers::runOneIteration (:244-255)
    al.rollback();
    for (int kind = 0; kind < 2; kind++)
      for (const StencilKey &x : found[kind]) al.add(kind, x);
    st.layers = al.deepest;
    if (found[0].empty() && found[1].empty()) {
      CCD_CUDA(cudaMemcpyAsync(qend, d_q, n3 * 8, cudaMemcpyDeviceToHost, s));
      CCD_CUDA(cudaStreamSynchronize(s));
      *result = iter;
      if (stats) *stats = st;
      return CCD_OK;
    }
  }
  *result = -3;  // MAXROLLBACKS_EXCEEDED
  if (stats) *stats = st;
  return CCD_OK;
}
