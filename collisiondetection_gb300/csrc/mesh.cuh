// Mesh-level pieces: static topology ranks (host) and the CTCD narrow phase
// over stencils (CTCDNarrowPhase::findCollisions, src/CTCDNarrowPhase.cpp:9-135).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace ccd {

// Ranks of a mesh's faces and edges in lexicographic order (computed once per
// mesh).  face_rank: rank of each face's ascending vertex triple (equal
// triples share a rank); face_edges: rank of edge (v_i, v_{i+1 mod 3}) among
// the ascending undirected edges.  Returns false on an out-of-range index.
struct HostTopology {
  std::vector<int32_t> face_rank, rank_triple, face_edges, rank_edge;
};
bool build_topology(int32_t nverts, int32_t nfaces, const int32_t *faces, HostTopology &out);

// Rows of the narrow-phase chain for `n` stencils (device arrays).
//   prim : VF or EE rows            [n][24]
//   ve   : vertex-edge rows         [n][3 or 4][18]
//   vv   : vertex-vertex rows       [n][3 or 4][12]
//   eta_* : per-row eta
// Start points follow History::stitchCommonHistory on a two-entry history:
// (1*start + 0*end)/1 (src/History.cpp:133); end points are the end positions.
// Stencils are canonicalised first (src/Stencils.h), as the reference's
// constructors do.
cudaError_t gather_stencil_rows(int kind, const int32_t *stencils, int64_t n, const double *qs, const double *qe,
                                const double *eta, int eta_per_row, double *prim, double *ve, double *vv,
                                double *eta_prim, double *eta_ve, double *eta_vv, cudaStream_t s);

// A multi-entry History: vertex v's entries are off[v] .. off[v+1]-1 of times
// and pos ([entries][3]).  The narrow phase runs its chain on every segment of
// each stencil's stitched common history (History::stitchCommonHistory,
// src/History.cpp:98-140; CTCDNarrowPhase.cpp:24-72, 74-135):
//   history_segment_counts: count[i] = segments of stencil i;
//   gather_history_rows: the chain rows of stencils [0, n), stencil i's
//     segments at rows seg_off[i] - base .. seg_off[i+1] - base - 1;
//   reduce_history_segments: per stencil, the first segment whose chain hits
//     (hit, t, which as combine_chain gives them per segment).
cudaError_t history_segment_counts(int kind, const int32_t *stencils, int64_t n, const int32_t *off,
                                   const double *times, const double *pos, uint32_t *count, cudaStream_t s);
cudaError_t gather_history_rows(int kind, const int32_t *stencils, int64_t n, const uint32_t *seg_off,
                                uint32_t base, const int32_t *off, const double *times, const double *pos,
                                const double *eta, int eta_per_row, double *prim, double *ve, double *vv,
                                double *eta_prim, double *eta_ve, double *eta_vv, cudaStream_t s);
cudaError_t reduce_history_segments(int64_t n, const uint32_t *seg_off, uint32_t base, const uint8_t *seg_hit,
                                    const double *seg_t, const int8_t *seg_which, uint8_t *hit, double *t,
                                    int8_t *which, cudaStream_t s);

// First hit along the reference's chain: primitive, then the vertex-edge
// tests, then the vertex-vertex tests (src/CTCDNarrowPhase.cpp:43-69, 92-129).
// which: 0 primitive, 1 vertex-edge, 2 vertex-vertex, -1 miss.
cudaError_t combine_chain(int kind, int64_t n, const uint8_t *h_prim, const double *t_prim, const uint8_t *h_ve,
                          const double *t_ve, const uint8_t *h_vv, const double *t_vv, uint8_t *hit, double *t,
                          int8_t *which, cudaStream_t s);

// Colliding stencils in input order: for the k-th i with hit[i] != 0,
// out[k] = stencils[i] and out_t[k] = t[i].  flags / pos hold n entries,
// temp scan_temp_bytes(n) bytes; *count (device) receives the number.
cudaError_t compact_hits(const int32_t *stencils, const uint8_t *hit, const double *t, int64_t n, uint32_t *flags,
                         uint32_t *pos, uint32_t *count, void *temp, size_t temp_bytes, int32_t *out, double *out_t,
                         cudaStream_t s);

}  // namespace ccd
