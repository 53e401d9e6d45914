/* ccd_gb300 -- continuous-time collision detection on one GB300 GPU.
 *
 * C ABI in front of the CUDA kernels (libccd_gb300.so).  Plain pointers and
 * sizes only.  Every function returns a ccd_status code; a failing call
 * leaves a message retrievable with ccd_last_error().
 *
 * Point layout of one swept primitive ("row"): the points of the reference's
 * argument list, all start positions first, then all end positions, each as
 * x,y,z doubles:
 *   vertex-face   q0s q1s q2s q3s q0e q1e q2e q3e   (24 doubles; q0 = vertex)
 *   edge-edge     q0s p0s q1s p1s q0e p0e q1e p1e   (24 doubles; edges q0-p0, q1-p1)
 *   vertex-edge   q0s q1s q2s q0e q1e q2e           (18 doubles; q0 = vertex)
 *   vertex-vertex q1s q2s q1e q2e                   (12 doubles)
 * Results follow the reference: hit = 1 if the primitives come within eta
 * during t in [0,1]; t is written only where hit = 1 (the reference leaves
 * its output argument untouched on a miss).
 */
#ifndef CCD_GB300_H
#define CCD_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ccd_context ccd_context;

typedef enum {
  CCD_OK = 0,
  CCD_ERR_INVALID_ARGUMENT = 1,
  CCD_ERR_CUDA = 2,
  CCD_ERR_OUT_OF_MEMORY = 3,
  CCD_ERR_NO_DEVICE = 4
} ccd_status;

typedef enum {
  CCD_VERTEX_FACE = 0,
  CCD_EDGE_EDGE = 1,
  CCD_VERTEX_EDGE = 2,
  CCD_VERTEX_VERTEX = 3
} ccd_prim_kind;

/* Execution path of a primitive batch. */
typedef enum {
  /* FP64 evaluation of every row, op-for-op with the reference. */
  CCD_PATH_FP64 = 0,
  /* Outward-bounded FP32 rejection of rows whose result is provably "no
   * hit", then the FP64 evaluation of the surviving rows only.  Same results
   * as CCD_PATH_FP64 (the FP32 stage never rejects a row that hits).
   * Vertex-vertex rows (one quadratic) are always evaluated in FP64. */
  CCD_PATH_CULL_REFINE = 1,
  /* No FP32 stage: every row through the FP64 refinement that
   * CCD_PATH_CULL_REFINE applies to its survivors (batched root solvers for
   * vertex-face and edge-edge rows).  Same results; the all-FP64 baseline
   * that isolates what the FP32 stage saves. */
  CCD_PATH_REFINE_ALL = 2
} ccd_path;

/* Counters of the most recent batch call on a context. */
typedef struct {
  int64_t rows;          /* rows evaluated */
  int64_t survivors;     /* rows the FP32 stage passed on (== rows for CCD_PATH_FP64) */
  int64_t hits;          /* rows with hit = 1 */
  int64_t status_flags;  /* rows whose root bound hit its iteration cap (non-finite input) */
} ccd_batch_stats;

/* Device time of the kernels launched on a context while profiling is on,
 * measured with CUDA events on the launching stream and summed over all
 * batches (and chunks) since ccd_context_set_profiling last switched it on.
 * Device-entry-point batches are included once ccd_context_synchronize has
 * returned; host-memory batches on return. */
typedef struct {
  float cull_ms;    /* FP32 rejection kernel */
  float refine_ms;  /* FP64 kernel over the surviving rows (or over all rows) */
  int32_t launches; /* kernels launched */
} ccd_batch_timings;

/* ------------------------------------------------------------------ context */
/* Creates a context on CUDA device `device` (owns device buffers and a
 * stream).  Contexts are independent; one context is not thread-safe. */
int ccd_context_create(int device, ccd_context **out);
int ccd_context_destroy(ccd_context *ctx);
/* Use `stream` (a cudaStream_t, or NULL for the context's own stream) for the
 * *_device entry points. */
int ccd_context_set_stream(ccd_context *ctx, void *stream);
int ccd_context_synchronize(ccd_context *ctx);
const char *ccd_last_error(const ccd_context *ctx);
const char *ccd_status_string(int status);
int ccd_last_batch_stats(const ccd_context *ctx, ccd_batch_stats *out);
/* Turns per-kernel event timing on (1) or off (0, the default); either way
 * waits for queued work and resets the accumulated timings. */
int ccd_context_set_profiling(ccd_context *ctx, int on);
int ccd_last_batch_timings(ccd_context *ctx, ccd_batch_timings *out);
/* Tuning options of a context, for the autotuner (results never change):
 *   "wave_steps"     root-solver steps taken in lock-step over all queued
 *                    polynomials of a large batch before the unfinished ones
 *                    continue in the per-warp pool solver (0: the pool
 *                    solver only); default 48, at most 4096
 *   "wave_min_rows"  smallest batch (rows) that uses those lock-step steps;
 *                    default 262144
 *   "count_slab_tests" 1: the broad phase counts its traversal's slab tests
 *                    (ccd_mesh_stats.slab_tests; a slower variant); default 0
 *   "tree_refit"     1: a mesh keeps its broad-phase tree between calls and,
 *                    while its kind and faces are unchanged, only refits the
 *                    node slabs to the new positions, rebuilding it when the
 *                    summed surface of its nodes has grown past
 *                    "tree_rebuild_pct" percent of its value after the build
 *                    or after "tree_max_refits" refits in a row; 0: every
 *                    call builds a new tree; defaults 1, 130, 64
 *   "traversal"      broad-phase tree traversal: 0 one thread per query face
 *                    with its own stack, 1 one warp per 32 query faces
 *                    adjacent in Morton order sharing one stack and each
 *                    node's loads, 2 as 0 with a smaller register budget
 *                    (more threads resident per SM), 3 four lanes per query
 *                    face, each loading and testing a quarter of every
 *                    13-DOP record (AABB trees take 0), 4 as 3 with a
 *                    smaller register budget; default 3
 *   "pool_budget"    further steps the unfinished polynomials get, many per
 *                    warp, before the last ones are finished one per warp
 *                    (0: no limit); default 0
 *   "pool_slots"     pool solver of a batch the wavefront does not take:
 *                    solver slots per warp, 64 (five warps per SM) or 32
 *                    (ten warps per SM); default 64
 *   "pool_slots_min" pool solver: a warp fills its share of the queued
 *                    polynomials (the queue over the grid's warps), but at
 *                    least this many of its 64 slots; a small share spreads
 *                    a small batch over more warps; in [1, 64], default 4
 *                    (64: the first warps fill all their slots)
 *   "pool_all"       pool solver: once the queue is drained, a warp with at
 *                    most this many solves left advances all of them at
 *                    every iteration, whatever their phases, instead of the
 *                    most populated phase's; in [0, 32], default 0
 *   "pool_phase_sync" pool solver of a batch the wavefront does not take:
 *                    0, or k: a warp advances the solver
 *                    phase of the current 2^k-cycle window of its SM's clock
 *                    (the same for the SM's warps, so they run one phase's
 *                    code at once) when it holds at least half as many
 *                    solves as the most populated phase; in [0, 30],
 *                    default 16
 *   "warp_finish"    how a warp finishes a solve it holds alone (the last of
 *                    its pool, or the one-per-warp finish): 0 on one lane,
 *                    1 on all 32 lanes with independent operations spread
 *                    over them, 2 each lane trying one of the stage's
 *                    remaining shifts, the first that converges kept (the
 *                    same results as the sequential order); default 1
 *   "shift_after"    warp_finish 2: shifts of a stage tried one at a time
 *                    before the remaining ones run at once; in [0, 19],
 *                    default 2
 *   "chunk_rows"     ccd_prim_batch: largest chunk (rows) streamed through
 *                    the device, two in flight; a batch is cut into equal
 *                    chunks; in [1024, 2^26], default 2^23
 *   "narrow_chunk"   mesh narrow phase (two-entry steps): stencils per chunk
 *                    of rows gathered and refined together (each chunk pays
 *                    the tail of its slowest root solves once; the row
 *                    scratch is about 200 B per stencil); in [1024, 2^24],
 *                    default 2^24
 *   "layer_events_per_launch" ccd_velocity_filter: firings per launch of the
 *                    event loop (it pauses and continues); default 2^20
 *   "layer_grid_min" ccd_velocity_filter: when a penalty group holds this
 *                    many stencils or vertices, each firing runs over the
 *                    whole GPU instead of one block; default 1024
 * Unknown names and out-of-range values return CCD_ERR_INVALID_ARGUMENT. */
int ccd_context_set_option(ccd_context *ctx, const char *name, int64_t value);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int ccd_version(void);

/* ---------------------------------------------------------- single queries
 * Replace the reference's static CTCD calls (include/CTCD.h:36-79):
 *   CTCD::vertexFaceCTCD   -> ccd_vertex_face_ctcd
 *   CTCD::edgeEdgeCTCD     -> ccd_edge_edge_ctcd
 *   CTCD::vertexEdgeCTCD   -> ccd_vertex_edge_ctcd
 *   CTCD::vertexVertexCTCD -> ccd_vertex_vertex_ctcd
 * `points` is one row in the layout above.  *hit receives 0/1; *t is written
 * only on a hit.  Each call is a batch of one (latency-bound); use the batch
 * entry points for throughput. */
int ccd_vertex_face_ctcd(ccd_context *ctx, const double *points, double eta, int *hit, double *t);
int ccd_edge_edge_ctcd(ccd_context *ctx, const double *points, double eta, int *hit, double *t);
int ccd_vertex_edge_ctcd(ccd_context *ctx, const double *points, double eta, int *hit, double *t);
int ccd_vertex_vertex_ctcd(ccd_context *ctx, const double *points, double eta, int *hit, double *t);

/* ---------------------------------------------------------- batches
 * n rows of one primitive kind (ccd_prim_kind), same semantics as n calls of
 * the reference's CTCD::*CTCD.  eta holds eta_count values: 1 (shared) or n
 * (per row).  hit[n] receives 0/1, t[n] is written only where hit = 1.
 *
 * ccd_prim_batch: all pointers are host memory; blocks until done.  Rows are
 * streamed through the device in chunks with copies overlapped with compute.
 * ccd_prim_batch_device: all pointers are device memory; enqueued on the
 * context's stream and returns without waiting.  status (optional, n bytes)
 * receives per-row status bits (0 = ok).
 * Stream capture: once the context has run a device batch of at least n rows
 * (which sizes its scratch) and with profiling off, ccd_prim_batch_device
 * enqueues only kernels, memsets and copies, so a caller may capture it on
 * the context's stream into a CUDA graph and replay it.  The graph keeps the
 * pointers and sizes it was captured with, and the context's scratch: replays
 * on one context must not overlap other work of that context.  A call that
 * would grow the scratch during capture fails with CCD_ERR_CUDA (and the
 * capture is invalidated). */
int ccd_prim_batch(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                   int64_t eta_count, uint8_t *hit, double *t);
int ccd_prim_batch_device(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                          int64_t eta_count, uint8_t *hit, double *t, uint8_t *status);

/* ---------------------------------------------------------- FP32 stage alone
 * No counterpart in the reference.  The FP32 conservative rejection of
 * CCD_PATH_CULL_REFINE without the refinement: rows (device memory, n rows of
 * a vertex-face, edge-edge or vertex-edge kind) that provably do not hit get
 * hit[i] = 0; the indices of the others go to survivors[] (device, room for n,
 * in no particular order) and their count to *n_survivors (host).  Blocks
 * until the count is known.  For callers that schedule the FP64 work
 * themselves, and for measuring what the FP32 stage passes on. */
int ccd_prim_cull_device(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                         int64_t eta_count, uint8_t *hit, int32_t *survivors, int64_t *n_survivors);

/* ---------------------------------------------------------- FP64 peak
 * No counterpart in the reference.  Measures the context device's FP64
 * arithmetic throughput with a kernel of independent add / multiply chains
 * and one of fused multiply-adds over every SM, timed with CUDA events on
 * the context's stream (best of `reps`).  ops_per_s counts one operation per
 * DADD or DMUL (the library is built without FMA contraction, so each of its
 * FP64 additions and multiplications is one such instruction); fma_flops_per_s
 * counts two per DFMA.  div_per_s is the same measure for correctly rounded
 * FP64 divisions.  The latencies come from one warp running one dependent
 * chain of each operation, timed with the SM clock (cycles per operation).
 * Blocks until done. */
typedef struct {
  double ops_per_s;           /* FP64 add + multiply instructions per second (lanes) */
  double fma_flops_per_s;     /* 2 x FP64 fused multiply-adds per second (lanes) */
  double ms;                  /* duration of the best add / multiply run */
  int64_t ops;                /* operations of one add / multiply run */
  double div_per_s;           /* FP64 divisions per second (lanes) */
  double add_latency_cycles;  /* dependent FP64 addition */
  double mul_latency_cycles;  /* dependent FP64 multiplication */
  double div_latency_cycles;  /* dependent FP64 division */
} ccd_fp64_peak_result;
int ccd_fp64_peak(ccd_context *ctx, int reps, ccd_fp64_peak_result *out);

/* ---------------------------------------------------------- autotuner
 * No counterpart in the reference (its narrow phase is one scalar call per
 * stencil).  Chooses the work split of the FP64 refinement for batches like
 * the given one: how many lock-step wavefront steps every queued root solve
 * takes ("wave_steps"), how many further steps the pool kernel gives each
 * unfinished solve ("pool_budget"), how the solves left after that finish
 * ("warp_finish", "shift_after"), and the batch size from which the
 * wavefront runs at all ("wave_min_rows").  It runs `rows` (device memory, a
 * vertex-face or edge-edge batch of n rows, CCD_PATH_CULL_REFINE) once to
 * warm up and `reps` timed times under the context's own split, the pool
 * kernel alone, each of 18 wavefront splits, 6 wavefront splits whose
 * leftovers after a short pool budget finish one per warp with their stages'
 * remaining shifts tried at once, and the context's own split once
 * more, checks that every split's hits and contact times equal the first
 * split's bit for bit, and sets the fastest matching split as the context's
 * options.  Blocks until done;
 * allocates its own output buffers.  Results of later batches never change,
 * only their speed. */
typedef struct {
  int32_t wave_steps;    /* the context's options after the call */
  int32_t pool_budget;
  int64_t wave_min_rows;
  int32_t candidates;    /* splits timed */
  int32_t mismatches;    /* splits whose output differed (never chosen; 0 expected) */
  int32_t chosen;        /* index of the chosen split in the order timed (0: the context's own) */
  int32_t warp_finish;   /* the context's options after the call */
  double default_ms;     /* median time of the context's own split */
  double best_ms;        /* median time of the chosen split */
  int32_t shift_after;
  int32_t reserved;
} ccd_tune_result;
int ccd_autotune_prim_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                            int64_t eta_count, int reps, ccd_tune_result *out);

/* ---------------------------------------------------------- allocation-free batch
 * No counterpart in the reference.  The same results as
 * ccd_prim_batch_device with CCD_PATH_CULL_REFINE (no per-row status), for
 * callers that must not allocate device memory while they run: every byte of
 * scratch comes from one fixed region of about 9.4 MB per device, set aside
 * when the library's device code is loaded.  Needs no context; all pointers
 * are device memory; enqueued on `stream` (a cudaStream_t, NULL for the
 * legacy default stream) of the current device; returns without waiting.
 *   - n > CCD_NOALLOC_MAX_ROWS is rejected with CCD_ERR_INVALID_ARGUMENT
 *     before any work is enqueued (split larger batches into calls);
 *   - the first call on a device does its setup (scratch address, SM count)
 *     with that device current; make it before any stream capture that should
 *     contain later calls;
 *   - the region is shared by all calls on a device: calls whose device work
 *     can overlap in time (different streams, several host threads) race and
 *     corrupt each other's results, so keep them on one stream or serialise
 *     them. */
#define CCD_NOALLOC_MAX_ROWS 65536
int ccd_prim_batch_device_noalloc(int kind, int64_t n, const double *rows, const double *eta, int64_t eta_count,
                                  uint8_t *hit, double *t, void *stream);

/* ------------------------------------------------------------------ meshes
 * A triangle mesh resident on its context's device: the faces of the
 * reference's Mesh (src/Mesh.h: Matrix3Xi faces, 3 x F, column-major, which
 * is [F][3] int32 in memory) and one step of its History with two entries,
 * start (time 0) and end (time 1) (src/History.h; VectorXd positions,
 * [V][3] doubles, xyz per vertex).  Stencils are int32 [n][4]:
 *   vertex-face  p q0 q1 q2   (VertexFaceStencil, src/Stencils.h:7-81)
 *   edge-edge    p0 p1 q0 q1  (EdgeEdgeStencil,   src/Stencils.h:83-137)
 * Candidate lists come out canonical (q0 <= q1 <= q2; p0 <= p1, q0 <= q1,
 * p0 <= q0) and in the reference's std::set order.  A mesh uses its
 * context's stream and is not thread-safe; it must be destroyed before its
 * context. */
typedef struct ccd_mesh ccd_mesh;

typedef enum {
  CCD_BROADPHASE_KDOP13 = 0, /* KDOPBroadPhase (src/KDOPBroadPhase.cpp) */
  CCD_BROADPHASE_AABB = 1,   /* AABBBroadPhase (src/AABBBroadPhase.cpp) */
  /* TrivialBroadPhase (src/TrivialBroadPhase.cpp:4-53), the brute-force
   * verifier: every stencil of a vertex and a face without it and of two
   * edges without a common vertex (all-fixed ones excepted), whatever the
   * positions and padding.  O(V F + E^2) stencils: for small meshes; single
   * meshes only (not ccd_mesh_create_instances). */
  CCD_BROADPHASE_TRIVIAL = 2
} ccd_broadphase_kind;

/* Counters of the most recent broad/narrow phase call on a mesh. */
typedef struct {
  int64_t face_pairs; /* face pairs whose swept volumes overlap, neighbours excluded */
  int64_t n_vf;       /* vertex-face stencils tested (candidates) */
  int64_t n_ee;       /* edge-edge stencils tested (candidates) */
  int64_t vf_hits;    /* colliding vertex-face stencils */
  int64_t ee_hits;    /* colliding edge-edge stencils */
  int64_t slab_tests; /* traversal slab tests (leaf and node), or -1 unless counting is on */
  float broadphase_ms; /* device time of the broad phase, traversal_ms of its tree */
  float traversal_ms;  /* traversal (both 0 unless the context's profiling is on) */
  double self_distance_eta; /* ccd_mesh_self_distance: its broad phase's padding, the least
                               qualifying vertex distance (+inf if none); 0 otherwise */
  int32_t tree_built;       /* 1: the broad phase built its tree; 0: it refitted the kept one */
  int32_t tree_refits;      /* refit-only broad phases since the tree was last built */
  int32_t graph_replay;     /* 1: ccd_mesh_detect_graph replayed its captured step */
  int32_t reserved;
} ccd_mesh_stats;

/* faces: nfaces x 3 vertex indices in [0, nverts).  Topology is fixed for the
 * mesh's lifetime; positions change per step. */
int ccd_mesh_create(ccd_context *ctx, int32_t nverts, int32_t nfaces, const int32_t *faces, ccd_mesh **out);
/* A mesh made of independent instances (no counterpart in the reference: it
 * is many reference meshes, each with its own broad and narrow phase, run as
 * one).  Instance i owns vertices vertex_offsets[i] .. vertex_offsets[i+1] - 1
 * and faces face_offsets[i] .. face_offsets[i+1] - 1; faces hold global
 * vertex indices and may only use their own instance's vertices.  The broad
 * phase never pairs faces of different instances, so every result is the
 * concatenation, in instance order, of what each instance gives alone (with
 * its vertex indices shifted by its offset).  Positions are [V][3] for all
 * instances together. */
int ccd_mesh_create_instances(ccd_context *ctx, int32_t ninst, const int32_t *vertex_offsets,
                              const int32_t *face_offsets, const int32_t *faces, ccd_mesh **out);
int ccd_mesh_destroy(ccd_mesh *mesh);
/* Start and end positions of the step (History entries at t = 0 and 1), host
 * memory; blocks until copied. */
int ccd_mesh_set_positions(ccd_mesh *mesh, const double *qstart, const double *qend);
/* The same from device memory; enqueued on the context's stream. */
int ccd_mesh_set_positions_device(ccd_mesh *mesh, const double *qstart, const double *qend);
/* A History with any number of entries per vertex (src/History.h; what
 * History::getVertexHistory(v) holds for every v): vertex v's entries are
 * offsets[v] .. offsets[v+1]-1 of times[] and positions[] ([entries][3]), in
 * time order, normally from time 0 (History's constructor) to time 1
 * (finishHistory) with the entries addHistory put between.  offsets has
 * nverts + 1 values, offsets[0] = 0, at least one entry per vertex.  Until
 * the next ccd_mesh_set_positions it replaces the two-entry step: the broad
 * phases take their slabs over every entry (src/KDOPBroadPhase.cpp:60-70),
 * and the narrow phase runs its chain on every segment of each stencil's
 * stitched common history (History::stitchCommonHistory,
 * src/History.cpp:98-140); a stencil collides when one segment does, and
 * its t is that segment's.  Host memory; blocks until copied. */
int ccd_mesh_set_history(ccd_mesh *mesh, const int32_t *offsets, const double *times, const double *positions);
/* fixedVerts as nverts bytes (non-zero = fixed), or NULL for none. */
int ccd_mesh_set_fixed(ccd_mesh *mesh, const uint8_t *fixed);

/* BroadPhase::findCollisionCandidates (src/RetrospectiveDetection.h:13;
 * KDOPBroadPhase.cpp:34-40, AABBBroadPhase.cpp:9-15): every vertex-face and
 * edge-edge stencil of the non-neighbouring face pairs whose swept volumes,
 * padded by outer_eta, overlap, minus stencils whose four vertices are all
 * fixed.  Writes the counts; the stencils stay on the device. */
int ccd_broadphase(ccd_mesh *mesh, int kind, double outer_eta, int64_t *n_vf, int64_t *n_ee);
/* Copies the last broad phase's stencils to host arrays of [n_vf][4] and
 * [n_ee][4] int32 (either may be NULL). */
int ccd_broadphase_get(ccd_mesh *mesh, int32_t *vf, int32_t *ee);

/* NarrowPhase::findCollisions with CTCDNarrowPhase (src/CTCDNarrowPhase.cpp:
 * 9-135) over caller stencils in host memory: hit[i] = 1 if stencil i
 * collides during the step with its eta (eta arrays hold 1 shared value or one
 * per stencil), tested as vertex-face (or edge-edge), then its 3 (4)
 * vertex-edge, then its 3 (4) vertex-vertex sub-tests.  The reference returns
 * the set of colliding stencils; here the caller gets one flag per input.
 * Optional outputs (NULL to skip): t of the first sub-test that hits (written
 * only where hit = 1; a vertex-vertex t can be negative, as in the reference),
 * and which sub-test hit (0 primitive, 1 vertex-edge, 2 vertex-vertex, -1
 * miss).  path: ccd_path of the primitive tests. */
int ccd_narrowphase(ccd_mesh *mesh, int path, int64_t n_vf, const int32_t *vf, const double *vf_eta,
                    int64_t vf_eta_count, int64_t n_ee, const int32_t *ee, const double *ee_eta, int64_t ee_eta_count,
                    uint8_t *vf_hit, uint8_t *ee_hit, double *vf_t, double *ee_t, int8_t *vf_which,
                    int8_t *ee_which);

/* SeparatingPlaneNarrowPhase::findCollisions (src/SeparatingPlaneNarrowPhase.cpp:
 * 11-278), the narrow phase the reference's velocity filter uses, over caller
 * stencils in host memory, on the mesh's history (ccd_mesh_set_history, or
 * the two-entry step): hit[i] = 1 if stencil i collides, by the reference's
 * separating-plane interval search with eps = History::computeMinimumGap()/4
 * and the CTCD chain on its short intervals.  Bit-identical to the
 * reference where it terminates.  On some inputs the reference's recursion
 * never ends (an interval ending exactly at a history entry time stops
 * shrinking) and it overflows its stack; such a stencil is stopped here with
 * status 1 (optional [n] outputs, 0 otherwise) and hit 0. */
int ccd_narrowphase_separating_plane(ccd_mesh *mesh, int64_t n_vf, const int32_t *vf, const double *vf_eta,
                                     int64_t vf_eta_count, int64_t n_ee, const int32_t *ee, const double *ee_eta,
                                     int64_t ee_eta_count, uint8_t *vf_hit, uint8_t *ee_hit, uint8_t *vf_status,
                                     uint8_t *ee_status);

/* One detection step on the device, as the reference's callers chain it
 * (example/AlecTest.cpp:97-111): broad phase with outer_eta, then the narrow
 * phase over every candidate with eta.  Writes the numbers of colliding
 * stencils (optional); the collisions stay on the device for
 * ccd_mesh_get_collisions, the candidates for ccd_broadphase_get. */
int ccd_mesh_detect(ccd_mesh *mesh, int broadphase_kind, double outer_eta, double eta, int path, int64_t *vf_hits,
                    int64_t *ee_hits);
/* No counterpart in the reference (it has no device work to capture).  The
 * same step and results as ccd_mesh_detect, for a mesh stepped repeatedly
 * with the same kind, paddings and path: the first call runs the step
 * directly, then captures its refit-only form -- the broad phase on the
 * kept tree, the narrow-phase chains and the compaction, with no host
 * synchronisation in between -- into a CUDA graph on the context's stream,
 * with room for twice the candidates that step found; later calls
 * replay the graph (one launch and one synchronisation).  The candidate
 * lists of a replay are padded to their capacity with stencils of four
 * padding vertices kept after the mesh's own, which never hit.  When a
 * replay finds more pairs or stencils than the capture has room for, when
 * the kept tree needs a rebuild, or when the context's options or the
 * mesh's buffers changed, the call runs the step directly (and captures a
 * new graph).  Needs the context's "tree_refit" on, profiling and
 * "count_slab_tests" off, a two-entry step (no ccd_mesh_set_history) and a
 * k-DOP or AABB broad phase; otherwise it is ccd_mesh_detect. */
int ccd_mesh_detect_graph(ccd_mesh *mesh, int broadphase_kind, double outer_eta, double eta, int path,
                          int64_t *vf_hits, int64_t *ee_hits);
/* Colliding stencils of the last ccd_mesh_detect(_graph) in the reference's set
 * order with the t of their first hitting sub-test; any pointer may be NULL. */
int ccd_mesh_get_collisions(ccd_mesh *mesh, int32_t *vf, double *vf_t, int32_t *ee, double *ee_t);
int ccd_mesh_last_stats(const ccd_mesh *mesh, ccd_mesh_stats *out);

/* ------------------------------------------------------------------ distances
 * The static queries of the reference's Distance class (include/Distance.h),
 * in FP64 with the reference's operation order: results are bit-identical.
 * Rows are 12 doubles, the reference's argument points in order:
 *   vertex-face, vertex-plane  p q0 q1 q2
 *   edge-edge, line-line       p0 p1 q0 q1 */
typedef enum {
  CCD_DISTANCE_VERTEX_FACE = 0, /* Distance::vertexFaceDistance (include/Distance.h:31-113) */
  CCD_DISTANCE_EDGE_EDGE = 1    /* Distance::edgeEdgeDistance (include/Distance.h:117-170) */
} ccd_distance_kind;

typedef enum {
  CCD_DISTANCE_VERTEX_PLANE = 0, /* Distance::vertexPlaneDistanceLessThan (include/Distance.h:13-19) */
  CCD_DISTANCE_LINE_LINE = 1     /* Distance::lineLineDistanceLessThan (include/Distance.h:21-27) */
} ccd_distance_predicate;

/* Per row: vec [n][3] the returned vector (closest point of the face or
 * segment minus p, or the shortest vector between the segments; its norm is
 * the distance); bary the barycentric coordinates the reference writes
 * through its reference arguments, [n][3] (q0, q1, q2) for vertex-face,
 * [n][4] (p0, p1, q0, q1) for edge-edge, or NULL.  Host memory. */
int ccd_distance_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, double *vec, double *bary);
/* The same on device memory, enqueued on the context's stream. */
int ccd_distance_batch_device(ccd_context *ctx, int kind, int64_t n, const double *rows, double *vec, double *bary);
/* Per row: out[i] = 1 if the predicate holds for eta (eta_count 1 shared value
 * or n, one per row).  Host memory. */
int ccd_distance_less_than_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                                 int64_t eta_count, uint8_t *out);

/* Distance::meshSelfDistance (src/Distance.cpp:12-66) on this mesh's faces
 * and fixed flags (ccd_mesh_set_fixed) at positions verts ([nverts][3] host
 * memory, which become both the start and end positions of the mesh):
 *   1. d = the least distance between a vertex i and a vertex of a face that
 *      does not contain i;
 *   2. the AABB broad phase with outer_eta = d on the motionless step;
 *   3. *distance = the least norm of vertexFaceDistance / edgeEdgeDistance
 *      over its stencils (+inf when there are none).
 * n_vf / n_ee (optional) receive the numbers of stencils checked, which the
 * reference prints.  The candidates stay available to ccd_broadphase_get.
 * A mesh made of instances is measured as the one mesh they form together. */
int ccd_mesh_self_distance(ccd_mesh *mesh, const double *verts, double *distance, int64_t *n_vf, int64_t *n_ee);
/* The same for a mesh given by value, as the reference's static call takes
 * it: faces [nfaces][3], fixed nverts flags or NULL. */
int ccd_self_distance(ccd_context *ctx, int32_t nverts, const double *verts, int32_t nfaces, const int32_t *faces,
                      const uint8_t *fixed, double *distance);

/* ------------------------------------------------------------------ penalty forces
 * PenaltyGroup::addForce (src/PenaltyGroup.cpp:34-52) for one group, with
 * the potentials of VertexFacePenaltyPotential::addForce and
 * EdgeEdgePenaltyPotential::addForce (src/PenaltyPotential.cpp:7-64): each
 * stencil whose primitives are closer than outer_eta (and not closer than
 * inner_eta) pushes them apart with stiffness (times cor when they are
 * separating); F += dt * (sum of the group's forces).  Bit-identical to the
 * reference: each vertex's forces are summed in the reference's order (the
 * vertex-face stencils in the order given, then the edge-edge ones).
 *   q, v, F     [nverts][3] positions, velocities, forces (F in and out)
 *   vf, ee      [n][4] stencils in the group's order (canonicalised as the
 *               stencil constructors do); *_isnew the stencils' isnew flags
 *               (NULL: none new)
 *   *_fired     optional [n] outputs: 1 where the stencil's potential fired
 *   newused     optional: 1 if a new stencil fired (the return value of
 *               PenaltyGroup::addForce)
 * Host memory; blocks until done. */
int ccd_penalty_group_force(ccd_context *ctx, int32_t nverts, const double *q, const double *v, int64_t n_vf,
                            const int32_t *vf, const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee,
                            const uint8_t *ee_isnew, double outer_eta, double inner_eta, double stiffness, double cor,
                            double dt, double *F, uint8_t *vf_fired, uint8_t *ee_fired, int *newused);
/* The same on device memory (q, v, F, stencils, flags; the fired arrays are
 * required here), on the context's stream; returns once newused is known
 * (the force kernels may still run; ccd_context_synchronize waits).  A
 * stencil vertex out of range fails the call with CCD_ERR_INVALID_ARGUMENT
 * (F is then left untouched). */
int ccd_penalty_group_force_device(ccd_context *ctx, int32_t nverts, const double *q, const double *v, int64_t n_vf,
                                   const int32_t *vf, const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee,
                                   const uint8_t *ee_isnew, double outer_eta, double inner_eta, double stiffness,
                                   double cor, double dt, double *F, uint8_t *vf_fired, uint8_t *ee_fired,
                                   int *newused);

/* ------------------------------------------------------------------ velocity filter
 * VelocityFilter::velocityFilter (include/VelocityFilter.h:45-46,
 * src/VelocityFilter.cpp:15-87) with the active layers it runs
 * (src/ActiveLayers.cpp): penalty groups fired in the order of their event
 * queue, the k-DOP broad phase over each iteration's history and the
 * separating-plane narrow phase, until no collision is left.  The event loop
 * of an iteration runs on the device in one persistent block; results are
 * the reference's bit for bit.
 *   qstart, qend  [nverts][3]; qend is overwritten with the filtered end
 *                 positions when *result >= 0 (as the reference does)
 *   faces         [nfaces][3]; invmasses [nverts][3] inverse mass per DOF
 * *result receives the reference's return value: the number of outer
 * iterations (>= 0), or -1 (a vertex in no face), -2 (the start is closer
 * than inner_eta), -3 (max_rollbacks iterations were not enough).  A search
 * of the separating-plane phase that the reference cannot finish (see
 * ccd_narrowphase_separating_plane) fails the call with
 * CCD_ERR_INVALID_ARGUMENT.  The reference's defaults: base_stiffness 1e-4,
 * base_substep 1e-4, cor 0.1, max_rollbacks 1000. */
typedef struct {
  int32_t iterations;      /* outer iterations run */
  int32_t layers;          /* penalty layers at the end */
  int64_t events;          /* group firings, all iterations */
  int64_t collisions;      /* colliding stencils found, all iterations */
  int64_t history_entries; /* entries of the last iteration's history */
  double start_distance;   /* Distance::meshSelfDistance of the start */
} ccd_velocity_filter_stats;

int ccd_velocity_filter(ccd_context *ctx, int32_t nverts, const double *qstart, double *qend, int32_t nfaces,
                        const int32_t *faces, const double *invmasses, double outer_eta, double inner_eta,
                        double base_stiffness, double base_substep, double cor, int32_t max_rollbacks,
                        int32_t *result, ccd_velocity_filter_stats *stats);

/* ------------------------------------------------------------------ serving
 * No counterpart in the reference (its detection runs in the caller's
 * thread).  A server runs collision queries for many callers at once on one
 * device.  A request is a mesh and a sequence of positions, frames 0..steps;
 * step k is one ccd_mesh_detect between frames k and k+1, which is the
 * reference's broad phase followed by CTCDNarrowPhase.
 *
 * The server has `slots` worker threads, each with its own context and
 * streams.  Requests wait in submission order and are admitted while the sum
 * of their estimated device footprints stays within memory_budget bytes. A
 * request larger than the whole budget runs alone.  An admitted request keeps
 * its mesh, positions and detection buffers resident for all of its steps.
 * Requests on different slots overlap on the device.  Results do not depend
 * on what else is running. */
typedef struct ccd_server ccd_server;

typedef struct {
  int32_t nverts, nfaces;
  const int32_t *faces;    /* [nfaces][3]; copied at submit */
  int32_t steps;           /* >= 1 */
  const double *frames;    /* [steps + 1][nverts][3] host memory, read until the request completes */
  const uint8_t *fixed;    /* nverts flags or NULL; copied at submit */
  int32_t broadphase_kind; /* ccd_broadphase_kind */
  int32_t path;            /* ccd_path of the primitive tests */
  double outer_eta, eta;   /* broad-phase padding, narrow-phase eta */
} ccd_request;

/* Results of a finished request; the arrays stay valid until
 * ccd_server_release. Step k's colliding stencils are rows
 * vf_offsets[k] .. vf_offsets[k + 1] of vf (and likewise ee), in set order,
 * with the t of their first hitting sub-test. */
typedef struct {
  int32_t status; /* ccd_status of the request */
  int32_t steps;  /* steps run */
  const int64_t *vf_hits, *ee_hits;       /* [steps] */
  const int64_t *vf_offsets, *ee_offsets; /* [steps + 1] */
  const int32_t *vf, *ee;                 /* [total][4] */
  const double *vf_t, *ee_t;              /* [total] */
  const double *step_ms;                  /* [steps] wall time of each step */
  double queue_ms;                        /* submit -> admitted */
  double total_ms;                        /* submit -> finished */
  const char *error;                      /* message when status != CCD_OK */
} ccd_request_result;

int ccd_server_create(int device, int slots, int64_t memory_budget, ccd_server **out);
/* Finishes the queued and running requests, then frees the server. */
int ccd_server_destroy(ccd_server *server);
int ccd_server_submit(ccd_server *server, const ccd_request *request, uint64_t *ticket);
/* *done = 1 once the request has finished. */
int ccd_server_poll(ccd_server *server, uint64_t ticket, int *done);
/* Blocks until the request has finished and describes its results. */
int ccd_server_wait(ccd_server *server, uint64_t ticket, ccd_request_result *out);
int ccd_server_release(ccd_server *server, uint64_t ticket);

#ifdef __cplusplus
}
#endif
#endif /* CCD_GB300_H */
