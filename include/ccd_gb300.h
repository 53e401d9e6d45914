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
   * as CCD_PATH_FP64 (the FP32 stage never rejects a row that hits). */
  CCD_PATH_CULL_REFINE = 1
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
 * receives per-row status bits (0 = ok). */
int ccd_prim_batch(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                   int64_t eta_count, uint8_t *hit, double *t);
int ccd_prim_batch_device(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                          int64_t eta_count, uint8_t *hit, double *t, uint8_t *status);

#ifdef __cplusplus
}
#endif
#endif /* CCD_GB300_H */
