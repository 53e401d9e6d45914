// The active layers' event loop on the device (velocity.cu): the inner loop of
// ActiveLayers::runOneIteration (src/ActiveLayers.cpp:91-156, 228-256).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

// The penalty groups of one iteration, flattened (device pointers).  Group g
// holds stencils st_off[g] .. st_off[g+1]-1 of st ([S][4], canonical; the
// first n_vf[g] are vertex-face, in the group's insertion order, then the
// edge-edge ones), its vertex set gv_off[g] .. gv_off[g+1]-1 of gv (ascending,
// PenaltyGroup::getGroupStencil), and for each of those vertex slots j the
// contributions co_off[j] .. co_off[j+1]-1 of co (stencil index within the
// group << 2 | slot), in the order the reference adds them.
struct LayerGroups {
  int ngroups;
  const double *dt, *eta, *inner, *stiffness, *cor;
  int *nextstep;
  const int64_t *st_off;
  const int32_t *n_vf;
  const int32_t *st;
  const int64_t *gv_off;
  const int32_t *gv;
  const int64_t *co_off;
  const int32_t *co;
  int *heap;       // the event queue (priority_queue layout, ccd_heap.h)
  int *heap_size;
};

// Where the grid-wide loop's leader publishes each firing (global memory).
struct GridStep {
  int action, group;
  double time;
};

// The simulation state and the history log.  The loop appends one entry
// (vertex, time, position) per touched vertex per event, in event order and
// ascending vertex order within an event (ActiveLayers::step's
// history_->addHistory).
struct LayerState {
  int nverts;
  double *q, *v, *lu;  // positions, velocities, last update times [3 nv]
  const double *minv;  // inverse masses per DOF [3 nv]
  double *newq, *newv; // scratch [3 nv]
  double *contrib;     // scratch [max group stencils][12]
  uint8_t *fired;      // scratch [max group stencils]
  int32_t *log_v;
  double *log_t, *log_p;
  int64_t log_cap;
  int64_t *log_n;
  double term;         // termination time (1.0)
  int *status;         // out: 1 finished, 2 paused (log full or event budget used)
  int64_t *events;     // events processed, accumulated
  GridStep *grid_step; // scratch of the grid-wide loop
};

// Runs events until the queue's next firing time reaches the termination
// time (status 1) or max_events events or the log's capacity stop it
// (status 2; call again to continue).  When the largest group holds
// grid_min or more stencils or vertices, the firings run over the whole GPU
// (a cooperative launch sized so that every block is resident); otherwise in
// one block.
// max_group: the largest group's stencil or vertex count.
cudaError_t launch_layer_events(const LayerGroups &g, const LayerState &s, int64_t max_events, int64_t max_group,
                                int64_t grid_min, cudaStream_t st);

// The final step (src/ActiveLayers.cpp:145-152): every coordinate advances to
// the termination time.
cudaError_t launch_layer_finish(const LayerState &s, cudaStream_t st);

// The iteration's History (History(q0), the logged entries, finishHistory at
// time 1.0) as offsets / times / positions: vertex v's entries are off[v] ..
// off[v+1]-1.  keys / keys_alt / temp: radix-sort scratch for n_log keys;
// count / scan / off: [nv + 1].  *min_gap receives History::computeMinimumGap (as a
// non-negative double's bits; the caller sets it to the bits of 1.0).
cudaError_t build_layer_history(int nverts, const double *q0, const double *qend, const int32_t *log_v,
                                const double *log_t, const double *log_p, int64_t n_log, uint64_t *keys,
                                uint64_t *keys_alt, void *temp, size_t temp_bytes, uint32_t *count, uint32_t *scan,
                                int32_t *off, double *times, double *pos, unsigned long long *min_gap,
                                cudaStream_t st);

}  // namespace ccd
