// The active layers' event loop on the device (velocity.cuh).
//
// ActiveLayers::step (src/ActiveLayers.cpp:91-156) fires one penalty group at
// a time, in the order of a priority queue keyed by the groups' next firing
// times; each firing moves the group's vertices to the firing time, applies
// the group's penalty impulses and logs the touched vertices' positions.
// Firings depend on one another through shared vertices, so they run in
// sequence -- here inside one persistent block, so that no firing costs a
// kernel launch: thread 0 keeps the queue (ccd_heap.h, the library heap's
// exact order), and the block's threads share each firing's vertices and
// stencils, with a barrier between the phases of a firing.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include <cooperative_groups.h>

#include "ccd_heap.h"
#include "penalty.cuh"
#include "radix_sort.cuh"
#include "velocity.cuh"

namespace ccd {

namespace {

// Groups whose queue state (heap, firing steps, time steps) fits in shared
// memory keep it there: every firing reads it several times on the loop's
// critical path.
constexpr int kSharedGroups = 4096;

// PenaltyGroupComparator (src/ActiveLayers.cpp:18-21): a ranks below b when
// b fires first; PenaltyGroup::nextFireTime is nextstep * dt.  With the queue
// in shared memory, each group's firing time is kept there too (key,
// recomputed by the same product whenever its step changes), so that a
// comparison on the loop's critical path is two loads and one FP64 compare
// instead of two conversions and two products.
struct FireLater {
  const int *nextstep;
  const double *dt;
  const double *key;  // null: computed from nextstep and dt
  __device__ bool operator()(int a, int b) const {
    if (key) return key[b] < key[a];
    return (double)nextstep[b] * dt[b] < (double)nextstep[a] * dt[a];
  }
};

__device__ __forceinline__ double fire_time(const int *nextstep, const double *dt, int grp) {
  return (double)nextstep[grp] * dt[grp];
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) layer_events(LayerGroups g, LayerState s, int64_t max_events) {
  constexpr int kWarps = THREADS / 32;
  extern __shared__ double smem[];
  __shared__ int sh_group, sh_action, sh_heap_size;
  __shared__ double sh_time;
  __shared__ int64_t sh_base;
  __shared__ int sh_warp[kWarps + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const bool in_shared = g.ngroups <= kSharedGroups;
  double *dt_q = in_shared ? smem : nullptr;
  double *key_q = in_shared ? smem + g.ngroups : nullptr;
  int *next_q = in_shared ? reinterpret_cast<int *>(smem + 2 * g.ngroups) : g.nextstep;
  int *heap = in_shared ? next_q + g.ngroups : g.heap;
  if (in_shared) {
    for (int i = tid; i < g.ngroups; i += THREADS) {
      dt_q[i] = g.dt[i];
      next_q[i] = g.nextstep[i];
      key_q[i] = fire_time(g.nextstep, g.dt, i);
    }
    for (int i = tid; i < *g.heap_size; i += THREADS) heap[i] = g.heap[i];
  } else {
    dt_q = const_cast<double *>(g.dt);
  }
  if (tid == 0) {
    sh_heap_size = *g.heap_size;
    sh_base = *s.log_n;
  }
  __syncthreads();
  const FireLater later{next_q, dt_q, key_q};
  int action = 0;
  int64_t done = 0;
  for (int64_t ev = 0;; ev++) {
    if (tid == 0) {
      int a = 0, grp = -1;
      double t = 0.0;
      if (sh_heap_size == 0) {
        a = 1;
      } else {
        grp = heap[0];
        t = key_q ? key_q[grp] : fire_time(next_q, dt_q, grp);
        if (!(t < s.term)) {
          a = 1;
        } else if (ev >= max_events || sh_base + (g.gv_off[grp + 1] - g.gv_off[grp]) > s.log_cap) {
          a = 2;
        } else {
          heap_pop(heap, &sh_heap_size, later);
        }
      }
      sh_action = a;
      sh_group = grp;
      sh_time = t;
    }
    __syncthreads();
    action = sh_action;
    if (action) break;
    const int grp = sh_group;
    const double t = sh_time;
    const int64_t v0 = g.gv_off[grp], v1 = g.gv_off[grp + 1];
    const int64_t s0 = g.st_off[grp], s1 = g.st_off[grp + 1];
    const int nvf = g.n_vf[grp];
    // (1) the group's vertices at the firing time (src/ActiveLayers.cpp:105-114)
    for (int64_t j = v0 + tid; j < v1; j += THREADS) {
      const int vert = g.gv[j];
      for (int c = 0; c < 3; c++) {
        const int64_t i = 3 * (int64_t)vert + c;
        const double dt = t - s.lu[i];
        const double nq = s.q[i] + (t - s.lu[i]) * s.v[i];
        s.newq[i] = nq;
        s.newv[i] = (nq - s.q[i]) / dt;
      }
    }
    __syncthreads();
    // (2) each stencil's potential (PenaltyGroup::addForce, src/PenaltyGroup.cpp:34-52)
    const PenaltyParams pp{g.eta[grp], g.inner[grp], g.stiffness[grp], g.cor[grp]};
    for (int64_t k = s0 + tid; k < s1; k += THREADS) {
      const int64_t local = k - s0;
      const int v4[4] = {g.st[4 * k], g.st[4 * k + 1], g.st[4 * k + 2], g.st[4 * k + 3]};
      v3d c[4];
      const bool f = local < nvf ? stencil_force<0>(s.newq, s.newv, v4, pp, c)
                                 : stencil_force<1>(s.newq, s.newv, v4, pp, c);
      s.fired[local] = f ? 1 : 0;
      if (f) {
        double *out = s.contrib + 12 * local;
        for (int q = 0; q < 4; q++) {
          out[3 * q] = c[q].x;
          out[3 * q + 1] = c[q].y;
          out[3 * q + 2] = c[q].z;
        }
      }
    }
    __syncthreads();
    // (3) per vertex: the group force summed in the reference's order, F =
    // 0 + group * dt, the impulse on touched vertices, and their history
    // entries in ascending vertex order (src/ActiveLayers.cpp:116-139)
    const double gdt = dt_q[grp];
    for (int64_t tile = v0; tile < v1; tile += THREADS) {
      const int64_t j = tile + tid;
      bool touched = false;
      int vert = 0;
      if (j < v1) {
        vert = g.gv[j];
        double acc[3] = {0.0, 0.0, 0.0};
        for (int64_t e = g.co_off[j]; e < g.co_off[j + 1]; e++) {
          const int code = g.co[e];
          const int local = code >> 2, slot = code & 3;
          if (!s.fired[local]) continue;
          const double *cv = s.contrib + 12 * (int64_t)local + 3 * slot;
          const bool minus = local < nvf ? slot == 0 : slot <= 1;
          for (int c = 0; c < 3; c++) acc[c] = minus ? acc[c] - cv[c] : acc[c] + cv[c];
        }
        double F[3];
        for (int c = 0; c < 3; c++) F[c] = 0.0 + acc[c] * gdt;
        touched = F[0] != 0.0 || F[1] != 0.0 || F[2] != 0.0;
        if (touched) {
          for (int c = 0; c < 3; c++) {
            const int64_t i = 3 * (int64_t)vert + c;
            s.v[i] = s.v[i] + s.minv[i] * F[c];
            s.q[i] = s.newq[i];
            s.lu[i] = t;
          }
        }
      }
      // exclusive block scan of the touched flags: ballots within warps,
      // then the warps' counts
      const unsigned ballot = __ballot_sync(0xffffffffu, touched);
      if (lane == 0) sh_warp[warp] = __popc(ballot);
      __syncthreads();
      if (tid == 0) {
        int acc = 0;
        for (int w = 0; w < kWarps; w++) {
          const int c = sh_warp[w];
          sh_warp[w] = acc;
          acc += c;
        }
        sh_warp[kWarps] = acc;
      }
      __syncthreads();
      if (touched) {
        const int64_t at = sh_base + sh_warp[warp] + __popc(ballot & ((1u << lane) - 1));
        s.log_v[at] = vert;
        s.log_t[at] = t;
        for (int c = 0; c < 3; c++) s.log_p[3 * at + c] = s.q[3 * (int64_t)vert + c];
      }
      __syncthreads();
      if (tid == 0) sh_base += sh_warp[kWarps];
    }
    if (tid == 0) {
      next_q[grp] += 1;  // PenaltyGroup::incrementTimeStep
      if (key_q) key_q[grp] = fire_time(next_q, dt_q, grp);
      heap_push(heap, &sh_heap_size, grp, later);
    }
    done++;
    __syncthreads();
  }
  // the queue's state back to global memory for the next launch and the host
  if (in_shared) {
    for (int i = tid; i < g.ngroups; i += THREADS) g.nextstep[i] = next_q[i];
    for (int i = tid; i < sh_heap_size; i += THREADS) g.heap[i] = heap[i];
  }
  if (tid == 0) {
    *g.heap_size = sh_heap_size;
    *s.log_n = sh_base;
    *s.events += done;
    *s.status = action;
  }
}

// Large groups: one firing spread over the whole GPU.  The block version
// above is bound by a single SM's FP64 rate (1/64 of its FP32 rate on this
// part) once a group holds thousands of stencils; here every SM takes a share
// of each phase, with a grid-wide barrier between phases (a cooperative
// launch, every block resident).  Block 0 keeps the queue.  Data that other
// SMs rewrite between barriers is read through L2 (__ldcg).  History entries
// are appended through an atomic counter: within one firing a vertex appears
// at most once, so each vertex's entries stay in firing order, which is all
// the history needs.
constexpr int kGridThreads = 256;

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }

// A vertex coordinate at the firing time t (src/ActiveLayers.cpp:109-112):
// newq = q + (t - lu) * v, newv = (newq - q) / (t - lu).  Every use below
// recomputes it from the same three loads, so the values are the same
// wherever they are needed.
struct Advance {
  const double *q, *v, *lu;
  double t;
  __device__ __forceinline__ double pos(int64_t i) const {
    const double lu_i = __ldcg(lu + i);
    return __ldcg(q + i) + (t - lu_i) * __ldcg(v + i);
  }
  __device__ __forceinline__ double vel(int64_t i) const {
    const double q_i = __ldcg(q + i), lu_i = __ldcg(lu + i);
    const double dt = t - lu_i;
    const double nq = q_i + (t - lu_i) * __ldcg(v + i);
    return (nq - q_i) / dt;
  }
  __device__ __forceinline__ v3d pos3(int vert) const {
    const int64_t i = 3 * (int64_t)vert;
    return v3d{pos(i), pos(i + 1), pos(i + 2)};
  }
  __device__ __forceinline__ v3d vel3(int vert) const {
    const int64_t i = 3 * (int64_t)vert;
    return v3d{vel(i), vel(i + 1), vel(i + 2)};
  }
};

// The group force of one vertex slot j, its contributions accumulated in
// order; the loads of eight contributions are issued before their additions.
__device__ __forceinline__ void ordered_sum(const LayerGroups &g, const LayerState &s, int64_t j, int nvf,
                                            double (&acc)[3]) {
  const int64_t e0 = g.co_off[j], e1 = g.co_off[j + 1];
  for (int64_t e = e0; e < e1; e += 8) {
    int code[8];
    uint8_t fired[8];
    double cv[8][3];
#pragma unroll
    for (int u = 0; u < 8; u++) code[u] = e + u < e1 ? g.co[e + u] : 0;
#pragma unroll
    for (int u = 0; u < 8; u++) fired[u] = e + u < e1 ? __ldcg(s.fired + (code[u] >> 2)) : 0;
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const double *p = s.contrib + 12 * (int64_t)(code[u] >> 2) + 3 * (code[u] & 3);
      for (int c = 0; c < 3; c++) cv[u][c] = fired[u] ? __ldcg(p + c) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (!fired[u]) continue;
      const int local = code[u] >> 2, slot = code[u] & 3;
      const bool minus = local < nvf ? slot == 0 : slot <= 1;
      for (int c = 0; c < 3; c++) acc[c] = minus ? acc[c] - cv[u][c] : acc[c] + cv[u][c];
    }
  }
}

__global__ void __launch_bounds__(kGridThreads) layer_events_grid(LayerGroups g, LayerState s, int64_t max_events,
                                                                 GridStep *step) {
  namespace cg = cooperative_groups;
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double smem[];
  __shared__ int sh_heap_size;
  const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const bool in_shared = g.ngroups <= kSharedGroups;
  double *dt_q = in_shared ? smem : const_cast<double *>(g.dt);
  double *key_q = in_shared ? smem + g.ngroups : nullptr;
  int *next_q = in_shared ? reinterpret_cast<int *>(smem + 2 * g.ngroups) : g.nextstep;
  int *heap = in_shared ? next_q + g.ngroups : g.heap;
  if (blockIdx.x == 0) {
    if (in_shared) {
      for (int i = threadIdx.x; i < g.ngroups; i += blockDim.x) {
        dt_q[i] = g.dt[i];
        next_q[i] = g.nextstep[i];
        key_q[i] = fire_time(g.nextstep, g.dt, i);
      }
      for (int i = threadIdx.x; i < *g.heap_size; i += blockDim.x) heap[i] = g.heap[i];
    }
    if (threadIdx.x == 0) sh_heap_size = *g.heap_size;
    __syncthreads();
  }
  const FireLater later{next_q, dt_q, key_q};
  // The leader decides the next firing: pops it from the queue, or stops
  // (1: the next firing time reaches the end; 2: the event budget or the
  // log's room, counting `pending` entries not yet appended, is used up).
  auto decide = [&](int64_t ev, int64_t pending) {
    int a = 0, grp = -1;
    double t = 0.0;
    if (sh_heap_size == 0) {
      a = 1;
    } else {
      grp = heap[0];
      t = key_q ? key_q[grp] : fire_time(next_q, dt_q, grp);
      if (!(t < s.term)) {
        a = 1;
      } else if (ev >= max_events || (int64_t)__ldcg((const long long *)s.log_n) + pending +
                                             (g.gv_off[grp + 1] - g.gv_off[grp]) > s.log_cap) {
        a = 2;
      } else {
        heap_pop(heap, &sh_heap_size, later);
      }
    }
    step->action = a;
    step->group = grp;
    step->time = t;
  };
  if (leader) decide(0, 0);
  grid.sync();
  int64_t done = 0;
  int action = 0;
  for (int64_t ev = 0;; ev++) {
    action = __ldcg(&step->action);
    if (action) break;
    const int grp = __ldcg(&step->group);
    const double t = __ldcg(&step->time);
    const int64_t v0 = g.gv_off[grp], v1 = g.gv_off[grp + 1];
    const int64_t s0 = g.st_off[grp], s1 = g.st_off[grp + 1];
    const int nvf = g.n_vf[grp];
    // (1, 2) each stencil's potential, its vertices advanced to the firing
    // time on the fly (no barrier between moving the vertices and using them)
    const Advance adv{s.q, s.v, s.lu, t};
    const PenaltyParams pp{g.eta[grp], g.inner[grp], g.stiffness[grp], g.cor[grp]};
    for (int64_t k = s0 + gtid; k < s1; k += gsize) {
      const int64_t local = k - s0;
      const int v4[4] = {g.st[4 * k], g.st[4 * k + 1], g.st[4 * k + 2], g.st[4 * k + 3]};
      const v3d x[4] = {adv.pos3(v4[0]), adv.pos3(v4[1]), adv.pos3(v4[2]), adv.pos3(v4[3])};
      const auto vel = [&](int kk) { return adv.vel3(v4[kk]); };
      v3d c[4];
      const bool f = local < nvf ? stencil_force_at<0>(x, vel, pp, c) : stencil_force_at<1>(x, vel, pp, c);
      s.fired[local] = f ? 1 : 0;
      if (f) {
        double *out = s.contrib + 12 * local;
        for (int q = 0; q < 4; q++) {
          out[3 * q] = c[q].x;
          out[3 * q + 1] = c[q].y;
          out[3 * q + 2] = c[q].z;
        }
      }
    }
    grid.sync();
    // the queue moves on while the vertices are summed: this group's next
    // firing goes back in, the next firing comes out (the queue holds only
    // firing times, which phase (3) does not touch)
    if (leader) {
      next_q[grp] += 1;  // PenaltyGroup::incrementTimeStep
      if (key_q) key_q[grp] = fire_time(next_q, dt_q, grp);
      heap_push(heap, &sh_heap_size, grp, later);
      decide(ev + 1, v1 - v0);
    }
    // (3) per vertex: the ordered group force, the impulse, the history entry
    const double gdt = g.dt[grp];  // every block: only block 0's shared memory holds the queue's copy
    for (int64_t base = v0; base < v1; base += gsize) {
      const int64_t j = base + gtid;
      bool touched = false;
      int vert = 0;
      if (j < v1) {
        vert = g.gv[j];
        double acc[3] = {0.0, 0.0, 0.0};
        ordered_sum(g, s, j, nvf, acc);
        double F[3];
        for (int c = 0; c < 3; c++) F[c] = 0.0 + acc[c] * gdt;
        touched = F[0] != 0.0 || F[1] != 0.0 || F[2] != 0.0;
        if (touched) {
          for (int c = 0; c < 3; c++) {
            const int64_t i = 3 * (int64_t)vert + c;
            const double nq = adv.pos(i);
            s.v[i] = ldcg(s.v + i) + s.minv[i] * F[c];
            s.q[i] = nq;
            s.lu[i] = t;
          }
        }
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, touched);
      unsigned long long first = 0;
      if (ballot) {
        const int lead = __ffs(ballot) - 1;
        if (lane == lead) first = atomicAdd((unsigned long long *)s.log_n, (unsigned long long)__popc(ballot));
        first = __shfl_sync(0xffffffffu, first, lead);
      }
      if (touched) {
        const int64_t at = (int64_t)first + __popc(ballot & ((1u << lane) - 1));
        s.log_v[at] = vert;
        s.log_t[at] = t;
        for (int c = 0; c < 3; c++) s.log_p[3 * at + c] = s.q[3 * (int64_t)vert + c];
      }
    }
    done++;
    grid.sync();
  }
  if (blockIdx.x == 0) {
    if (in_shared) {
      for (int i = threadIdx.x; i < g.ngroups; i += blockDim.x) g.nextstep[i] = next_q[i];
      for (int i = threadIdx.x; i < sh_heap_size; i += blockDim.x) g.heap[i] = heap[i];
    }
    if (threadIdx.x == 0) {
      *g.heap_size = sh_heap_size;
      *s.events += done;
      *s.status = action;
    }
  }
}

__global__ void __launch_bounds__(256) layer_finish(int64_t n3, double *q, const double *v, double *lu, double term) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n3) return;
  q[i] += (term - lu[i]) * v[i];
  lu[i] = term;
}

__global__ void __launch_bounds__(256) count_log(const int32_t *log_v, int64_t n, uint32_t *count, uint64_t *keys) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  atomicAdd(&count[log_v[i]], 1u);
  keys[i] = ((uint64_t)(uint32_t)log_v[i] << 32) | (uint64_t)i;
}

// Vertex v's entries: History's first (time 0, q0), its logged entries in
// log order, finishHistory's (time 1.0, qend).  scan = exclusive prefix of the
// logged counts, so off[v] = 2 v + scan[v].
__global__ void __launch_bounds__(256) place_ends(int nv, const uint32_t *scan, const double *q0, const double *qend,
                                                  int32_t *off, double *times, double *pos) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v > nv) return;
  const int64_t first = 2 * (int64_t)v + scan[v];
  off[v] = (int32_t)first;
  if (v == nv) return;
  const int64_t last = 2 * (int64_t)(v + 1) + scan[v + 1] - 1;
  times[first] = 0.0;
  times[last] = 1.0;
  for (int c = 0; c < 3; c++) {
    pos[3 * first + c] = q0[3 * (int64_t)v + c];
    pos[3 * last + c] = qend[3 * (int64_t)v + c];
  }
}

// Sorted position i of a logged entry of vertex v lands at 2 v + 1 + i.
__global__ void __launch_bounds__(256) place_log(const uint64_t *keys, int64_t n, const double *log_t,
                                                 const double *log_p, double *times, double *pos) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  const int64_t v = (int64_t)(k >> 32), e = (int64_t)(k & 0xffffffffull);
  const int64_t at = 2 * v + 1 + i;
  times[at] = log_t[e];
  for (int c = 0; c < 3; c++) pos[3 * at + c] = log_p[3 * e + c];
}

// History::computeMinimumGap (src/History.cpp:82-96): the least gap between
// consecutive entries of a vertex, at most 1.0 (times are non-decreasing, so
// the gaps are non-negative and their bits order like the doubles).
__global__ void __launch_bounds__(256) min_gap(int nv, const int32_t *off, const double *times,
                                               unsigned long long *best) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= off[nv]) return;
  // the vertex of entry e: the last v with off[v] <= e
  int lo = 0, hi = nv - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (off[mid] <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  if (e == off[lo]) return;
  const double gap = times[e] - times[e - 1];
  atomicMin(best, (unsigned long long)__double_as_longlong(gap));
}

unsigned grid_of(int64_t n, int threads) { return (unsigned)std::max<int64_t>(1, (n + threads - 1) / threads); }

}  // namespace

cudaError_t launch_layer_events(const LayerGroups &g, const LayerState &s, int64_t max_events, int64_t max_group,
                                int64_t grid_min, cudaStream_t st) {
  const size_t shared =
      g.ngroups <= kSharedGroups ? (size_t)g.ngroups * (2 * sizeof(double) + 2 * sizeof(int)) + 16 : 0;
  if (max_group >= grid_min) {
    // every block must be resident at once: size the grid by occupancy
    if (shared > 48 * 1024)
      cudaFuncSetAttribute(layer_events_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared);
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, layer_events_grid, kGridThreads,
                                                                            shared);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int64_t want = (max_group + kGridThreads - 1) / kGridThreads;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
    GridStep *step = s.grid_step;
    LayerGroups gg = g;
    LayerState ss = s;
    void *args[] = {&gg, &ss, &max_events, &step};
    return cudaLaunchCooperativeKernel((void *)layer_events_grid, blocks, kGridThreads, args, shared, st);
  }
  if (shared > 48 * 1024) {
    cudaFuncSetAttribute(layer_events<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared);
    cudaFuncSetAttribute(layer_events<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared);
    cudaFuncSetAttribute(layer_events<512>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shared);
  }
  // small groups: a small block, whose barriers are cheap (one warp for
  // groups of at most 32 stencils and vertices)
  if (max_group <= 32)
    layer_events<32><<<1, 32, shared, st>>>(g, s, max_events);
  else if (max_group <= 256)
    layer_events<128><<<1, 128, shared, st>>>(g, s, max_events);
  else
    layer_events<512><<<1, 512, shared, st>>>(g, s, max_events);
  return cudaGetLastError();
}

cudaError_t launch_layer_finish(const LayerState &s, cudaStream_t st) {
  const int64_t n3 = 3 * (int64_t)s.nverts;
  layer_finish<<<grid_of(n3, 256), 256, 0, st>>>(n3, s.q, s.v, s.lu, s.term);
  return cudaGetLastError();
}

cudaError_t build_layer_history(int nverts, const double *q0, const double *qend, const int32_t *log_v,
                                const double *log_t, const double *log_p, int64_t n_log, uint64_t *keys,
                                uint64_t *keys_alt, void *temp, size_t temp_bytes, uint32_t *count, uint32_t *scan,
                                int32_t *off, double *times, double *pos, unsigned long long *best, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(count, 0, ((size_t)nverts + 1) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (n_log > 0) {
    count_log<<<grid_of(n_log, 256), 256, 0, st>>>(log_v, n_log, count, keys);
    int vbits = 1;
    while (vbits < 31 && ((int64_t)1 << vbits) < nverts) vbits++;
    e = radix_sort_u64(keys, keys_alt, nullptr, nullptr, n_log, 0, 32 + vbits, temp, temp_bytes, st);
    if (e != cudaSuccess) return e;
  }
  e = exclusive_scan_u32(count, scan, nverts, scan + nverts, temp, temp_bytes, st);
  if (e != cudaSuccess) return e;
  place_ends<<<grid_of((int64_t)nverts + 1, 256), 256, 0, st>>>(nverts, scan, q0, qend, off, times, pos);
  if (n_log > 0) place_log<<<grid_of(n_log, 256), 256, 0, st>>>(keys, n_log, log_t, log_p, times, pos);
  const int64_t entries = 2 * (int64_t)nverts + n_log;
  min_gap<<<grid_of(entries, 256), 256, 0, st>>>(nverts, off, times, best);
  return cudaGetLastError();
}

}  // namespace ccd
