// Swept-volume candidate search (broadphase.cuh).
#include <math.h>

#include <algorithm>

#include <string.h>

#include "broadphase.cuh"
#include "ccd_common.h"
#include "ccd_distance.h"
#include "radix_sort.cuh"

namespace ccd {

namespace {

constexpr int kThreads = 256;
constexpr int kStack = 128;
constexpr uint64_t kNoKey = ~0ull;

// Bit widths of the packed keys: Morton code << fbits | face (Morton keys),
// vertex << rbits | face rank (vertex-face), edge rank << ebits | edge rank
// (edge-edge).  An emitted key stays below 2^(width of the key), so kNoKey
// sorts after every emitted key when the sort covers one more bit.
struct KeyBits {
  int fbits, rbits, ebits;
  int mbits;          // Morton code bits kept (30, fewer when instances and faces need the room)
  int ibits, ishift;  // instance id above the Morton code: key >> ishift
  uint64_t fmask, rmask, emask;
};

inline int bits_for(int64_t x) {
  int b = 1;
  while (b < 62 && ((int64_t)1 << b) <= x) b++;
  return b;
}

inline KeyBits key_bits(const MeshTopology &t) {
  KeyBits k;
  k.fbits = bits_for(t.nf - 1);
  k.rbits = bits_for(std::max(t.nranks - 1, 1));
  k.ebits = bits_for(std::max(t.nedges - 1, 1));
  k.ibits = t.ninst > 1 ? bits_for(t.ninst - 1) : 0;
  // A shorter Morton code only makes the tree less tight, never the candidate
  // set different (that depends on the leaf slabs alone).
  k.mbits = std::min(30, 63 - k.fbits - k.ibits);
  k.ishift = k.mbits + k.fbits;
  k.fmask = ((uint64_t)1 << k.fbits) - 1;
  k.rmask = ((uint64_t)1 << k.rbits) - 1;
  k.emask = ((uint64_t)1 << k.ebits) - 1;
  return k;
}
// Face pairs per call: 9 edge-edge keys per pair stay below the sort's 2^31.
constexpr int64_t kMaxPairs = (int64_t)1 << 27;

struct Axes {
  double a[13][3];
};

inline unsigned grid_of(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

// ------------------------------------------------------------------ leaves
template <int K>
__global__ void __launch_bounds__(kThreads) leaf_slabs(MeshTopology topo, BroadphaseParams p, Axes ax, double *lo64,
                                                       double *hi64, float *flo, float *fhi, float *bounds) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (f < topo.nf) {
    double lo[K], hi[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
    for (int j = 0; j < 3; j++) {
      const int v = topo.faces[3 * f + j];
      // every History entry of the vertex (src/KDOPBroadPhase.cpp:60-70): the
      // two of a step, or the entries of a multi-entry history
      const int e0 = p.hoff ? p.hoff[v] : 0, e1 = p.hoff ? p.hoff[v + 1] : 2;
      for (int e = e0; e < e1; e++) {
        const double *pos = p.hoff ? p.hpos + 3 * (int64_t)e : (e ? p.qe : p.qs) + 3 * (int64_t)v;
        const double px = pos[0], py = pos[1], pz = pos[2];
#pragma unroll
        for (int k = 0; k < K; k++) {
          // KDOPBroadPhase.cpp:66-67 (pos . axis) / AABBBroadPhase.cpp:38-39 (pos[k])
          const double val = (K == 13) ? (px * ax.a[k][0] + py * ax.a[k][1]) + pz * ax.a[k][2]
                                       : (k == 0 ? px : (k == 1 ? py : pz));
          lo[k] = smin(val - p.eta, lo[k]);
          hi[k] = smax(val + p.eta, hi[k]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      lo64[(int64_t)k * topo.nf + f] = lo[k];
      hi64[(int64_t)k * topo.nf + f] = hi[k];
      flo[(int64_t)k * topo.nf + f] = __double2float_rd(lo[k]);
      fhi[(int64_t)k * topo.nf + f] = __double2float_ru(hi[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float c = 0.5f * (__double2float_rd(lo[k]) + __double2float_ru(hi[k]));
      cmin[k] = c;
      cmax[k] = c;
    }
  }
  // Bounds of the slab centres (for the Morton grid): warp reduce, then
  // atomics on the order-preserving integer image of the floats.
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      cmin[k] = fminf(cmin[k], __shfl_xor_sync(0xffffffffu, cmin[k], o));
      cmax[k] = fmaxf(cmax[k], __shfl_xor_sync(0xffffffffu, cmax[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; k++) {
      if (cmin[k] <= cmax[k]) {
        atomicMin((int *)&bounds[k], __float_as_int(cmin[k]) >= 0 ? __float_as_int(cmin[k])
                                                                   : (int)(0x80000000u - (unsigned)__float_as_int(cmin[k])));
        atomicMax((int *)&bounds[3 + k], __float_as_int(cmax[k]) >= 0 ? __float_as_int(cmax[k])
                                                                       : (int)(0x80000000u - (unsigned)__float_as_int(cmax[k])));
      }
    }
  }
}

__device__ __forceinline__ float ordered_to_float(int v) {
  return v >= 0 ? __int_as_float(v) : __int_as_float((int)(0x80000000u - (unsigned)v));
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 1023u;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void __launch_bounds__(kThreads) morton_keys(int nf, const float *flo, const float *fhi, const float *bounds,
                                                        const int32_t *face_inst, KeyBits kb, uint64_t *keys) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  uint32_t m = 0;
  for (int k = 0; k < 3; k++) {
    const float lo = ordered_to_float(((const int *)bounds)[k]);
    const float hi = ordered_to_float(((const int *)bounds)[3 + k]);
    const float c = 0.5f * (flo[(int64_t)k * nf + f] + fhi[(int64_t)k * nf + f]);
    float u = (hi > lo) ? (c - lo) / (hi - lo) : 0.5f;
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    uint32_t q = (uint32_t)(u * 1023.0f);
    m |= spread10(q) << (2 - k);
  }
  const uint64_t inst = face_inst ? (uint64_t)(uint32_t)face_inst[f] : 0;
  keys[f] = (inst << kb.ishift) | ((uint64_t)(m >> (30 - kb.mbits)) << kb.fbits) | (uint32_t)f;
}

// FP32 slab boxes of the tree, one contiguous record per leaf or node: lower
// bounds at [0, K), upper bounds at [H, H + K), H = 16 for the 13-DOP (128 B,
// one cache line per record) and 4 for the AABB (32 B); a slab test reads
// whole records with 16-byte loads.
template <int K>
struct BoxLayout {
  static constexpr int H = K > 4 ? 16 : 4;  // floats per half
  static constexpr int S = 2 * H;           // floats per record
  static constexpr int V = H / 4;           // float4 per half
};

template <int K>
__device__ __forceinline__ void load_box(const float *rec, float (&lo)[K], float (&hi)[K]) {
  typedef BoxLayout<K> L;
  const float4 *q = reinterpret_cast<const float4 *>(rec);
  float tmp[L::S];
#pragma unroll
  for (int v = 0; v < 2 * L::V; v++) {
    const float4 x = __ldg(q + v);
    tmp[4 * v] = x.x;
    tmp[4 * v + 1] = x.y;
    tmp[4 * v + 2] = x.z;
    tmp[4 * v + 3] = x.w;
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    lo[k] = tmp[k];
    hi[k] = tmp[L::H + k];
  }
}

// The same through L2 (records written by other blocks of the same launch).
template <int K>
__device__ __forceinline__ void load_box_cg(const float *rec, float (&lo)[K], float (&hi)[K]) {
  typedef BoxLayout<K> L;
  const float4 *q = reinterpret_cast<const float4 *>(rec);
  float tmp[L::S];
#pragma unroll
  for (int v = 0; v < 2 * L::V; v++) {
    const float4 x = __ldcg(q + v);
    tmp[4 * v] = x.x;
    tmp[4 * v + 1] = x.y;
    tmp[4 * v + 2] = x.z;
    tmp[4 * v + 3] = x.w;
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    lo[k] = tmp[k];
    hi[k] = tmp[L::H + k];
  }
}

template <int K>
__device__ __forceinline__ void store_box_cg(float *rec, const float (&lo)[K], const float (&hi)[K]) {
  typedef BoxLayout<K> L;
  float tmp[L::S];
#pragma unroll
  for (int k = 0; k < L::S; k++) tmp[k] = 0.0f;
#pragma unroll
  for (int k = 0; k < K; k++) {
    tmp[k] = lo[k];
    tmp[L::H + k] = hi[k];
  }
  float4 *q = reinterpret_cast<float4 *>(rec);
#pragma unroll
  for (int v = 0; v < 2 * L::V; v++) __stcg(q + v, make_float4(tmp[4 * v], tmp[4 * v + 1], tmp[4 * v + 2], tmp[4 * v + 3]));
}

// Leaf boxes in Morton order.
template <int K>
__global__ void __launch_bounds__(kThreads) gather_leaves(int nf, const uint64_t *keys, uint64_t fmask,
                                                          const float *flo, const float *fhi, float *leaf_box) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nf) return;
  const int f = (int)(keys[s] & fmask);
  float lo[K], hi[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    lo[k] = flo[(int64_t)k * nf + f];
    hi[k] = fhi[(int64_t)k * nf + f];
  }
  store_box_cg<K>(leaf_box + (int64_t)s * BoxLayout<K>::S, lo, hi);
}

// ------------------------------------------------------------------ LBVH (Karras 2012)
__device__ __forceinline__ int key_delta(const uint64_t *keys, int n, int i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);  // keys are unique
}

__global__ void __launch_bounds__(kThreads) build_lbvh(int n, const uint64_t *keys, int32_t *child, int32_t *range,
                                                       int32_t *parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (key_delta(keys, n, i, i + 1) - key_delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = key_delta(keys, n, i, i - d);
  int64_t lmax = 2;
  while (key_delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int64_t l = 0;
  for (int64_t t = lmax / 2; t >= 1; t /= 2)
    if (key_delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = (int)(i + l * d);
  const int dnode = key_delta(keys, n, i, j);
  int64_t sp = 0;
  for (int64_t div = 2;; div *= 2) {
    const int64_t t = (l + div - 1) / div;
    if (key_delta(keys, n, i, i + (sp + t) * d) > dnode) sp += t;
    if (t <= 1) break;
  }
  const int gamma = (int)(i + sp * d) + (d < 0 ? -1 : 0);
  const int first = i < j ? i : j, last = i < j ? j : i;
  const int left = (first == gamma) ? ~gamma : gamma;
  const int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  child[2 * i] = left;
  child[2 * i + 1] = right;
  range[2 * i] = first;
  range[2 * i + 1] = last;
  parent[left >= 0 ? left : (n - 1) + ~left] = i;
  parent[right >= 0 ? right : (n - 1) + ~right] = i;
  if (i == 0) parent[0] = -1;
}

// The surface of a box over its first three slabs (the x, y, z axes of both
// layouts): the tree-quality measure behind the rebuild decision of
// refit-only calls.
template <int K>
__device__ __forceinline__ float box_surface(const float (&lo)[K], const float (&hi)[K]) {
  const float x = fmaxf(hi[0] - lo[0], 0.0f), y = fmaxf(hi[1] - lo[1], 0.0f), z = fmaxf(hi[2] - lo[2], 0.0f);
  const float a = x * y + y * z + z * x;
  return isfinite(a) ? a : 0.0f;
}

// Bottom-up walk from leaf s: the second child to arrive at a node builds its
// FP32 slab union.  Returns the surface of the nodes this walk built.
template <int K>
__device__ __forceinline__ float refit_walk(int s, int n, const int32_t *child, const int32_t *parent,
                                            uint32_t *arrive, const float *leaf_box, float *node_box,
                                            unsigned long long *counters) {
  typedef BoxLayout<K> L;
  float area = 0.0f;
  int node = parent[(n - 1) + s];
  // Unique 64-bit keys bound the depth by 65; a longer walk means a broken
  // tree and is reported instead of followed.
  for (int level = 0; node >= 0; level++) {
    if (level > 70) {
      atomicOr(&counters[3], 2ull);
      return area;
    }
    __threadfence();
    if (atomicAdd(&arrive[node], 1u) == 0) return area;
    __threadfence();
    const int c0 = child[2 * node], c1 = child[2 * node + 1];
    float lo0[K], hi0[K], lo1[K], hi1[K];
    if (c0 >= 0)
      load_box_cg<K>(node_box + (int64_t)c0 * L::S, lo0, hi0);
    else
      load_box_cg<K>(leaf_box + (int64_t)(~c0) * L::S, lo0, hi0);
    if (c1 >= 0)
      load_box_cg<K>(node_box + (int64_t)c1 * L::S, lo1, hi1);
    else
      load_box_cg<K>(leaf_box + (int64_t)(~c1) * L::S, lo1, hi1);
#pragma unroll
    for (int k = 0; k < K; k++) {
      lo0[k] = fminf(lo0[k], lo1[k]);
      hi0[k] = fmaxf(hi0[k], hi1[k]);
    }
    store_box_cg<K>(node_box + (int64_t)node * L::S, lo0, hi0);
    area += box_surface<K>(lo0, hi0);
    node = parent[node];
  }
  return area;
}

// Node slabs of the whole tree; the summed node surface goes to counters[5]
// (a float), one atomic per warp.
template <int K>
__global__ void __launch_bounds__(kThreads) refit(int n, const int32_t *child, const int32_t *parent, uint32_t *arrive,
                                                  const float *leaf_box, float *node_box,
                                                  unsigned long long *counters) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  float area = 0.0f;
  if (s < n) area = refit_walk<K>(s, n, child, parent, arrive, leaf_box, node_box, counters);
  for (int o = 16; o > 0; o >>= 1) area += __shfl_xor_sync(0xffffffffu, area, o);
  if ((threadIdx.x & 31) == 0 && area != 0.0f) atomicAdd(reinterpret_cast<float *>(&counters[5]), area);
}

// ------------------------------------------------------------------ traversal
// The links a traversal needs, in 16-byte records beside the slab records so
// that visiting a node costs one memory round trip:
//   node_links[i] = (child 0, child 1, split, last leaf)   (child < 0: leaf ~child)
//   leaf_links[j] = (face, its three vertices)
//   leaf_end[j]   = first sorted leaf of a later instance (instance meshes)
// Child 0 of node i covers the sorted leaves [first, split] and child 1
// [split + 1, last], so a stack entry that carries a node's links tells,
// before any load, which children can hold a partner of the query (a later
// leaf of the same instance); only those children's slab and link records
// are then loaded, together.
__global__ void __launch_bounds__(kThreads) link_tree(int n, const uint64_t *keys, uint64_t fmask, int ishift,
                                                      bool multi, const int32_t *faces, const int32_t *child,
                                                      const int32_t *range, int4 *node_links, int4 *leaf_links,
                                                      int32_t *leaf_end) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i < n - 1) {
    const int c0 = child[2 * i];
    const int split = c0 < 0 ? ~c0 : range[2 * c0 + 1];
    node_links[i] = make_int4(c0, child[2 * i + 1], split, range[2 * i + 1]);
  }
  const int f = (int)(keys[i] & fmask);
  leaf_links[i] = make_int4(f, faces[3 * f], faces[3 * f + 1], faces[3 * f + 2]);
  if (multi) {
    // keys are sorted by instance first: binary search for the first leaf of
    // a later instance
    const uint64_t inst = keys[i] >> ishift;
    int lo = i + 1, hi = n;
    while (lo < hi) {
      const int mid = lo + ((hi - lo) >> 1);
      if ((keys[mid] >> ishift) > inst)
        hi = mid;
      else
        lo = mid + 1;
    }
    leaf_end[i] = lo;
  }
}

// A node on a traversal stack: its links (child 0, child 1, split, last).
// Every node pushed has its first leaf before the query's instance end (the
// root starts at leaf 0; child 1 is checked below; child 0 starts where its
// parent does), so the stack need not carry it.
struct StackEntry {
  int4 lk;
};

// Which of an entry's children can hold a partner of query leaf s: a later
// leaf (each pair once) of the same instance (before my_end).
__device__ __forceinline__ bool child_wanted(const StackEntry &e, int c, int s, int my_end) {
  return c ? (e.lk.w > s && e.lk.z + 1 < my_end) : (e.lk.z > s);
}

__device__ __forceinline__ StackEntry child_entry(const StackEntry &, int, const int4 &lk) { return StackEntry{lk}; }

// The part of a face-pair test after the conservative FP32 slab test:
// Mesh::neighboringFaces (src/Mesh.cpp:13-20) first -- most overlapping leaf
// pairs are adjacent faces, and this integer test spares them the FP64 one
// (FP64 compares run at 1/64 of the FP32 rate) -- then the reference's exact
// FP64 slab test (KDOPBroadPhase.cpp:132-137, strict '<').
__device__ __forceinline__ bool adjacent(const int4 &a, const int4 &b) {
  return a.y == b.y || a.y == b.z || a.y == b.w || a.z == b.y || a.z == b.z || a.z == b.w || a.w == b.y ||
         a.w == b.z || a.w == b.w;
}

template <int K>
__device__ __forceinline__ bool exact_pair(const MeshTopology &topo, const int4 &a, const int4 &b, const double *lo64,
                                           const double *hi64) {
  if (adjacent(a, b)) return false;
  const int fa = a.x, fb = b.x;
  for (int k = 0; k < K; k++)
    if ((hi64[(int64_t)k * topo.nf + fa] < lo64[(int64_t)k * topo.nf + fb]) ||
        (hi64[(int64_t)k * topo.nf + fb] < lo64[(int64_t)k * topo.nf + fa]))
      return false;
  return true;
}

template <int K>
__device__ __forceinline__ bool slabs_overlap(const float (&qlo)[K], const float (&qhi)[K], const float (&blo)[K],
                                              const float (&bhi)[K]) {
  bool sep = false;
#pragma unroll
  for (int k = 0; k < K; k++) sep |= (qhi[k] < blo[k]) || (bhi[k] < qlo[k]);
  return !sep;
}

__device__ __forceinline__ StackEntry root_entry(const int4 *node_links) { return StackEntry{__ldg(node_links)}; }

// One thread per query leaf s, over the leaves after s in sorted order (each
// pair once) and of the same instance.  COUNT: also count the slab tests
// (leaf and node), for the traversal's algorithmic bytes; a separate variant
// so that timed runs carry no counter.
template <int K, bool COUNT, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) find_pairs(MeshTopology topo, int n, const int4 *node_links,
                                                             const int4 *leaf_links, const int32_t *leaf_end,
                                                             const float *leaf_box, const float *node_box,
                                                             const double *lo64, const double *hi64, uint32_t *pairs,
                                                             uint64_t cap, unsigned long long *counters) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || n < 2) return;
  typedef BoxLayout<K> L;
  float qlo[K], qhi[K];
  load_box<K>(leaf_box + (int64_t)s * L::S, qlo, qhi);
  const int4 me = __ldg(leaf_links + s);
  const int my_end = leaf_end ? leaf_end[s] : n;
  // The visited node stays in registers: a visit with one overlapping
  // internal child goes on with it, and only the second of two goes through
  // the stack (the same visits as pushing every child, in another order).
  StackEntry stack[kStack];
  int sp = 0;
  StackEntry e = root_entry(node_links);
  bool have = true;
  unsigned long long tests = 0;
  // A valid tree is visited at most once per node (n - 1 internal nodes).
  for (int visits = 0; have || sp > 0; visits++) {
    if (visits >= n) {
      atomicOr(&counters[3], 2ull);
      return;
    }
    if (!have) e = stack[--sp];
    have = false;
    StackEntry next{make_int4(0, 0, 0, 0)};
    bool want[2];
    int4 lk[2];
    float blo[2][K], bhi[2][K];
#pragma unroll
    for (int c = 0; c < 2; c++) {  // the wanted children's records at once
      want[c] = child_wanted(e, c, s, my_end);
      const int ch = c ? e.lk.y : e.lk.x;
      if (!want[c]) continue;
      if (ch < 0) {
        lk[c] = __ldg(leaf_links + ~ch);
        load_box<K>(leaf_box + (int64_t)(~ch) * L::S, blo[c], bhi[c]);
      } else {
        lk[c] = __ldg(node_links + ch);
        load_box<K>(node_box + (int64_t)ch * L::S, blo[c], bhi[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 2; c++) {
      if (!want[c]) continue;
      if (COUNT) tests++;
      if (!slabs_overlap<K>(qlo, qhi, blo[c], bhi[c])) continue;
      const int ch = c ? e.lk.y : e.lk.x;
      if (ch < 0) {
        if (!exact_pair<K>(topo, me, lk[c], lo64, hi64)) continue;
        const unsigned long long idx = atomicAdd(&counters[0], 1ull);
        if (idx < cap) {
          pairs[2 * (int64_t)idx] = (uint32_t)me.x;
          pairs[2 * (int64_t)idx + 1] = (uint32_t)lk[c].x;
        }
      } else if (!have) {
        next = child_entry(e, c, lk[c]);
        have = true;
      } else if (sp < kStack) {
        stack[sp++] = child_entry(e, c, lk[c]);
      } else {
        atomicOr(&counters[3], 1ull);  // stack overflow: reported as an error
      }
    }
    if (have) e = next;
  }
  if (COUNT && tests) atomicAdd(&counters[4], tests);
}

// Four lanes per query face (13-DOP records only).  Lane q of a quad loads
// the q-th 16-byte piece of the lower-bound half and of the upper-bound half
// of every record it visits and tests the query's slabs 4q .. 4q+3 (the pad
// slots past slab 12 hold zero in both the query and the node, so they never
// separate); two shuffles within the quad combine the four answers.  A
// record's four pieces are thus read by four neighbouring lanes -- one
// 128-byte line per quad per load instruction instead of one line per lane
// -- and each lane needs a quarter of the registers, so more warps stay
// resident.  The quad follows one traversal, so it never diverges; lane 0 of
// the quad keeps the stack and hands each popped entry to the others.  Each
// quad performs exactly the per-face traversal's slab tests.
__device__ __forceinline__ int quad_bcast(unsigned qmask, int x) { return __shfl_sync(qmask, x, 0, 4); }

template <bool COUNT, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) find_pairs_quad(MeshTopology topo, int n, const int4 *node_links,
                                                                  const int4 *leaf_links, const int32_t *leaf_end,
                                                                  const float *leaf_box, const float *node_box,
                                                                  const double *lo64, const double *hi64,
                                                                  uint32_t *pairs, uint64_t cap,
                                                                  unsigned long long *counters) {
  typedef BoxLayout<13> L;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int s = (int)(t >> 2), q = (int)(t & 3);
  const unsigned lane = threadIdx.x & 31;
  const unsigned qmask = 0xfu << (lane & ~3u);
  if (s >= n || n < 2) return;  // whole quads leave together
  const float4 *qrec = reinterpret_cast<const float4 *>(leaf_box + (int64_t)s * L::S);
  const float4 qlo = __ldg(qrec + q), qhi = __ldg(qrec + L::V + q);
  const int4 me = __ldg(leaf_links + s);
  const int my_end = leaf_end ? leaf_end[s] : n;
  // The node being visited sits in registers of all four lanes: a visit that
  // finds one overlapping internal child goes on with it directly, and only
  // when both overlap does one go through the stack (lane 0's, broadcast to
  // the quad when popped).  The set of visits, and so of slab tests, is the
  // same as with every child pushed; only their order differs.
  StackEntry stack[kStack];  // kept by lane 0 of the quad
  int sp = 0;
  StackEntry e = root_entry(node_links);
  bool have = true;
  unsigned long long tests = 0;
  for (int visits = 0; have || sp > 0; visits++) {
    if (visits >= n) {
      if (q == 0) atomicOr(&counters[3], 2ull);
      return;
    }
    if (!have) {
      StackEntry p{make_int4(0, 0, 0, 0)};
      if (q == 0) p = stack[sp - 1];
      sp--;
      e.lk.x = quad_bcast(qmask, p.lk.x);
      e.lk.y = quad_bcast(qmask, p.lk.y);
      e.lk.z = quad_bcast(qmask, p.lk.z);
      e.lk.w = quad_bcast(qmask, p.lk.w);
    }
    have = false;
    StackEntry next{make_int4(0, 0, 0, 0)};
    bool want[2];
    int4 lk[2];
    float4 blo[2], bhi[2];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      want[c] = child_wanted(e, c, s, my_end);
      if (!want[c]) continue;
      const int ch = c ? e.lk.y : e.lk.x;
      const float4 *rec = reinterpret_cast<const float4 *>(ch < 0 ? leaf_box + (int64_t)(~ch) * L::S
                                                                   : node_box + (int64_t)ch * L::S);
      lk[c] = __ldg(ch < 0 ? leaf_links + ~ch : node_links + ch);
      blo[c] = __ldg(rec + q);
      bhi[c] = __ldg(rec + L::V + q);
    }
#pragma unroll
    for (int c = 0; c < 2; c++) {
      if (!want[c]) continue;  // uniform within the quad
      if (COUNT && q == 0) tests++;
      bool sep = (qhi.x < blo[c].x) || (bhi[c].x < qlo.x) || (qhi.y < blo[c].y) || (bhi[c].y < qlo.y) ||
                 (qhi.z < blo[c].z) || (bhi[c].z < qlo.z) || (qhi.w < blo[c].w) || (bhi[c].w < qlo.w);
      sep |= __shfl_xor_sync(qmask, sep, 1, 4);
      sep |= __shfl_xor_sync(qmask, sep, 2, 4);
      if (sep) continue;
      const int ch = c ? e.lk.y : e.lk.x;
      if (ch >= 0) {
        if (!have) {  // every lane loaded lk[c]: no broadcast needed
          next = child_entry(e, c, lk[c]);
          have = true;
        } else if (sp < kStack) {
          if (q == 0) stack[sp] = child_entry(e, c, lk[c]);
          sp++;
        } else if (q == 0) {
          atomicOr(&counters[3], 1ull);  // stack overflow: reported as an error
        }
        continue;
      }
      // Mesh::neighboringFaces, then the exact FP64 test with its slabs
      // split over the quad as above.
      const int4 b = lk[c];
      if (adjacent(me, b)) continue;
      bool xsep = false;
      for (int k = 4 * q; k < 4 * q + 4 && k < 13; k++)
        xsep |= (hi64[(int64_t)k * topo.nf + me.x] < lo64[(int64_t)k * topo.nf + b.x]) ||
                (hi64[(int64_t)k * topo.nf + b.x] < lo64[(int64_t)k * topo.nf + me.x]);
      xsep |= __shfl_xor_sync(qmask, xsep, 1, 4);
      xsep |= __shfl_xor_sync(qmask, xsep, 2, 4);
      if (xsep || q != 0) continue;
      const unsigned long long idx = atomicAdd(&counters[0], 1ull);
      if (idx < cap) {
        pairs[2 * (int64_t)idx] = (uint32_t)me.x;
        pairs[2 * (int64_t)idx + 1] = (uint32_t)b.x;
      }
    }
    if (have) e = next;
  }
  if (COUNT && tests) atomicAdd(&counters[4], tests);
}

// Warp-cooperative (packet) traversal.  A warp takes 32 consecutive leaves in
// Morton order -- spatially close queries -- and walks the tree once for all
// of them: each stack entry holds a node and the mask of lanes whose query
// overlapped it (a lane whose query misses a node misses its whole subtree,
// since a parent's slab contains its children's).  At each pop every lane in
// the mask tests its own query against the child records, which all lanes
// load from the same addresses (one memory request per 16-byte piece for the
// warp instead of one per lane); the lanes that pass make up the child's
// mask.  Each lane therefore performs exactly the slab tests of its own
// per-leaf traversal; the stack and the loads are shared, and the chain of
// visits is the union of the lanes' traversals.  Pairs that pass the exact
// test are appended with one atomic per warp (ballot + prefix of the lanes
// that emit).
constexpr int kPacketWarps = 4;
constexpr int kPacketStack = 128;

__device__ __forceinline__ void emit_pairs(bool emit, int fa, int fb, uint32_t *pairs, uint64_t cap,
                                           unsigned long long *counters) {
  const unsigned m = __ballot_sync(0xffffffffu, emit);
  if (!m) return;
  const unsigned lane = threadIdx.x & 31;
  unsigned long long base = 0;
  const int leader = __ffs(m) - 1;
  if ((int)lane == leader) base = atomicAdd(&counters[0], (unsigned long long)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (emit) {
    const unsigned long long idx = base + __popc(m & ((1u << lane) - 1u));
    if (idx < cap) {
      pairs[2 * (int64_t)idx] = (uint32_t)fa;
      pairs[2 * (int64_t)idx + 1] = (uint32_t)fb;
    }
  }
}

template <int K, bool COUNT>
__global__ void __launch_bounds__(kPacketWarps * 32, 4)
    find_pairs_packet(MeshTopology topo, int n, const int4 *node_links, const int4 *leaf_links,
                      const int32_t *leaf_end, const float *leaf_box, const float *node_box, const double *lo64,
                      const double *hi64, uint32_t *pairs, uint64_t cap, unsigned long long *counters) {
  typedef BoxLayout<K> L;
  __shared__ StackEntry st_node[kPacketWarps][kPacketStack];
  __shared__ unsigned st_mask[kPacketWarps][kPacketStack];
  const unsigned lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int64_t first = ((int64_t)blockIdx.x * kPacketWarps + w) * 32;
  if (first >= n || n < 2) return;  // whole warps leave together
  const int s = (int)(first + lane);
  const bool valid = s < n;
  float qlo[K], qhi[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    qlo[k] = INFINITY;  // an empty box for lanes past the last leaf
    qhi[k] = -INFINITY;
  }
  int4 me = make_int4(0, -1, -1, -1);
  int my_end = n;
  if (valid) {
    load_box<K>(leaf_box + (int64_t)s * L::S, qlo, qhi);
    me = __ldg(leaf_links + s);
    if (leaf_end) my_end = leaf_end[s];
  }
  const unsigned all = __ballot_sync(0xffffffffu, valid);
  if (lane == 0) {
    st_node[w][0] = root_entry(node_links);
    st_mask[w][0] = all;
  }
  int sp = 1;
  __syncwarp();
  unsigned long long tests = 0;
  for (int visits = 0; sp > 0; visits++) {
    if (visits >= n) {
      if (lane == 0) atomicOr(&counters[3], 2ull);
      return;
    }
    sp--;
    const StackEntry e = st_node[w][sp];
    const unsigned mask = st_mask[w][sp];
    __syncwarp();
    const bool mine = (mask >> lane) & 1u;
    bool want[2];
    int4 lk[2];
    float blo[2][K], bhi[2][K];
#pragma unroll
    for (int c = 0; c < 2; c++) {
      want[c] = mine && child_wanted(e, c, s, my_end);
      const int ch = c ? e.lk.y : e.lk.x;
      if (!__any_sync(0xffffffffu, want[c])) continue;
      if (ch < 0) {
        lk[c] = __ldg(leaf_links + ~ch);
        load_box<K>(leaf_box + (int64_t)(~ch) * L::S, blo[c], bhi[c]);
      } else {
        lk[c] = __ldg(node_links + ch);
        load_box<K>(node_box + (int64_t)ch * L::S, blo[c], bhi[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < 2; c++) {
      if (!__any_sync(0xffffffffu, want[c])) continue;
      if (COUNT && want[c]) tests++;
      const bool hit = want[c] && slabs_overlap<K>(qlo, qhi, blo[c], bhi[c]);
      const int ch = c ? e.lk.y : e.lk.x;
      if (ch < 0) {
        emit_pairs(hit && exact_pair<K>(topo, me, lk[c], lo64, hi64), me.x, lk[c].x, pairs, cap, counters);
      } else {
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (m) {
          if (sp >= kPacketStack) {  // deeper than any valid tree: reported as an error
            if (lane == 0) atomicOr(&counters[3], 1ull);
            return;
          }
          if (lane == 0) {
            st_node[w][sp] = child_entry(e, c, lk[c]);
            st_mask[w][sp] = m;
          }
          sp++;
          __syncwarp();
        }
      }
    }
  }
  if (COUNT) {
    tests = __reduce_add_sync(0xffffffffu, (unsigned)tests);
    if (lane == 0 && tests) atomicAdd(&counters[4], tests);
  }
}

// ------------------------------------------------------------------ stencils
// KDOPBroadPhase.cpp:150-183: 6 vertex-face and 9 edge-edge stencils per
// pair, skipping those whose four vertices are all fixed.
__global__ void __launch_bounds__(kThreads) stencil_keys(MeshTopology topo, KeyBits kb, const uint8_t *fixed,
                                                         const uint32_t *pairs, int64_t npairs,
                                                         const unsigned long long *count, uint64_t *vf_keys,
                                                         uint64_t *ee_keys) {
  const int64_t pi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pi >= npairs) return;
  // With a device count (the graph step), slots past it hold no pair: their
  // keys are kNoKey, which sort last and are never decoded.
  if (count && (unsigned long long)pi >= *count) {
    for (int k = 0; k < 6; k++) vf_keys[6 * pi + k] = kNoKey;
    for (int k = 0; k < 9; k++) ee_keys[9 * pi + k] = kNoKey;
    return;
  }
  const int fa = (int)pairs[2 * pi], fb = (int)pairs[2 * pi + 1];
  int A[3], B[3];
  bool FA[3], FB[3];
  for (int i = 0; i < 3; i++) {
    A[i] = topo.faces[3 * fa + i];
    B[i] = topo.faces[3 * fb + i];
    FA[i] = fixed && fixed[A[i]];
    FB[i] = fixed && fixed[B[i]];
  }
  const bool allA = FA[0] && FA[1] && FA[2], allB = FB[0] && FB[1] && FB[2];
  const uint64_t ra = (uint32_t)topo.face_rank[fa], rb = (uint32_t)topo.face_rank[fb];
  for (int i = 0; i < 3; i++) {
    vf_keys[6 * pi + 2 * i] = (FA[i] && allB) ? kNoKey : ((uint64_t)(uint32_t)A[i] << kb.rbits) | rb;
    vf_keys[6 * pi + 2 * i + 1] = (FB[i] && allA) ? kNoKey : ((uint64_t)(uint32_t)B[i] << kb.rbits) | ra;
    for (int j = 0; j < 3; j++) {
      const bool all = FA[i] && FA[(i + 1) % 3] && FB[j] && FB[(j + 1) % 3];
      const uint32_t e1 = (uint32_t)topo.face_edges[3 * fa + i], e2 = (uint32_t)topo.face_edges[3 * fb + j];
      ee_keys[9 * pi + 3 * i + j] =
          all ? kNoKey : (((uint64_t)(e1 < e2 ? e1 : e2) << kb.ebits) | (uint64_t)(e1 < e2 ? e2 : e1));
    }
  }
}

// Every stencil slot of [0, cap) := the same stencil (the graph step's
// padding: slots past the real candidates).
__global__ void __launch_bounds__(kThreads) fill_stencils(int32_t *out, int64_t cap, int4 st) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cap) reinterpret_cast<int4 *>(out)[i] = st;
}

__global__ void __launch_bounds__(kThreads) first_of_run(const uint64_t *keys, int64_t n, uint32_t *flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t k = keys[i];
  flags[i] = (k != kNoKey && (i == 0 || keys[i - 1] != k)) ? 1u : 0u;
}

// Unique keys -> stencils (reference order: keys are sorted).
__global__ void __launch_bounds__(kThreads) decode_vf(MeshTopology topo, KeyBits kb, const uint64_t *keys,
                                                      const uint32_t *flags,
                                                      const uint32_t *pos, int64_t n, int32_t *out, int64_t cap) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flags[i]) return;
  const uint64_t k = keys[i];
  const int64_t o = pos[i];
  if (o >= cap) return;
  const int r = (int)(k & kb.rmask);
  out[4 * o] = (int32_t)(k >> kb.rbits);
  out[4 * o + 1] = topo.rank_triple[3 * r];
  out[4 * o + 2] = topo.rank_triple[3 * r + 1];
  out[4 * o + 3] = topo.rank_triple[3 * r + 2];
}

__global__ void __launch_bounds__(kThreads) decode_ee(MeshTopology topo, KeyBits kb, const uint64_t *keys,
                                                      const uint32_t *flags,
                                                      const uint32_t *pos, int64_t n, int32_t *out, int64_t cap) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flags[i]) return;
  const uint64_t k = keys[i];
  const int64_t o = pos[i];
  if (o >= cap) return;
  const int r1 = (int)(k >> kb.ebits), r2 = (int)(k & kb.emask);
  out[4 * o] = topo.rank_edge[2 * r1];
  out[4 * o + 1] = topo.rank_edge[2 * r1 + 1];
  out[4 * o + 2] = topo.rank_edge[2 * r2];
  out[4 * o + 3] = topo.rank_edge[2 * r2 + 1];
}

template <class T>
cudaError_t grow(T **p, int64_t *cap, int64_t need) {
  if (*cap >= need && *p) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  int64_t c = std::max<int64_t>(need, 1);
  cudaError_t e = cudaMalloc(p, (size_t)c * sizeof(T));
  if (e == cudaSuccess) *cap = c;
  return e;
}

Axes make_axes() {
  // The 13 k-DOP directions of KDOPBroadPhase.cpp:12-31, normalised as the
  // reference does (component / norm, norm = sqrt((x*x + y*y) + z*z)).
  static const double dirs[13][3] = {{1, 0, 0},  {0, 1, 0},  {0, 0, 1},  {1, 1, 0},  {1, -1, 0},
                                     {0, 1, 1},  {0, 1, -1}, {1, 0, 1},  {1, 0, -1}, {1, 1, 1},
                                     {1, 1, -1}, {1, -1, 1}, {1, -1, -1}};
  Axes ax;
  for (int k = 0; k < 13; k++) {
    volatile double x = dirs[k][0], y = dirs[k][1], z = dirs[k][2];
    volatile double xx = x * x, yy = y * y, zz = z * z;
    volatile double s = xx + yy;
    s = s + zz;
    const double nrm = sqrt((double)s);
    ax.a[k][0] = x / nrm;
    ax.a[k][1] = y / nrm;
    ax.a[k][2] = z / nrm;
  }
  return ax;
}

// ------------------------------------------------------------------ trivial candidates
// TrivialBroadPhase::findCollisionCandidates (src/TrivialBroadPhase.cpp:4-53)
// in set order without a sort.  Vertex-face stencils are the pairs (vertex i,
// face rank r) with i not in r's sorted triple, in (i, r) order -- the set
// order of (p, q0, q1, q2), each distinct triple once.  Edge-edge stencils are
// the pairs of edge ranks (a < b) whose edges share no vertex, in (a, b) order
// -- the set order of (p0, p1, q0, q1), since the smaller-ranked edge has the
// smaller first vertex.  A chunk of the index space is flagged, scanned and
// written out at its running offset.
__device__ __forceinline__ bool all_fixed4(const uint8_t *fixed, int a, int b, int c, int d) {
  return fixed && fixed[a] && fixed[b] && fixed[c] && fixed[d];
}

__global__ void __launch_bounds__(kThreads) trivial_flags(MeshTopology topo, const uint8_t *fixed, int which,
                                                          int64_t begin, int64_t count, uint32_t *flags) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int64_t idx = begin + t;
  bool keep;
  if (which == 0) {
    const int i = (int)(idx / topo.nranks), r = (int)(idx % topo.nranks);
    const int a = topo.rank_triple[3 * r], b = topo.rank_triple[3 * r + 1], c = topo.rank_triple[3 * r + 2];
    keep = i != a && i != b && i != c && !all_fixed4(fixed, i, a, b, c);
  } else {
    const int ea = (int)(idx / topo.nedges), eb = (int)(idx % topo.nedges);
    const int a0 = topo.rank_edge[2 * ea], a1 = topo.rank_edge[2 * ea + 1];
    const int b0 = topo.rank_edge[2 * eb], b1 = topo.rank_edge[2 * eb + 1];
    keep = ea < eb && a0 != b0 && a0 != b1 && a1 != b0 && a1 != b1 && !all_fixed4(fixed, a0, a1, b0, b1);
  }
  flags[t] = keep ? 1u : 0u;
}

__global__ void __launch_bounds__(kThreads) trivial_emit(MeshTopology topo, int which, int64_t begin, int64_t count,
                                                         const uint32_t *flags, const uint32_t *pos, int64_t base,
                                                         int32_t *out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= count || !flags[t]) return;
  const int64_t idx = begin + t;
  int4 st;
  if (which == 0) {
    const int i = (int)(idx / topo.nranks), r = (int)(idx % topo.nranks);
    st = make_int4(i, topo.rank_triple[3 * r], topo.rank_triple[3 * r + 1], topo.rank_triple[3 * r + 2]);
  } else {
    const int ea = (int)(idx / topo.nedges), eb = (int)(idx % topo.nedges);
    st = make_int4(topo.rank_edge[2 * ea], topo.rank_edge[2 * ea + 1], topo.rank_edge[2 * eb],
                   topo.rank_edge[2 * eb + 1]);
  }
  reinterpret_cast<int4 *>(out)[base + pos[t]] = st;
}

// ------------------------------------------------------------------ closest vertex pair
// The vertex scan of Distance::meshSelfDistance (src/Distance.cpp:21-34):
// the least (x_i - x_v).squaredNorm() over vertices i and vertices v of a face
// that does not contain i.  A pair (i, v) qualifies exactly when some face
// incident to v misses i; a vertex in no face is never the far end v.

// Vertex -> face incidence (CSR): each face once per distinct vertex.
__global__ void __launch_bounds__(kThreads) incidence_count(int nf, const int32_t *faces, uint32_t *count) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
  atomicAdd(&count[a], 1u);
  if (b != a) atomicAdd(&count[b], 1u);
  if (c != a && c != b) atomicAdd(&count[c], 1u);
}

__global__ void __launch_bounds__(kThreads) incidence_fill(int nf, const int32_t *faces, const uint32_t *off,
                                                           uint32_t *cursor, int32_t *list) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
  list[off[a] + atomicAdd(&cursor[a], 1u)] = f;
  if (b != a) list[off[b] + atomicAdd(&cursor[b], 1u)] = f;
  if (c != a && c != b) list[off[c] + atomicAdd(&cursor[c], 1u)] = f;
}

__device__ __forceinline__ bool finite3(const double *x) {
  return isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
}

// Point boxes (outward-rounded FP32) of the vertices that can be a far end:
// in some face and with finite coordinates (a non-finite coordinate makes
// every squared distance NaN or infinite, which never lowers the reference's
// running minimum).  Other vertices get the empty box [+inf, -inf], which no
// test passes.
__global__ void __launch_bounds__(kThreads) point_slabs(int nv, const double *x, const uint32_t *degree, float *flo,
                                                        float *fhi, float *bounds) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  float cmin[3] = {INFINITY, INFINITY, INFINITY}, cmax[3] = {-INFINITY, -INFINITY, -INFINITY};
  if (v < nv) {
    const double *p = x + 3 * (int64_t)v;
    const bool far_end = degree[v] > 0 && finite3(p);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float lo = far_end ? __double2float_rd(p[k]) : INFINITY;
      const float hi = far_end ? __double2float_ru(p[k]) : -INFINITY;
      flo[(int64_t)k * nv + v] = lo;
      fhi[(int64_t)k * nv + v] = hi;
      if (far_end) cmin[k] = cmax[k] = 0.5f * (lo + hi);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      cmin[k] = fminf(cmin[k], __shfl_xor_sync(0xffffffffu, cmin[k], o));
      cmax[k] = fmaxf(cmax[k], __shfl_xor_sync(0xffffffffu, cmax[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; k++) {
      if (cmin[k] <= cmax[k]) {
        atomicMin((int *)&bounds[k], __float_as_int(cmin[k]) >= 0 ? __float_as_int(cmin[k])
                                                                   : (int)(0x80000000u - (unsigned)__float_as_int(cmin[k])));
        atomicMax((int *)&bounds[3 + k], __float_as_int(cmax[k]) >= 0 ? __float_as_int(cmax[k])
                                                                       : (int)(0x80000000u - (unsigned)__float_as_int(cmax[k])));
      }
    }
  }
}

// Does some face incident to v miss vertex i?  (Mesh::vertexOfFace,
// src/Mesh.cpp:5-11, negated, over v's faces.)
__device__ __forceinline__ bool far_end_of(int i, int v, const uint32_t *off, const int32_t *list,
                                           const int32_t *faces) {
  const uint32_t e = off[v + 1];
  for (uint32_t k = off[v]; k < e; k++) {
    const int f = list[k];
    if (faces[3 * f] != i && faces[3 * f + 1] != i && faces[3 * f + 2] != i) return true;
  }
  return false;
}

__device__ __forceinline__ double sq_dist(const double *a, const double *b) {
  return vertex_distance_sq(v3d{a[0], a[1], a[2]}, v3d{b[0], b[1], b[2]});
}

// Lowers *best (the bits of a non-negative double) to d, one atomic per warp.
__device__ __forceinline__ void warp_min_to(double d, unsigned long long *best) {
  unsigned long long b = (unsigned long long)__double_as_longlong(d);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
    b = other < b ? other : b;
  }
  if ((threadIdx.x & 31) == 0 && b < __ldcg(best)) atomicMin(best, b);
}

constexpr int kSeedReach = 4;

// A first bound: each vertex against its Morton-order neighbours.
__global__ void __launch_bounds__(kThreads) pair_seed(int n, const uint64_t *keys, uint64_t vmask, const double *x,
                                                      const uint32_t *off, const int32_t *list, const int32_t *faces,
                                                      unsigned long long *best) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double local = INFINITY;
  if (s < n) {
    const int i = (int)(keys[s] & vmask);
    const double *xi = x + 3 * (int64_t)i;
    if (finite3(xi)) {
      for (int d = -kSeedReach; d <= kSeedReach; d++) {
        const int j = s + d;
        if (d == 0 || j < 0 || j >= n) continue;
        const int v = (int)(keys[j] & vmask);
        const double dd = sq_dist(xi, x + 3 * (int64_t)v);
        if (dd < local && off[v + 1] > off[v] && far_end_of(i, v, off, list, faces)) local = dd;
      }
    }
  }
  warp_min_to(local, best);
}

// Every vertex i against the tree of far-end vertices, pruned by the running
// global minimum.  A node is skipped when a lower bound of its squared
// distance to x_i exceeds the minimum by a relative 2^-40, far more than the
// rounding of the FP64 squared distances (a few ulps) -- so no pair whose
// FP64 squared distance is at most the final minimum is ever skipped.
__global__ void __launch_bounds__(kThreads) pair_search(int n, const uint64_t *keys, uint64_t vmask, const double *x,
                                                        const uint32_t *off, const int32_t *list, const int32_t *faces,
                                                        const int32_t *child, const float *leaf_box,
                                                        const float *node_box, unsigned long long *best,
                                                        unsigned long long *counters) {
  typedef BoxLayout<3> L;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || n < 2) return;
  const int i = (int)(keys[s] & vmask);
  const double *xi = x + 3 * (int64_t)i;
  if (!finite3(xi)) return;
  float qlo[3], qhi[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    qlo[k] = __double2float_rd(xi[k]);
    qhi[k] = __double2float_ru(xi[k]);
  }
  const double keep = 1.0 - 0x1p-40;
  double cur = __longlong_as_double((long long)__ldcg(best));
  int stack[kStack];
  int sp = 0;
  stack[sp++] = 0;  // root
  int64_t visits = 0;
  while (sp > 0) {
    if (cur == 0.0) return;  // nothing lies below zero
    const int node = stack[--sp];
    if (++visits > 4 * (int64_t)n) {
      atomicOr(&counters[3], 2ull);
      return;
    }
    if ((visits & 7) == 0) cur = fmin(cur, __longlong_as_double((long long)__ldcg(best)));
#pragma unroll
    for (int c = 0; c < 2; c++) {
      const int ch = child[2 * node + c];
      float blo[3], bhi[3];
      if (ch >= 0)
        load_box<3>(node_box + (int64_t)ch * L::S, blo, bhi);
      else
        load_box<3>(leaf_box + (int64_t)(~ch) * L::S, blo, bhi);
      float lb = 0.0f;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const float g = fmaxf(0.0f, fmaxf(__fsub_rd(blo[k], qhi[k]), __fsub_rd(qlo[k], bhi[k])));
        lb = __fadd_rd(lb, __fmul_rd(g, g));
      }
      if ((double)lb * keep > cur) continue;
      if (ch >= 0) {
        if (sp >= kStack) {
          atomicOr(&counters[3], 1ull);
          return;
        }
        stack[sp++] = ch;
        continue;
      }
      const int v = (int)(keys[~ch] & vmask);
      if (v == i) continue;
      const double dd = sq_dist(xi, x + 3 * (int64_t)v);
      if (dd < cur && far_end_of(i, v, off, list, faces)) {
        cur = dd;
        atomicMin(best, (unsigned long long)__double_as_longlong(dd));
      }
    }
  }
}

// Enqueues the traversal kernel the parameters choose; pairs past cap are
// counted but not written.
void enqueue_traversal(const MeshTopology &topo, const BroadphaseParams &p, BroadphaseBuffers &b, const KeyBits &kb,
                       uint64_t cap, cudaStream_t s) {
  const int nf = topo.nf;
  const bool kdop = p.kind == kBvhKdop13;
  const int32_t *lend = topo.ninst > 1 ? b.leaf_end : nullptr;
  if ((p.traversal == kTraversalQuad || p.traversal == kTraversalQuadDense) && kdop) {
    const unsigned grid = (unsigned)((4 * (int64_t)nf + kThreads - 1) / kThreads);
#define BP_QUAD(CC, MB)                                                                                  \
  find_pairs_quad<CC, MB><<<grid, kThreads, 0, s>>>(topo, nf, b.node_links, b.leaf_links, lend, b.leaf_box, \
                                                  b.node_box, b.lo64, b.hi64, b.pairs,                   \
                                                  cap, b.counters)
    if (p.traversal == kTraversalQuadDense) {
      if (p.count_tests) BP_QUAD(true, 5);
      else BP_QUAD(false, 5);
    } else {
      if (p.count_tests) BP_QUAD(true, 3);
      else BP_QUAD(false, 3);
    }
#undef BP_QUAD
    return;
  }
  if (p.traversal == kTraversalPacket) {
    const unsigned grid = (unsigned)((nf + 32 * kPacketWarps - 1) / (32 * kPacketWarps));
#define BP_FIND(KK, CC)                                                                                         \
  find_pairs_packet<KK, CC><<<grid, kPacketWarps * 32, 0, s>>>(topo, nf, b.node_links, b.leaf_links, lend,     \
                                                             b.leaf_box, b.node_box, b.lo64, b.hi64,         \
                                                             b.pairs, cap, b.counters)
    if (kdop && p.count_tests) BP_FIND(13, true);
    else if (kdop) BP_FIND(13, false);
    else if (p.count_tests) BP_FIND(3, true);
    else BP_FIND(3, false);
#undef BP_FIND
    return;
  }
#define BP_FIND(KK, CC, MB)                                                                                       \
  find_pairs<KK, CC, MB><<<grid_of(nf), kThreads, 0, s>>>(topo, nf, b.node_links, b.leaf_links, lend, b.leaf_box, \
                                                        b.node_box, b.lo64, b.hi64, b.pairs,                  \
                                                        cap, b.counters)
  if (p.traversal == kTraversalThreadDense) {
    if (kdop && p.count_tests) BP_FIND(13, true, 3);
    else if (kdop) BP_FIND(13, false, 3);
    else if (p.count_tests) BP_FIND(3, true, 3);
    else BP_FIND(3, false, 3);
  } else {
    if (kdop && p.count_tests) BP_FIND(13, true, 2);
    else if (kdop) BP_FIND(13, false, 2);
    else if (p.count_tests) BP_FIND(3, true, 2);
    else BP_FIND(3, false, 2);
  }
#undef BP_FIND
}

}  // namespace

void broadphase_free(BroadphaseBuffers &b) {
  void *ptrs[] = {b.lo64, b.hi64, b.face_lo, b.face_hi, b.leaf_box, b.node_box, b.node_child, b.node_range,
                  b.node_links, b.leaf_links, b.leaf_end, b.parent,
                  b.arrive, b.keys, b.keys_alt, b.vals, b.vals_alt, b.bounds, b.counters, b.pairs, b.vf_keys,
                  b.ee_keys, b.flags, b.scan, b.temp};
  for (void *p : ptrs) cudaFree(p);
  b = BroadphaseBuffers{};
}

#define BP_CUDA(call)        \
  do {                       \
    cudaError_t e_ = (call); \
    if (e_ != cudaSuccess) { \
      *err = e_;             \
      return 2;              \
    }                        \
  } while (0)

// Returns 0 on success, 2 on a CUDA error (*err), 3 on a malformed tree
// (traversal stack overflow or a walk longer than the tree allows), 4 when the
// candidate face pairs exceed 2^27.
int broadphase_run(const MeshTopology &topo, const BroadphaseParams &p, BroadphaseBuffers &b, int32_t **vf_out,
                   int64_t *vf_cap, int32_t **ee_out, int64_t *ee_cap, int64_t *n_vf, int64_t *n_ee,
                   int64_t *n_pairs, int64_t *slab_tests, int num_sms, cudaStream_t s, cudaError_t *err,
                   bool *rebuilt) {
  (void)num_sms;
  *n_vf = *n_ee = *n_pairs = 0;
  const int nf = topo.nf;
  if (nf < 2) return 0;
  const bool kdop = p.kind == kBvhKdop13;
  // Buffers sized by the face count.
  if (b.cap_faces < nf) {
    broadphase_free(b);
    const size_t F = (size_t)nf;
    BP_CUDA(cudaMalloc(&b.lo64, 13 * F * sizeof(double)));
    BP_CUDA(cudaMalloc(&b.hi64, 13 * F * sizeof(double)));
    BP_CUDA(cudaMalloc(&b.face_lo, 13 * F * sizeof(float)));  // [axis][face]
    BP_CUDA(cudaMalloc(&b.face_hi, 13 * F * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.leaf_box, 32 * F * sizeof(float)));  // [sorted leaf][record]
    BP_CUDA(cudaMalloc(&b.node_box, 32 * F * sizeof(float)));  // [node][record]
    BP_CUDA(cudaMalloc(&b.node_child, 2 * F * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.node_range, 2 * F * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.node_links, F * sizeof(int4)));
    BP_CUDA(cudaMalloc(&b.leaf_links, F * sizeof(int4)));
    BP_CUDA(cudaMalloc(&b.leaf_end, F * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.parent, 2 * F * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.arrive, F * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.keys, F * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.vals, F * sizeof(uint64_t)));  // second Morton key buffer
    BP_CUDA(cudaMalloc(&b.bounds, 8 * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.counters, 8 * sizeof(unsigned long long)));
    b.cap_faces = nf;
  }
  // Pair-sized buffers; grown when a traversal reports more pairs.
  auto ensure_pairs = [&](int64_t cap) -> int {
    if (b.cap_pairs >= cap && b.pairs) return 0;
    void *ptrs[] = {b.pairs, b.vf_keys, b.ee_keys, b.keys_alt, b.flags, b.scan, b.temp};
    for (void *q : ptrs) cudaFree(q);
    b.pairs = nullptr;
    b.vf_keys = b.ee_keys = b.keys_alt = nullptr;
    b.flags = b.scan = nullptr;
    b.temp = nullptr;
    b.cap_pairs = 0;
    const int64_t nkeys = std::max<int64_t>(9 * cap, nf);
    BP_CUDA(cudaMalloc(&b.pairs, (size_t)cap * 2 * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.vf_keys, (size_t)6 * cap * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.ee_keys, (size_t)9 * cap * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.keys_alt, (size_t)nkeys * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.flags, (size_t)nkeys * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.scan, (size_t)nkeys * sizeof(uint32_t)));
    b.temp_bytes = std::max(radix_sort_temp_bytes(nkeys), scan_temp_bytes(nkeys));
    BP_CUDA(cudaMalloc(&b.temp, b.temp_bytes));
    b.cap_pairs = cap;
    return 0;
  };
  int rc = ensure_pairs(std::max<int64_t>(b.cap_pairs, std::min<int64_t>(std::max<int64_t>(8 * (int64_t)nf, 4096), kMaxPairs)));
  if (rc) return rc;

  if (p.ev[0]) BP_CUDA(cudaEventRecord(p.ev[0], s));
  float *flo = b.face_lo, *fhi = b.face_hi;
  const Axes ax = make_axes();
  {
    // centre bounds as order-preserving ints: +inf for minima, -inf for maxima
    const int pinf = 0x7f800000, ninf = (int)(0x80000000u - 0xff800000u);
    int hb[6] = {pinf, pinf, pinf, ninf, ninf, ninf};
    BP_CUDA(cudaMemcpyAsync(b.bounds, hb, sizeof(hb), cudaMemcpyHostToDevice, s));
  }
  if (kdop)
    leaf_slabs<13><<<grid_of(nf), kThreads, 0, s>>>(topo, p, ax, b.lo64, b.hi64, flo, fhi, b.bounds);
  else
    leaf_slabs<3><<<grid_of(nf), kThreads, 0, s>>>(topo, p, ax, b.lo64, b.hi64, flo, fhi, b.bounds);
  BP_CUDA(cudaGetLastError());
  const KeyBits kb = key_bits(topo);
  // Refit only: the kept tree's leaf order and links stay, its node slabs are
  // rebuilt from the new leaf slabs.  Otherwise a new tree: Morton keys of
  // the slab centres, radix sort, Karras hierarchy.
  const bool reuse = p.refit && b.tree_kind == p.kind && b.tree_nf == nf && b.tree_ninst == topo.ninst &&
                     !b.rebuild_next && b.refits < p.max_refits;
  if (rebuilt) *rebuilt = !reuse;
  if (!reuse) {
    morton_keys<<<grid_of(nf), kThreads, 0, s>>>(nf, flo, fhi, b.bounds, topo.ninst > 1 ? topo.face_inst : nullptr,
                                                  kb, b.keys);
    BP_CUDA(cudaGetLastError());
    BP_CUDA(radix_sort_u64(b.keys, (uint64_t *)b.vals, nullptr, nullptr, nf, 0, kb.ishift + kb.ibits, b.temp,
                           b.temp_bytes, s));
  }
  if (kdop)
    gather_leaves<13><<<grid_of(nf), kThreads, 0, s>>>(nf, b.keys, kb.fmask, flo, fhi, b.leaf_box);
  else
    gather_leaves<3><<<grid_of(nf), kThreads, 0, s>>>(nf, b.keys, kb.fmask, flo, fhi, b.leaf_box);
  if (!reuse) {
    build_lbvh<<<grid_of(nf - 1), kThreads, 0, s>>>(nf, b.keys, b.node_child, b.node_range, b.parent);
    link_tree<<<grid_of(nf), kThreads, 0, s>>>(nf, b.keys, kb.fmask, kb.ishift, topo.ninst > 1, topo.faces,
                                               b.node_child, b.node_range, b.node_links, b.leaf_links, b.leaf_end);
    b.tree_kind = p.kind;
    b.tree_nf = nf;
    b.tree_ninst = topo.ninst;
    b.refits = 0;
    b.build_area = -1.0f;
  } else {
    b.refits++;
  }
  b.rebuild_next = false;
  BP_CUDA(cudaMemsetAsync(b.arrive, 0, (size_t)nf * sizeof(uint32_t), s));
  BP_CUDA(cudaMemsetAsync(b.counters, 0, 8 * sizeof(unsigned long long), s));
  if (kdop)
    refit<13><<<grid_of(nf), kThreads, 0, s>>>(nf, b.node_child, b.parent, b.arrive, b.leaf_box, b.node_box,
                                               b.counters);
  else
    refit<3><<<grid_of(nf), kThreads, 0, s>>>(nf, b.node_child, b.parent, b.arrive, b.leaf_box, b.node_box,
                                              b.counters);
  BP_CUDA(cudaGetLastError());

  if (p.ev[0]) BP_CUDA(cudaEventRecord(p.ev[1], s));
  auto traverse = [&]() { enqueue_traversal(topo, p, b, kb, (uint64_t)b.cap_pairs, s); };
  for (;;) {
    // pairs, vf, ee and the slab-test count; keeps the error word
    BP_CUDA(cudaMemsetAsync(b.counters, 0, 3 * sizeof(unsigned long long), s));
    BP_CUDA(cudaMemsetAsync(b.counters + 4, 0, sizeof(unsigned long long), s));
    traverse();
    BP_CUDA(cudaGetLastError());
    if (p.ev[0]) BP_CUDA(cudaEventRecord(p.ev[2], s));
    unsigned long long hc[6];
    BP_CUDA(cudaMemcpyAsync(hc, b.counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
    BP_CUDA(cudaStreamSynchronize(s));
    if (hc[3]) {
      b.tree_kind = -1;  // never refit a tree that failed
      return 3;
    }
    {
      // Tree quality: the summed node surface against its value after the
      // build; a kept tree whose nodes have grown too much is rebuilt next.
      float area;
      const uint32_t bits = (uint32_t)hc[5];
      memcpy(&area, &bits, sizeof(area));
      if (b.build_area < 0.0f)
        b.build_area = area;
      else if (!(area <= p.rebuild_ratio * b.build_area))
        b.rebuild_next = true;
    }
    *n_pairs = hc[0];
    if (slab_tests) *slab_tests = (int64_t)hc[4];
    if ((int64_t)hc[0] <= b.cap_pairs) break;
    if ((int64_t)hc[0] > kMaxPairs) return 4;
    rc = ensure_pairs(std::min<int64_t>(2 * (int64_t)hc[0], kMaxPairs));  // the tree stays valid; only the pair buffers grow
    if (rc) return rc;
  }
  const int64_t np = *n_pairs;
  if (np == 0) {
    if (p.ev[0]) BP_CUDA(cudaEventRecord(p.ev[3], s));
    BP_CUDA(cudaStreamSynchronize(s));
    return 0;
  }
  stencil_keys<<<grid_of(np), kThreads, 0, s>>>(topo, kb, p.fixed, b.pairs, np, nullptr, b.vf_keys, b.ee_keys);
  BP_CUDA(cudaGetLastError());
  // Sort, mark the first of each run of equal keys, scan, decode.
  for (int which = 0; which < 2; which++) {
    uint64_t *keys = which == 0 ? b.vf_keys : b.ee_keys;
    const int64_t n = (which == 0 ? 6 : 9) * np;
    // One bit above the packed key so that kNoKey (all ones) sorts last.
    const int key_bits_used = which == 0 ? bits_for(std::max(topo.nv - 1, 1)) + kb.rbits : 2 * kb.ebits;
    BP_CUDA(radix_sort_u64(keys, b.keys_alt, nullptr, nullptr, n, 0, key_bits_used + 1, b.temp, b.temp_bytes, s));
    first_of_run<<<grid_of(n), kThreads, 0, s>>>(keys, n, b.flags);
    BP_CUDA(cudaGetLastError());
    uint32_t *total = (uint32_t *)(b.counters + 1 + which);
    BP_CUDA(exclusive_scan_u32(b.flags, b.scan, n, total, b.temp, b.temp_bytes, s));
    uint32_t count = 0;
    BP_CUDA(cudaMemcpyAsync(&count, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    BP_CUDA(cudaStreamSynchronize(s));
    if (which == 0) {
      BP_CUDA(grow(vf_out, vf_cap, 4 * (int64_t)count));
      decode_vf<<<grid_of(n), kThreads, 0, s>>>(topo, kb, keys, b.flags, b.scan, n, *vf_out, INT64_MAX);
      *n_vf = count;
    } else {
      BP_CUDA(grow(ee_out, ee_cap, 4 * (int64_t)count));
      decode_ee<<<grid_of(n), kThreads, 0, s>>>(topo, kb, keys, b.flags, b.scan, n, *ee_out, INT64_MAX);
      *n_ee = count;
    }
    BP_CUDA(cudaGetLastError());
  }
  if (p.ev[0]) BP_CUDA(cudaEventRecord(p.ev[3], s));
  BP_CUDA(cudaStreamSynchronize(s));
  return 0;
}


int broadphase_enqueue_refit(const MeshTopology &topo, const BroadphaseParams &p, BroadphaseBuffers &b,
                             int64_t cap_pairs, int32_t *vf_out, int64_t cap_vf, int32_t *ee_out, int64_t cap_ee,
                             int4 dummy, cudaStream_t s, cudaError_t *err) {
  const int nf = topo.nf;
  if (nf < 2 || b.tree_kind != p.kind || b.tree_nf != nf || b.tree_ninst != topo.ninst || cap_pairs > b.cap_pairs)
    return 5;
  const bool kdop = p.kind == kBvhKdop13;
  const Axes ax = make_axes();
  if (kdop)
    leaf_slabs<13><<<grid_of(nf), kThreads, 0, s>>>(topo, p, ax, b.lo64, b.hi64, b.face_lo, b.face_hi, b.bounds);
  else
    leaf_slabs<3><<<grid_of(nf), kThreads, 0, s>>>(topo, p, ax, b.lo64, b.hi64, b.face_lo, b.face_hi, b.bounds);
  const KeyBits kb = key_bits(topo);
  if (kdop)
    gather_leaves<13><<<grid_of(nf), kThreads, 0, s>>>(nf, b.keys, kb.fmask, b.face_lo, b.face_hi, b.leaf_box);
  else
    gather_leaves<3><<<grid_of(nf), kThreads, 0, s>>>(nf, b.keys, kb.fmask, b.face_lo, b.face_hi, b.leaf_box);
  BP_CUDA(cudaMemsetAsync(b.arrive, 0, (size_t)nf * sizeof(uint32_t), s));
  BP_CUDA(cudaMemsetAsync(b.counters, 0, 8 * sizeof(unsigned long long), s));
  if (kdop)
    refit<13><<<grid_of(nf), kThreads, 0, s>>>(nf, b.node_child, b.parent, b.arrive, b.leaf_box, b.node_box,
                                               b.counters);
  else
    refit<3><<<grid_of(nf), kThreads, 0, s>>>(nf, b.node_child, b.parent, b.arrive, b.leaf_box, b.node_box,
                                              b.counters);
  enqueue_traversal(topo, p, b, kb, (uint64_t)cap_pairs, s);
  stencil_keys<<<grid_of(cap_pairs), kThreads, 0, s>>>(topo, kb, p.fixed, b.pairs, cap_pairs, b.counters, b.vf_keys,
                                                       b.ee_keys);
  BP_CUDA(cudaGetLastError());
  for (int which = 0; which < 2; which++) {
    uint64_t *keys = which == 0 ? b.vf_keys : b.ee_keys;
    const int64_t n = (which == 0 ? 6 : 9) * cap_pairs;
    const int key_bits_used = which == 0 ? bits_for(std::max(topo.nv - 1, 1)) + kb.rbits : 2 * kb.ebits;
    BP_CUDA(radix_sort_u64(keys, b.keys_alt, nullptr, nullptr, n, 0, key_bits_used + 1, b.temp, b.temp_bytes, s));
    first_of_run<<<grid_of(n), kThreads, 0, s>>>(keys, n, b.flags);
    uint32_t *total = (uint32_t *)(b.counters + 1 + which);
    BP_CUDA(exclusive_scan_u32(b.flags, b.scan, n, total, b.temp, b.temp_bytes, s));
    int32_t *out = which == 0 ? vf_out : ee_out;
    const int64_t cap = which == 0 ? cap_vf : cap_ee;
    fill_stencils<<<grid_of(cap), kThreads, 0, s>>>(out, cap, dummy);
    if (which == 0)
      decode_vf<<<grid_of(n), kThreads, 0, s>>>(topo, kb, keys, b.flags, b.scan, n, out, cap);
    else
      decode_ee<<<grid_of(n), kThreads, 0, s>>>(topo, kb, keys, b.flags, b.scan, n, out, cap);
    BP_CUDA(cudaGetLastError());
  }
  return 0;
}

void point_tree_free(PointTreeBuffers &b) {
  void *ptrs[] = {b.pt_lo, b.pt_hi, b.leaf_box, b.node_box, b.node_child, b.node_range, b.parent, b.arrive, b.keys,
                  b.keys_alt, b.degree, b.off, b.list, b.bounds, b.counters, b.temp};
  for (void *p : ptrs) cudaFree(p);
  b = PointTreeBuffers{};
}

// Returns 0 on success, 2 on a CUDA error (*err), 3 on a malformed tree.
int closest_vertex_pair(int nv, int nf, const int32_t *faces, const double *x, PointTreeBuffers &b, double *d2,
                        cudaStream_t s, cudaError_t *err) {
  *d2 = INFINITY;
  if (nv < 2 || nf < 1) return 0;
  if (b.cap_verts < nv || b.cap_faces < nf) {
    point_tree_free(b);
    const size_t V = (size_t)nv, F = (size_t)nf;
    BP_CUDA(cudaMalloc(&b.pt_lo, 3 * V * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.pt_hi, 3 * V * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.leaf_box, 8 * V * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.node_box, 8 * V * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.node_child, 2 * V * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.node_range, 2 * V * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.parent, 2 * V * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.arrive, V * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.keys, V * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.keys_alt, V * sizeof(uint64_t)));
    BP_CUDA(cudaMalloc(&b.degree, V * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.off, (V + 1) * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&b.list, 3 * F * sizeof(int32_t)));
    BP_CUDA(cudaMalloc(&b.bounds, 8 * sizeof(float)));
    BP_CUDA(cudaMalloc(&b.counters, 8 * sizeof(unsigned long long)));
    b.temp_bytes = std::max(radix_sort_temp_bytes(nv), scan_temp_bytes(nv));
    BP_CUDA(cudaMalloc(&b.temp, b.temp_bytes));
    b.cap_verts = nv;
    b.cap_faces = nf;
  }
  // Incidence lists.
  BP_CUDA(cudaMemsetAsync(b.degree, 0, (size_t)nv * sizeof(uint32_t), s));
  incidence_count<<<grid_of(nf), kThreads, 0, s>>>(nf, faces, b.degree);
  BP_CUDA(cudaGetLastError());
  BP_CUDA(exclusive_scan_u32(b.degree, b.off, nv, b.off + nv, b.temp, b.temp_bytes, s));
  BP_CUDA(cudaMemsetAsync(b.degree, 0, (size_t)nv * sizeof(uint32_t), s));
  incidence_fill<<<grid_of(nf), kThreads, 0, s>>>(nf, faces, b.off, b.degree, b.list);
  BP_CUDA(cudaGetLastError());
  // Point tree over the far-end vertices.
  {
    const int pinf = 0x7f800000, ninf = (int)(0x80000000u - 0xff800000u);
    int hb[6] = {pinf, pinf, pinf, ninf, ninf, ninf};
    BP_CUDA(cudaMemcpyAsync(b.bounds, hb, sizeof(hb), cudaMemcpyHostToDevice, s));
    // counters[0]: the minimum's bits (+inf); [3]: error word
    unsigned long long hc[8] = {0x7ff0000000000000ull, 0, 0, 0, 0, 0, 0, 0};
    BP_CUDA(cudaMemcpyAsync(b.counters, hc, sizeof(hc), cudaMemcpyHostToDevice, s));
  }
  point_slabs<<<grid_of(nv), kThreads, 0, s>>>(nv, x, b.degree, b.pt_lo, b.pt_hi, b.bounds);
  BP_CUDA(cudaGetLastError());
  KeyBits kb{};
  kb.fbits = bits_for(nv - 1);
  kb.mbits = std::min(30, 63 - kb.fbits);
  kb.ishift = kb.mbits + kb.fbits;
  kb.fmask = ((uint64_t)1 << kb.fbits) - 1;
  morton_keys<<<grid_of(nv), kThreads, 0, s>>>(nv, b.pt_lo, b.pt_hi, b.bounds, nullptr, kb, b.keys);
  BP_CUDA(cudaGetLastError());
  BP_CUDA(radix_sort_u64(b.keys, b.keys_alt, nullptr, nullptr, nv, 0, kb.ishift, b.temp, b.temp_bytes, s));
  gather_leaves<3><<<grid_of(nv), kThreads, 0, s>>>(nv, b.keys, kb.fmask, b.pt_lo, b.pt_hi, b.leaf_box);
  build_lbvh<<<grid_of(nv - 1), kThreads, 0, s>>>(nv, b.keys, b.node_child, b.node_range, b.parent);
  BP_CUDA(cudaMemsetAsync(b.arrive, 0, (size_t)nv * sizeof(uint32_t), s));
  refit<3><<<grid_of(nv), kThreads, 0, s>>>(nv, b.node_child, b.parent, b.arrive, b.leaf_box, b.node_box,
                                            b.counters);
  BP_CUDA(cudaGetLastError());
  // Seed the bound, then search.
  pair_seed<<<grid_of(nv), kThreads, 0, s>>>(nv, b.keys, kb.fmask, x, b.off, b.list, faces, b.counters);
  pair_search<<<grid_of(nv), kThreads, 0, s>>>(nv, b.keys, kb.fmask, x, b.off, b.list, faces, b.node_child,
                                               b.leaf_box, b.node_box, b.counters, b.counters);
  BP_CUDA(cudaGetLastError());
  unsigned long long hc[4];
  BP_CUDA(cudaMemcpyAsync(hc, b.counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  BP_CUDA(cudaStreamSynchronize(s));
  if (hc[3]) return 3;
  double d;
  memcpy(&d, &hc[0], sizeof(d));
  *d2 = d;
  return 0;
}


// Returns 0, 2 on a CUDA error (*err), 4 when a stencil list would pass 2^31.
int trivial_candidates(const MeshTopology &topo, const uint8_t *fixed, int32_t **vf_out, int64_t *vf_cap,
                       int32_t **ee_out, int64_t *ee_cap, int64_t *n_vf, int64_t *n_ee, cudaStream_t s,
                       cudaError_t *err) {
  *n_vf = *n_ee = 0;
  const int64_t space[2] = {(int64_t)topo.nv * topo.nranks, (int64_t)topo.nedges * topo.nedges};
  const int64_t chunk = std::min<int64_t>(std::max(space[0], space[1]), (int64_t)1 << 26);
  if (chunk <= 0) return 0;
  uint32_t *flags = nullptr, *pos = nullptr, *total = nullptr;
  void *temp = nullptr;
  const size_t temp_bytes = scan_temp_bytes(chunk);
  int rc = 0;
  auto run = [&]() -> int {
    BP_CUDA(cudaMalloc(&flags, (size_t)chunk * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&pos, (size_t)chunk * sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&total, sizeof(uint32_t)));
    BP_CUDA(cudaMalloc(&temp, temp_bytes));
    for (int which = 0; which < 2; which++) {
      int32_t **out = which == 0 ? vf_out : ee_out;
      int64_t *cap = which == 0 ? vf_cap : ee_cap;
      // pass 0 counts, pass 1 writes
      int64_t n = 0;
      for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
          if (n >= ((int64_t)1 << 31)) return 4;
          BP_CUDA(grow(out, cap, 4 * std::max<int64_t>(n, 1)));
        }
        int64_t base = 0;
        for (int64_t begin = 0; begin < space[which]; begin += chunk) {
          const int64_t count = std::min(chunk, space[which] - begin);
          const unsigned grid = (unsigned)((count + kThreads - 1) / kThreads);
          trivial_flags<<<grid, kThreads, 0, s>>>(topo, fixed, which, begin, count, flags);
          BP_CUDA(cudaGetLastError());
          BP_CUDA(exclusive_scan_u32(flags, pos, count, total, temp, temp_bytes, s));
          if (pass == 1) {
            trivial_emit<<<grid, kThreads, 0, s>>>(topo, which, begin, count, flags, pos, base, *out);
            BP_CUDA(cudaGetLastError());
          }
          uint32_t h = 0;
          BP_CUDA(cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, s));
          BP_CUDA(cudaStreamSynchronize(s));
          base += h;
        }
        n = base;
      }
      *(which == 0 ? n_vf : n_ee) = n;
    }
    return 0;
  };
  rc = run();
  cudaFree(flags);
  cudaFree(pos);
  cudaFree(total);
  cudaFree(temp);
  return rc;
}

}  // namespace ccd
