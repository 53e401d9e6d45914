// Swept-volume candidate search on the GPU: the candidate set of the
// reference's KDOPBroadPhase / AABBBroadPhase::findCollisionCandidates
// (src/KDOPBroadPhase.cpp:34-185, src/AABBBroadPhase.cpp:9-152) on a
// two-entry history (start, end).
//
// The reference builds a median-split tree over per-face swept slabs and
// self-intersects it; a face pair is reached exactly when its two leaf slabs
// overlap on every axis (a parent's slab contains its children's), so the
// candidate set is a function of the leaf slabs alone.  Here:
//   1. leaf slabs in FP64 with the reference's arithmetic (pos . axis -+ eta,
//      min/max over 3 vertices x 2 history entries), plus outward-rounded FP32
//      copies (lower bounds rounded down, upper bounds up);
//   2. Morton codes of the FP32 slab centres, radix sort, Karras LBVH,
//      bottom-up refit of FP32 slabs (atomic arrival counters);
//   3. stack traversal per leaf over leaves later in Morton order with the
//      conservative FP32 test, then the reference's exact FP64 test
//      (strict '<' rejection) and neighbour exclusion (any shared vertex);
//   4. 6 vertex-face + 9 edge-edge stencils per pair (fixed-vertex filter),
//      as integer keys (vertex, face rank) and (edge rank, edge rank), packed
//      into as few bits as the mesh needs, whose order is the reference's
//      std::set order; radix sort over those bits + unique.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

enum BvhKind : int { kBvhKdop13 = 0, kBvhAabb = 1 };

// Static topology of a mesh, ranks computed on the host once per mesh.
struct MeshTopology {
  int32_t nv, nf;
  int32_t nranks, nedges;      // distinct sorted face triples, distinct edges
  const int32_t *faces;        // [nf][3]
  const int32_t *face_rank;    // [nf] rank of the face's sorted vertex triple
  const int32_t *rank_triple;  // [nranks][3] sorted triple of each face rank
  const int32_t *face_edges;   // [nf][3] rank of edge (v_i, v_{i+1 mod 3})
  const int32_t *rank_edge;    // [nedges][2] (a <= b) of each edge rank
  // Independent instances in one mesh (null / 1: a single mesh).  Faces of
  // different instances are never paired.
  const int32_t *face_inst;    // [nf] instance of each face
  int32_t ninst;
};

// Device buffers of one broad-phase call; grown by the caller.
struct BroadphaseBuffers {
  int64_t cap_faces = 0, cap_pairs = 0;
  // per face / node
  double *lo64 = nullptr, *hi64 = nullptr;        // [13][nf]
  float *face_lo = nullptr, *face_hi = nullptr;   // [13][nf]   outward-rounded FP32 slabs by face
  float *leaf_box = nullptr;                      // [nf][32]   slab records by sorted position
  float *node_box = nullptr;                      // [nf-1][32] internal nodes
  int32_t *node_child = nullptr;                  // [nf-1][2]  >= 0 internal, < 0 leaf ~s
  int32_t *node_range = nullptr;                  // [nf-1][2]  first, last sorted leaf
  int32_t *parent = nullptr;                      // [2 nf]     internal then leaves
  int4 *node_links = nullptr;                     // [nf-1]     children, first and last leaf of each node
  int4 *leaf_links = nullptr;                     // [nf]       face and its vertices of each sorted leaf
  int32_t *leaf_end = nullptr;                    // [nf]       first sorted leaf of a later instance
  uint32_t *arrive = nullptr;                     // [nf]
  uint64_t *keys = nullptr, *keys_alt = nullptr;  // [max(nf, 9 pairs)]
  uint32_t *vals = nullptr, *vals_alt = nullptr;  // [2 nf]: second Morton key buffer
  float *bounds = nullptr;                        // [6]
  unsigned long long *counters = nullptr;         // [8] pairs, vf, ee, overflow, slab tests
  uint32_t *pairs = nullptr;                      // [cap_pairs][2]
  uint64_t *vf_keys = nullptr, *ee_keys = nullptr;
  uint32_t *flags = nullptr, *scan = nullptr;
  void *temp = nullptr;
  size_t temp_bytes = 0;
  // The tree kept from the last call (leaf order, links) for refit-only
  // calls: valid for this kind, face count and instance count.
  int tree_kind = -1, tree_nf = 0, tree_ninst = 0;
  int refits = 0;            // refit-only calls since the last build
  float build_area = -1.0f;  // summed node surface after the last build (-1: not yet measured)
  bool rebuild_next = false;
};

// Traversal kernels: one thread per query leaf with a private stack (two
// register budgets: up to 112 registers, or 80 with three blocks per SM),
// one warp per 32 consecutive query leaves with a shared stack, or four lanes
// per query leaf, each testing a quarter of the slabs (13-DOP trees; AABB
// trees take the thread kernel), with two register budgets.
enum TraversalKind : int {
  kTraversalThread = 0,
  kTraversalPacket = 1,
  kTraversalThreadDense = 2,
  kTraversalQuad = 3,
  kTraversalQuadDense = 4
};

struct BroadphaseParams {
  int kind;
  double eta;
  const double *qs, *qe;  // [nv][3]: a two-entry history (start, end) ...
  const int32_t *hoff;    // ... or, when non-null, every entry: vertex v's are hoff[v] .. hoff[v+1]-1
  const double *hpos;     // [entries][3]
  const uint8_t *fixed;   // [nv] or null
  bool count_tests;       // count the traversal's slab tests (a slower, counting variant)
  int traversal;          // TraversalKind
  // Keep the last call's tree and only refit its node slabs when the mesh
  // and kind are unchanged, until the summed surface of its nodes grows by
  // more than rebuild_ratio over its value after the build (or max_refits
  // calls in a row).  The candidate set depends on the leaf slabs alone, so
  // this changes speed only.
  bool refit;
  float rebuild_ratio;
  int max_refits;
  cudaEvent_t ev[4];      // optional (all null or all set): start, before / after the traversal, end
};

// Runs the candidate search; on return (stream synchronised) n_vf / n_ee
// hold the counts and vf_out / ee_out (device, [n][4] int32) the stencils in
// the reference's order.  The output arrays are grown as needed.
// *rebuilt (optional) tells whether this call built its tree (or refitted
// the kept one).
int broadphase_run(const MeshTopology &topo, const BroadphaseParams &p, BroadphaseBuffers &buf, int32_t **vf_out,
                   int64_t *vf_cap, int32_t **ee_out, int64_t *ee_cap, int64_t *n_vf, int64_t *n_ee,
                   int64_t *n_pairs, int64_t *slab_tests, int num_sms, cudaStream_t s, cudaError_t *err,
                   bool *rebuilt = nullptr);

// The step of a captured graph: the same candidate search on the kept tree
// (refit only) with no host synchronisation, so that it can be captured.
// Pairs beyond cap_pairs are counted (counters[0]) but not written; the
// unique vertex-face / edge-edge counts go to counters[1] / counters[2] (as
// uint32), and vf_out / ee_out (capacities cap_vf / cap_ee stencils) hold the
// candidates in set order followed by copies of `dummy` up to the capacity.
// The caller compares the counts with the capacities afterwards.  Returns 0,
// 2 on a CUDA error (*err), 5 when no tree of this mesh and kind is kept or
// cap_pairs exceeds the pair buffers.
int broadphase_enqueue_refit(const MeshTopology &topo, const BroadphaseParams &p, BroadphaseBuffers &buf,
                             int64_t cap_pairs, int32_t *vf_out, int64_t cap_vf, int32_t *ee_out, int64_t cap_ee,
                             int4 dummy, cudaStream_t s, cudaError_t *err);

void broadphase_free(BroadphaseBuffers &buf);

// TrivialBroadPhase::findCollisionCandidates (src/TrivialBroadPhase.cpp:4-53):
// every vertex-face stencil of a vertex and a face without it and every
// edge-edge stencil of two edges without a common vertex, minus stencils
// whose four vertices are all fixed; positions and padding are not used.
// Same outputs as broadphase_run (synchronised on return).  Returns 0, 2 on
// a CUDA error (*err), 4 when a list would reach 2^31 stencils.
int trivial_candidates(const MeshTopology &topo, const uint8_t *fixed, int32_t **vf_out, int64_t *vf_cap,
                       int32_t **ee_out, int64_t *ee_cap, int64_t *n_vf, int64_t *n_ee, cudaStream_t s,
                       cudaError_t *err);

// Device buffers of the closest-vertex-pair search; grown by the caller.
struct PointTreeBuffers {
  int64_t cap_verts = 0, cap_faces = 0;
  float *pt_lo = nullptr, *pt_hi = nullptr;       // [3][nv] outward-rounded FP32 points (empty for non-far ends)
  float *leaf_box = nullptr, *node_box = nullptr; // [nv][8] point-tree records (AABB layout)
  int32_t *node_child = nullptr, *node_range = nullptr, *parent = nullptr;
  uint32_t *arrive = nullptr;
  uint64_t *keys = nullptr, *keys_alt = nullptr;  // Morton code << vbits | vertex
  uint32_t *degree = nullptr;                     // [nv] faces per vertex
  uint32_t *off = nullptr;                        // [nv + 1] incidence offsets
  int32_t *list = nullptr;                        // [<= 3 nf] faces of each vertex
  float *bounds = nullptr;
  unsigned long long *counters = nullptr;         // [0] minimum (bits of a double), [3] error word
  void *temp = nullptr;
  size_t temp_bytes = 0;
};

// The vertex scan of Distance::meshSelfDistance (src/Distance.cpp:21-34):
// *d2 = the least squared distance (x_i - x_v).squaredNorm(), in the
// reference's FP64 arithmetic, over vertex pairs (i, v) where some face
// contains v but not i; +inf when there is none.  x is [nv][3] on the device.
// Exact: a point LBVH with conservative FP32 bounds prunes only pairs whose
// FP64 squared distance exceeds the running minimum.  Returns 0, 2 on a CUDA
// error (*err), 3 on a malformed tree.
int closest_vertex_pair(int nv, int nf, const int32_t *faces, const double *x, PointTreeBuffers &buf, double *d2,
                        cudaStream_t s, cudaError_t *err);

void point_tree_free(PointTreeBuffers &buf);

}  // namespace ccd
