/* ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's continuous-time collision detection
 * path (evouga/collisiondetection): the primitive CTCD tests (src/CTCD.cpp),
 * the Jenkins-Traub root finder they use (src/rpoly.h), the swept k-DOP / AABB
 * candidate search (src/KDOPBroadPhase.cpp, src/AABBBroadPhase.cpp) and the
 * CTCD narrow phase over stencils (src/CTCDNarrowPhase.cpp) for the two-entry
 * (start, end) history.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only to check results.  It is pinned against the reference's
 * own sources (oracle/_ref, built from the reference tree by oracle/Makefile)
 * through the fixtures in tests/golden/.
 */
#ifndef CCD_ORACLE_H
#define CCD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Primitive tests; x holds the points in the reference's argument order
 * (include/CTCD.h:36-79): VF/EE 8 points (24 doubles), VE 6 (18), VV 4 (12).
 * Return 1 on a hit and write *t; on a miss *t is left untouched. */
int oracle_vf(const double *x, double eta, double *t);
int oracle_ee(const double *x, double eta, double *t);
int oracle_ve(const double *x, double eta, double *t);
int oracle_vv(const double *x, double eta, double *t);

/* Batched form over n primitives of one kind (0=VF 1=EE 2=VE 3=VV), using
 * nthreads host threads (<=1: the calling thread only).  eta has n entries
 * when eta_per_test, else one.  t[i] is written only where hit[i]==1. */
void oracle_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit, double *t,
                  int nthreads);

/* Swept-primitive candidate search.  kind 0 = 13-DOP (KDOPBroadPhase),
 * 1 = AABB (AABBBroadPhase), 2 = TrivialBroadPhase (every stencil of a
 * vertex and a face without it and of two edges without a common vertex;
 * positions and eta unused).  faces is F x 3 (row per face), fixed is NULL or
 * one byte per vertex.  Results are held until oracle_broadphase_get copies
 * them out (VF rows p,q0,q1,q2; EE rows p0,p1,q0,q1), in the reference's
 * std::set order.  Returns 0, or -1 on allocation failure. */
int oracle_broadphase(int kind, int nverts, const double *qstart, const double *qend, int nfaces,
                      const int32_t *faces, double eta, const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee);
void oracle_broadphase_get(int32_t *vf, int32_t *ee);
/* Number of non-neighbouring face pairs whose swept volumes overlap in the
 * last oracle_broadphase call. */
int64_t oracle_broadphase_face_pairs(void);

/* CTCD narrow phase over stencils (CTCDNarrowPhase::checkVFS / checkEES) on
 * the history qstart (t=0) -> qend (t=1).  hit[i] = stencil i collides;
 * t[i] = contact time reported by the first test in the chain that hit
 * (untouched on a miss); which[i] = 0 primitive (VF/EE), 1 vertex-edge,
 * 2 vertex-vertex, -1 miss.  Any of t / which may be NULL. */
void oracle_narrowphase(int nverts, const double *qstart, const double *qend, int64_t n_vf, const int32_t *vf,
                        const double *vf_eta, int64_t n_ee, const int32_t *ee, const double *ee_eta, uint8_t *vf_hit,
                        uint8_t *ee_hit, double *vf_t, double *ee_t, int8_t *vf_which, int8_t *ee_which,
                        int nthreads);

/* Distance (include/Distance.h): rows of 12 doubles, (p, q0, q1, q2) for
 * kind 0 and (p0, p1, q0, q1) for kind 1.  oracle_distance_batch:
 * vertexFaceDistance (0) / edgeEdgeDistance (1), vec [n][3], bary [n][3|4] or
 * NULL.  oracle_distance_less_than: vertexPlaneDistanceLessThan (0) /
 * lineLineDistanceLessThan (1). */
void oracle_distance_batch(int kind, int64_t n, const double *rows, double *vec, double *bary);
void oracle_distance_less_than(int kind, int64_t n, const double *rows, const double *eta, int eta_per_row,
                               uint8_t *out);
/* Distance::meshSelfDistance (src/Distance.cpp:12-66), its O(V F) vertex scan
 * included; n_vf / n_ee receive the stencil counts it checks (may be NULL). */
double oracle_mesh_self_distance(int nverts, const double *verts, int nfaces, const int32_t *faces,
                                 const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee);

/* That vertex scan alone over vertices [i0, i1): the least squared distance. */
double oracle_vertex_scan(int nverts, const double *verts, int nfaces, const int32_t *faces, int i0, int i1);

/* PenaltyGroup::addForce (src/PenaltyGroup.cpp:34-52) with the potentials of
 * src/PenaltyPotential.cpp:7-64: F += dt * group force; *_fired (may be NULL)
 * receive the per-stencil flags; returns newused (or -1 on allocation
 * failure). */
int oracle_penalty_group_force(int nverts, const double *q, const double *v, int64_t n_vf, const int32_t *vf,
                               const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee, const uint8_t *ee_isnew,
                               double outer_eta, double inner_eta, double stiffness, double cor, double dt,
                               double *F, uint8_t *vf_fired, uint8_t *ee_fired);

/* The same two phases on a multi-entry History (src/History.h): vertex v's
 * entries are offsets[v] .. offsets[v+1]-1 of times / positions ([E][3]).
 * The broad phase takes slabs over every entry; the narrow phase runs its
 * chain on every segment of each stencil's stitched common history
 * (History::stitchCommonHistory) and reports the first segment that hits. */
int oracle_broadphase_history(int kind, int nverts, const int32_t *offsets, const double *positions, int nfaces,
                              const int32_t *faces, double eta, const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee);
int oracle_narrowphase_history(int nverts, const int32_t *offsets, const double *times, const double *positions,
                               int64_t n_vf, const int32_t *vf, const double *vf_eta, int64_t n_ee, const int32_t *ee,
                               const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit, double *vf_t, double *ee_t,
                               int8_t *vf_which, int8_t *ee_which);

/* SeparatingPlaneNarrowPhase::findCollisions (src/SeparatingPlaneNarrowPhase.cpp)
 * on a multi-entry history: hit flags per stencil; *_status (may be NULL)
 * 1 where the stencil's interval recursion stalled (the reference recurses
 * until its stack overflows there) and was stopped, hit then 0.  Returns
 * the number of such stencils. */
int64_t oracle_separating_plane(int nverts, const int32_t *offsets, const double *times, const double *positions,
                                int64_t n_vf, const int32_t *vf, const double *vf_eta, int64_t n_ee,
                                const int32_t *ee, const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit,
                                uint8_t *vf_status, uint8_t *ee_status);

/* VelocityFilter::velocityFilter (src/VelocityFilter.cpp:15-87) with the
 * ActiveLayers it runs (src/ActiveLayers.cpp): returns the reference's value
 * (iterations >= 0, -1, -2, -3), or -4 when a separating-plane search stalls
 * (the reference overflows its stack there); qend is overwritten on success.
 * *events (may be NULL) receives the number of group firings. */
int oracle_velocity_filter(int nverts, const double *qstart, double *qend, int nfaces, const int32_t *faces,
                           const double *invmasses, double outer_eta, double inner_eta, double base_stiffness,
                           double base_substep, double cor, int max_rollbacks, int64_t *events);

/* Stencil canonical forms (src/Stencils.h): writes the canonical 4-tuple. */
void oracle_vf_canon(int p, int q0, int q1, int q2, int32_t *out);
void oracle_ee_canon(int p0, int p1, int q0, int q1, int32_t *out);

#ifdef __cplusplus
}
#endif
#endif
