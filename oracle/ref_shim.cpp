// ORACLE / TEST INFRASTRUCTURE ONLY.  Never linked into the product.
//
// extern "C" wrapper over the reference library's own, unmodified sources
// (src/CTCD.cpp, src/History.cpp, src/Mesh.cpp, src/KDOPBroadPhase.cpp,
// src/AABBBroadPhase.cpp, src/TrivialBroadPhase.cpp, src/CTCDNarrowPhase.cpp,
// src/Distance.cpp, src/PenaltyPotential.cpp, src/PenaltyGroup.cpp,
// src/SeparatingPlaneNarrowPhase.cpp, src/ActiveLayers.cpp,
// src/VelocityFilter.cpp), compiled by
// oracle/Makefile against the project-written Eigen-API subset.  It exists so
// that tests/golden/make_golden.py can pin the C restatement (ccd_oracle.c)
// against the reference itself.  The reference tree is only present in the
// development container, so this library is never built on the GPU host.
#include <stdint.h>

#include <set>
#include <vector>

#include "CTCD.h"
#include "CTCDNarrowPhase.h"
#include "Distance.h"
#include "PenaltyGroup.h"
#include "PenaltyPotential.h"
#include "SeparatingPlaneNarrowPhase.h"
#include "VelocityFilter.h"
#include "History.h"
#include "KDOPBroadPhase.h"
#include "Mesh.h"
#include "TrivialBroadPhase.h"

using Eigen::Vector3d;

// AABBBroadPhase.h and KDOPBroadPhase.h both define a class NodeComparator, so
// the AABB broad phase is driven from its own translation unit.
void ref_aabb_candidates(const History &h, const Mesh &m, double eta, std::set<VertexFaceStencil> &vfs,
                         std::set<EdgeEdgeStencil> &ees, const std::set<int> &fixedVerts);

static Vector3d v3(const double *p) { return Vector3d(p[0], p[1], p[2]); }

extern "C" {

// One call of each primitive test, argument order of include/CTCD.h:36-79.
// Returns hit (0/1); *t is written only on a hit, as in the reference.
int ref_vf(const double *x, double eta, double *t) {
  return CTCD::vertexFaceCTCD(v3(x + 0), v3(x + 3), v3(x + 6), v3(x + 9), v3(x + 12), v3(x + 15), v3(x + 18),
                              v3(x + 21), eta, *t);
}
int ref_ee(const double *x, double eta, double *t) {
  return CTCD::edgeEdgeCTCD(v3(x + 0), v3(x + 3), v3(x + 6), v3(x + 9), v3(x + 12), v3(x + 15), v3(x + 18),
                            v3(x + 21), eta, *t);
}
int ref_ve(const double *x, double eta, double *t) {
  return CTCD::vertexEdgeCTCD(v3(x + 0), v3(x + 3), v3(x + 6), v3(x + 9), v3(x + 12), v3(x + 15), eta, *t);
}
int ref_vv(const double *x, double eta, double *t) {
  return CTCD::vertexVertexCTCD(v3(x + 0), v3(x + 3), v3(x + 6), v3(x + 9), eta, *t);
}

// Batched form: kind 0=VF(24 doubles) 1=EE(24) 2=VE(18) 3=VV(12).
// eta has n entries when eta_per_test, else one.
void ref_batch(int kind, int64_t n, const double *x, const double *eta, int eta_per_test, uint8_t *hit,
               double *t) {
  static const int width[4] = {24, 24, 18, 12};
  for (int64_t i = 0; i < n; i++) {
    const double *xi = x + i * width[kind];
    double e = eta_per_test ? eta[i] : eta[0];
    int h = 0;
    switch (kind) {
      case 0: h = ref_vf(xi, e, &t[i]); break;
      case 1: h = ref_ee(xi, e, &t[i]); break;
      case 2: h = ref_ve(xi, e, &t[i]); break;
      default: h = ref_vv(xi, e, &t[i]); break;
    }
    hit[i] = (uint8_t)h;
  }
}

// ---------------------------------------------------------------- mesh path
static std::vector<int32_t> g_vf, g_ee;

static void build_mesh(int nverts, const double *q, int nfaces, const int32_t *faces, Mesh &m) {
  m.vertices.resize(3 * nverts);
  for (int i = 0; i < 3 * nverts; i++) m.vertices[i] = q[i];
  m.faces.resize(3, nfaces);
  for (int f = 0; f < nfaces; f++)
    for (int j = 0; j < 3; j++) m.faces.coeffRef(j, f) = faces[3 * f + j];
}

static Eigen::VectorXd vecx(int nverts, const double *q) {
  Eigen::VectorXd v(3 * nverts);
  for (int i = 0; i < 3 * nverts; i++) v[i] = q[i];
  return v;
}

// Runs KDOPBroadPhase (kind 0), AABBBroadPhase (kind 1) or TrivialBroadPhase
// (kind 2) on the 2-entry
// history (qstart at t=0, qend at t=1).  fixed may be NULL.  Results are kept
// until ref_broadphase_get copies them out, in std::set iteration order.
void ref_broadphase(int kind, int nverts, const double *qstart, const double *qend, int nfaces, const int32_t *faces,
                    double eta, const uint8_t *fixed, int64_t *n_vf, int64_t *n_ee) {
  Mesh m;
  build_mesh(nverts, qstart, nfaces, faces, m);
  History h(vecx(nverts, qstart));
  h.finishHistory(vecx(nverts, qend));
  std::set<int> fixedVerts;
  if (fixed)
    for (int i = 0; i < nverts; i++)
      if (fixed[i]) fixedVerts.insert(i);
  std::set<VertexFaceStencil> vfs;
  std::set<EdgeEdgeStencil> ees;
  if (kind == 0) {
    KDOPBroadPhase bp;
    bp.findCollisionCandidates(h, m, eta, vfs, ees, fixedVerts);
  } else if (kind == 2) {
    TrivialBroadPhase bp;
    bp.findCollisionCandidates(h, m, eta, vfs, ees, fixedVerts);
  } else {
    ref_aabb_candidates(h, m, eta, vfs, ees, fixedVerts);
  }
  g_vf.clear();
  g_ee.clear();
  for (std::set<VertexFaceStencil>::const_iterator it = vfs.begin(); it != vfs.end(); ++it) {
    g_vf.push_back(it->p); g_vf.push_back(it->q0); g_vf.push_back(it->q1); g_vf.push_back(it->q2);
  }
  for (std::set<EdgeEdgeStencil>::const_iterator it = ees.begin(); it != ees.end(); ++it) {
    g_ee.push_back(it->p0); g_ee.push_back(it->p1); g_ee.push_back(it->q0); g_ee.push_back(it->q1);
  }
  *n_vf = (int64_t)(g_vf.size() / 4);
  *n_ee = (int64_t)(g_ee.size() / 4);
}

void ref_broadphase_get(int32_t *vf, int32_t *ee) {
  for (size_t i = 0; i < g_vf.size(); i++) vf[i] = g_vf[i];
  for (size_t i = 0; i < g_ee.size(); i++) ee[i] = g_ee[i];
}

// CTCDNarrowPhase::findCollisions over canonical stencils with per-stencil eta;
// hit[i] = whether stencil i is in the returned set.
void ref_narrowphase(int nverts, const double *qstart, const double *qend, int64_t n_vf, const int32_t *vf,
                     const double *vf_eta, int64_t n_ee, const int32_t *ee, const double *ee_eta, uint8_t *vf_hit,
                     uint8_t *ee_hit) {
  History h(vecx(nverts, qstart));
  h.finishHistory(vecx(nverts, qend));
  std::set<std::pair<VertexFaceStencil, double> > cvf;
  std::set<std::pair<EdgeEdgeStencil, double> > cee;
  for (int64_t i = 0; i < n_vf; i++)
    cvf.insert(std::make_pair(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]), vf_eta[i]));
  for (int64_t i = 0; i < n_ee; i++)
    cee.insert(std::make_pair(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]), ee_eta[i]));
  std::set<VertexFaceStencil> ovf;
  std::set<EdgeEdgeStencil> oee;
  CTCDNarrowPhase np;
  np.findCollisions(h, cvf, cee, ovf, oee);
  for (int64_t i = 0; i < n_vf; i++)
    vf_hit[i] = (uint8_t)ovf.count(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]));
  for (int64_t i = 0; i < n_ee; i++)
    ee_hit[i] = (uint8_t)oee.count(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]));
}

// ---------------------------------------------------------------- distances
// Distance::vertexFaceDistance (kind 0) / edgeEdgeDistance (kind 1) over rows
// of 12 doubles; vec [n][3], bary [n][3|4].
void ref_distance_batch(int kind, int64_t n, const double *x, double *vec, double *bary) {
  for (int64_t i = 0; i < n; i++) {
    const double *r = x + 12 * i;
    Vector3d v;
    if (kind == 0) {
      double *b = bary + 3 * i;
      v = Distance::vertexFaceDistance(v3(r), v3(r + 3), v3(r + 6), v3(r + 9), b[0], b[1], b[2]);
    } else {
      double *b = bary + 4 * i;
      v = Distance::edgeEdgeDistance(v3(r), v3(r + 3), v3(r + 6), v3(r + 9), b[0], b[1], b[2], b[3]);
    }
    for (int k = 0; k < 3; k++) vec[3 * i + k] = v[k];
  }
}

// Distance::vertexPlaneDistanceLessThan (kind 0) / lineLineDistanceLessThan (kind 1).
void ref_distance_less_than(int kind, int64_t n, const double *x, const double *eta, int eta_per_row, uint8_t *out) {
  for (int64_t i = 0; i < n; i++) {
    const double *r = x + 12 * i;
    const double e = eta_per_row ? eta[i] : eta[0];
    out[i] = (uint8_t)(kind == 0 ? Distance::vertexPlaneDistanceLessThan(v3(r), v3(r + 3), v3(r + 6), v3(r + 9), e)
                                 : Distance::lineLineDistanceLessThan(v3(r), v3(r + 3), v3(r + 6), v3(r + 9), e));
  }
}

// Distance::meshSelfDistance (src/Distance.cpp:12-66); fixed may be NULL.
double ref_mesh_self_distance(int nverts, const double *q, int nfaces, const int32_t *faces, const uint8_t *fixed) {
  Mesh m;
  build_mesh(nverts, q, nfaces, faces, m);
  std::set<int> fixedVerts;
  if (fixed)
    for (int i = 0; i < nverts; i++)
      if (fixed[i]) fixedVerts.insert(i);
  return Distance::meshSelfDistance(vecx(nverts, q), m.faces, fixedVerts);
}

// ---------------------------------------------------------------- multi-entry history
// A History built through the reference's own API: the constructor takes each
// vertex's first entry (time 0), addHistory the others in order.
static History *make_history(int nverts, const int32_t *off, const double *times, const double *pos) {
  Eigen::VectorXd q0(3 * nverts);
  for (int v = 0; v < nverts; v++)
    for (int k = 0; k < 3; k++) q0[3 * v + k] = pos[3 * (size_t)off[v] + k];
  History *h = new History(q0);
  for (int v = 0; v < nverts; v++)
    for (int e = off[v] + 1; e < off[v + 1]; e++) h->addHistory(v, times[e], v3(pos + 3 * (size_t)e));
  return h;
}

void ref_broadphase_history(int kind, int nverts, const int32_t *off, const double *times, const double *pos,
                            int nfaces, const int32_t *faces, double eta, const uint8_t *fixed, int64_t *n_vf,
                            int64_t *n_ee) {
  History *h = make_history(nverts, off, times, pos);
  Mesh m;
  std::vector<double> q0(3 * (size_t)nverts);
  for (int v = 0; v < nverts; v++)
    for (int k = 0; k < 3; k++) q0[3 * (size_t)v + k] = pos[3 * (size_t)off[v] + k];
  build_mesh(nverts, q0.data(), nfaces, faces, m);
  std::set<int> fixedVerts;
  if (fixed)
    for (int i = 0; i < nverts; i++)
      if (fixed[i]) fixedVerts.insert(i);
  std::set<VertexFaceStencil> vfs;
  std::set<EdgeEdgeStencil> ees;
  if (kind == 0) {
    KDOPBroadPhase bp;
    bp.findCollisionCandidates(*h, m, eta, vfs, ees, fixedVerts);
  } else {
    ref_aabb_candidates(*h, m, eta, vfs, ees, fixedVerts);
  }
  delete h;
  g_vf.clear();
  g_ee.clear();
  for (std::set<VertexFaceStencil>::const_iterator it = vfs.begin(); it != vfs.end(); ++it) {
    g_vf.push_back(it->p); g_vf.push_back(it->q0); g_vf.push_back(it->q1); g_vf.push_back(it->q2);
  }
  for (std::set<EdgeEdgeStencil>::const_iterator it = ees.begin(); it != ees.end(); ++it) {
    g_ee.push_back(it->p0); g_ee.push_back(it->p1); g_ee.push_back(it->q0); g_ee.push_back(it->q1);
  }
  *n_vf = (int64_t)(g_vf.size() / 4);
  *n_ee = (int64_t)(g_ee.size() / 4);
}

void ref_narrowphase_history(int nverts, const int32_t *off, const double *times, const double *pos, int64_t n_vf,
                             const int32_t *vf, const double *vf_eta, int64_t n_ee, const int32_t *ee,
                             const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit) {
  History *h = make_history(nverts, off, times, pos);
  std::set<std::pair<VertexFaceStencil, double> > cvf;
  std::set<std::pair<EdgeEdgeStencil, double> > cee;
  for (int64_t i = 0; i < n_vf; i++)
    cvf.insert(std::make_pair(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]), vf_eta[i]));
  for (int64_t i = 0; i < n_ee; i++)
    cee.insert(std::make_pair(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]), ee_eta[i]));
  std::set<VertexFaceStencil> ovf;
  std::set<EdgeEdgeStencil> oee;
  CTCDNarrowPhase np;
  np.findCollisions(*h, cvf, cee, ovf, oee);
  delete h;
  for (int64_t i = 0; i < n_vf; i++)
    vf_hit[i] = (uint8_t)ovf.count(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]));
  for (int64_t i = 0; i < n_ee; i++)
    ee_hit[i] = (uint8_t)oee.count(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]));
}

// SeparatingPlaneNarrowPhase::findCollisions on a history built as above.
void ref_separating_plane(int nverts, const int32_t *off, const double *times, const double *pos, int64_t n_vf,
                          const int32_t *vf, const double *vf_eta, int64_t n_ee, const int32_t *ee,
                          const double *ee_eta, uint8_t *vf_hit, uint8_t *ee_hit) {
  History *h = make_history(nverts, off, times, pos);
  std::set<std::pair<VertexFaceStencil, double> > cvf;
  std::set<std::pair<EdgeEdgeStencil, double> > cee;
  for (int64_t i = 0; i < n_vf; i++)
    cvf.insert(std::make_pair(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]), vf_eta[i]));
  for (int64_t i = 0; i < n_ee; i++)
    cee.insert(std::make_pair(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]), ee_eta[i]));
  std::set<VertexFaceStencil> ovf;
  std::set<EdgeEdgeStencil> oee;
  SeparatingPlaneNarrowPhase np;
  np.findCollisions(*h, cvf, cee, ovf, oee);
  delete h;
  for (int64_t i = 0; i < n_vf; i++)
    vf_hit[i] = (uint8_t)ovf.count(VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]));
  for (int64_t i = 0; i < n_ee; i++)
    ee_hit[i] = (uint8_t)oee.count(EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]));
}

// ---------------------------------------------------------------- velocity filter
// VelocityFilter::velocityFilter (src/VelocityFilter.cpp:15-87); qend is
// overwritten, the return value is the reference's.
int ref_velocity_filter(int nverts, const double *qstart, double *qend, int nfaces, const int32_t *faces,
                        const double *invmasses, double outer_eta, double inner_eta, double base_stiffness,
                        double base_substep, double cor, int max_rollbacks) {
  Mesh m;
  build_mesh(nverts, qstart, nfaces, faces, m);
  Eigen::VectorXd q1 = vecx(nverts, qstart), q2 = vecx(nverts, qend), minv = vecx(nverts, invmasses);
  const int r = VelocityFilter::velocityFilter(q1, q2, m.faces, minv, outer_eta, inner_eta, base_stiffness,
                                               base_substep, cor, max_rollbacks);
  for (int i = 0; i < 3 * nverts; i++) qend[i] = q2[i];
  return r;
}

// ---------------------------------------------------------------- penalty forces
// PenaltyGroup::addForce on one group built from the given stencils (with
// their isnew flags); F is updated in place; *_fired from the potentials'
// own addForce on a scratch vector.  Returns newused.
int ref_penalty_group_force(int nverts, const double *q, const double *v, int64_t n_vf, const int32_t *vf,
                            const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee, const uint8_t *ee_isnew,
                            double outer_eta, double inner_eta, double stiffness, double cor, double dt, double *F,
                            uint8_t *vf_fired, uint8_t *ee_fired) {
  Eigen::VectorXd Q = vecx(nverts, q), Vv = vecx(nverts, v), FF = vecx(nverts, F), scratch(3 * nverts);
  PenaltyGroup g(dt, outer_eta, inner_eta, stiffness, cor);
  for (int64_t i = 0; i < n_vf; i++) {
    VertexFaceStencil st(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]);
    st.isnew = vf_isnew ? vf_isnew[i] != 0 : false;
    g.addVFStencil(st);
    scratch.setZero();
    vf_fired[i] = (uint8_t)VertexFacePenaltyPotential::addForce(Q, Vv, scratch, st, outer_eta, inner_eta, stiffness,
                                                                 cor);
  }
  for (int64_t i = 0; i < n_ee; i++) {
    EdgeEdgeStencil st(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]);
    st.isnew = ee_isnew ? ee_isnew[i] != 0 : false;
    g.addEEStencil(st);
    scratch.setZero();
    ee_fired[i] = (uint8_t)EdgeEdgePenaltyPotential::addForce(Q, Vv, scratch, st, outer_eta, inner_eta, stiffness,
                                                               cor);
  }
  const bool used = g.addForce(Q, Vv, FF);
  for (int i = 0; i < 3 * nverts; i++) F[i] = FF[i];
  return used ? 1 : 0;
}

}  // extern "C"
