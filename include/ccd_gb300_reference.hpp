// Drop-in adapters between the reference's C++ types (evouga/collisiondetection)
// and the C ABI of libccd_gb300.so (ccd_gb300.h).  Header-only; compiled
// inside the reference's own build, with its headers (CTCD.h, History.h,
// Mesh.h, Stencils.h, RetrospectiveDetection.h) and Eigen on the include path.
//
//   ccd_gb300::vertexFaceCTCD ... vertexVertexCTCD
//       same signatures and results as the CTCD statics (include/CTCD.h:36-79);
//       the body of each CTCD static can forward to them
//   ccd_gb300::GpuKDOPBroadPhase, ccd_gb300::GpuAABBBroadPhase : BroadPhase
//       findCollisionCandidates (src/RetrospectiveDetection.h:13)
//   ccd_gb300::GpuCTCDNarrowPhase : NarrowPhase
//       findCollisions (src/RetrospectiveDetection.h:20), CTCDNarrowPhase's results
//
// The GPU path covers histories of two entries per vertex (start at time 0,
// end at time 1: History(qstart) + finishHistory(qend)); a longer history
// raises std::runtime_error.  Errors of the C ABI raise std::runtime_error
// with the library's message.
#ifndef CCD_GB300_REFERENCE_HPP
#define CCD_GB300_REFERENCE_HPP

#include <stdint.h>

#include <algorithm>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "CTCD.h"
#include "History.h"
#include "Mesh.h"
#include "RetrospectiveDetection.h"
#include "Stencils.h"
#include "ccd_gb300.h"

namespace ccd_gb300 {

inline void check(ccd_context *ctx, int rc, const char *what) {
  if (rc != CCD_OK)
    throw std::runtime_error(std::string(what) + ": " + ccd_status_string(rc) + ": " + ccd_last_error(ctx));
}

// One process-wide context on device 0, created on first use.
inline ccd_context *default_context() {
  static ccd_context *ctx = [] {
    ccd_context *c = nullptr;
    const int rc = ccd_context_create(0, &c);
    if (rc != CCD_OK) throw std::runtime_error(std::string("ccd_context_create: ") + ccd_status_string(rc));
    return c;
  }();
  return ctx;
}

inline void put(double *dst, const Eigen::Vector3d &v) {
  dst[0] = v[0];
  dst[1] = v[1];
  dst[2] = v[2];
}

// ------------------------------------------------------------------ CTCD statics
inline bool edgeEdgeCTCD(const Eigen::Vector3d &q0start, const Eigen::Vector3d &p0start,
                         const Eigen::Vector3d &q1start, const Eigen::Vector3d &p1start,
                         const Eigen::Vector3d &q0end, const Eigen::Vector3d &p0end, const Eigen::Vector3d &q1end,
                         const Eigen::Vector3d &p1end, double eta, double &t) {
  double x[24];
  const Eigen::Vector3d *pts[8] = {&q0start, &p0start, &q1start, &p1start, &q0end, &p0end, &q1end, &p1end};
  for (int i = 0; i < 8; i++) put(x + 3 * i, *pts[i]);
  int hit = 0;
  check(default_context(), ccd_edge_edge_ctcd(default_context(), x, eta, &hit, &t), "ccd_edge_edge_ctcd");
  return hit != 0;
}

inline bool vertexFaceCTCD(const Eigen::Vector3d &q0start, const Eigen::Vector3d &q1start,
                           const Eigen::Vector3d &q2start, const Eigen::Vector3d &q3start,
                           const Eigen::Vector3d &q0end, const Eigen::Vector3d &q1end, const Eigen::Vector3d &q2end,
                           const Eigen::Vector3d &q3end, double eta, double &t) {
  double x[24];
  const Eigen::Vector3d *pts[8] = {&q0start, &q1start, &q2start, &q3start, &q0end, &q1end, &q2end, &q3end};
  for (int i = 0; i < 8; i++) put(x + 3 * i, *pts[i]);
  int hit = 0;
  check(default_context(), ccd_vertex_face_ctcd(default_context(), x, eta, &hit, &t), "ccd_vertex_face_ctcd");
  return hit != 0;
}

inline bool vertexEdgeCTCD(const Eigen::Vector3d &q0start, const Eigen::Vector3d &q1start,
                           const Eigen::Vector3d &q2start, const Eigen::Vector3d &q0end, const Eigen::Vector3d &q1end,
                           const Eigen::Vector3d &q2end, double eta, double &t) {
  double x[18];
  const Eigen::Vector3d *pts[6] = {&q0start, &q1start, &q2start, &q0end, &q1end, &q2end};
  for (int i = 0; i < 6; i++) put(x + 3 * i, *pts[i]);
  int hit = 0;
  check(default_context(), ccd_vertex_edge_ctcd(default_context(), x, eta, &hit, &t), "ccd_vertex_edge_ctcd");
  return hit != 0;
}

inline bool vertexVertexCTCD(const Eigen::Vector3d &q1start, const Eigen::Vector3d &q2start,
                             const Eigen::Vector3d &q1end, const Eigen::Vector3d &q2end, double eta, double &t) {
  double x[12];
  const Eigen::Vector3d *pts[4] = {&q1start, &q2start, &q1end, &q2end};
  for (int i = 0; i < 4; i++) put(x + 3 * i, *pts[i]);
  int hit = 0;
  check(default_context(), ccd_vertex_vertex_ctcd(default_context(), x, eta, &hit, &t), "ccd_vertex_vertex_ctcd");
  return hit != 0;
}

// ------------------------------------------------------------------ Distance statics
// The reference's Distance class (include/Distance.h) with the same
// signatures, evaluated on the device with bit-identical results.  Reference
// arguments written in order, so aliased outputs (meshSelfDistance passes
// t, t, t) end with the same value as in the reference.
inline Eigen::Vector3d vertexFaceDistance(const Eigen::Vector3d &p, const Eigen::Vector3d &q0,
                                          const Eigen::Vector3d &q1, const Eigen::Vector3d &q2, double &q0bary,
                                          double &q1bary, double &q2bary) {
  double x[12], v[3], b[3];
  put(x, p), put(x + 3, q0), put(x + 6, q1), put(x + 9, q2);
  check(default_context(), ccd_distance_batch(default_context(), CCD_DISTANCE_VERTEX_FACE, 1, x, v, b),
        "ccd_distance_batch");
  q0bary = b[0];
  q1bary = b[1];
  q2bary = b[2];
  return Eigen::Vector3d(v[0], v[1], v[2]);
}

inline Eigen::Vector3d edgeEdgeDistance(const Eigen::Vector3d &p0, const Eigen::Vector3d &p1,
                                        const Eigen::Vector3d &q0, const Eigen::Vector3d &q1, double &p0bary,
                                        double &p1bary, double &q0bary, double &q1bary) {
  double x[12], v[3], b[4];
  put(x, p0), put(x + 3, p1), put(x + 6, q0), put(x + 9, q1);
  check(default_context(), ccd_distance_batch(default_context(), CCD_DISTANCE_EDGE_EDGE, 1, x, v, b),
        "ccd_distance_batch");
  p0bary = b[0];
  p1bary = b[1];
  q0bary = b[2];
  q1bary = b[3];
  return Eigen::Vector3d(v[0], v[1], v[2]);
}

inline bool vertexPlaneDistanceLessThan(const Eigen::Vector3d &p, const Eigen::Vector3d &q0,
                                        const Eigen::Vector3d &q1, const Eigen::Vector3d &q2, double eta) {
  double x[12];
  uint8_t out = 0;
  put(x, p), put(x + 3, q0), put(x + 6, q1), put(x + 9, q2);
  check(default_context(),
        ccd_distance_less_than_batch(default_context(), CCD_DISTANCE_VERTEX_PLANE, 1, x, &eta, 1, &out),
        "ccd_distance_less_than_batch");
  return out != 0;
}

inline bool lineLineDistanceLessThan(const Eigen::Vector3d &p0, const Eigen::Vector3d &p1,
                                     const Eigen::Vector3d &q0, const Eigen::Vector3d &q1, double eta) {
  double x[12];
  uint8_t out = 0;
  put(x, p0), put(x + 3, p1), put(x + 6, q0), put(x + 9, q1);
  check(default_context(),
        ccd_distance_less_than_batch(default_context(), CCD_DISTANCE_LINE_LINE, 1, x, &eta, 1, &out),
        "ccd_distance_less_than_batch");
  return out != 0;
}

// Distance::meshSelfDistance (src/Distance.cpp:12-66).  The reference also
// prints the numbers of stencils it checks; ccd_mesh_self_distance returns
// them instead.
inline double meshSelfDistance(const Eigen::VectorXd &verts, const Eigen::Matrix3Xi &faces,
                               const std::set<int> &fixedVerts) {
  const int nv = (int)(verts.size() / 3), nf = (int)faces.cols();
  std::vector<double> x((size_t)3 * nv);
  for (int i = 0; i < 3 * nv; i++) x[(size_t)i] = verts[i];
  std::vector<int32_t> f((size_t)3 * nf);
  for (int c = 0; c < nf; c++)
    for (int j = 0; j < 3; j++) f[(size_t)3 * c + j] = faces.coeff(j, c);
  std::vector<uint8_t> fixed((size_t)nv, 0);
  for (std::set<int>::const_iterator it = fixedVerts.begin(); it != fixedVerts.end(); ++it)
    if (*it >= 0 && *it < nv) fixed[(size_t)*it] = 1;
  double d = 0;
  check(default_context(),
        ccd_self_distance(default_context(), nv, x.data(), nf, f.data(), fixedVerts.empty() ? nullptr : fixed.data(),
                          &d),
        "ccd_self_distance");
  return d;
}

// ------------------------------------------------------------------ velocity filter
// VelocityFilter::velocityFilter (include/VelocityFilter.h:45-46) with the
// same signature and return values; qend is overwritten as the reference
// does.  The active layers, broad phase and narrow phase run on the device.
inline int velocityFilter(const Eigen::VectorXd &qstart, Eigen::VectorXd &qend, const Eigen::Matrix3Xi &faces,
                          const Eigen::VectorXd &masses, double outerEta, double innerEta,
                          double baseStiffness = .0001, double baseSubstepSize = 0.0001, double CoR = 0.1,
                          int maxRollbacks = 1000) {
  const int nv = (int)(qstart.size() / 3), nf = (int)faces.cols();
  std::vector<double> qs(qstart.data(), qstart.data() + 3 * nv), qe(qend.data(), qend.data() + 3 * nv),
      mi(masses.data(), masses.data() + 3 * nv);
  std::vector<int32_t> f((size_t)3 * nf);
  for (int c = 0; c < nf; c++)
    for (int j = 0; j < 3; j++) f[(size_t)3 * c + j] = faces.coeff(j, c);
  int32_t result = 0;
  check(default_context(),
        ccd_velocity_filter(default_context(), nv, qs.data(), qe.data(), nf, f.data(), mi.data(), outerEta, innerEta,
                            baseStiffness, baseSubstepSize, CoR, maxRollbacks, &result, nullptr),
        "ccd_velocity_filter");
  if (result >= 0)
    for (int i = 0; i < 3 * nv; i++) qend[i] = qe[(size_t)i];
  return result;
}

// ------------------------------------------------------------------ penalty groups
// PenaltyGroup (src/PenaltyGroup.h) with the same interface; addForce runs on
// the device (ccd_penalty_group_force) with bit-identical forces.
class GpuPenaltyGroup {
 public:
  GpuPenaltyGroup(double dt, double outerEta, double innerEta, double stiffness, double CoR)
      : nextstep_(1), dt_(dt), outerEta_(outerEta), innerEta_(innerEta), stiffness_(stiffness), CoR_(CoR) {}

  void addVFStencil(VertexFaceStencil stencil) {
    vf_.push_back(stencil);
    groupStencil_.insert(stencil.p);
    groupStencil_.insert(stencil.q0);
    groupStencil_.insert(stencil.q1);
    groupStencil_.insert(stencil.q2);
  }
  void addEEStencil(EdgeEdgeStencil stencil) {
    ee_.push_back(stencil);
    groupStencil_.insert(stencil.p0);
    groupStencil_.insert(stencil.p1);
    groupStencil_.insert(stencil.q0);
    groupStencil_.insert(stencil.q1);
  }
  bool addForce(const Eigen::VectorXd &q, const Eigen::VectorXd &v, Eigen::VectorXd &F) {
    const int nv = (int)(q.size() / 3);
    std::vector<int32_t> vf(4 * vf_.size()), ee(4 * ee_.size());
    std::vector<uint8_t> vfn(vf_.size()), een(ee_.size());
    for (size_t i = 0; i < vf_.size(); i++) {
      vf[4 * i] = vf_[i].p, vf[4 * i + 1] = vf_[i].q0, vf[4 * i + 2] = vf_[i].q1, vf[4 * i + 3] = vf_[i].q2;
      vfn[i] = vf_[i].isnew ? 1 : 0;
    }
    for (size_t i = 0; i < ee_.size(); i++) {
      ee[4 * i] = ee_[i].p0, ee[4 * i + 1] = ee_[i].p1, ee[4 * i + 2] = ee_[i].q0, ee[4 * i + 3] = ee_[i].q1;
      een[i] = ee_[i].isnew ? 1 : 0;
    }
    std::vector<double> qq(q.data(), q.data() + 3 * nv), vv(v.data(), v.data() + 3 * nv),
        ff(F.data(), F.data() + 3 * nv);
    int used = 0;
    check(default_context(),
          ccd_penalty_group_force(default_context(), nv, qq.data(), vv.data(), (int64_t)vf_.size(), vf.data(),
                                  vfn.data(), (int64_t)ee_.size(), ee.data(), een.data(), outerEta_, innerEta_,
                                  stiffness_, CoR_, dt_, ff.data(), nullptr, nullptr, &used),
          "ccd_penalty_group_force");
    for (int i = 0; i < 3 * nv; i++) F[i] = ff[(size_t)i];
    return used != 0;
  }
  void incrementTimeStep() { nextstep_++; }
  double nextFireTime() const { return nextstep_ * dt_; }
  void rollback() {
    nextstep_ = 1;
    for (size_t i = 0; i < vf_.size(); i++) vf_[i].isnew = false;
    for (size_t i = 0; i < ee_.size(); i++) ee_[i].isnew = false;
  }
  double getDt() { return dt_; }
  double getOuterEta() { return outerEta_; }
  const std::set<int> &getGroupStencil() { return groupStencil_; }

 private:
  GpuPenaltyGroup(const GpuPenaltyGroup &);
  GpuPenaltyGroup &operator=(const GpuPenaltyGroup &);
  std::vector<VertexFaceStencil> vf_;
  std::vector<EdgeEdgeStencil> ee_;
  std::set<int> groupStencil_;
  int nextstep_;
  double dt_, outerEta_, innerEta_, stiffness_, CoR_;
};

// ------------------------------------------------------------------ meshes
// A device mesh that follows the faces of the reference Mesh it is given:
// re-created when the topology changes, positions uploaded on every call.
class DeviceMesh {
 public:
  explicit DeviceMesh(ccd_context *ctx = default_context()) : ctx_(ctx) {}
  ~DeviceMesh() { ccd_mesh_destroy(mesh_); }
  DeviceMesh(const DeviceMesh &) = delete;
  DeviceMesh &operator=(const DeviceMesh &) = delete;

  // Uploads faces (if changed), the two history entries and the fixed set.
  ccd_mesh *sync(const History &h, const Mesh &m, const std::set<int> *fixedVerts) {
    const int nf = (int)m.faces.cols();
    std::vector<int32_t> faces(3 * (size_t)nf);
    for (int f = 0; f < nf; f++)
      for (int j = 0; j < 3; j++) faces[3 * (size_t)f + j] = m.faces.coeff(j, f);
    const int nv = (int)(m.vertices.size() / 3);
    if (!mesh_ || faces != faces_ || nv != nv_) {
      ccd_mesh_destroy(mesh_);
      mesh_ = nullptr;
      check(ctx_, ccd_mesh_create(ctx_, nv, nf, faces.data(), &mesh_), "ccd_mesh_create");
      faces_.swap(faces);
      nv_ = nv;
    }
    qs_.resize(3 * (size_t)nv);
    qe_.resize(3 * (size_t)nv);
    for (int v = 0; v < nv; v++) {
      const std::vector<HistoryEntry> &e = h.getVertexHistory(v);
      if (e.size() != 2) throw std::runtime_error("ccd_gb300: only two-entry histories (start, end) are supported");
      put(&qs_[3 * (size_t)v], e.front().pos);
      put(&qe_[3 * (size_t)v], e.back().pos);
    }
    check(ctx_, ccd_mesh_set_positions(mesh_, qs_.data(), qe_.data()), "ccd_mesh_set_positions");
    if (fixedVerts) {
      std::vector<uint8_t> fx((size_t)nv, 0);
      bool any = false;
      for (int v : *fixedVerts)
        if (v >= 0 && v < nv) fx[(size_t)v] = 1, any = true;
      check(ctx_, ccd_mesh_set_fixed(mesh_, any ? fx.data() : nullptr), "ccd_mesh_set_fixed");
    }
    return mesh_;
  }
  ccd_context *context() const { return ctx_; }

 private:
  ccd_context *ctx_;
  ccd_mesh *mesh_ = nullptr;
  std::vector<int32_t> faces_;
  int nv_ = -1;
  std::vector<double> qs_, qe_;
};

// ------------------------------------------------------------------ broad phases
template <int Kind>
class GpuBroadPhase : public BroadPhase {
 public:
  explicit GpuBroadPhase(ccd_context *ctx = default_context()) : mesh_(ctx) {}

  // Clears and fills the sets, as KDOPBroadPhase.cpp:34-40 does.
  virtual void findCollisionCandidates(const History &h, const Mesh &m, double outerEta,
                                       std::set<VertexFaceStencil> &vfs, std::set<EdgeEdgeStencil> &ees,
                                       const std::set<int> &fixedVerts) {
    vfs.clear();
    ees.clear();
    ccd_mesh *dm = mesh_.sync(h, m, &fixedVerts);
    int64_t nvf = 0, nee = 0;
    check(mesh_.context(), ccd_broadphase(dm, Kind, outerEta, &nvf, &nee), "ccd_broadphase");
    std::vector<int32_t> vf(4 * (size_t)nvf), ee(4 * (size_t)nee);
    check(mesh_.context(), ccd_broadphase_get(dm, vf.data(), ee.data()), "ccd_broadphase_get");
    // The lists are in set order: append at the end.
    for (int64_t i = 0; i < nvf; i++)
      vfs.insert(vfs.end(), VertexFaceStencil(vf[4 * i], vf[4 * i + 1], vf[4 * i + 2], vf[4 * i + 3]));
    for (int64_t i = 0; i < nee; i++)
      ees.insert(ees.end(), EdgeEdgeStencil(ee[4 * i], ee[4 * i + 1], ee[4 * i + 2], ee[4 * i + 3]));
  }

 private:
  DeviceMesh mesh_;
};

typedef GpuBroadPhase<CCD_BROADPHASE_KDOP13> GpuKDOPBroadPhase;
typedef GpuBroadPhase<CCD_BROADPHASE_AABB> GpuAABBBroadPhase;
// TrivialBroadPhase (src/TrivialBroadPhase.cpp): the brute-force verifier.
typedef GpuBroadPhase<CCD_BROADPHASE_TRIVIAL> GpuTrivialBroadPhase;

// ------------------------------------------------------------------ narrow phase
class GpuCTCDNarrowPhase : public NarrowPhase {
 public:
  explicit GpuCTCDNarrowPhase(ccd_context *ctx = default_context(), int path = CCD_PATH_CULL_REFINE)
      : ctx_(ctx), path_(path) {}

  // Appends the colliding stencils to vfs / ees (which are not cleared), as
  // CTCDNarrowPhase::findCollisions does (src/CTCDNarrowPhase.cpp:9-24).  The
  // mesh positions come from the history; the narrow phase needs no faces.
  virtual void findCollisions(const History &h, const std::set<std::pair<VertexFaceStencil, double> > &candidateVFS,
                              const std::set<std::pair<EdgeEdgeStencil, double> > &candidateEES,
                              std::set<VertexFaceStencil> &vfs, std::set<EdgeEdgeStencil> &ees) {
    int nv = 0;
    for (const auto &c : candidateVFS) nv = std::max(nv, std::max(c.first.p, c.first.q2) + 1);
    for (const auto &c : candidateEES) nv = std::max(nv, std::max(c.first.p1, c.first.q1) + 1);
    if (nv == 0) return;
    Mesh points;
    points.vertices.resize(3 * nv);
    points.faces.resize(3, 0);
    ccd_mesh *dm = mesh_for(h, points);
    std::vector<int32_t> vf, ee;
    std::vector<double> vfe, eee;
    for (const auto &c : candidateVFS) {
      vf.insert(vf.end(), {c.first.p, c.first.q0, c.first.q1, c.first.q2});
      vfe.push_back(c.second);
    }
    for (const auto &c : candidateEES) {
      ee.insert(ee.end(), {c.first.p0, c.first.p1, c.first.q0, c.first.q1});
      eee.push_back(c.second);
    }
    std::vector<uint8_t> vh(vfe.size()), eh(eee.size());
    check(ctx_,
          ccd_narrowphase(dm, path_, (int64_t)vfe.size(), vf.data(), vfe.data(), (int64_t)vfe.size(),
                          (int64_t)eee.size(), ee.data(), eee.data(), (int64_t)eee.size(), vh.data(), eh.data(),
                          nullptr, nullptr, nullptr, nullptr),
          "ccd_narrowphase");
    size_t i = 0;
    for (const auto &c : candidateVFS)
      if (vh[i++]) vfs.insert(c.first);
    i = 0;
    for (const auto &c : candidateEES)
      if (eh[i++]) ees.insert(c.first);
  }

 private:
  ccd_mesh *mesh_for(const History &h, const Mesh &points) {
    if (!dev_) dev_.reset(new DeviceMesh(ctx_));
    return dev_->sync(h, points, nullptr);
  }
  ccd_context *ctx_;
  int path_;
  std::unique_ptr<DeviceMesh> dev_;
};

}  // namespace ccd_gb300

#endif  // CCD_GB300_REFERENCE_HPP
