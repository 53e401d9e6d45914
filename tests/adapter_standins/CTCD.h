// Stand-in for the reference's include/CTCD.h.  The adapters' forwarders
// take the CTCD statics' argument lists; nothing here is defined or called.
#ifndef CTCD_H
#define CTCD_H

#include <Eigen/Core>

class CTCD {
 public:
  static bool vertexFaceCTCD(const Eigen::Vector3d &q0start, const Eigen::Vector3d &q1start,
                             const Eigen::Vector3d &q2start, const Eigen::Vector3d &q3start,
                             const Eigen::Vector3d &q0end, const Eigen::Vector3d &q1end,
                             const Eigen::Vector3d &q2end, const Eigen::Vector3d &q3end, double eta, double &t);
};

#endif
