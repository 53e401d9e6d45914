// Static closest-point queries of the reference's Distance class
// (include/Distance.h), op-for-op in FP64 with one rounding per operation
// (no contraction: see ccd_common.h) and the Eigen contract for dot (see
// ccd_ctcd64.h).  Eigen evaluates `(q0 + v*ab) - p` coefficient-wise, i.e.
// (q0[k] + v*ab[k]) - p[k], which is what the v3d operators below compute.
#pragma once

#include "ccd_ctcd64.h"

namespace ccd {

// Distance::clamp (include/Distance.h:182-185): std::min(1.0, std::max(u, 0.0)).
// A NaN argument gives 1.0, as std::min/std::max do.
CCD_HD double dist_clamp(double u) { return smin(1.0, smax(u, 0.0)); }

// Distance::vertexFaceDistance (include/Distance.h:31-113): the vector from p
// to the closest point of triangle (q0, q1, q2), and that point's barycentric
// coordinates b.
CCD_HD v3d vertex_face_closest(v3d p, v3d q0, v3d q1, v3d q2, double (&b)[3]) {
  const v3d ab = q1 - q0;
  const v3d ac = q2 - q0;
  const v3d ap = p - q0;
  const double d1 = dot(ab, ap);
  const double d2 = dot(ac, ap);
  if (d1 <= 0 && d2 <= 0) {
    b[0] = 1.0, b[1] = 0.0, b[2] = 0.0;
    return q0 - p;
  }
  const v3d bp = p - q1;
  const double d3 = dot(ab, bp);
  const double d4 = dot(ac, bp);
  if (d3 >= 0 && d4 <= d3) {
    b[0] = 0.0, b[1] = 1.0, b[2] = 0.0;
    return q1 - p;
  }
  const double vc = d1 * d4 - d3 * d2;
  if ((vc <= 0) && (d1 >= 0) && (d3 <= 0)) {
    const double v = d1 / (d1 - d3);
    b[0] = 1.0 - v, b[1] = v, b[2] = 0;
    return (q0 + v * ab) - p;
  }
  const v3d cp = p - q2;
  const double d5 = dot(ab, cp);
  const double d6 = dot(ac, cp);
  if (d6 >= 0 && d5 <= d6) {
    b[0] = 0, b[1] = 0, b[2] = 1.0;
    return q2 - p;
  }
  const double vb = d5 * d2 - d1 * d6;
  if ((vb <= 0) && (d2 >= 0) && (d6 <= 0)) {
    const double w = d2 / (d2 - d6);
    b[0] = 1 - w, b[1] = 0, b[2] = w;
    return (q0 + w * ac) - p;
  }
  const double va = d3 * d6 - d5 * d4;
  if ((va <= 0) && (d4 - d3 >= 0) && (d5 - d6 >= 0)) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    b[0] = 0, b[1] = 1.0 - w, b[2] = w;
    return (q1 + w * (q2 - q1)) - p;
  }
  const double denom = 1.0 / (va + vb + vc);
  const double v = vb * denom;
  const double w = vc * denom;
  const double u = 1.0 - v - w;
  b[0] = u, b[1] = v, b[2] = w;
  return (u * q0 + v * q1 + w * q2) - p;
}

// Distance::edgeEdgeDistance (include/Distance.h:117-170): the shortest vector
// from segment (p0, p1) to segment (q0, q1), and the barycentric coordinates
// (p0, p1, q0, q1) of its end points.
CCD_HD v3d edge_edge_closest(v3d p0, v3d p1, v3d q0, v3d q1, double (&bary)[4]) {
  const v3d d1 = p1 - p0;
  const v3d d2 = q1 - q0;
  const v3d r = p0 - q0;
  const double a = dot(d1, d1);
  const double e = dot(d2, d2);
  const double f = dot(d2, r);
  double s, t;
  const double c = dot(d1, r);
  const double b = dot(d1, d2);
  const double denom = a * e - b * b;
  if (denom != 0.0)
    s = dist_clamp((b * f - c * e) / denom);
  else
    s = 0;  // parallel or degenerate edges
  const double tnom = b * s + f;
  if (tnom < 0 || e == 0) {
    t = 0;
    s = (a == 0) ? 0 : dist_clamp(-c / a);
  } else if (tnom > e) {
    t = 1.0;
    s = (a == 0) ? 0 : dist_clamp((b - c) / a);
  } else {
    t = tnom / e;
  }
  const v3d c1 = p0 + s * d1;
  const v3d c2 = q0 + t * d2;
  bary[0] = 1.0 - s;
  bary[1] = s;
  bary[2] = 1.0 - t;
  bary[3] = t;
  return c2 - c1;
}

// Distance::vertexPlaneDistanceLessThan (include/Distance.h:13-19).
CCD_HD bool vertex_plane_distance_less_than(v3d p, v3d q0, v3d q1, v3d q2, double eta) {
  const v3d c = cross(q1 - q0, q2 - q0);
  return dot(c, p - q0) * dot(c, p - q0) < eta * eta * dot(c, c);
}

// Distance::lineLineDistanceLessThan (include/Distance.h:21-27).
CCD_HD bool line_line_distance_less_than(v3d p0, v3d p1, v3d q0, v3d q1, double eta) {
  const v3d c = cross(p1 - p0, q1 - q0);
  return dot(c, q0 - p0) * dot(c, q0 - p0) < eta * eta * dot(c, c);
}

// The squared distance of Distance::meshSelfDistance's vertex scan
// (src/Distance.cpp:28): (verts_i - verts_v).squaredNorm().
CCD_HD double vertex_distance_sq(v3d a, v3d b) {
  const v3d d = a - b;
  return dot(d, d);
}

}  // namespace ccd
