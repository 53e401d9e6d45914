// The penalty potentials of the reference (src/PenaltyPotential.cpp:7-64) as
// device functions, shared by the group-force kernels (penalty.cu) and the
// active layers' event loop (velocity.cu).
#pragma once

#include "ccd_distance.h"

namespace ccd {

__device__ __forceinline__ v3d ldv(const double *x, int v) { return ld3(x + 3 * (int64_t)v); }

__device__ __forceinline__ void swap_i(int &a, int &b) {
  const int t = a;
  a = b;
  b = t;
}

// The canonical forms the stencil constructors produce (src/Stencils.h:13-57,
// 86-117).
__device__ __forceinline__ void canonical(int kind, int *v) {
  if (kind == 0) {
    if (v[1] > v[2]) swap_i(v[1], v[2]);
    if (v[2] > v[3]) swap_i(v[2], v[3]);
    if (v[1] > v[2]) swap_i(v[1], v[2]);
  } else {
    if (v[0] > v[1]) swap_i(v[0], v[1]);
    if (v[2] > v[3]) swap_i(v[2], v[3]);
    if (v[0] > v[2]) {
      swap_i(v[0], v[2]);
      swap_i(v[1], v[3]);
    }
  }
}

struct PenaltyParams {
  double outer_eta, inner_eta, stiffness, cor;
};

// One stencil's potential.  Returns whether it fires; then c[slot] holds the
// vector the reference adds to (slot with sign +) or subtracts from (sign -)
// the group force of vertex v[slot]: vertex-face p -, q0 q1 q2 +; edge-edge
// p0 p1 -, q0 q1 +.
// Position / velocity loads: plain, or through L2 only (data that other SMs
// rewrite between a kernel's grid-wide barriers).
struct PlainLoad {
  __device__ v3d operator()(const double *x, int v) const { return ldv(x, v); }
};
struct L2Load {
  __device__ v3d operator()(const double *x, int v) const {
    const double *p = x + 3 * (int64_t)v;
    return v3d{__ldcg(p), __ldcg(p + 1), __ldcg(p + 2)};
  }
};

// The potential from the stencil's four positions x; vel(k) gives vertex k's
// velocity and is called only when the potential fires, in the reference's
// order of the relative-velocity sum.
template <int KIND, class Vel>
__device__ __forceinline__ bool stencil_force_at(const v3d (&x)[4], Vel vel, PenaltyParams pp, v3d (&c)[4]) {
  double stiffness = pp.stiffness;
  if constexpr (KIND == 0) {
    // VertexFacePenaltyPotential::addForce (src/PenaltyPotential.cpp:7-34)
    if (!vertex_plane_distance_less_than(x[0], x[1], x[2], x[3], pp.outer_eta)) return false;
    double b[3];
    const v3d cv = vertex_face_closest(x[0], x[1], x[2], x[3], b);
    const double dist = norm(cv);
    if (dist >= pp.outer_eta || dist < pp.inner_eta) return false;
    const v3d vp = vel(0);
    const v3d relvel = (((v3d{-vp.x, -vp.y, -vp.z}) + b[0] * vel(1)) + b[1] * vel(2)) + b[2] * vel(3);
    if (dot(relvel, cv) > 0) stiffness *= pp.cor;
    const double s = stiffness * (pp.outer_eta - dist) / (pp.outer_eta - pp.inner_eta);
    const v3d sc = s * cv;
    const v3d lf = v3d{sc.x / dist, sc.y / dist, sc.z / dist};
    c[0] = lf;
    c[1] = b[0] * lf;
    c[2] = b[1] * lf;
    c[3] = b[2] * lf;
  } else {
    // EdgeEdgePenaltyPotential::addForce (src/PenaltyPotential.cpp:36-64)
    if (!line_line_distance_less_than(x[0], x[1], x[2], x[3], pp.outer_eta)) return false;
    double b[4];
    const v3d cv = edge_edge_closest(x[0], x[1], x[2], x[3], b);
    const double dist = norm(cv);
    if (dist >= pp.outer_eta || dist < pp.inner_eta) return false;
    const v3d relvel = (((-b[0]) * vel(0) - b[1] * vel(1)) + b[2] * vel(2)) + b[3] * vel(3);
    if (dot(relvel, cv) > 0) stiffness *= pp.cor;
    const double s = stiffness * (pp.outer_eta - dist) / (pp.outer_eta - pp.inner_eta);
    const v3d sc = s * cv;
    const v3d lf = v3d{sc.x / dist, sc.y / dist, sc.z / dist};
    c[0] = b[0] * lf;
    c[1] = b[1] * lf;
    c[2] = b[2] * lf;
    c[3] = b[3] * lf;
  }
  return true;
}

// The same from position and velocity arrays indexed by vertex.
template <int KIND, class Load = PlainLoad>
__device__ __forceinline__ bool stencil_force(const double *q, const double *vel, const int *v, PenaltyParams pp,
                                              v3d (&c)[4], Load ldv = Load()) {
  const v3d x[4] = {ldv(q, v[0]), ldv(q, v[1]), ldv(q, v[2]), ldv(q, v[3])};
  return stencil_force_at<KIND>(x, [&](int k) { return ldv(vel, v[k]); }, pp, c);
}

}  // namespace ccd
