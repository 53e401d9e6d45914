// Stand-in for the reference's src/Stencils.h: the two stencil types with
// canonical vertex order and lexicographic ordering (src/Stencils.h:6-132).
#ifndef STENCILS_H
#define STENCILS_H

#include <algorithm>
#include <utility>

struct VertexFaceStencil {
  int p;
  int q0, q1, q2;  // ascending
  bool isnew;
  VertexFaceStencil(int p_, int a, int b, int c) : p(p_), isnew(true) {
    int q[3] = {a, b, c};
    std::sort(q, q + 3);
    q0 = q[0];
    q1 = q[1];
    q2 = q[2];
  }
  bool operator<(const VertexFaceStencil &o) const {
    if (p != o.p) return p < o.p;
    if (q0 != o.q0) return q0 < o.q0;
    if (q1 != o.q1) return q1 < o.q1;
    return q2 < o.q2;
  }
};

struct EdgeEdgeStencil {
  int p0, p1;  // each edge ascending, the edge with the smaller first vertex first
  int q0, q1;
  bool isnew;
  EdgeEdgeStencil(int a0, int a1, int b0, int b1) : isnew(true) {
    p0 = std::min(a0, a1);
    p1 = std::max(a0, a1);
    q0 = std::min(b0, b1);
    q1 = std::max(b0, b1);
    if (p0 > q0) {
      std::swap(p0, q0);
      std::swap(p1, q1);
    }
  }
  bool operator<(const EdgeEdgeStencil &o) const {
    if (p0 != o.p0) return p0 < o.p0;
    if (p1 != o.p1) return p1 < o.p1;
    if (q0 != o.q0) return q0 < o.q0;
    return q1 < o.q1;
  }
};

#endif
