// ORACLE / TEST INFRASTRUCTURE ONLY: drives the reference's AABBBroadPhase
// (src/AABBBroadPhase.cpp) for ref_shim.cpp; see that file's header.
#include <set>

#include "AABBBroadPhase.h"
#include "History.h"
#include "Mesh.h"

void ref_aabb_candidates(const History &h, const Mesh &m, double eta, std::set<VertexFaceStencil> &vfs,
                         std::set<EdgeEdgeStencil> &ees, const std::set<int> &fixedVerts) {
  AABBBroadPhase bp;
  bp.findCollisionCandidates(h, m, eta, vfs, ees, fixedVerts);
}
