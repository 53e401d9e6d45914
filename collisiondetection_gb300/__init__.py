"""GB300-native continuous-time collision detection (CTCD).

A drop-in accelerator for the collision path of evouga/collisiondetection:
the primitive CTCD tests (CTCD::vertexFaceCTCD / edgeEdgeCTCD / vertexEdgeCTCD /
vertexVertexCTCD), the swept k-DOP / AABB broad phases, the CTCD narrow phase
over stencils and the Distance queries (meshSelfDistance and the closest-point
primitives), as hand-written CUDA kernels for sm_103a behind the C ABI in
include/ccd_gb300.h.  This package holds the build helper, the ctypes binding
and the synthetic workload generators.
"""
from . import workloads  # noqa: F401
from ._native import (BROADPHASE_AABB, BROADPHASE_KDOP13, BROADPHASE_TRIVIAL, DISTANCE_EDGE_EDGE, DISTANCE_LINE_LINE,  # noqa: F401
                      DISTANCE_VERTEX_FACE, DISTANCE_VERTEX_PLANE, EDGE_EDGE, PATH_CULL_REFINE, PATH_FP64,
                      PATH_REFINE_ALL,
                      ROW_WIDTH, VERTEX_EDGE, VERTEX_FACE, VERTEX_VERTEX, CcdError, Context, Mesh, Server,
                      header_functions, load)

__version__ = "0.1.0"
