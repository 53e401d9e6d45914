"""GB300-native continuous-time collision detection (CTCD).

A drop-in accelerator for the collision path of evouga/collisiondetection:
the primitive CTCD tests (CTCD::vertexFaceCTCD / edgeEdgeCTCD / vertexEdgeCTCD /
vertexVertexCTCD) as hand-written CUDA kernels for sm_103a behind the C ABI in
include/ccd_gb300.h.  This package holds the build helper, the ctypes binding
and the synthetic workload generators.
"""
from . import workloads  # noqa: F401
from ._native import (BROADPHASE_AABB, BROADPHASE_KDOP13, EDGE_EDGE, PATH_CULL_REFINE, PATH_FP64,  # noqa: F401
                      ROW_WIDTH, VERTEX_EDGE, VERTEX_FACE, VERTEX_VERTEX, CcdError, Context, Mesh, Server,
                      header_functions, load)

__version__ = "0.1.0"
