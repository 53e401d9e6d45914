"""The header-only C++ adapters (include/ccd_gb300_reference.hpp) compile
against the reference's own headers (CTCD.h, History.h, Mesh.h, Stencils.h,
RetrospectiveDetection.h, Distance.h) and the Eigen API subset: the classes
derive from the reference's BroadPhase / NarrowPhase and the CTCD and Distance
forwarders keep the statics' signatures.  Needs the reference tree (skipped without it)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_TREE = os.environ.get("CCD_REFERENCE_TREE", "/root/reference")

CHECK = r'''
#include "ccd_gb300_reference.hpp"
#include "Distance.h"
#include "PenaltyGroup.h"
#include "VelocityFilter.h"
#include <type_traits>
static_assert(std::is_base_of<BroadPhase, ccd_gb300::GpuKDOPBroadPhase>::value, "k-DOP adapter");
static_assert(std::is_base_of<BroadPhase, ccd_gb300::GpuAABBBroadPhase>::value, "AABB adapter");
static_assert(std::is_base_of<BroadPhase, ccd_gb300::GpuTrivialBroadPhase>::value, "trivial adapter");
static_assert(std::is_base_of<NarrowPhase, ccd_gb300::GpuCTCDNarrowPhase>::value, "narrow-phase adapter");
// The forwarders take exactly the CTCD statics' argument lists.
static_assert(std::is_same<decltype(&CTCD::vertexFaceCTCD), decltype(&ccd_gb300::vertexFaceCTCD)>::value, "vf");
static_assert(std::is_same<decltype(&CTCD::edgeEdgeCTCD), decltype(&ccd_gb300::edgeEdgeCTCD)>::value, "ee");
static_assert(std::is_same<decltype(&CTCD::vertexEdgeCTCD), decltype(&ccd_gb300::vertexEdgeCTCD)>::value, "ve");
static_assert(std::is_same<decltype(&CTCD::vertexVertexCTCD), decltype(&ccd_gb300::vertexVertexCTCD)>::value, "vv");
// ... and the Distance statics'.
static_assert(std::is_same<decltype(&Distance::vertexFaceDistance), decltype(&ccd_gb300::vertexFaceDistance)>::value, "vfd");
static_assert(std::is_same<decltype(&Distance::edgeEdgeDistance), decltype(&ccd_gb300::edgeEdgeDistance)>::value, "eed");
static_assert(std::is_same<decltype(&Distance::vertexPlaneDistanceLessThan),
                           decltype(&ccd_gb300::vertexPlaneDistanceLessThan)>::value, "vpl");
static_assert(std::is_same<decltype(&Distance::lineLineDistanceLessThan),
                           decltype(&ccd_gb300::lineLineDistanceLessThan)>::value, "lll");
static_assert(std::is_same<decltype(&Distance::meshSelfDistance), decltype(&ccd_gb300::meshSelfDistance)>::value, "msd");
static_assert(std::is_same<decltype(&VelocityFilter::velocityFilter), decltype(&ccd_gb300::velocityFilter)>::value,
              "velocity filter");
// GpuPenaltyGroup keeps PenaltyGroup's interface (src/PenaltyGroup.h).
static bool (ccd_gb300::GpuPenaltyGroup::*add_force)(const Eigen::VectorXd &, const Eigen::VectorXd &,
                                                       Eigen::VectorXd &) = &ccd_gb300::GpuPenaltyGroup::addForce;
static bool (PenaltyGroup::*ref_add_force)(const Eigen::VectorXd &, const Eigen::VectorXd &, Eigen::VectorXd &) =
    &PenaltyGroup::addForce;
static void (ccd_gb300::GpuPenaltyGroup::*add_vf)(VertexFaceStencil) = &ccd_gb300::GpuPenaltyGroup::addVFStencil;
static void (PenaltyGroup::*ref_add_vf)(VertexFaceStencil) = &PenaltyGroup::addVFStencil;
static double (ccd_gb300::GpuPenaltyGroup::*next_fire)() const = &ccd_gb300::GpuPenaltyGroup::nextFireTime;
static double (PenaltyGroup::*ref_next_fire)() const = &PenaltyGroup::nextFireTime;
int main() { return add_force && ref_add_force && add_vf && ref_add_vf && next_fire && ref_next_fire ? 0 : 1; }
'''


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_TREE, "src")), reason="reference tree not present")
def test_adapters_compile_against_reference_headers(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "check.cpp"
    src.write_text(CHECK)
    cmd = [cxx, "-std=c++11", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
           "-I" + os.path.join(ROOT, "collisiondetection_gb300", "eigen_subset"),
           "-I" + os.path.join(REF_TREE, "include"), "-I" + os.path.join(REF_TREE, "src"),
           "-I" + os.path.join(ROOT, "include"), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
