"""VelocityFilter::velocityFilter on the GPU (ccd_velocity_filter) against the
golden fixtures made by the reference's own VelocityFilter / ActiveLayers.

Parity bar: the same return value and filtered end positions equal bit for
bit (the event order, every impulse and every history entry are the
reference's)."""
import json
import os

import numpy as np
import pytest

import collisiondetection_gb300 as C

pytestmark = pytest.mark.gpu

SCENES = ["triangles", "sheets", "spheres", "intersecting_start", "dangling"]


@pytest.fixture(scope="module")
def ctx():
    from collisiondetection_gb300 import build as B

    B.build_library()
    c = C.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("scene", SCENES)
def test_velocity_filter_matches_reference(ctx, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "velocity_filter.json")))[scene]
    g = np.load(os.path.join(golden_dir, "velocity_filter.npz"))
    q0, q1, f, mi = g[f"{scene}_qstart"], g[f"{scene}_qend"], g[f"{scene}_faces"], g[f"{scene}_invmasses"]
    res, qe, st = ctx.velocity_filter(q0, q1, f, mi, meta["outer_eta"], meta["inner_eta"])
    assert res == meta["return"]
    expect = g[f"{scene}_result"].ravel()
    bad = np.nonzero(expect.view(np.uint64) != qe.view(np.uint64))[0]
    assert bad.size == 0, f"end positions differ at coordinates {bad[:10]} (max {np.abs(qe - expect).max()})"
    if res >= 0:
        assert st["iterations"] == res + 1 and st["events"] >= 0
        if res > 0:
            assert st["events"] > 0 and st["layers"] >= 5
