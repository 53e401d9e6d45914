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


@pytest.mark.parametrize("scene", ["triangles", "sheets", "spheres"])
def test_grid_wide_firings_match_reference(ctx, golden_dir, scene):
    """The grid-wide event loop (forced on for every group) gives the same
    bits as the block loop and the reference."""
    meta = json.load(open(os.path.join(golden_dir, "velocity_filter.json")))[scene]
    g = np.load(os.path.join(golden_dir, "velocity_filter.npz"))
    q0, q1, f, mi = g[f"{scene}_qstart"], g[f"{scene}_qend"], g[f"{scene}_faces"], g[f"{scene}_invmasses"]
    ctx.set_option("layer_grid_min", 1)
    try:
        res, qe, st = ctx.velocity_filter(q0, q1, f, mi, meta["outer_eta"], meta["inner_eta"])
    finally:
        ctx.set_option("layer_grid_min", 1024)
    assert res == meta["return"]
    assert np.array_equal(qe.view(np.uint64), g[f"{scene}_result"].ravel().view(np.uint64))


def test_larger_sheets_match_oracle(ctx, oracle):
    """Two 12x12 sheets (contact groups of a few thousand stencils: the grid
    loop) against the oracle's restatement of the whole filter."""
    from collisiondetection_gb300 import workloads as W

    gsz = 12
    v, f = W.grid_sheet(gsz, gsz)
    v = np.asarray(v).reshape(-1, 3)
    n = v.shape[0]
    upper = v.copy()
    upper[:, 2] += 0.02
    q0 = np.concatenate([v, upper])
    q1 = q0.copy()
    q1[n:, 2] -= 0.04
    ff = np.concatenate([f, f + n]).astype(np.int32)
    mi = np.ones(q0.size)
    mi[: 3 * n] = 0
    sp = 1.0 / (gsz - 1)
    res, qe, st = ctx.velocity_filter(q0, q1, ff, mi, 0.2 * sp, 0.1 * sp)
    r2, q2, ev = oracle.velocity_filter(q0, q1, ff, mi, 0.2 * sp, 0.1 * sp)
    assert res == r2 and st["events"] == ev
    assert np.array_equal(qe.view(np.uint64), q2.view(np.uint64))
