"""Serving engine on the GPU (ccd_server_*): requests of different sizes run
concurrently on several slots give exactly the results they give alone, and
those match the mesh entry points and the oracle.

Parity bar: identical colliding-stencil lists per step; contact times equal
bit for bit between the mixed and the alone runs (same kernels), and within
1e-12 relative of the oracle."""
import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REQUESTS = [(2000, 2), (20000, 4), (5000, 7), (20000, 3), (1000, 11), (8000, 12)]


@pytest.fixture(scope="module")
def built():
    from collisiondetection_gb300 import build as B

    B.build_library()
    return [W.motion_request(tris, seed, steps=3) for tris, seed in REQUESTS]


def _run(server, reqs):
    tickets = [server.submit(f, fr) for f, fr in reqs]
    return [server.wait(t) for t in tickets]


def _same(a, b):
    assert len(a["steps"]) == len(b["steps"])
    for (vf1, vft1, ee1, eet1), (vf2, vft2, ee2, eet2) in zip(a["steps"], b["steps"]):
        np.testing.assert_array_equal(vf1, vf2)
        np.testing.assert_array_equal(ee1, ee2)
        np.testing.assert_array_equal(vft1, vft2)
        np.testing.assert_array_equal(eet1, eet2)


def test_results_same_alone_and_in_the_mix(built):
    with C.Server(0, slots=1) as s:
        alone = [_run(s, [r])[0] for r in built]
    with C.Server(0, slots=4) as s:
        mixed = _run(s, built)
    for a, b in zip(alone, mixed):
        _same(a, b)
    assert sum(len(st[0]) + len(st[2]) for r in mixed for st in r["steps"]) > 0  # some collisions


def test_tight_budget_serialises_but_agrees(built):
    with C.Server(0, slots=4, memory_budget=1) as s:  # every request exceeds it: one at a time
        tight = _run(s, built)
    with C.Server(0, slots=4) as s:
        loose = _run(s, built)
    for a, b in zip(tight, loose):
        _same(a, b)


def test_server_matches_mesh_entry_point_and_oracle(built, oracle):
    f, fr = built[1]
    with C.Server(0, slots=2) as s:
        res = _run(s, [(f, fr)])[0]
    ctx = C.Context(0)
    with C.Mesh(ctx, f, fr[0], fr[1]) as m:
        for k in range(fr.shape[0] - 1):
            m.set_positions(fr[k], fr[k + 1])
            vf, vft, ee, eet = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
            svf, svft, see, seet = res["steps"][k]
            np.testing.assert_array_equal(vf, svf)
            np.testing.assert_array_equal(ee, see)
    ctx.close()
    # First step against the oracle: broad phase, then the narrow phase.
    cvf, cee = oracle.broadphase(0, fr[0], fr[1], f, 1e-6)
    r = oracle.narrowphase(fr[0], fr[1], cvf, 1e-6, cee, 1e-6)
    svf, svft, see, seet = res["steps"][0]
    np.testing.assert_array_equal(svf, cvf[r["vf_hit"] == 1])
    np.testing.assert_array_equal(see, cee[r["ee_hit"] == 1])
    for t, rt in ((svft, r["vf_t"][r["vf_hit"] == 1]), (seet, r["ee_t"][r["ee_hit"] == 1])):
        assert t.size == 0 or (np.abs(t - rt) / np.maximum(np.abs(rt), 1e-300)).max() <= 1e-12


def test_invalid_requests_are_rejected(built):
    f, fr = built[0]
    with C.Server(0, slots=1) as s:
        bad = f.copy()
        bad[0, 0] = fr.shape[1] // 3  # vertex out of range
        with pytest.raises(C.CcdError):
            s.submit(bad, fr)
        with pytest.raises(C.CcdError):
            s.submit(f, fr[:1])  # no step
        t = s.submit(f, fr)
        assert len(s.wait(t)["steps"]) == fr.shape[0] - 1
