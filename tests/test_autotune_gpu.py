"""The work-split autotuner (ccd_autotune_prim_batch) through the C ABI.

A split only reschedules the root solves of the FP64 refinement, so every
candidate must reproduce the context's own output bit for bit (the tuner
counts the ones that do not), and batches run after tuning must give the
same hits and contact times as before it and as the oracle: identical hit
flags, contact times within 1e-12 relative."""
import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    from collisiondetection_gb300 import build as B

    B.build_library()
    ctx = C.Context(0)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    yield torch, ctx, stream
    ctx.close()


def _run(torch, ctx, stream, kind, d_rows, d_eta, n):
    dev = d_rows.device
    with torch.cuda.stream(stream):
        hit = torch.zeros(n, dtype=torch.uint8, device=dev)
        t = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    ctx.prim_batch_device(kind, n, d_rows.data_ptr(), d_eta.data_ptr(), 1, hit.data_ptr(), t.data_ptr())
    ctx.synchronize()
    return hit.cpu().numpy(), t.cpu().numpy()


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_autotune_keeps_results_and_sets_a_split(setup, oracle, kind):
    torch, ctx, stream = setup
    # Above the default wavefront threshold (2^18 rows), so both kinds of
    # split are timed.
    n = 400_000
    rows = W.primitive_batch(kind, n, seed=40 + kind)
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        d_rows = torch.from_numpy(rows).to(dev)
        d_eta = torch.tensor([1e-6], dtype=torch.float64, device=dev)
    stream.synchronize()
    h0, t0 = _run(torch, ctx, stream, kind, d_rows, d_eta, n)

    res = ctx.autotune_prim_batch(kind, n, d_rows.data_ptr(), d_eta.data_ptr(), 1, reps=2)
    assert res["candidates"] == 26
    assert res["mismatches"] == 0
    assert 0 <= res["chosen"] < res["candidates"]
    assert 0 < res["best_ms"] <= res["default_ms"]
    assert 0 <= res["wave_steps"] <= 4096 and res["pool_budget"] >= 0 and res["wave_min_rows"] >= 0
    assert res["warp_finish"] in (0, 1, 2) and 0 <= res["shift_after"] < 20

    h1, t1 = _run(torch, ctx, stream, kind, d_rows, d_eta, n)
    assert np.array_equal(h0, h1)
    m = h0 == 1
    assert np.array_equal(t0[m].view(np.uint64), t1[m].view(np.uint64))

    k = 20_000
    h_ref, t_ref = oracle.batch(kind, rows[:k], 1e-6)
    assert np.array_equal(h1[:k], h_ref)
    mr = h_ref == 1
    if mr.any():
        rel = np.abs(t1[:k][mr] - t_ref[mr]) / np.maximum(np.abs(t_ref[mr]), 1e-300)
        assert rel.max() <= TOL


def test_autotune_rejects_bad_arguments(setup):
    torch, ctx, stream = setup
    dev = torch.device("cuda", 0)
    d_rows = torch.zeros((16, 24), dtype=torch.float64, device=dev)
    d_eta = torch.tensor([1e-6], dtype=torch.float64, device=dev)
    with pytest.raises(C.CcdError, match="invalid argument"):
        ctx.autotune_prim_batch(C.VERTEX_VERTEX, 16, d_rows.data_ptr(), d_eta.data_ptr(), 1)
    with pytest.raises(C.CcdError, match="invalid argument"):
        ctx.autotune_prim_batch(C.VERTEX_FACE, 16, d_rows.data_ptr(), d_eta.data_ptr(), 1, reps=0)
    with pytest.raises(C.CcdError, match="invalid argument"):
        ctx.autotune_prim_batch(C.VERTEX_FACE, 16, d_rows.data_ptr(), d_eta.data_ptr(), 3)
