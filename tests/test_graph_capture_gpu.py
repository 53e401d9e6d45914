"""ccd_prim_batch_device captured into a CUDA graph and replayed.

Once a context has run one batch of at least n rows of a kind on a path
(which sizes its scratch), a device batch enqueues only kernels, memsets and
copies, so a caller can capture it on the context's stream and replay it.
The replays must give the results of a direct call bit for bit: identical
hit flags and contact times (the same kernels on the same inputs).  Both
refinement branches are covered: the pool solver alone (a small batch) and
the lock-step wavefront (a batch above its 2^18-row threshold)."""
import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
@pytest.mark.parametrize("n", [20_000, 300_000])
def test_captured_batch_replays_bit_for_bit(setup, kind, n):
    torch, ctx, stream = setup
    rows = W.primitive_batch(kind, n, seed=70 + kind)
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        d_rows = torch.from_numpy(rows).to(dev)
        d_eta = torch.tensor([1e-6], dtype=torch.float64, device=dev)
        hit = torch.zeros(n, dtype=torch.uint8, device=dev)
        t = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)

    def call():
        ctx.prim_batch_device(kind, n, d_rows.data_ptr(), d_eta.data_ptr(), 1, hit.data_ptr(), t.data_ptr())

    # a direct call: the expected output, and the scratch sized for n rows
    call()
    ctx.synchronize()
    h0, t0 = hit.cpu().numpy(), t.cpu().numpy()
    hits0 = ctx.stats()["hits"]
    assert h0.sum() == hits0 > 0

    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        call()
    for rep in range(2):
        with torch.cuda.stream(stream):  # replay() launches on the current stream
            hit.zero_()
            t.fill_(float("nan"))
            g.replay()
        ctx.synchronize()
        h1, t1 = hit.cpu().numpy(), t.cpu().numpy()
        assert np.array_equal(h0, h1)
        assert np.array_equal(t0.view(np.uint64), t1.view(np.uint64))
        if rep == 0:
            # the counters the captured call copies back arrive with the replay
            assert ctx.stats()["hits"] == hits0
    del g
