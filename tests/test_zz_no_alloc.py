"""The allocation-free batch entry point (ccd_prim_batch_device_noalloc)
against the context batch entry point (ccd_prim_batch_device, cull + refine)
and the oracle on the same device inputs: two full-size calls in a row, then
smaller calls over the scratch the last one left, with the device's free
memory unchanged across them.  Collected last on purpose: it must pass after
the other GPU tests as well as alone in a fresh process.

Tolerance: identical hit flags; contact times within 1e-12 relative (the two
entry points run the same kernels, so they agree exactly in practice)."""
import ctypes
import os
import re

import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _max_rows() -> int:
    text = open(C._native.HEADER).read()
    return int(re.search(r"#define CCD_NOALLOC_MAX_ROWS (\d+)", text).group(1))


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    from collisiondetection_gb300 import build as B

    B.build_library()
    ctx = C.Context(0)
    lib = ctx.lib
    fn = lib.ccd_prim_batch_device_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    yield torch, ctx, fn, stream
    ctx.close()


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE, C.VERTEX_EDGE, C.VERTEX_VERTEX])
@pytest.mark.parametrize("per_row_eta", [False, True])
def test_noalloc_matches_batch_entry_point(setup, oracle, kind, per_row_eta):
    torch, ctx, fn, stream = setup
    n = _max_rows()
    rows = W.primitive_batch(kind, n, seed=11 + kind)
    eta = 10.0 ** np.random.default_rng(kind).uniform(-7, -2, n) if per_row_eta else np.array([1e-6])
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        d_rows = torch.from_numpy(rows).to(dev)
        d_eta = torch.from_numpy(eta).to(dev)
        ref_hit = torch.zeros(n, dtype=torch.uint8, device=dev)
        ref_t = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        hit = torch.zeros(n, dtype=torch.uint8, device=dev)
        t = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    ctx.prim_batch_device(kind, n, d_rows.data_ptr(), d_eta.data_ptr(), eta.size, ref_hit.data_ptr(),
                          ref_t.data_ptr(), None, path=C.PATH_CULL_REFINE)
    ctx.synchronize()
    h_ref, t_ref = ref_hit.cpu().numpy(), ref_t.cpu().numpy()
    assert h_ref.any()
    # the oracle agrees with the context entry point on these rows
    h_orc, t_orc = oracle.batch(kind, rows, eta if per_row_eta else eta[0], nthreads=os.cpu_count() or 4)
    np.testing.assert_array_equal(h_ref, h_orc)

    def call(m):
        """The first m rows through the allocation-free entry point, with hit
        starting at a sentinel so that a row it never writes shows."""
        with torch.cuda.stream(stream):
            hit.fill_(7)
            t.fill_(float("nan"))
        e = eta.size if eta.size == 1 else m
        rc = fn(kind, m, d_rows.data_ptr(), d_eta.data_ptr(), e, hit.data_ptr(), t.data_ptr(), stream.cuda_stream)
        assert rc == 0, f"status {rc}"
        stream.synchronize()
        h, tt = hit.cpu().numpy(), t.cpu().numpy()
        assert np.isin(h[:m], (0, 1)).all() and (h[m:] == 7).all()
        np.testing.assert_array_equal(h[:m], h_ref[:m])
        mk = h_ref[:m] == 1
        for ref in (t_ref, t_orc):
            rel = np.abs(tt[:m][mk] - ref[:m][mk]) / np.maximum(np.abs(ref[:m][mk]), 1e-300)
            assert not mk.any() or rel.max() <= TOL
        assert np.isnan(tt[:m][~mk]).all()  # t is written only where hit

    call(n)  # the first call on the device may do the setup
    free0 = torch.cuda.mem_get_info()[0]
    for m in (n, n, 1, 5000):  # two full calls in a row, then smaller ones over the last call's scratch
        call(m)
    assert torch.cuda.mem_get_info()[0] == free0  # nothing was allocated


def test_noalloc_rejects_oversized_and_bad_arguments(setup):
    torch, ctx, fn, stream = setup
    n = _max_rows()
    dev = torch.device("cuda", 0)
    rows = torch.zeros((n + 1) * 24, dtype=torch.float64, device=dev)
    eta = torch.full((1,), 1e-6, dtype=torch.float64, device=dev)
    hit = torch.full((n + 1,), 7, dtype=torch.uint8, device=dev)
    t = torch.zeros(n + 1, dtype=torch.float64, device=dev)
    args = (rows.data_ptr(), eta.data_ptr(), 1, hit.data_ptr(), t.data_ptr(), stream.cuda_stream)
    assert fn(C.VERTEX_FACE, n + 1, *args) == 1  # CCD_ERR_INVALID_ARGUMENT
    assert fn(9, 10, *args) == 1
    assert fn(C.EDGE_EDGE, 10, rows.data_ptr(), eta.data_ptr(), 3, hit.data_ptr(), t.data_ptr(),
              stream.cuda_stream) == 1
    assert fn(C.VERTEX_FACE, 0, *args) == 0
    stream.synchronize()
    assert int((hit != 7).sum()) == 0  # nothing was enqueued
