"""Primitive CTCD kernels on the GPU through the C ABI, against the golden
fixtures (produced by the reference itself) and the oracle.

Parity bar: identical hit flags; contact times within 1e-12 relative (the
reference's host exp/log are not correctly rounded on ~0.1% of inputs, the
device ones are, so a contact time may differ in the last bits)."""
import json
import os

import numpy as np
import pytest

import collisiondetection_gb300 as C

pytestmark = pytest.mark.gpu

KINDS = [C.VERTEX_FACE, C.EDGE_EDGE, C.VERTEX_EDGE, C.VERTEX_VERTEX]
PATHS = [C.PATH_FP64, C.PATH_CULL_REFINE, C.PATH_REFINE_ALL]
TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    from collisiondetection_gb300 import build as B

    B.build_library()
    c = C.Context(0)
    yield c
    c.close()


def _assert_same(h, t, h_ref, t_ref, what):
    bad = np.nonzero(h != h_ref)[0]
    assert bad.size == 0, f"{what}: hit differs at rows {bad[:10]}"
    m = h_ref == 1
    rel = np.abs(t[m] - t_ref[m]) / np.maximum(np.abs(t_ref[m]), 1e-300)
    assert not m.any() or rel.max() <= TOL, f"{what}: contact time off by {rel.max():.3g}"


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("path", PATHS)
def test_golden_fixtures(ctx, golden_dir, kind, path):
    g = np.load(os.path.join(golden_dir, "prims.npz"))
    h, t = ctx.prim_batch(kind, g[f"x{kind}"], g[f"eta{kind}"], path=path)
    _assert_same(h, t, g[f"hit{kind}"], g[f"t{kind}"], f"kind {kind} path {path}")
    st = ctx.stats()
    assert st["hits"] == int(g[f"hit{kind}"].sum()) and st["status_flags"] == 0


def test_testctcd_known_answers_single_calls(ctx, golden_dir):
    kat = json.load(open(os.path.join(golden_dir, "kat_testctcd.json")))
    kinds = {"vf": C.VERTEX_FACE, "ee": C.EDGE_EDGE, "ve": C.VERTEX_EDGE, "vv": C.VERTEX_VERTEX}
    for case in kat:
        h, t = ctx.single(kinds[case["kind"]], case["points"], case["eta"])
        assert h == case["hit"] == 1
        assert abs(t - case["t"]) <= TOL * abs(case["t"])


@pytest.mark.parametrize("kind", KINDS)
def test_random_batches_match_oracle(ctx, oracle, kind):
    rows = C.workloads.primitive_batch(kind, 100000, seed=2024)
    h_ref, t_ref = oracle.batch(kind, rows, 1e-6, nthreads=os.cpu_count() or 4)
    for path in PATHS:
        h, t = ctx.prim_batch(kind, rows, 1e-6, path=path)
        _assert_same(h, t, h_ref, t_ref, f"kind {kind} path {path}")


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_cull_refine_equals_fp64_at_scale(ctx, kind):
    # Size-independent property at a size the oracle does not finish quickly:
    # the FP32 stage never changes a result, and rejects most rows.
    rows = C.workloads.primitive_batch(kind, 2_000_000, seed=99)
    h64, t64 = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_FP64)
    assert ctx.stats()["survivors"] == rows.shape[0]
    h32, t32 = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
    st = ctx.stats()
    np.testing.assert_array_equal(h32, h64)
    np.testing.assert_array_equal(t32[h64 == 1], t64[h64 == 1])
    assert st["survivors"] < 0.4 * rows.shape[0]
    assert st["hits"] == int(h64.sum())


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_wavefront_batch_matches_oracle(ctx, oracle, kind):
    # 400k rows: large enough for the wavefront root solver (batches of at
    # least 2^18 rows), small enough for the oracle.
    rows = C.workloads.primitive_batch(kind, 400_000, seed=4242)
    h_ref, t_ref = oracle.batch(kind, rows, 1e-6, nthreads=os.cpu_count() or 4)
    ctx.set_profiling(True)
    h, t = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
    tm = ctx.timings()
    ctx.set_profiling(False)
    _assert_same(h, t, h_ref, t_ref, f"kind {kind} wavefront")
    assert tm["launches"] > 10  # cull, build, wavefront steps, tail, combine


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_refine_all_equals_fp64_at_wavefront_size(ctx, kind):
    # Every row through the staged refinement (no FP32 stage): the wavefront
    # solver runs (more than 2^18 rows) and every result is the plain
    # kernel's, bit for bit.
    rows = C.workloads.primitive_batch(kind, 600_000, seed=77)
    h64, t64 = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_FP64)
    ha, ta = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_REFINE_ALL)
    st = ctx.stats()
    np.testing.assert_array_equal(ha, h64)
    np.testing.assert_array_equal(ta[h64 == 1].view(np.uint64), t64[h64 == 1].view(np.uint64))
    assert st["survivors"] == rows.shape[0] and st["hits"] == int(h64.sum())


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
@pytest.mark.parametrize("n", [4096, 600_000])
def test_warp_finish_is_bit_identical(ctx, kind, n):
    # The slowest solves advanced by all 32 lanes of a warp (1: independent
    # divisions and K terms spread over lanes; 2: each lane trying one of the
    # stage's remaining shifts, from the first shift on or after two failed
    # ones) against one lane alone (0): the same operations on the same
    # operands, so the same bits.  4,096 rows take the pool kernel alone (its
    # last solve per warp), 600,000 the wavefront and the one-solve-per-warp
    # finish.
    rows = C.workloads.primitive_batch(kind, n, seed=505)
    out = {}
    for mode, after in ((0, 2), (1, 2), (2, 0), (2, 2)):
        ctx.set_option("warp_finish", mode)
        ctx.set_option("shift_after", after)
        try:
            out[mode, after] = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
        finally:
            ctx.set_option("warp_finish", 1)
            ctx.set_option("shift_after", 2)
    ref = out[0, 2]
    m = ref[0] == 1
    assert m.any()
    for key, got in out.items():
        np.testing.assert_array_equal(ref[0], got[0])
        np.testing.assert_array_equal(ref[1][m].view(np.uint64), got[1][m].view(np.uint64))


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_pool_spreading_is_bit_identical(ctx, kind):
    # How many slots a pool warp has and fills, whether a drained warp steps
    # all its remaining solves at once and which phase a warp prefers change
    # only which warp and lane advance a solve, never its operations.
    rows = C.workloads.primitive_batch(kind, 4096, seed=507)
    out = {}
    try:
        for pool, slots, every, sync in ((64, 64, 0, 0), (64, 4, 0, 16), (64, 1, 0, 0), (64, 4, 32, 16),
                                         (64, 64, 32, 12), (32, 4, 0, 16), (32, 32, 8, 0)):
            ctx.set_option("pool_slots", pool)
            ctx.set_option("pool_slots_min", slots)
            ctx.set_option("pool_all", every)
            ctx.set_option("pool_phase_sync", sync)
            out[pool, slots, every, sync] = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
    finally:
        ctx.set_option("pool_slots", 64)
        ctx.set_option("pool_slots_min", 4)
        ctx.set_option("pool_all", 0)
        ctx.set_option("pool_phase_sync", 16)
    ref = out[64, 64, 0, 0]
    m = ref[0] == 1
    assert m.any()
    for got in out.values():
        np.testing.assert_array_equal(ref[0], got[0])
        np.testing.assert_array_equal(ref[1][m].view(np.uint64), got[1][m].view(np.uint64))


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE])
def test_one_per_warp_finish_is_bit_identical(ctx, kind):
    # A pool budget hands the solves still running after it to the
    # one-solve-per-warp finish kernel (wave_finish), which then runs with
    # each of its three modes; every mode gives the same bits.
    rows = C.workloads.primitive_batch(kind, 600_000, seed=506)
    out = {}
    ctx.set_option("pool_budget", 16)
    try:
        ctx.set_option("shift_after", 0)
        for mode in (0, 1, 2):
            ctx.set_option("warp_finish", mode)
            out[mode] = ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
    finally:
        ctx.set_option("warp_finish", 1)
        ctx.set_option("shift_after", 2)
        ctx.set_option("pool_budget", 0)
    m = out[0][0] == 1
    assert m.any()
    for mode in (1, 2):
        np.testing.assert_array_equal(out[0][0], out[mode][0])
        np.testing.assert_array_equal(out[0][1][m].view(np.uint64), out[mode][1][m].view(np.uint64))


@pytest.mark.parametrize("kind", [C.VERTEX_FACE, C.EDGE_EDGE, C.VERTEX_EDGE])
def test_cull_alone_keeps_every_hit(ctx, oracle, kind):
    torch = pytest.importorskip("torch")
    rows = C.workloads.primitive_batch(kind, 100_000, seed=31)
    h_ref, _ = oracle.batch(kind, rows, 1e-6, nthreads=os.cpu_count() or 4)
    n = rows.shape[0]
    d_rows = torch.from_numpy(rows).cuda()
    d_eta = torch.full((1,), 1e-6, dtype=torch.float64, device="cuda")
    d_hit = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    d_surv = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ns = ctx.prim_cull_device(kind, n, d_rows.data_ptr(), d_eta.data_ptr(), 1, d_hit.data_ptr(), d_surv.data_ptr())
    surv = np.sort(d_surv.cpu().numpy()[:ns])
    hit = d_hit.cpu().numpy()
    assert 0 < ns < n and np.unique(surv).size == ns and surv[0] >= 0 and surv[-1] < n
    kept = np.zeros(n, bool)
    kept[surv] = True
    assert np.all(hit[~kept] == 0) and np.all(hit[kept] == 7)  # rejected rows only are written
    assert not np.any((h_ref == 1) & ~kept)  # no hit is rejected
    # the same survivors as the cull + refine path counts
    ctx.prim_batch(kind, rows, 1e-6, path=C.PATH_CULL_REFINE)
    assert ctx.stats()["survivors"] == ns
    with pytest.raises(C.CcdError):
        ctx.prim_cull_device(C.VERTEX_VERTEX, n, d_rows.data_ptr(), d_eta.data_ptr(), 1, d_hit.data_ptr(),
                             d_surv.data_ptr())


def test_fp64_peak_is_plausible(ctx):
    p = ctx.fp64_peak(reps=2)
    # GB300: about 1.2 TFLOP/s of FP64 FMA; DADD / DMUL issue at the same rate
    assert 1e11 < p["ops_per_s"] < 1e13 and 1e11 < p["fma_flops_per_s"] < 1e13
    assert p["ms"] > 0 and p["ops"] > 0
    # a correctly rounded division is several dependent FP64 operations
    assert 1e9 < p["div_per_s"] < p["ops_per_s"]
    for op in ("add", "mul"):
        assert 1.0 < p[op + "_latency_cycles"] < 1000.0
    assert p["add_latency_cycles"] < p["div_latency_cycles"] < 10000.0


def test_t_untouched_on_miss_and_eta_per_row(ctx):
    rows = C.workloads.primitive_batch(C.VERTEX_FACE, 5000, seed=5)
    sentinel = np.full(rows.shape[0], -7.25)
    h, t = ctx.prim_batch(C.VERTEX_FACE, rows, 1e-6, t=sentinel)
    assert np.all(t[h == 0] == -7.25)
    assert np.all(t[h == 1] >= 0.0)
    eta = np.full(rows.shape[0], 1e-6)
    h2, t2 = ctx.prim_batch(C.VERTEX_FACE, rows, eta, t=sentinel)
    np.testing.assert_array_equal(h, h2)
    np.testing.assert_array_equal(t, t2)


def test_device_entry_point_matches_host(ctx):
    torch = pytest.importorskip("torch")
    rows = C.workloads.primitive_batch(C.EDGE_EDGE, 50000, seed=8)
    h_ref, t_ref = ctx.prim_batch(C.EDGE_EDGE, rows, 1e-6)
    d_rows = torch.from_numpy(rows).cuda()
    d_eta = torch.full((1,), 1e-6, dtype=torch.float64, device="cuda")
    d_hit = torch.zeros(rows.shape[0], dtype=torch.uint8, device="cuda")
    d_t = torch.full((rows.shape[0],), float("nan"), dtype=torch.float64, device="cuda")
    d_st = torch.zeros(rows.shape[0], dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    ctx.prim_batch_device(C.EDGE_EDGE, rows.shape[0], d_rows.data_ptr(), d_eta.data_ptr(), 1, d_hit.data_ptr(),
                          d_t.data_ptr(), d_st.data_ptr())
    ctx.synchronize()
    np.testing.assert_array_equal(d_hit.cpu().numpy(), h_ref)
    np.testing.assert_array_equal(d_t.cpu().numpy()[h_ref == 1], t_ref[h_ref == 1])
    assert int(d_st.sum()) == 0
    assert ctx.stats()["hits"] == int(h_ref.sum())


def test_profiling_timings(ctx):
    rows = C.workloads.primitive_batch(C.VERTEX_FACE, 200000, seed=6)
    ctx.set_profiling(True)
    ctx.prim_batch(C.VERTEX_FACE, rows, 1e-6, path=C.PATH_CULL_REFINE)
    tm = ctx.timings()
    ctx.set_profiling(False)
    # cull, then build + (wavefront steps +) roots + combine for the one tile
    assert tm["launches"] >= 4 and tm["cull_ms"] > 0 and tm["refine_ms"] > 0


def test_empty_and_invalid_batches(ctx):
    h, t = ctx.prim_batch(C.VERTEX_FACE, np.zeros((0, 24)), 1e-6)
    assert h.size == 0
    rows = C.workloads.primitive_batch(C.VERTEX_FACE, 10, seed=1)
    with pytest.raises(C.CcdError):
        ctx.prim_batch(C.VERTEX_FACE, rows, np.full(3, 1e-6))  # eta_count neither 1 nor n
    with pytest.raises(C.CcdError):
        ctx.prim_batch(7, rows, 1e-6)


def test_nonfinite_rows_terminate(ctx):
    # The reference loops forever on NaN coefficients (src/rpoly.h:151-158);
    # the device code caps that loop and reports it through the status bits.
    rows = C.workloads.primitive_batch(C.VERTEX_FACE, 64, seed=3)
    rows[::2, 5] = np.nan
    rows[1::4, 20] = np.inf
    for path in PATHS:
        h, _ = ctx.prim_batch(C.VERTEX_FACE, rows, 1e-6, path=path)
        st = ctx.stats()
        assert st["rows"] == 64
    good = C.workloads.primitive_batch(C.VERTEX_FACE, 64, seed=3)
    h2, _ = ctx.prim_batch(C.VERTEX_FACE, good, 1e-6)
    assert ctx.stats()["status_flags"] == 0
