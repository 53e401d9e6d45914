"""The device arithmetic (csrc/*.h) compiled for the host, against the oracle
and the golden fixtures.  CPU only."""
import ctypes

import numpy as np
import pytest

from hostcheck.build import core_lib, math_lib

P = ctypes.c_void_p


def _run(lib, fn, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    getattr(lib, fn)(x.ctypes.data_as(P), y.ctypes.data_as(P), ctypes.c_int64(x.size))
    return y


def test_exp_log_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    lib = math_lib()
    rng = np.random.default_rng(3)
    xl = np.concatenate([rng.uniform(0.5, 2.0, 2000), np.exp(rng.uniform(-700, 700, 2000)), [1.0, 2.0, 5e-324]])
    yl = _run(lib, "hc_log", xl)
    for x, y in zip(xl, yl):
        assert y == float(mpmath.log(mpmath.mpf(float(x)))), x
    xe = np.concatenate([rng.uniform(-745, 709, 2000), rng.normal(0, 1e-6, 500), [0.0, 1.0, -1.0]])
    ye = _run(lib, "hc_exp", xe)
    for x, y in zip(xe, ye):
        assert y == float(mpmath.exp(mpmath.mpf(float(x)))), x


def test_exp_log_agree_with_host_libm_mostly():
    # The host C library is not correctly rounded on every input; the device
    # versions are.  They must agree on all but a small fraction.
    lib = math_lib()
    rng = np.random.default_rng(4)
    x = np.exp(rng.uniform(-700, 700, 200000))
    assert np.mean(_run(lib, "hc_log", x) != _run(lib, "hc_libm_log", x)) < 2e-3
    x = rng.uniform(-700, 700, 200000)
    assert np.mean(_run(lib, "hc_exp", x) != _run(lib, "hc_libm_exp", x)) < 2e-3
    specials = np.array([0.0, np.inf, -1.0])
    y = _run(lib, "hc_log", specials)
    assert y[0] == -np.inf and y[1] == np.inf and np.isnan(y[2])
    y = _run(lib, "hc_exp", np.array([1000.0, -1000.0, np.nan]))
    assert y[0] == np.inf and y[1] == 0.0 and np.isnan(y[2])


def _core(kind, x, eta):
    lib = core_lib()
    x = np.ascontiguousarray(x)
    n = x.shape[0]
    e = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, np.float64)))
    per = int(e.size == n and n != 1)
    h = np.zeros(n, np.uint8)
    t = np.full(n, np.nan)
    st = np.zeros(n, np.uint8)
    lib.hc_batch(kind, ctypes.c_int64(n), x.ctypes.data_as(P), e.ctypes.data_as(P), per, h.ctypes.data_as(P),
                 t.ctypes.data_as(P), st.ctypes.data_as(P))
    return h, t, st


def _cull(kind, x, eta):
    lib = core_lib()
    x = np.ascontiguousarray(x)
    n = x.shape[0]
    e = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, np.float64)))
    per = int(e.size == n and n != 1)
    r = np.zeros(n, np.uint8)
    lib.hc_cull(kind, ctypes.c_int64(n), x.ctypes.data_as(P), e.ctypes.data_as(P), per, r.ctypes.data_as(P))
    return r


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_fp64_core_matches_golden(golden_dir, kind):
    g = np.load(f"{golden_dir}/prims.npz")
    h, t, st = _core(kind, g[f"x{kind}"], g[f"eta{kind}"])
    np.testing.assert_array_equal(h, g[f"hit{kind}"])
    m = h == 1
    tr = g[f"t{kind}"][m]
    assert np.all(np.abs(t[m] - tr) <= 1e-12 * np.maximum(np.abs(tr), 1e-300))
    assert st.sum() == 0


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_fp64_core_matches_oracle_random(oracle, kind):
    from collisiondetection_gb300 import workloads as W

    x = W.primitive_batch(kind, 20000, seed=321)
    h_ref, t_ref = oracle.batch(kind, x, 1e-6, nthreads=4)
    h, t, _ = _core(kind, x, 1e-6)
    np.testing.assert_array_equal(h, h_ref)
    m = h == 1
    assert np.all(np.abs(t[m] - t_ref[m]) <= 1e-12 * np.maximum(np.abs(t_ref[m]), 1e-300))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_fp32_cull_has_no_false_negatives(oracle, golden_dir, kind):
    from collisiondetection_gb300 import workloads as W

    g = np.load(f"{golden_dir}/prims.npz")
    cases = [(g[f"x{kind}"], g[f"eta{kind}"]), (W.primitive_batch(kind, 50000, seed=77), 1e-6)]
    if kind == 2:
        # Larger eta: many distance hits; small motion: near-static rows.
        cases.append((W.primitive_batch(kind, 50000, seed=78), 3e-2))
        cases.append((W.primitive_batch(kind, 50000, seed=79, sigma=1e-3), 1e-3))
    for x, eta in cases:
        h, _ = oracle.batch(kind, x, eta, nthreads=4)
        rej = _cull(kind, x, eta)
        assert not np.any((rej == 1) & (h == 1))
        assert rej.mean() > 0.5  # the stage does reject most random rows


def test_vertex_edge_cull_on_mesh_stencils(oracle):
    """Vertex-edge rows of the narrow-phase chain on a real candidate set
    (two icospheres closing in): no false negatives, most rows rejected."""
    from collisiondetection_gb300 import workloads as W

    qs, qe, f = W.two_spheres(seed=1)
    vf, _ = oracle.broadphase(0, qs, qe, f, 1e-6)
    P0, P1 = qs.reshape(-1, 3), qe.reshape(-1, 3)
    rows = []
    for e in range(3):
        ids = np.stack([vf[:, 0], vf[:, 1 + e], vf[:, 1 + (e + 1) % 3]], 1)
        rows.append(np.concatenate([P0[ids].reshape(-1, 9), P1[ids].reshape(-1, 9)], 1))
    x = np.ascontiguousarray(np.concatenate(rows))
    for eta in (1e-6, 1e-2):
        h, _ = oracle.batch(2, x, eta, nthreads=4)
        rej = _cull(2, x, eta)
        assert not np.any((rej == 1) & (h == 1))
        assert rej.mean() > 0.85


def test_fp32_cull_never_rejects_nonfinite():
    for kind, w in ((0, 24), (1, 24), (2, 18)):
        x = np.random.default_rng(0).uniform(0, 1, (8, w))
        x[0, 3] = np.nan
        x[1, w - 4] = np.inf
        x[2, :] = 1e30  # overflows FP32
        rej = _cull(kind, x[:3], 1e-6)
        assert rej.sum() == 0
        assert _cull(kind, x[3:4], np.nan).sum() == 0


def test_fast_exp_log_equal_slow_exact_paths():
    # The table-driven fast paths either prove their rounding or fall back;
    # both must give the correctly rounded double of the series versions.
    lib = math_lib()
    rng = np.random.default_rng(12)
    xl = np.concatenate([rng.uniform(0.5, 2, 200000), np.exp(rng.uniform(-744, 709, 200000)),
                         1 + rng.normal(0, 1e-9, 20000), 1 - np.abs(rng.normal(0, 1e-12, 20000)),
                         [1.0, 0.75, 1.5, 5e-324, 1.7e308, np.nextafter(1.0, 0.0), np.nextafter(1.0, 2.0)]])
    np.testing.assert_array_equal(_run(lib, "hc_log", xl).view(np.uint64), _run(lib, "hc_log_slow", xl).view(np.uint64))
    xe = np.concatenate([rng.uniform(-745, 709.7, 200000), rng.normal(0, 1e-8, 20000),
                         [0.0, -0.0, 699.99, -699.99, 700.1, -700.1, 709.78, -745.1]])
    np.testing.assert_array_equal(_run(lib, "hc_exp", xe).view(np.uint64), _run(lib, "hc_exp_slow", xe).view(np.uint64))


def test_event_heap_matches_priority_queue():
    """The event queue's heap (csrc/ccd_heap.h) pops in std::priority_queue's
    order on the same operations, ties and keys changed under a built heap
    included (the active layers' rollback re-queues groups whose firing times
    were reset)."""
    lib = core_lib()
    rng = np.random.default_rng(12)
    for trial in range(40):
        nkeys = int(rng.integers(1, 60))
        key = rng.integers(0, 6, nkeys).astype(np.float64) * 0.25  # many ties
        n = int(rng.integers(1, 400))
        op = np.where(rng.random(n) < 0.55, rng.integers(0, nkeys, n), -1).astype(np.int32)
        op_key = np.where(rng.random(n) < 0.2, rng.integers(0, nkeys, n), -1).astype(np.int32)
        newkey = rng.integers(0, 6, n).astype(np.float64) * 0.25
        ours = np.full(n, -2, np.int32)
        theirs = np.full(n, -3, np.int32)
        lib.hc_heap_replay(ctypes.c_int(n), op.ctypes.data_as(P), op_key.ctypes.data_as(P), newkey.ctypes.data_as(P),
                           key.ctypes.data_as(P), ctypes.c_int(nkeys), ours.ctypes.data_as(P),
                           theirs.ctypes.data_as(P))
        npop = int((op < 0).sum())
        np.testing.assert_array_equal(ours[:npop], theirs[:npop])
