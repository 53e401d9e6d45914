"""Host-side logic of the bench on the CPU: the parity report that checks the
headline path's hits and contact times against a reference result (the
FP32 cull's false negatives must be 0)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_compare_results_counts_misses_and_time_error():
    h_ref = np.array([1, 1, 0, 1, 0], np.uint8)
    t_ref = np.array([0.5, 0.25, np.nan, 0.75, np.nan])
    h = np.array([1, 0, 1, 1, 0], np.uint8)
    t = np.array([0.5, np.nan, 0.1, 0.75 * (1 + 1e-13), np.nan])
    r = bench.compare_results(h_ref, t_ref, h, t)
    assert r["hits"] == 3 and r["false_negatives"] == 1 and r["false_positives"] == 1
    assert 0.9e-13 < r["max_rel_t_err"] < 1.1e-13 and not r["t_bit_identical"]


def test_compare_results_identical():
    rng = np.random.default_rng(0)
    h = (rng.random(1000) < 0.3).astype(np.uint8)
    t = np.where(h == 1, rng.random(1000), np.nan)
    r = bench.compare_results(h, t, h.copy(), t.copy())
    assert r["false_negatives"] == r["false_positives"] == 0
    assert r["max_rel_t_err"] == 0.0 and r["t_bit_identical"]
    r = bench.compare_results(np.zeros(4, np.uint8), np.full(4, np.nan), np.zeros(4, np.uint8), np.full(4, np.nan))
    assert r["hits"] == 0 and r["max_rel_t_err"] == 0.0 and r["t_bit_identical"]
