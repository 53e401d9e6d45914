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


def _result(hits, fn=0, fp=0, err=0.0, same=True):
    return {"hits": hits, "false_negatives": fn, "false_positives": fp, "max_rel_t_err": err,
            "t_bit_identical": same}


def test_parity_summary_prefers_the_oracle():
    parity = {"cull_refine_vs_fp64_path": {"vf": _result(5), "ee": _result(7)},
              "refine_all_vs_fp64_path": {"vf": _result(5), "ee": _result(7)},
              "cull_refine_vs_oracle": {"vf": _result(5, fn=1), "ee": _result(7, err=2e-13, same=False)}}
    s = bench.parity_summary(parity)
    assert s["vs"] == "oracle" and s["hits"] == 12 and s["false_negatives"] == 1 and s["false_positives"] == 0
    assert s["max_rel_t_err"] == 2e-13 and not s["t_bit_identical"] and s["staged_fp64_identical"]
    del parity["cull_refine_vs_oracle"]
    assert bench.parity_summary(parity)["vs"] == "fp64_path"
    assert bench.parity_summary(None) is None


def test_mesh_summary_and_identity():
    par = {"identical_candidates": True, "identical_collisions": True, "max_rel_t_err": 0.0, "steps": [48, 25, 0]}
    mesh = {"two_spheres_kdop": {"ms_per_step": 5.0, "parity": par},
            "cloth_on_sphere_kdop": {"faces": 211970, "ms_per_step": 2.0, "parity": par,
                                     "traversal": {"frac": 0.5, "achieved_gbs": 3000.0, "traversal_ms": 0.3}}}
    uneven = {"instances": 32, "faces": 10, "one_call": {"ms": 1.0, "value": 2.0}, "per_instance_calls": {"ms": 3.0},
              "parity": dict(par, max_rel_t_err=1e-11)}
    s = bench.mesh_summary(mesh, uneven)
    assert s["two_spheres"]["identical"] and s["cloth_on_sphere"]["identical"]
    assert s["cloth_on_sphere"]["checked_steps"] == [48, 25, 0] and s["cloth_on_sphere"]["traversal"]["frac"] == 0.5
    assert s["uneven_batch"]["identical"] is False  # contact times beyond 1e-12 relative
    assert bench.mesh_summary(None, None) is None


def test_round_floats_keeps_the_line_short():
    x = {"a": 1.0 / 3.0, "b": [2.0 / 3.0, 5], "c": {"d": 123456789.123}, "e": "x", "f": None, "g": True}
    r = bench.round_floats(x)
    assert r["a"] == 0.33333 and r["b"] == [0.66667, 5] and r["c"]["d"] == 123460000.0
    assert r["e"] == "x" and r["f"] is None and r["g"] is True


def test_small_batch_summary():
    g = {"rows_per_kind": 4096, "iters": 50, "direct": {"device_us_per_step": 3081.8, "wall_us_per_step": 3082.0},
         "graph": {"device_us_per_step": 2983.9, "wall_us_per_step": 2984.2}, "replays_match_direct_call": True}
    r = bench.small_batch_summary(g)
    assert r["rows_per_kind"] == 4096 and r["replays_match"] is True
    assert abs(r["ms_direct"] - 3.0818) < 1e-12 and abs(r["ms_graph"] - 2.9839) < 1e-12
    assert bench.small_batch_summary(None) is None
    assert bench.small_batch_summary({"error": "CcdError: x"}) == {"error": "CcdError: x"}
