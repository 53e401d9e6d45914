"""Benchmark: swept primitive-pair CTCD tests per second on one GB300.

Workload (the raw narrow-phase batch): 10M vertex-face + 10M edge-edge swept
quadruples in FP64, start ~ U[0,1]^3, end = start + N(0, 0.1), eta = 1e-6,
20% built near-degenerate (coplanar / parallel to 1e-9, tangential double
roots); seeded synthetic data (collisiondetection_gb300/workloads.py).

One step = every row of both kinds through the FP32-cull + FP64-refine path
(the two kinds on two contexts and streams, which overlaps each batch's
latency-bound tail with the other's bulk).
  value : tests/s with rows resident in HBM (device entry point), CUDA events
  e2e   : tests/s through ccd_prim_batch with host buffers, copies included
          (one host thread per kind)
Also reported: the plain all-FP64 GPU path on the same rows, the roofline of
the dominant kernel, the CPU baseline (oracle restatement, all host cores).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "swept prim-pair tests/s (10M VF + 10M EE swept quadruples, FP64)"
UNIT = "tests/s"
ETA = 1e-6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-vf", type=int, default=10_000_000)
    ap.add_argument("--n-ee", type=int, default=10_000_000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-sample", type=int, default=0,
                    help="reference arm: rows per kind per step (0: every row, the same config as this arm)")
    ap.add_argument("--mesh", type=int, default=1, help="also time the mesh configurations (1) or not (0)")
    ap.add_argument("--uneven-parity", type=int, default=32,
                    help="instances of the uneven batch checked against the oracle")
    ap.add_argument("--uneven-instances", type=int, default=512,
                    help="instances of the uneven-batch sample (0: skip; the configuration has 512)")
    ap.add_argument("--distance", type=int, default=1,
                    help="also time meshSelfDistance, the closest-point batches and the penalty forces (1) or not (0)")
    ap.add_argument("--velocity", type=int, default=1, help="also time the velocity filter (1) or not (0)")
    ap.add_argument("--vf-grid", type=int, default=16, help="sheet resolution of the velocity-filter scene")
    ap.add_argument("--vf-events-per-launch", type=int, default=0,
                    help="velocity filter: firings per event-loop launch (0: the library's default); short launches "
                         "for profilers")
    ap.add_argument("--serve", type=int, default=1, help="also run the serving loop (1) or not (0)")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[100.0, 200.0, 500.0, 1000.0, 2000.0, 5000.0])
    ap.add_argument("--serve-fp64-requests", type=int, default=6)
    ap.add_argument("--graph-rows", type=int, default=4096,
                    help="rows per kind of the small-batch CUDA-graph comparison (0: skip it)")
    ap.add_argument("--graph-iters", type=int, default=50)
    ap.add_argument("--autotune", type=int, default=1,
                    help="choose each context's refinement work split with ccd_autotune_prim_batch first (1) or not (0)")
    ap.add_argument("--only", default="all", choices=["all", "device", "mesh"],
                    help="device: only the resident cull + refine steps; mesh: only the mesh configurations "
                         "(two spheres, cloth on sphere), printing their summary (short runs for profilers)")
    ap.add_argument("--cloth-grid", type=int, default=256)
    ap.add_argument("--cloth-level", type=int, default=6)
    ap.add_argument("--cloth-steps", type=int, default=50)
    ap.add_argument("--detail-out", default=os.path.join(ROOT, "gpurun_out", "bench_detail.json"),
                    help="where the full results go (the printed line is their summary)")
    return ap.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def workload(n_vf, n_ee):
    from collisiondetection_gb300 import workloads as W

    return (W.primitive_batch(W.KIND_VF, n_vf, seed=1), W.primitive_batch(W.KIND_EE, n_ee, seed=2))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def compare_results(h_ref, t_ref, h, t):
    """Hit sets and contact times of (h, t) against a reference result of the
    same rows: rows the reference hits and (h, t) misses (false negatives),
    the converse, and the largest relative contact-time error over common
    hits (t is only defined where hit)."""
    ref = np.asarray(h_ref).astype(bool)
    got = np.asarray(h).astype(bool)
    both = ref & got
    tr, tg = np.asarray(t_ref)[both], np.asarray(t)[both]
    rel = np.abs(tg - tr) / np.maximum(np.abs(tr), 1e-300)
    return {"hits": int(ref.sum()), "false_negatives": int((ref & ~got).sum()),
            "false_positives": int((~ref & got).sum()), "max_rel_t_err": float(rel.max()) if rel.size else 0.0,
            "t_bit_identical": bool(np.array_equal(tr.view(np.uint64), tg.view(np.uint64)))}


def workload_config(args) -> dict:
    """The workload both arms run (identical in the reference arm's line)."""
    return {"workload": f"raw narrow-phase batch, {args.n_vf:,} VF + {args.n_ee:,} EE swept quadruples, eta=1e-6, "
                        "20% near-degenerate",
            "rows_per_step": args.n_vf + args.n_ee, "bytes_per_step": 192 * (args.n_vf + args.n_ee),
            "l2": "inputs larger than L2 (129 MB); no flush"}


def compact(d, keys):
    return None if d is None else {k: d[k] for k in keys if k in d}


def round_floats(x, digits=5):
    """Shortens the floats of the bench line (the line must stay a few KB)."""
    if isinstance(x, float):
        return float(f"{x:.{digits}g}")
    if isinstance(x, dict):
        return {k: round_floats(v, digits) for k, v in x.items()}
    if isinstance(x, list):
        return [round_floats(v, digits) for v in x]
    return x


def parity_summary(parity):
    """False negatives / positives and contact-time error of the headline
    path over every row, against the oracle (else the plain FP64 GPU path)."""
    if not parity:
        return None
    ref = parity.get("cull_refine_vs_oracle") or parity["cull_refine_vs_fp64_path"]
    out = {"vs": "oracle" if "cull_refine_vs_oracle" in parity else "fp64_path",
           "rows": "all rows of both kinds"}
    for key in ("false_negatives", "false_positives"):
        out[key] = sum(ref[k][key] for k in ref)
    out["hits"] = sum(ref[k]["hits"] for k in ref)
    out["max_rel_t_err"] = max(ref[k]["max_rel_t_err"] for k in ref)
    out["t_bit_identical"] = all(ref[k]["t_bit_identical"] for k in ref)
    st = parity.get("refine_all_vs_fp64_path")
    if st:
        out["staged_fp64_identical"] = all(st[k]["false_negatives"] == 0 and st[k]["false_positives"] == 0 and
                                           st[k]["t_bit_identical"] for k in st)
    return out


def mesh_summary(mesh, uneven):
    """Mesh configurations in a few numbers: step time, parity against the
    oracle (identical candidate and colliding sets) and the traversal's
    roofline."""
    if not mesh and not uneven:
        return None
    out = {}
    if mesh:
        c1 = mesh.get("two_spheres_kdop", {})
        out["two_spheres"] = {"ms_per_step": c1.get("ms_per_step"),
                              "identical": _identical(c1.get("parity"))}
        c3 = mesh.get("cloth_on_sphere_kdop", {})
        tr = c3.get("traversal", {})
        out["cloth_on_sphere"] = {"faces": c3.get("faces"), "ms_per_step": c3.get("ms_per_step"),
                                  "graph_ms_per_step": (c3.get("graph") or {}).get("ms_per_step"),
                                  "identical": _identical(c3.get("parity")),
                                  "checked_steps": (c3.get("parity") or {}).get("steps"),
                                  "traversal": {"frac": tr.get("frac"), "achieved_gbs": tr.get("achieved_gbs"),
                                                "ms": tr.get("traversal_ms"),
                                                "frac_built_tree": (tr.get("built") or {}).get("frac"),
                                                "ms_built_tree": (tr.get("built") or {}).get("traversal_ms")}}
    if uneven:
        out["uneven_batch"] = {"instances": uneven.get("instances"), "faces": uneven.get("faces"),
                               "ms": uneven["one_call"]["ms"], "value": uneven["one_call"]["value"],
                               "graph_ms": uneven.get("one_call_graph", {}).get("ms"),
                               "per_instance_ms": uneven.get("per_instance_calls", {}).get("ms"),
                               "identical": _identical(uneven.get("parity"))}
    return out


def serving_summary(serving):
    """Per arrival rate: throughput and per-step latency percentiles."""
    if not serving or "rates" not in serving:
        return None
    r = serving["rates"]
    return {"requests": serving.get("requests"), "rates": [x["arrival_rate"] for x in r],
            "req_s": [x["throughput_req_s"] for x in r], "step_ms_p50": [x["step_ms_p50"] for x in r],
            "step_ms_p95": [x["step_ms_p95"] for x in r], "step_ms_p99": [x["step_ms_p99"] for x in r],
            "collisions": [x["collisions"] for x in r],
            "fp64_one_at_a_time_req_s": serving.get("fp64_one_at_a_time", {}).get("throughput_req_s")}


def small_batch_summary(graph):
    """The small-batch step (4,096 + 4,096 rows by default) issued directly
    and replayed from a CUDA graph: ms per step on the device."""
    if not graph:
        return None
    if "error" in graph:
        return {"error": graph["error"]}
    return {"rows_per_kind": graph.get("rows_per_kind"),
            "ms_direct": graph["direct"]["device_us_per_step"] / 1e3,
            "ms_graph": graph["graph"]["device_us_per_step"] / 1e3,
            "replays_match": graph.get("replays_match_direct_call")}


def _identical(par):
    if not par:
        return None
    return bool(par["identical_candidates"] and par["identical_collisions"] and par["max_rel_t_err"] <= 1e-12)


def write_detail(args, detail) -> str:
    """Writes the bench's full results beside the one-line summary."""
    path = args.detail_out
    try:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "w") as fh:
            json.dump(detail, fh, indent=1, default=str)
    except OSError as exc:
        return f"not written: {exc}"
    return os.path.relpath(path, ROOT) if os.path.abspath(path).startswith(ROOT) else path


def cpu_baseline(vf, ee, max_rows=None, results=None):
    """The oracle restatement of the reference's CPU path on all host cores.
    With `results` (a dict), the oracle's (hit, t) per kind go into it too:
    the bench checks the GPU's results against them."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    orc = O.Oracle()
    threads = os.cpu_count() or 1
    if max_rows:
        vf, ee = vf[:max_rows], ee[:max_rows]
    t0 = time.perf_counter()
    out_vf = orc.batch(0, vf, ETA, nthreads=threads)
    out_ee = orc.batch(1, ee, ETA, nthreads=threads)
    dt = time.perf_counter() - t0
    if results is not None:
        results["vf"], results["ee"] = out_vf, out_ee
    rows = vf.shape[0] + ee.shape[0]
    return {"value": rows / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{vf.shape[0]} VF + {ee.shape[0]} EE rows of the same workload, {dt:.2f} s wall"}


def mesh_section(ctx, stream, rank, args):
    """Mesh configurations through the mesh entry points, one detection step
    = set positions (host -> device) + broad phase + narrow phase over every
    candidate + read back the colliding stencils.  Unit: candidate stencil
    tests per second (the reference's exact candidate set; broad phase in
    the wall time).  The oracle times the same steps on the host cores."""
    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    orc = O.Oracle()
    threads = os.cpu_count() or 1
    out = {}

    def run_steps(m, frames, kind, eta, reps, graph=False):
        ctx.synchronize()
        tests, hits, dts = 0, 0, []
        for _ in range(reps):
            for k in range(len(frames) - 1):
                torch_sync()
                t0 = time.perf_counter()
                m.set_positions(frames[k], frames[k + 1])
                vf, vft, ee, eet = m.detect(kind, eta, eta, path=C.PATH_CULL_REFINE, graph=graph)
                dts.append(time.perf_counter() - t0)
                st = m.stats()
                tests += st["n_vf"] + st["n_ee"]
                hits += vf.shape[0] + ee.shape[0]
        return tests, hits, dts

    def torch_sync():
        import torch

        torch.cuda.synchronize()

    def oracle_steps(m, frames, faces, eta, idx):
        """The oracle's broad and narrow phase on steps idx, timed, and each
        step's candidate and colliding sets checked against the GPU's (the
        graph-step entry point, as the timed steps use)."""
        t_bp = t_np = 0.0
        checks = []
        for k in idx:
            m.set_positions(frames[k], frames[k + 1])
            col = m.detect(C.BROADPHASE_KDOP13, eta, eta, path=C.PATH_CULL_REFINE, graph=True)
            cand = m.candidates()
            t0 = time.perf_counter()
            vf, ee = orc.broadphase(0, frames[k], frames[k + 1], faces, eta)
            t1 = time.perf_counter()
            out = orc.narrowphase(frames[k], frames[k + 1], vf, eta, ee, eta, nthreads=threads)
            t2 = time.perf_counter()
            t_bp += t1 - t0
            t_np += t2 - t1
            checks.append(O.compare_step_results(vf, ee, out, cand, col))
        return 1e3 * t_bp / len(idx), 1e3 * t_np / len(idx), O.merge_checks(checks, idx)

    # Two level-3 icospheres (2 x 642 v / 1,280 f), 0.8 approach + N(0, 0.01) jitter.
    qs, qe, f = W.two_spheres(seed=1)
    frames = np.stack([qs, qe])
    with C.Mesh(ctx, f, qs, qe) as m:
        for label, kind in (("kdop", C.BROADPHASE_KDOP13), ("aabb", C.BROADPHASE_AABB)):
            run_steps(m, frames, kind, 1e-6, 3)  # warm-up
            tests, hits, dts = run_steps(m, frames, kind, 1e-6, 20)
            ms = 1e3 * statistics.median(dts)
            out[f"two_spheres_{label}"] = {
                "ms_per_step": ms, "stencil_tests_per_step": tests // 20, "collisions_per_step": hits // 20,
                "value": (tests // 20) / (ms / 1e3), "unit": "stencil tests/s"}
        if rank == 0:
            bp, nph, par = oracle_steps(m, frames, f, 1e-6, [0])
            out["two_spheres_kdop"]["cpu_oracle"] = {"broadphase_ms": bp, "narrowphase_ms": nph,
                                                     "cores": {"broadphase": 1, "narrowphase": threads}}
            out["two_spheres_kdop"]["parity"] = par
    # Cloth on sphere: sheet + level-6 icosphere, one step per frame pair.
    faces, frames = W.cloth_frames(grid=args.cloth_grid, level=args.cloth_level, seed=0, steps=args.cloth_steps)
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        run_steps(m, frames[:4], C.BROADPHASE_KDOP13, 1e-6, 1)  # warm-up
        tests, hits, dts = run_steps(m, frames, C.BROADPHASE_KDOP13, 1e-6, 1)
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        # the same steps through ccd_mesh_detect_graph (captured step replayed)
        run_steps(m, frames[:4], C.BROADPHASE_KDOP13, 1e-6, 1, graph=True)  # warm-up
        gtests, ghits, gdts = run_steps(m, frames, C.BROADPHASE_KDOP13, 1e-6, 1, graph=True)
        total = sum(dts)
        out["cloth_on_sphere_kdop"] = {
            "faces": int(faces.shape[0]), "vertices": int(frames.shape[1] // 3), "steps": len(dts),
            "entry_point": "ccd_mesh_detect", "ms_per_step": 1e3 * total / len(dts),
            "ms_per_step_p50": 1e3 * statistics.median(dts), "ms_per_step_max": 1e3 * max(dts),
            "stencil_tests": tests, "collisions": hits, "value": tests / total, "unit": "stencil tests/s",
            "graph": {"entry_point": "ccd_mesh_detect_graph", "ms_per_step": 1e3 * sum(gdts) / len(gdts),
                      "ms_per_step_p50": 1e3 * statistics.median(gdts),
                      "same_as_direct": bool(gtests == tests and ghits == hits)}}
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        run_steps(m, frames[:4], C.BROADPHASE_KDOP13, 1e-6, 1)
        for k in range(len(frames) // 2):  # the kept tree as the stepping leaves it
            m.set_positions(frames[k], frames[k + 1])
            m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, fetch=False)
        # Traversal roofline of one step (k = steps / 2): slab tests from a
        # counting run, device time from timed runs without the counter; on
        # the tree the stepping kept and refitted since the first step, and
        # on a tree built for this step.
        k = len(frames) // 2
        m.set_positions(frames[k], frames[k + 1])
        peak, src = measured_peaks()

        def traversal(label):
            ctx.set_option("count_slab_tests", 1)
            m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
            tests = m.stats()["slab_tests"]
            pairs = m.stats()["face_pairs"]
            ctx.set_option("count_slab_tests", 0)
            ctx.set_profiling(True)
            trav, bpms = [], []
            for _ in range(9):
                m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
                trav.append(m.stats()["traversal_ms"])
                bpms.append(m.stats()["broadphase_ms"])
            ctx.set_profiling(False)
            tms = statistics.median(trav)
            algo = tests * 13 * 2 * 4 + pairs * 8  # 13-DOP FP32 slab per test, a pair written per hit
            return {"tree": label, "kernel": "find_pairs_quad (four lanes per query face)", "slab_tests": tests,
                    "face_pairs": pairs, "traversal_ms": tms, "broadphase_ms": statistics.median(bpms),
                    "algorithmic_bytes": algo, "achieved_gbs": algo / (tms / 1e3) / 1e9, "peak_gbs": peak,
                    "frac": algo / (tms / 1e3) / 1e9 / peak}

        refitted = traversal("kept since the first step, refitted")
        ctx.set_option("tree_refit", 0)
        built = traversal("built for this step")
        ctx.set_option("tree_refit", 1)
        out["cloth_on_sphere_kdop"]["traversal"] = dict(
            refitted, built=built,
            note="the tree (about 300 B per face: two 128 B slab records and the links) fits in L2, so DRAM is not "
                 "what bounds this traversal")
        if rank == 0:
            idx = [len(frames) - 2, len(frames) // 2, (4 * len(frames)) // 5]
            bp, nph, par = oracle_steps(m, frames, faces, 1e-6, idx)
            out["cloth_on_sphere_kdop"]["cpu_oracle"] = {"broadphase_ms": bp, "narrowphase_ms": nph,
                                                        "sample_steps": idx,
                                                        "cores": {"broadphase": 1, "narrowphase": threads}}
            out["cloth_on_sphere_kdop"]["parity"] = par
    return out


def distance_section(ctx, stream, rank, args):
    """Distance::meshSelfDistance (src/Distance.cpp:12-66) and the closest-point
    batch kernels.

    self_distance: wall time of ccd_mesh_self_distance (positions copied from
    host memory, the vertex scan on a point tree, the AABB broad phase, the
    stencil minimum, result read back) on the two-sphere start frame (2,560
    faces) and on one sheet-on-sphere frame (211,970 faces).  The oracle is
    timed beside it on one core: the whole call on the spheres; on the sheet,
    its O(V F) vertex scan over a bounded sample of vertices, scaled to all of
    them, plus its broad phase and stencil stage at the same padding.

    closest_point_batch: 10M vertex-face + 10M edge-edge rows of 12 doubles
    resident in HBM through ccd_distance_batch_device (vectors and barycentric
    coordinates out), timed with CUDA events on the launching stream; HBM
    roofline with 96 B in + 24 B vector + 24 (32) B barycentrics per row."""
    import torch

    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    orc = O.Oracle()
    out = {}
    qs, _, f_sph = W.two_spheres(seed=1)
    f_cl, frames = W.cloth_frames(grid=args.cloth_grid, level=args.cloth_level, seed=0, steps=2)
    cases = (("two_spheres", qs.reshape(-1, 3), f_sph), ("cloth_on_sphere", frames[1].reshape(-1, 3), f_cl))
    for name, v, f in cases:
        v = np.ascontiguousarray(v, np.float64)
        with C.Mesh(ctx, f, nverts=v.shape[0]) as m:
            for _ in range(3):
                m.self_distance(v)
            dts = []
            for _ in range(10):
                t0 = time.perf_counter()
                d, nvf, nee = m.self_distance(v)
                dts.append(time.perf_counter() - t0)
            eta = m.stats()["self_distance_eta"]
        entry = {"faces": int(f.shape[0]), "vertices": int(v.shape[0]), "distance": d, "padding": eta,
                 "stencils": {"vf": nvf, "ee": nee}, "ms": 1e3 * statistics.median(dts),
                 "ms_min": 1e3 * min(dts)}
        if rank == 0:
            nv = v.shape[0]
            if f.shape[0] <= 10_000:
                t0 = time.perf_counter()
                d_ref, _, _ = orc.mesh_self_distance(v, f)
                entry["cpu_oracle"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": 1, "sample": "whole call",
                                       "same_result": float(d_ref).hex() == float(d).hex()}
            else:
                sample = max(1, nv // 128)
                t0 = time.perf_counter()
                orc.vertex_scan(v, f, 0, sample)
                scan_ms = 1e3 * (time.perf_counter() - t0) * nv / sample
                t0 = time.perf_counter()
                vf, ee = orc.broadphase(1, v.ravel(), v.ravel(), f, eta)
                orc.distance(0, v[vf].reshape(-1, 12))
                orc.distance(1, v[ee].reshape(-1, 12))
                rest_ms = 1e3 * (time.perf_counter() - t0)
                entry["cpu_oracle"] = {"ms": scan_ms + rest_ms, "vertex_scan_ms": scan_ms,
                                       "broadphase_and_stencils_ms": rest_ms, "cores": 1,
                                       "sample": f"vertex scan over {sample} of {nv} vertices, scaled"}
        out[name] = entry
    # closest-point batch throughput, rows resident in HBM
    n = 10_000_000
    g = torch.Generator(device="cuda").manual_seed(7)
    peak, src = measured_peaks()
    batch = {}
    total_ms, total_bytes = 0.0, 0
    for kind, label, nb in ((C.DISTANCE_VERTEX_FACE, "vertex_face", 3), (C.DISTANCE_EDGE_EDGE, "edge_edge", 4)):
        rows = torch.rand((n, 12), generator=g, device="cuda", dtype=torch.float64)
        vec = torch.empty((n, 3), device="cuda", dtype=torch.float64)
        bary = torch.empty((n, nb), device="cuda", dtype=torch.float64)
        for _ in range(3):
            ctx.distance_device(kind, n, rows.data_ptr(), vec.data_ptr(), bary.data_ptr())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        e0.record(stream)
        for _ in range(reps):
            ctx.distance_device(kind, n, rows.data_ptr(), vec.data_ptr(), bary.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        nbytes = n * (96 + 24 + 8 * nb)
        batch[label] = {"rows": n, "ms_per_launch": ms, "rows_per_s": n / (ms / 1e3),
                        "achieved_gbs": nbytes / (ms / 1e3) / 1e9}
        total_ms += ms
        total_bytes += nbytes
        del rows, vec, bary
    batch["roofline"] = {"kernel": "distance_rows<0|1>", "bound": "hbm", "achieved": total_bytes / (total_ms / 1e3) / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": total_bytes / (total_ms / 1e3) / 1e9 / peak,
                         "peak_source": f"{src} hbm_gbs",
                         "note": "inputs (0.96 GB per kind) larger than L2; algorithmic bytes per row "
                                 "96 in + 24 vector + 24 (32) barycentrics"}
    out["closest_point_batch"] = batch
    return out


def penalty_section(ctx, rank, args):
    """PenaltyGroup::addForce (src/PenaltyGroup.cpp:34-52) on one group made of
    every k-DOP candidate of one sheet-on-sphere frame (211,970 faces) at a
    padding of 0.005 (about a third of the sheet's spacing): wall time of
    ccd_penalty_group_force (positions, velocities, forces and stencils from
    host memory, forces and fired flags back), with the oracle's sequential
    restatement timed beside it on one core."""
    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    f, frames = W.cloth_frames(grid=args.cloth_grid, level=args.cloth_level, seed=0, steps=50)
    q = frames[40]
    v = (frames[41] - frames[39]) / 2
    eta = 0.005
    with C.Mesh(ctx, f, q, q) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, eta)
    F0 = np.zeros_like(q)
    args_ = (q, v, F0, vf, ee, eta, 1e-6, 1.0, 0.1, 1e-3)
    for _ in range(2):
        ctx.penalty_group_force(*args_)
    dts = []
    for _ in range(5):
        t0 = time.perf_counter()
        F, vfire, efire, _used = ctx.penalty_group_force(*args_)
        dts.append(time.perf_counter() - t0)
    # the same group resident on the device (ccd_penalty_group_force_device)
    import torch

    d = {k: torch.from_numpy(np.ascontiguousarray(a)).cuda() for k, a in (("q", q), ("v", v), ("vf", vf), ("ee", ee))}
    dF = torch.zeros(q.size, dtype=torch.float64, device="cuda")
    dvf = torch.zeros(vf.shape[0], dtype=torch.uint8, device="cuda")
    dee = torch.zeros(ee.shape[0], dtype=torch.uint8, device="cuda")

    def dev_call():
        ctx.penalty_group_force_device(q.size // 3, d["q"].data_ptr(), d["v"].data_ptr(), vf.shape[0],
                                       d["vf"].data_ptr(), ee.shape[0], d["ee"].data_ptr(), eta, 1e-6, 1.0, 0.1, 1e-3,
                                       dF.data_ptr(), dvf.data_ptr(), dee.data_ptr())

    for _ in range(2):
        dev_call()
    torch.cuda.synchronize()
    ddts = []
    for _ in range(5):
        dF.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_call()
        ctx.synchronize()
        ddts.append(time.perf_counter() - t0)
    same_dev = bool(np.array_equal(dF.cpu().numpy().view(np.uint64), F.view(np.uint64)))
    out = {"faces": int(f.shape[0]), "stencils": {"vf": int(vf.shape[0]), "ee": int(ee.shape[0])},
           "fired": {"vf": int(vfire.sum()), "ee": int(efire.sum())},
           "host_memory": {"ms": 1e3 * statistics.median(dts),
                           "stencils_per_s": (vf.shape[0] + ee.shape[0]) / statistics.median(dts),
                           "entry_point": "ccd_penalty_group_force (pageable host buffers, 0.42 GB of stencils in)"},
           "device_memory": {"ms": 1e3 * statistics.median(ddts),
                             "stencils_per_s": (vf.shape[0] + ee.shape[0]) / statistics.median(ddts),
                             "entry_point": "ccd_penalty_group_force_device", "same_forces": same_dev}}
    if rank == 0:
        orc = O.Oracle()
        t0 = time.perf_counter()
        Fr = orc.penalty_group_force(*args_)[0]
        out["cpu_oracle"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": 1, "sample": "whole group",
                             "same_forces": bool(np.array_equal(Fr.view(np.uint64), F.view(np.uint64)))}
    return out


def velocity_filter_section(ctx, rank, args):
    """VelocityFilter::velocityFilter (src/VelocityFilter.cpp:15-87) through
    ccd_velocity_filter, wall time of the whole call (host memory in and out),
    with the oracle's sequential restatement timed beside it on one core:
      sheets: a 16x16 sheet (512 vertices with the fixed lower one) dropped
        onto a fixed sheet, layers of 0.2 / 0.1 of the sheet spacing; one
        rollback iteration, 282,050 group firings over groups spanning the
        contact (thousands of stencils each);
      triangles: a triangle falling through a fixed one (2 stencils per
        group, 1.7 M firings): the latency-bound extreme."""
    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    orc = O.Oracle()
    scenes = {}
    g = args.vf_grid
    v, f = W.grid_sheet(g, g)
    v = np.asarray(v).reshape(-1, 3)
    n = v.shape[0]
    upper = v.copy()
    upper[:, 2] += 0.02
    q0 = np.concatenate([v, upper])
    q1 = q0.copy()
    q1[n:, 2] -= 0.04
    mi = np.ones(q0.size)
    mi[: 3 * n] = 0
    sp = 1.0 / (g - 1)
    scenes["sheets"] = (q0, q1, np.concatenate([f, f + n]).astype(np.int32), mi, 0.2 * sp, 0.1 * sp)
    t0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.1], [1.2, 0.2, 0.1], [0.2, 1.2, 0.1]], float)
    t1 = t0.copy()
    t1[3:, 2] = -0.1
    tm = np.ones(18)
    tm[:9] = 0
    scenes["triangles"] = (t0, t1, np.array([[0, 1, 2], [3, 4, 5]], np.int32), tm, 0.01, 0.005)
    out = {}
    if args.vf_events_per_launch:
        ctx.set_option("layer_events_per_launch", args.vf_events_per_launch)
    for name, (a, b, ff, m, oe, ie) in scenes.items():
        t = time.perf_counter()
        res, qe, st = ctx.velocity_filter(a, b, ff, m, oe, ie)
        gpu_s = time.perf_counter() - t
        entry = {"vertices": int(a.size // 3), "faces": int(ff.shape[0]), "result": res,
                 "iterations": st["iterations"], "layers": st["layers"], "firings": st["events"],
                 "gpu_s": gpu_s, "firings_per_s": st["events"] / gpu_s if gpu_s > 0 else None}
        if rank == 0:
            t = time.perf_counter()
            r2, q2, ev = orc.velocity_filter(a, b, ff, m, oe, ie)
            entry["cpu_oracle"] = {"s": time.perf_counter() - t, "cores": 1, "sample": "whole call",
                                   "same_result": bool(r2 == res and np.array_equal(q2.view(np.uint64),
                                                                                    qe.view(np.uint64)))}
        out[name] = entry
    return out


def serving_section(args):
    """Serving loop: Poisson arrivals of collision queries (a mesh pair that
    closes in and touches halfway through 10 steps of seeded rigid + jitter
    motion, triangle counts log-uniform in [1e3, 5e5])
    through the serving engine (ccd_server_*, 4 slots, 60 GB admission
    budget).  Reports throughput and per-step latency percentiles at each
    arrival rate, beside the same queries one at a time on the plain FP64
    path (a subset)."""
    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    rng = np.random.default_rng(7)
    n_req = args.serve_requests
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(5e5), n_req)).astype(int)
    reqs = [W.pair_request(int(t), 1000 + i, steps=10) for i, t in enumerate(sizes)]
    out = {"requests": n_req, "steps_per_request": 10, "faces_mean": float(np.mean([f.shape[0] for f, _ in reqs])),
           "slots": 4, "memory_budget_gb": 60, "rates": []}

    def pct(x, q):
        return float(np.percentile(np.asarray(x), q)) if len(x) else None

    with C.Server(0, slots=4, memory_budget=60 << 30) as srv:
        # warm-up: one small query per slot
        for t in [srv.submit(*reqs[int(np.argmin(sizes))]) for _ in range(4)]:
            srv.wait(t)
        for rate in args.serve_rates:
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
            t0 = time.perf_counter()
            tickets = []
            for (f, fr), at in zip(reqs, arrivals):
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(f, fr))
            results = [srv.wait(t) for t in tickets]
            wall = time.perf_counter() - t0
            step_ms = np.concatenate([r["step_ms"] for r in results])
            req_ms = [r["total_ms"] for r in results]
            out["rates"].append({
                "arrival_rate": rate, "throughput_req_s": n_req / wall,
                "step_ms_p50": pct(step_ms, 50), "step_ms_p95": pct(step_ms, 95), "step_ms_p99": pct(step_ms, 99),
                "request_ms_p50": pct(req_ms, 50), "request_ms_p95": pct(req_ms, 95),
                "request_ms_p99": pct(req_ms, 99), "collisions": int(sum(len(st[0]) + len(st[2])
                                                                          for r in results for st in r["steps"]))})
    # Plain FP64 path, one query at a time (a subset of the same queries).
    sub = list(range(min(args.serve_fp64_requests, n_req)))
    with C.Server(0, slots=1, memory_budget=60 << 30) as srv:
        t0 = time.perf_counter()
        res = [srv.wait(srv.submit(*reqs[i], path=C.PATH_FP64)) for i in sub]
        wall = time.perf_counter() - t0
    step_ms = np.concatenate([r["step_ms"] for r in res])
    out["fp64_one_at_a_time"] = {"requests": len(sub), "throughput_req_s": len(sub) / wall,
                                 "step_ms_p50": pct(step_ms, 50), "step_ms_p99": pct(step_ms, 99)}
    return out


def uneven_section(args, rank):
    """Uneven batch: independent mesh instances (icospheres and grid-sheet
    pairs, triangle counts log-uniform in [200, 2e5], rigid + jitter motion)
    detected in one call on a mesh of instances, against the same instances
    one call each.  Unit: candidate stencil tests per second."""
    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import workloads as W

    n = args.uneven_instances
    faces, frames, vo, fo = W.uneven_batch(n, seed=0)
    ctx = C.Context(0)
    out = {"instances": n, "of_config_instances": 512, "faces": int(faces.shape[0]),
           "vertices": int(frames.shape[1] // 3)}
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3, instances=(vo, fo)) as m:
        m.set_positions(frames[0], frames[1])
        m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, fetch=False)  # warm-up
        t0 = time.perf_counter()
        m.set_positions(frames[0], frames[1])
        col = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
        dt = time.perf_counter() - t0
        st = m.stats()
        cand = m.candidates()
        # The same step from a captured graph (ccd_mesh_detect_graph: the
        # first call runs it directly and captures, the second replays).
        m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, fetch=False, graph=True)
        t0 = time.perf_counter()
        m.set_positions(frames[0], frames[1])
        gcol = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, graph=True)
        gdt = time.perf_counter() - t0
        greplay = m.stats()["graph_replay"]
    tests = st["n_vf"] + st["n_ee"]
    out["one_call"] = {"ms": 1e3 * dt, "stencil_tests": tests, "collisions": st["vf_hits"] + st["ee_hits"],
                       "value": tests / dt, "unit": "stencil tests/s", "entry_point": "ccd_mesh_detect"}
    out["one_call_graph"] = {"ms": 1e3 * gdt, "value": tests / gdt, "unit": "stencil tests/s",
                             "entry_point": "ccd_mesh_detect_graph", "replayed": bool(greplay),
                             "same_as_direct": all(np.array_equal(a, b) for a, b in zip(gcol, col))}
    if rank == 0:
        # The first `uneven_parity` instances through the oracle, each alone
        # (instances are never paired), against the one call's results for
        # them: stencils come out ordered by vertex, and instances own
        # consecutive vertex ranges, so they are the stencils below vo[np_].
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        np_ = min(n, args.uneven_parity)
        lim = vo[np_]

        def below(st):
            return st.max(axis=1) < lim if st.size else np.zeros(0, bool)

        mv, me_ = below(col[0]), below(col[2])
        col = (col[0][mv], col[1][mv], col[2][me_], col[3][me_])
        cand = (cand[0][below(cand[0])], cand[1][below(cand[1])])
        orc = O.Oracle()
        parts = {"vf_c": [], "ee_c": [], "vf_hit": [], "ee_hit": [], "vf_t": [], "ee_t": []}
        t0 = time.perf_counter()
        for i in range(np_):
            a, b = 3 * vo[i], 3 * vo[i + 1]
            qs, qe = frames[0][a:b], frames[1][a:b]
            fi = faces[fo[i]:fo[i + 1]] - vo[i]
            vf_c, ee_c = orc.broadphase(0, qs, qe, fi, 1e-6)
            r = orc.narrowphase(qs, qe, vf_c, 1e-6, ee_c, 1e-6, nthreads=os.cpu_count() or 1)
            parts["vf_c"].append(vf_c + vo[i])
            parts["ee_c"].append(ee_c + vo[i])
            for k in ("vf_hit", "ee_hit", "vf_t", "ee_t"):
                parts[k].append(r[k])
        cat = {k: np.concatenate(v) for k, v in parts.items()}
        par = O.compare_step_results(cat["vf_c"], cat["ee_c"], cat, cand, col)
        par["instances"] = np_
        par["oracle_s"] = time.perf_counter() - t0
        out["parity"] = par
    # One mesh at a time (created, warmed up and freed outside the timed
    # steps, as the one call was).
    hits, dt1 = 0, 0.0
    for i in range(n):
        with C.Mesh(ctx, faces[fo[i]:fo[i + 1]] - vo[i], nverts=int(vo[i + 1] - vo[i])) as mi:
            a, b = 3 * vo[i], 3 * vo[i + 1]
            mi.set_positions(frames[0][a:b], frames[1][a:b])
            mi.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, fetch=False)
            t0 = time.perf_counter()
            mi.set_positions(frames[0][a:b], frames[1][a:b])
            vf, vft, ee, eet = mi.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
            dt1 += time.perf_counter() - t0
            hits += vf.shape[0] + ee.shape[0]
    out["per_instance_calls"] = {"ms": 1e3 * dt1, "collisions": hits, "value": tests / dt1,
                                 "unit": "stencil tests/s"}
    ctx.close()
    return out


def graph_section(ctx, stream, args):
    """Small device batches issued directly and replayed from a CUDA graph.

    One step is `graph_rows` vertex-face rows and as many edge-edge rows
    through ccd_prim_batch_device on one context and stream: the size of a
    serving step's narrow phase, where launch costs are a visible share.  The
    step is captured once (after a direct call that sizes the context's
    scratch) and replayed; replays must reproduce the direct call's hits and
    contact times bit for bit.  Errors are reported, not raised, so that
    this section cannot stop the bench line."""
    import torch

    import collisiondetection_gb300 as C

    try:
        n = args.graph_rows
        ctx.set_profiling(False)
        bufs = {}
        with torch.cuda.stream(stream):
            for kind in (C.VERTEX_FACE, C.EDGE_EDGE):
                rows = C.workloads.primitive_batch(kind, n, seed=90 + kind)
                bufs[kind] = (torch.from_numpy(rows).cuda(), torch.zeros(n, dtype=torch.uint8, device="cuda"),
                              torch.full((n,), float("nan"), dtype=torch.float64, device="cuda"))
            d_eta = torch.full((1,), ETA, dtype=torch.float64, device="cuda")
        stream.synchronize()

        def step():
            for kind, (r, h, t) in bufs.items():
                ctx.prim_batch_device(kind, n, r.data_ptr(), d_eta.data_ptr(), 1, h.data_ptr(), t.data_ptr())

        step()
        ctx.synchronize()
        ref = {k: (h.cpu().numpy(), t.cpu().numpy()) for k, (_, h, t) in bufs.items()}
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            step()

        def timeit(fn, iters):
            for _ in range(3):
                fn()
            stream.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            e0.record(stream)
            for _ in range(iters):
                fn()
            e1.record(stream)
            stream.synchronize()
            wall = time.perf_counter() - t0
            return e0.elapsed_time(e1) * 1e3 / iters, wall * 1e6 / iters

        with torch.cuda.stream(stream):  # replay() launches on the current stream
            dev_direct, wall_direct = timeit(step, args.graph_iters)
            dev_graph, wall_graph = timeit(g.replay, args.graph_iters)
        same = all(np.array_equal(ref[k][0], h.cpu().numpy()) and
                   np.array_equal(ref[k][1].view(np.uint64), t.cpu().numpy().view(np.uint64))
                   for k, (_, h, t) in bufs.items())
        del g
        return {"rows_per_kind": n, "iters": args.graph_iters,
                "direct": {"device_us_per_step": dev_direct, "wall_us_per_step": wall_direct},
                "graph": {"device_us_per_step": dev_graph, "wall_us_per_step": wall_graph},
                "tests_per_s": {"direct": 2 * n / (dev_direct / 1e6), "graph": 2 * n / (dev_graph / 1e6)},
                "replays_match_direct_call": bool(same)}
    except Exception as exc:  # noqa: BLE001 - reported in the bench line instead
        return {"error": f"{type(exc).__name__}: {exc}"}


def run_reference(args, rank, world, pg):
    """The reference's CPU path (the oracle restatement, all host threads) on
    the same workload and config as this arm's line: every row of both kinds
    per step unless --ref-sample bounds it."""
    if rank != 0:
        return
    vf, ee = workload(args.n_vf, args.n_ee)
    m_vf = min(args.ref_sample, vf.shape[0]) if args.ref_sample else vf.shape[0]
    m_ee = min(args.ref_sample, ee.shape[0]) if args.ref_sample else ee.shape[0]
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    orc = O.Oracle()
    threads = os.cpu_count() or 1
    times = []
    for step in range(args.warmup + args.steps):
        o_vf = (step * m_vf) % max(1, vf.shape[0] - m_vf + 1)
        o_ee = (step * m_ee) % max(1, ee.shape[0] - m_ee + 1)
        t0 = time.perf_counter()
        orc.batch(0, vf[o_vf:o_vf + m_vf], ETA, nthreads=threads)
        orc.batch(1, ee[o_ee:o_ee + m_ee], ETA, nthreads=threads)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = (m_vf + m_ee) * len(times) / total
    sample = (f"{m_vf} VF + {m_ee} EE rows per step ({'all rows' if m_vf + m_ee == vf.shape[0] + ee.shape[0] else 'a sample'}), "
              f"{args.steps} steps")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_mesh_only(args, rank, local):
    """The mesh configurations alone (a short run for profilers)."""
    import torch

    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import build as B

    B.build_library()
    torch.cuda.set_device(local)
    ctx = C.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    mesh = mesh_section(ctx, stream, rank, args)
    if rank == 0:
        print(json.dumps(round_floats({"mode": "mesh only", "mesh": mesh_summary(mesh, None)})), flush=True)
    ctx.close()


def run_ours(args, rank, world, local, pg):
    import torch

    import collisiondetection_gb300 as C
    from collisiondetection_gb300 import build as B

    if args.only == "mesh":
        run_mesh_only(args, rank, local)
        return
    B.build_library()
    torch.cuda.set_device(local)
    vf, ee = workload(args.n_vf, args.n_ee)
    n_vf, n_ee = vf.shape[0], ee.shape[0]
    rows_per_step = n_vf + n_ee

    ctx = C.Context(local)
    # A dedicated stream: the context launches on it and the events below are
    # recorded on it (handle 0, the legacy stream, selects the context's own).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    # The two kinds are independent batches: the edge-edge one runs on a
    # second context and stream, so that each batch's latency-bound tail
    # overlaps the other's bulk.
    ctx_ee = C.Context(local)
    stream_ee = torch.cuda.Stream()
    ctx_ee.set_stream(stream_ee.cuda_stream)
    kind_ctx = {"vf": ctx, "ee": ctx_ee}
    d = {}
    for name, arr in (("vf", vf), ("ee", ee)):
        d[name] = {
            "rows": torch.from_numpy(arr).cuda(),
            "hit": torch.zeros(arr.shape[0], dtype=torch.uint8, device="cuda"),
            "t": torch.full((arr.shape[0],), float("nan"), dtype=torch.float64, device="cuda"),
        }
    d_eta = torch.full((1,), ETA, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    # the work split of each kind's refinement, chosen by the autotuner on the
    # batch itself (outside the timed regions; results never change)
    tune = None
    if args.autotune:
        tune = {}
        for kind, name in ((C.VERTEX_FACE, "vf"), (C.EDGE_EDGE, "ee")):
            b = d[name]
            try:
                tune[name] = kind_ctx[name].autotune_prim_batch(kind, b["rows"].shape[0], b["rows"].data_ptr(),
                                                                d_eta.data_ptr(), 1, reps=2)
            except C.CcdError as exc:  # the context keeps its own split; reported in the line
                tune[name] = {"error": str(exc)}
        torch.cuda.synchronize()

    def step(path):
        for kind, name in ((C.VERTEX_FACE, "vf"), (C.EDGE_EDGE, "ee")):
            b = d[name]
            kind_ctx[name].prim_batch_device(kind, b["rows"].shape[0], b["rows"].data_ptr(), d_eta.data_ptr(), 1,
                                             b["hit"].data_ptr(), b["t"].data_ptr(), None, path=path)

    def sync_all():
        ctx.synchronize()
        ctx_ee.synchronize()

    def timed(path, steps, warmup, profile=False):
        for _ in range(warmup):
            step(path)
        sync_all()
        if profile:
            ctx.set_profiling(True)
            ctx_ee.set_profiling(True)
        barrier(pg)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stream_ee.wait_event(e0)  # the second stream starts with the first
        for _ in range(steps):
            step(path)
        joined = torch.cuda.Event()
        joined.record(stream_ee)
        stream.wait_event(joined)  # the end event waits for both streams
        e1.record(stream)
        sync_all()
        torch.cuda.synchronize()
        barrier(pg)
        ms = e0.elapsed_time(e1)
        tm = None
        if profile:
            t_vf, t_ee = ctx.timings(), ctx_ee.timings()
            tm = {k: t_vf[k] + t_ee[k] for k in t_vf}
            tm["per_kind"] = {"vf": t_vf, "ee": t_ee}
            ctx.set_profiling(False)
            ctx_ee.set_profiling(False)
        return ms, tm

    # The all-FP64 GPU paths on the same rows (the comparison points of the
    # metric): the plain kernel (one thread per row, the whole test inline)
    # and the staged refinement of every row with no FP32 stage.
    full = args.only == "all"
    fp64_tps = staged_tps = None
    if full:
        ms64, _ = timed(C.PATH_FP64, max(1, min(args.steps, 3)), 1)
        fp64_tps = rows_per_step * max(1, min(args.steps, 3)) / (ms64 / 1e3)
        # the plain FP64 path's results, to check the cull path against
        fp64_out = {name: (d[name]["hit"].cpu().numpy(), d[name]["t"].cpu().numpy()) for name in ("vf", "ee")}
        ms_st, _ = timed(C.PATH_REFINE_ALL, 1, 1)
        staged_tps = rows_per_step / (ms_st / 1e3)
        staged_out = {name: (d[name]["hit"].cpu().numpy(), d[name]["t"].cpu().numpy()) for name in ("vf", "ee")}
    # FP64 add / multiply rate of this GPU: the refinement's roofline peak
    peak64 = ctx.fp64_peak(reps=3)

    # headline: FP32 cull + FP64 refine, rows resident in HBM; clocks sampled meanwhile
    with ClockSampler(local) as clk:
        ms, tm = timed(C.PATH_CULL_REFINE, args.steps, args.warmup, profile=True)
    ms = max_over_ranks(pg, ms)
    value = world * rows_per_step * args.steps / (ms / 1e3)

    # counters of one step (survivors / hits per kind)
    counts = {}
    for kind, name in ((C.VERTEX_FACE, "vf"), (C.EDGE_EDGE, "ee")):
        b = d[name]
        c = kind_ctx[name]
        c.prim_batch_device(kind, b["rows"].shape[0], b["rows"].data_ptr(), d_eta.data_ptr(), 1,
                            b["hit"].data_ptr(), b["t"].data_ptr(), None, path=C.PATH_CULL_REFINE)
        c.synchronize()
        counts[name] = c.stats()
    gpu_out = {name: (d[name]["hit"].cpu().numpy(), d[name]["t"].cpu().numpy()) for name in ("vf", "ee")}

    # end to end through the host-memory entry point (copies inside the timed
    # region), from pinned host buffers
    keep = []

    def pinned(arr):
        t = torch.empty(arr.shape, dtype=getattr(torch, str(arr.dtype)), pin_memory=True)
        keep.append(t)
        out = t.numpy()
        out[...] = arr
        return out

    if args.only == "all":
        host = {"vf": (pinned(vf), pinned(np.zeros(n_vf, np.uint8)), pinned(np.full(n_vf, np.nan))),
                "ee": (pinned(ee), pinned(np.zeros(n_ee, np.uint8)), pinned(np.full(n_ee, np.nan)))}
        eta_h = pinned(np.array([ETA]))

    def e2e_kind(kind, name):
        c = kind_ctx[name]
        rows, hit, t = host[name]
        rc = c.lib.ccd_prim_batch(c.handle, kind, C.PATH_CULL_REFINE, rows.shape[0], rows.ctypes.data,
                                  eta_h.ctypes.data, 1, hit.ctypes.data, t.ctypes.data)
        if rc != 0:
            raise C.CcdError(c.lib.ccd_last_error(c.handle).decode())

    def e2e_step():
        # one host thread per kind, each on its own context (ctypes releases
        # the interpreter lock for the call)
        import threading

        errors = []

        def run(kind, name):
            try:
                e2e_kind(kind, name)
            except Exception as exc:  # noqa: BLE001 - re-raised below
                errors.append(exc)

        th = threading.Thread(target=run, args=(C.EDGE_EDGE, "ee"))
        th.start()
        run(C.VERTEX_FACE, "vf")
        th.join()
        if errors:
            raise errors[0]

    e2e = None
    if full:
        e2e_step()
        barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
        e2e_value = world * rows_per_step * args.e2e_steps / e2e_s
        h2d = vf.nbytes + ee.nbytes + 8 * rows_per_step + 16
        d2h = rows_per_step * (1 + 8)
        # agreement of the two entry points on this workload
        same = bool(np.array_equal(host["vf"][1], d["vf"]["hit"].cpu().numpy())
                    and np.array_equal(host["ee"][1], d["ee"]["hit"].cpu().numpy()))
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "entry_point": "ccd_prim_batch (pinned host buffers; the two kinds from two host threads, one "
                              "context each)", "matches_device_path": same}

    # The refinement's roofline: the reference's FP64 operations on the rows
    # the FP32 stage passes on (counted by the oracle over a counting
    # scalar), per second of the refinement's launches (CUDA events on each
    # kind's stream), against this GPU's FP64 add / multiply rate.
    oracle_out = {}
    cpu = cpu_baseline(vf, ee, results=oracle_out) if rank == 0 and full else None
    flops = {}
    if rank == 0 and full:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        fc = O.FlopCounter()
        threads = os.cpu_count() or 1
        for kind, name, arr in ((C.VERTEX_FACE, "vf", vf), (C.EDGE_EDGE, "ee", ee)):
            n = arr.shape[0]
            surv = torch.empty(n, dtype=torch.int32, device="cuda")
            htmp = torch.empty(n, dtype=torch.uint8, device="cuda")
            ns = kind_ctx[name].prim_cull_device(kind, n, d[name]["rows"].data_ptr(), d_eta.data_ptr(), 1,
                                                 htmp.data_ptr(), surv.data_ptr())
            idx = surv[:ns].cpu().numpy()
            _, _, fl, tot = fc.batch(kind, arr, ETA, nthreads=threads)
            flops[name] = {"survivors": int(ns), "flops_all_rows": int(fl.astype(np.int64).sum()),
                           "flops_survivors": int(fl[idx].astype(np.int64).sum()), "ops": tot}
            del surv, htmp
    pk = tm["per_kind"]
    refine_ms_launch = {k: pk[k]["refine_ms"] / args.steps for k in ("vf", "ee")}
    cull_ms_launch = {k: pk[k]["cull_ms"] / args.steps for k in ("vf", "ee")}
    roofline = None
    if flops:
        f_step = flops["vf"]["flops_survivors"] + flops["ee"]["flops_survivors"]
        ms_launches = refine_ms_launch["vf"] + refine_ms_launch["ee"]
        achieved = f_step / (ms_launches / 1e3) / 1e9
        peak = peak64["ops_per_s"] / 1e9
        roofline = {"kernel": "staged FP64 refine of the FP32 survivors (stage_build, wave_step, stage_roots, "
                              "wave_finish, stage_combine)",
                    "bound": "fp64", "achieved": achieved, "peak": peak, "unit": "GFLOP/s", "frac": achieved / peak,
                    "peak_source": "measured: ccd_fp64_peak (own DADD/DMUL kernel, CUDA events)",
                    "traffic": None,
                    "flops_per_survivor": {k: flops[k]["flops_survivors"] / max(1, flops[k]["survivors"])
                                           for k in ("vf", "ee")},
                    "refine_ms_per_launch": refine_ms_launch, "cull_ms_per_launch": cull_ms_launch,
                    "share_refine": (tm["refine_ms"] / (tm["cull_ms"] + tm["refine_ms"]))}
        # The same work priced at the measured rates of each operation: adds,
        # multiplies and square roots at the add / multiply rate, divisions at
        # the division rate (several FP64 instructions each).  The survivors'
        # share of each kind's operation mix is taken as their share of its
        # flops.
        t_peak = 0.0
        for k in ("vf", "ee"):
            ops, share = flops[k]["ops"], flops[k]["flops_survivors"] / max(1, flops[k]["flops_all_rows"])
            t_peak += share * ((ops["add"] + ops["mul"] + ops["sqrt"]) / peak64["ops_per_s"]
                               + ops["div"] / peak64["div_per_s"])
        roofline["frac_division_priced"] = t_peak * 1e3 / ms_launches
        roofline["fp64_latency_cycles"] = {op: round(peak64[op + "_latency_cycles"], 1) for op in ("add", "mul", "div")}
    # the FP32 cull's false negatives and the contact-time error of the
    # headline path, against the oracle (all rows) and the all-FP64 GPU paths
    parity = None
    if full:
        parity = {"cull_refine_vs_fp64_path": {k: compare_results(*fp64_out[k], *gpu_out[k]) for k in gpu_out},
                  "refine_all_vs_fp64_path": {k: compare_results(*fp64_out[k], *staged_out[k]) for k in gpu_out}}
        if oracle_out:
            parity["cull_refine_vs_oracle"] = {k: compare_results(*oracle_out[k], *gpu_out[k]) for k in gpu_out}
    mesh = mesh_section(ctx, stream, rank, args) if args.mesh and full else None
    distance = distance_section(ctx, stream, rank, args) if args.distance and full else None
    penalty = penalty_section(ctx, rank, args) if args.distance and full else None
    velocity = velocity_filter_section(ctx, rank, args) if args.velocity and full and world == 1 else None
    serving = serving_section(args) if args.serve and full and world == 1 else None
    uneven = uneven_section(args, rank) if args.uneven_instances and full and world == 1 else None
    graph = graph_section(ctx, stream, args) if args.graph_rows and full else None

    if rank == 0:
        detail = {
            "fp64_peak": peak64, "flops": flops, "survivors": {"vf": counts["vf"]["survivors"] / n_vf,
                                                                "ee": counts["ee"]["survivors"] / n_ee},
            "hits": {"vf": counts["vf"]["hits"], "ee": counts["ee"]["hits"]},
            "status_flags": counts["vf"]["status_flags"] + counts["ee"]["status_flags"], "timings": tm,
            "roofline": roofline, "parity": parity, "autotune": tune, "mesh": mesh, "distance": distance,
            "penalty": penalty, "velocity_filter": velocity, "serving": serving, "uneven_batch": uneven,
            "graph_small_batches": graph, "e2e": e2e}
        detail_path = write_detail(args, detail)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(args),
            "path": "FP32 cull + FP64 refine; the two kinds on two contexts / streams",
            "gpu_launches": int(tm["launches"]),
            "e2e": compact(e2e, ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step", "matches_device_path")),
            "roofline": compact(roofline, ("kernel", "bound", "achieved", "peak", "unit", "frac", "peak_source",
                                           "traffic", "flops_per_survivor", "frac_division_priced",
                                           "fp64_latency_cycles")),
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "fp64_path": ({"plain": fp64_tps, "staged": staged_tps, "speedup_vs_plain": value / (world * fp64_tps),
                           "speedup_vs_staged": value / (world * staged_tps)} if fp64_tps else None),
            "parity": parity_summary(parity),
            "mesh": mesh_summary(mesh, uneven),
            "small_batch": small_batch_summary(graph),
            "serving": serving_summary(serving),
            "detail": detail_path,
        }
        print(json.dumps(round_floats(line)), flush=True)
    ctx.close()
    ctx_ee.close()


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
    else:
        run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
