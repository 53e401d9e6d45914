"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference library's own sources, compiled unmodified by
``make -C oracle ref`` (oracle/_ref/libccd_ref.so), on seeded inputs and on
the reference's example meshes, and writes:

* ``kat_testctcd.json`` -- the four hand-built cases of the reference's
  example/testCTCD.cpp (it prints hit and t; the values here are the ones the
  reference computes).
* ``prims.npz`` -- seeded swept primitives of the four kinds (random,
  near-degenerate and hand-built edge cases) with the reference's hit / t.
* ``meshes.npz`` -- the two-sphere scene and the reference's start/end mesh
  pairs meshes/test1.obj -> test2.obj and meshes/V0_prob3_402.obj ->
  V1_prob3_402.obj, with digests of the reference's k-DOP and AABB candidate
  sets and its CTCD narrow-phase result.
* ``distances.npz`` / ``distances.json`` -- the reference's Distance class:
  vertexFaceDistance / edgeEdgeDistance vectors and barycentric coordinates
  and the two distance predicates on seeded and hand-built rows, and
  meshSelfDistance (with the stencil counts it prints) on the meshes above, on
  meshes/V0_prob11_835.obj, on a small sheet over a sphere and on hand-built
  small meshes.
* ``trivial.json`` -- digests of TrivialBroadPhase's candidate sets on the
  meshes of ``meshes.npz``, free and with fixed vertices.
* ``penalty.npz`` / ``penalty.json`` -- PenaltyGroup::addForce on three
  groups (two spheres in contact, a sheet on a sphere, hand-built stencils
  with repeated and coincident vertices), in shuffled group order with
  non-canonical and repeated stencils, with and without new stencils: the
  forces, the per-stencil fired flags (from the potentials' own addForce) and
  the returned newused flag.
* ``history.npz`` / ``history.json`` -- multi-entry histories (built with
  History's constructor and addHistory) for the two spheres, a sheet on a
  sphere and two hand-built triangles: k-DOP and AABB candidate digests, free
  and with fixed vertices, CTCDNarrowPhase's colliding stencils and
  SeparatingPlaneNarrowPhase's hit flags (stencils on which its recursion
  never ends, found by the oracle, are recorded instead of run: the
  reference overflows its stack there).
* ``velocity_filter.npz`` / ``velocity_filter.json`` --
  VelocityFilter::velocityFilter on small scenes (a triangle and a sheet
  falling onto fixed ones, two spheres thrown together) and on its two early
  exits: the return value and the filtered end positions.

Only runs where the reference tree exists:
    python tests/golden/make_golden.py [--only distances|trivial|penalty|history|velocity_filter]
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_TREE = os.environ.get("CCD_REFERENCE_TREE", "/root/reference")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from collisiondetection_gb300 import workloads as W  # noqa: E402
import oracle as O  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def load_obj(path):
    """The reference's examples read 'v x y z' and 1-based 'f a b c' lines
    (example/AlecTest.cpp:9-55)."""
    V, F = [], []
    with open(path) as fh:
        for line in fh:
            s = line.split()
            if not s:
                continue
            if s[0] == "v":
                V.append([float(a) for a in s[1:4]])
            elif s[0] == "f":
                F.append([int(a) - 1 for a in s[1:4]])
    return np.array(V, np.float64), np.array(F, np.int32)


KAT = [
    ("ee", [[0, 0, 0], [1, 0, 0], [2, 0, 0], [2, 1, 0], [0, 0, 0], [1, 0, 0], [2, 1, 0], [-1, -1, 0]]),
    ("vf", [[.5, .5, 1], [0, 0, 0], [1, 0, 0], [0, 1, 0], [.5, .5, 1], [0, 0, 0], [1, 0, 3], [0, 1, 0]]),
    ("ve", [[.5, 0, 1], [0, 0, 0], [1, 0, 0], [.5, 0, -3], [0, 0, 0], [1, 0, 0]]),
    ("vv", [[0, 0, 0], [1, 0, 0], [6, 0, 0], [1, 0, 0]]),
]


def edge_cases(kind: int) -> np.ndarray:
    """Hand-built degenerate inputs for one primitive kind."""
    k = W.NPTS[kind]
    rng = np.random.default_rng(1000 + kind)
    rows = []
    base_s = rng.uniform(0, 1, size=(k, 3))
    base_e = base_s + rng.normal(0, 0.1, size=(k, 3))
    rows.append(np.concatenate([base_s.ravel(), base_s.ravel()]))                     # no motion
    rows.append(np.zeros(6 * k))                                                        # all points equal
    pts = np.tile(rng.uniform(0, 1, size=3), (k, 1))
    rows.append(np.concatenate([pts.ravel(), (pts + rng.normal(0, .1, 3)).ravel()]))    # all coincide, move together
    flat_s, flat_e = base_s.copy(), base_e.copy()
    flat_s[:, 2] = 0.25
    flat_e[:, 2] = 0.25
    rows.append(np.concatenate([flat_s.ravel(), flat_e.ravel()]))                       # exactly coplanar (z const)
    line_s = np.outer(np.linspace(0, 1, k), [1, 2, 3]) * 0.3
    rows.append(np.concatenate([line_s.ravel(), (line_s + 0.1).ravel()]))               # collinear, translating
    rows.append(np.concatenate([base_s.ravel() * 1e3, base_e.ravel() * 1e3]))           # large coordinates
    rows.append(np.concatenate([base_s.ravel() * 1e-3, base_e.ravel() * 1e-3]))         # small coordinates
    rows.append(np.concatenate([base_s.ravel() + 1e3, base_e.ravel() + 1e3]))           # far from origin
    sw = base_s.copy()
    sw[0] = base_e[0]
    rows.append(np.concatenate([base_s.ravel(), sw.ravel()]))                           # one point jumps
    if kind == W.KIND_VF:
        tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
        for z0, z1 in ((1, -1), (0, 0), (1e-7, -1e-7), (5e-7, 5e-7), (0, 1)):
            for xy in ((0.2, 0.2), (1.0, 0.0), (0.5, 0.5), (2, 2)):
                v0 = np.array([xy[0], xy[1], z0])
                v1 = np.array([xy[0], xy[1], z1])
                rows.append(np.concatenate([np.vstack([v0, tri]).ravel(), np.vstack([v1, tri]).ravel()]))
    if kind == W.KIND_EE:
        for dz in (1e-7, 0.0, 5e-7, 2e-6):
            e0 = np.array([[0, 0, 0], [1, 0, 0]], float)
            e1s = np.array([[0.5, -1, 1], [0.5, 1, 1]], float)
            e1e = np.array([[0.5, -1, -1], [0.5, 1, -1]], float)
            rows.append(np.concatenate([np.vstack([e0, e1s]).ravel(), np.vstack([e0, e1e]).ravel()]))
            par_s = np.array([[0, 0, 0], [1, 0, 0], [0, 0, dz], [1, 0, dz]], float)      # parallel edges
            rows.append(np.concatenate([par_s.ravel(), (par_s + [0, 0.1, 0]).ravel()]))
            rows.append(np.concatenate([par_s.ravel(), par_s.ravel()]))
    return np.array(rows, np.float64)


def distance_rows(kind: int) -> np.ndarray:
    """Seeded and hand-built rows (12 doubles) for one Distance query kind:
    0 = (p, q0, q1, q2), 1 = (p0, p1, q0, q1)."""
    rng = np.random.default_rng(5000 + kind)
    rows = [rng.uniform(-1, 1, size=(600, 12)), rng.normal(0, 1e-3, size=(100, 12)) + rng.uniform(0, 1, (1, 12))]
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    if kind == 0:
        # every Voronoi region of a triangle, above, on and below its plane
        for x in (-0.5, 0.0, 0.25, 0.5, 1.0, 1.5):
            for y in (-0.5, 0.0, 0.25, 0.5, 1.0, 1.5):
                for z in (-1.0, 0.0, 1e-9, 1.0):
                    rows.append(np.concatenate([[x, y, z], tri.ravel()])[None])
        degenerate = [
            [[0.3, 0.3, 1], [0, 0, 0], [1, 1, 1], [2, 2, 2]],    # collinear triangle
            [[0.3, 0.3, 1], [1, 1, 1], [1, 1, 1], [1, 1, 1]],    # all three vertices coincide
            [[1, 1, 1], [1, 1, 1], [1, 1, 1], [1, 1, 1]],        # everything coincides
            [[0.2, 0.2, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0]],    # p inside the triangle
            [[0.5, 0, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0]],      # p on an edge
            [[1, 0, 0], [0, 0, 0], [1, 0, 0], [0, 1, 0]],        # p on a vertex
            [[0.5, 0.5, 0.5], [0, 0, 0], [1, 0, 0], [1, 0, 0]],  # two coincident vertices
        ]
    else:
        degenerate = [
            [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]],        # parallel (denominator 0)
            [[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]],        # collinear, apart
            [[0, 0, 0], [2, 0, 0], [1, 0, 0], [3, 0, 0]],        # collinear, overlapping
            [[0, 0, 0], [0, 0, 0], [1, 1, 1], [2, 0, 1]],        # first edge a point
            [[0, 0, 0], [1, 0, 0], [1, 1, 1], [1, 1, 1]],        # second edge a point
            [[1, 1, 1], [1, 1, 1], [1, 1, 1], [1, 1, 1]],        # both points, coincident
            [[0, 0, 0], [1, 0, 0], [0.5, -1, 0], [0.5, 1, 0]],   # crossing
            [[0, 0, 0], [1, 0, 0], [0.5, -1, 1], [0.5, 1, 1]],   # skew, closest inside both
            [[0, 0, 0], [1, 0, 0], [2, -1, 1], [2, 1, 1]],       # skew, clamped
            [[0, 0, 0], [1, 0, 0], [-2, 1, 0], [-1, 1, 1e-12]],  # nearly parallel
        ]
    rows.append(np.array(degenerate, float).reshape(-1, 12))
    base = rng.uniform(0, 1, size=(50, 12))
    rows += [base * 1e6, base * 1e-6, base + 1e4]
    nonfinite = base[:4].copy()
    nonfinite[0, 0] = np.nan
    nonfinite[1, 4] = np.inf
    nonfinite[2, 9] = -np.inf
    nonfinite[3, :] = np.nan
    rows.append(nonfinite)
    return np.concatenate(rows).astype(np.float64)


def small_meshes():
    """Hand-built small meshes for meshSelfDistance: (verts [V][3], faces)."""
    out = {}
    out["one_triangle"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float), np.array([[0, 1, 2]], np.int32))
    out["two_triangles"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.5], [1.2, 0.2, 0.5],
                                      [0.2, 1.2, 0.6]], float), np.array([[0, 1, 2], [3, 4, 5]], np.int32))
    out["shared_edge"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.1]], float),
                          np.array([[0, 1, 2], [1, 3, 2]], np.int32))
    out["coincident_copies"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]] * 2, float),
                                np.array([[0, 1, 2], [3, 4, 5]], np.int32))
    out["isolated_vertex"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.3, 0.3, 0.01]], float),
                              np.array([[0, 1, 2]], np.int32))
    out["repeated_index"] = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float),
                             np.array([[0, 0, 1], [2, 3, 3]], np.int32))
    return out


def stdout_of(fn, *args):
    """Runs fn(*args) and returns (its result, what it wrote to file
    descriptor 1): the reference prints its stencil counts there."""
    sys.stdout.flush()
    saved = os.dup(1)
    with tempfile.TemporaryFile() as tmp:
        os.dup2(tmp.fileno(), 1)
        try:
            result = fn(*args)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        tmp.seek(0)
        text = tmp.read().decode()
    return result, text


def distance_fixtures(ref) -> None:
    arrays, meta = {}, {"queries": {}, "self_distance": {}}
    for kind in (0, 1):
        rows = distance_rows(kind)
        vec, bary = ref.distance(kind, rows)
        eta = np.random.default_rng(6000 + kind).uniform(0, 0.5, rows.shape[0])
        less = ref.distance_less_than(kind, rows, eta)
        arrays[f"rows{kind}"] = rows
        arrays[f"vec{kind}"] = vec
        arrays[f"bary{kind}"] = bary
        arrays[f"eta{kind}"] = eta
        arrays[f"less{kind}"] = less
        meta["queries"][str(kind)] = {"rows": int(rows.shape[0]), "less_true": int(less.sum())}
    meshes = {}
    qs, _, f = W.two_spheres(seed=1)
    meshes["spheres"] = (qs.reshape(-1, 3), f)
    v0, f0 = load_obj(os.path.join(REF_TREE, "meshes", "test1.obj"))
    meshes["test1"] = (v0, f0)
    v0, f0 = load_obj(os.path.join(REF_TREE, "meshes", "V0_prob3_402.obj"))
    meshes["prob3"] = (v0, f0)
    v0, f0 = load_obj(os.path.join(REF_TREE, "meshes", "V0_prob11_835.obj"))
    meshes["prob11"] = (v0, f0)
    f, frames = W.cloth_frames(grid=24, level=2, seed=3, steps=1)
    meshes["cloth"] = (frames[0].reshape(-1, 3), f)
    meshes.update(small_meshes())
    for name, (v, f) in meshes.items():
        v = np.ascontiguousarray(v, np.float64)
        f = np.ascontiguousarray(f, np.int32)
        arrays[f"mesh_{name}_verts"] = v
        arrays[f"mesh_{name}_faces"] = f
        fixed = np.zeros(v.shape[0], np.uint8)
        fixed[: v.shape[0] // 2] = 1
        arrays[f"mesh_{name}_fixed"] = fixed
        entry = {}
        for label, fx in (("free", None), ("fixed", fixed)):
            d, text = stdout_of(ref.mesh_self_distance, v, f, fx)
            m = re.search(r"Checking (\d+) vertex-face and (\d+) edge-edge stencils", text)
            entry[label] = {"distance_hex": float(d).hex(), "distance": d,
                            "n_vf": int(m.group(1)), "n_ee": int(m.group(2))}
        meta["self_distance"][name] = entry
    np.savez_compressed(os.path.join(HERE, "distances.npz"), **arrays)
    with open(os.path.join(HERE, "distances.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def trivial_fixtures(ref) -> None:
    """Digests of TrivialBroadPhase's candidate sets (src/TrivialBroadPhase.cpp)
    on the fixture meshes, free and with their fixed vertices."""
    g = np.load(os.path.join(HERE, "meshes.npz"))
    meta = {}
    for name in ("test12", "prob3", "spheres"):
        qs, qe, f, fixed = g[f"{name}_qstart"], g[f"{name}_qend"], g[f"{name}_faces"], g[f"{name}_fixed"]
        entry = {}
        for label, fx in (("free", None), ("fixed", fixed)):
            vf, ee = ref.broadphase(2, qs, qe, f, 1e-6, fx)
            entry[label] = {"n_vf": int(vf.shape[0]), "n_ee": int(ee.shape[0]), "digest": digest(vf, ee)}
        meta[name] = entry
    with open(os.path.join(HERE, "trivial.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def penalty_scenes():
    """Groups for PenaltyGroup::addForce: (q, v, F, vf, vf_isnew, ee, ee_isnew,
    outer_eta, inner_eta, stiffness, cor, dt)."""
    rng = np.random.default_rng(90)
    scenes = {}

    def jumble(st, kind):
        """Group order shuffled, a tenth of the stencils written
        non-canonically, a few listed twice."""
        st = st[rng.permutation(st.shape[0])].copy()
        pick = rng.random(st.shape[0]) < 0.1
        if kind == 0:
            st[pick, 1:] = st[pick][:, [2, 3, 1]]
        else:
            st[pick] = st[pick][:, [3, 2, 1, 0]]
        return np.concatenate([st, st[: max(1, st.shape[0] // 50)]])

    qs, qe, f = W.two_spheres(seed=1)
    q = qs + 0.62 * (qe - qs)
    vf, ee = O.Oracle().broadphase(0, q, q, f, 0.05)
    v = (qe - qs) + rng.normal(0, 0.05, qs.shape)
    scenes["spheres"] = (q, v, rng.normal(0, 1, qs.shape), jumble(vf, 0), None, jumble(ee, 1), None,
                         0.05, 1e-4, 10.0, 0.1, 1e-3)
    f2, frames = W.cloth_frames(grid=24, level=2, seed=6, steps=30)
    q = frames[28]
    vf, ee = O.Oracle().broadphase(0, q, q, f2, 0.02)
    v = (frames[29] - frames[27]) / 2 + rng.normal(0, 1e-3, q.shape)
    scenes["cloth"] = (q, v, np.zeros(q.shape), jumble(vf, 0), None, jumble(ee, 1), None, 0.02, 0.0, 1.0, 0.5, 0.01)
    # hand-built: repeated vertices, coincident points, both signs of relative velocity
    q = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.01], [0.2, 0.2, 0.01], [0.3, 0.3, -0.005],
                  [0.5, -0.5, 0.002], [0.5, 0.5, 0.002], [1, 1, 0]], float)
    v = rng.normal(0, 1, q.shape)
    vf = np.array([[3, 0, 1, 2], [4, 2, 1, 0], [5, 0, 1, 2], [3, 0, 0, 1], [3, 0, 1, 2], [8, 0, 1, 2]], np.int32)
    ee = np.array([[6, 7, 0, 1], [0, 1, 6, 7], [1, 0, 7, 6], [3, 4, 0, 1], [0, 2, 1, 8], [6, 7, 2, 8]], np.int32)
    scenes["hand"] = (q.ravel(), v.ravel(), np.full(q.size, -0.0), vf, None, ee, None, 0.05, 1e-3, 2.0, 0.25, 0.5)
    out = {}
    for name, sc in scenes.items():
        q, v, F, vf, _, ee, _, oe, ie, k, cor, dt = sc
        vfn = rng.integers(0, 2, vf.shape[0]).astype(np.uint8)
        een = (rng.random(ee.shape[0]) < 0.05).astype(np.uint8)
        out[name] = (np.ascontiguousarray(q, np.float64).ravel(), np.ascontiguousarray(v, np.float64).ravel(),
                     np.ascontiguousarray(F, np.float64).ravel(), vf, vfn, ee, een, oe, ie, k, cor, dt)
    return out


def penalty_fixtures(ref) -> None:
    arrays, meta = {}, {}
    for name, (q, v, F, vf, vfn, ee, een, oe, ie, k, cor, dt) in penalty_scenes().items():
        for label, (vn, en) in (("new", (vfn, een)), ("old", (None, None))):
            Fo, vfire, efire, used = ref.penalty_group_force(q, v, F, vf, ee, oe, ie, k, cor, dt, vn, en)
            arrays[f"{name}_{label}_F"] = Fo
            arrays[f"{name}_{label}_vf_fired"] = vfire
            arrays[f"{name}_{label}_ee_fired"] = efire
            meta[f"{name}_{label}"] = {"newused": bool(used), "vf_fired": int(vfire.sum()),
                                       "ee_fired": int(efire.sum())}
        for key, val in (("q", q), ("v", v), ("F0", F), ("vf", vf), ("vf_isnew", vfn), ("ee", ee),
                         ("ee_isnew", een)):
            arrays[f"{name}_{key}"] = val
        meta[name] = {"outer_eta": oe, "inner_eta": ie, "stiffness": k, "cor": cor, "dt": dt}
    np.savez_compressed(os.path.join(HERE, "penalty.npz"), **arrays)
    with open(os.path.join(HERE, "penalty.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def history_fixtures(ref) -> None:
    """KDOPBroadPhase / AABBBroadPhase candidate digests and CTCDNarrowPhase
    results on multi-entry histories built through History's own API."""
    scenes = {}
    qs, qe, f = W.two_spheres(seed=1)
    scenes["spheres"] = (W.multi_entry_history(qs, qe, seed=5), f, 1e-3)
    f2, frames = W.cloth_frames(grid=24, level=2, seed=6, steps=30)
    scenes["cloth"] = (W.multi_entry_history(frames[26], frames[28], seed=6, active=0.5, max_entries=10,
                                             jitter=0.004), f2, 2e-3)
    # vertices whose histories start late / hold one entry only / repeat a time
    q0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.3], [1.2, 0.2, 0.3], [0.2, 1.2, 0.3]], float)
    q1 = q0.copy()
    q1[3:, 2] -= 0.6  # the upper triangle passes through the lower one
    off, tt, pp = W.multi_entry_history(q0, q1, seed=7, active=1.0, max_entries=4, jitter=0.01, pool=3)
    scenes["hand"] = ((off, tt, pp), np.array([[0, 1, 2], [3, 4, 5]], np.int32), 1e-2)
    arrays, meta = {}, {}
    for name, ((off, tt, pp), f, eta) in scenes.items():
        arrays[f"{name}_offsets"], arrays[f"{name}_times"], arrays[f"{name}_positions"] = off, tt, pp
        arrays[f"{name}_faces"] = f
        fixed = np.zeros(off.size - 1, np.uint8)
        fixed[: (off.size - 1) // 2] = 1
        arrays[f"{name}_fixed"] = fixed
        entry = {"eta": eta}
        for kind, label in ((0, "kdop"), (1, "aabb")):
            for fx_label, fx in (("", None), ("_fixed", fixed)):
                vf, ee = ref.broadphase_history(kind, off, tt, pp, f, eta, fx)
                entry[f"{label}{fx_label}"] = {"n_vf": int(vf.shape[0]), "n_ee": int(ee.shape[0]),
                                               "digest": digest(vf, ee)}
        vf, ee = ref.broadphase_history(0, off, tt, pp, f, eta)
        vh, eh = ref.narrowphase_history(off, tt, pp, vf, eta, ee, eta)
        arrays[f"{name}_hit_vf"] = vf[vh.astype(bool)]
        arrays[f"{name}_hit_ee"] = ee[eh.astype(bool)]
        entry["narrow"] = {"n_vf_hit": int(vh.sum()), "n_ee_hit": int(eh.sum()), "digest": digest(vh, eh)}
        # SeparatingPlaneNarrowPhase on the same candidates.  Its recursion
        # never ends on some stencils (the reference overflows its stack);
        # the oracle finds those first, and they are kept out of the
        # reference's run and recorded as such.
        o = O.Oracle()
        _, _, vs, es = o.separating_plane(off, tt, pp, vf, eta, ee, eta)
        svh, seh = ref.separating_plane(off, tt, pp, vf[vs == 0], eta, ee[es == 0], eta)
        arrays[f"{name}_sp_vf_hit"] = svh
        arrays[f"{name}_sp_ee_hit"] = seh
        arrays[f"{name}_sp_vf_stalled"] = vs
        arrays[f"{name}_sp_ee_stalled"] = es
        entry["separating_plane"] = {"n_vf_hit": int(svh.sum()), "n_ee_hit": int(seh.sum()),
                                     "n_stalled": int(vs.sum() + es.sum())}
        meta[name] = entry
    np.savez_compressed(os.path.join(HERE, "history.npz"), **arrays)
    with open(os.path.join(HERE, "history.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def velocity_filter_scenes():
    """Scenes for VelocityFilter::velocityFilter: (qstart, qend, faces,
    invmasses, outer_eta, inner_eta)."""
    scenes = {}
    # a triangle falling through a fixed one
    q0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.1], [1.2, 0.2, 0.1], [0.2, 1.2, 0.1]], float)
    q1 = q0.copy()
    q1[3:, 2] = -0.1
    mi = np.ones(18)
    mi[:9] = 0
    scenes["triangles"] = (q0, q1, np.array([[0, 1, 2], [3, 4, 5]], np.int32), mi, 0.01, 0.005)
    # a 6x6 sheet falling onto a fixed one
    v, f = W.grid_sheet(6, 6)
    v = np.asarray(v).reshape(-1, 3)
    n = v.shape[0]
    upper = v.copy()
    upper[:, 2] += 0.05
    q0 = np.concatenate([v, upper])
    q1 = q0.copy()
    q1[n:, 2] -= 0.1
    mi = np.ones(q0.size)
    mi[: 3 * n] = 0
    scenes["sheets"] = (q0, q1, np.concatenate([f, f + n]).astype(np.int32), mi, 0.01, 0.005)
    # two small spheres thrown into each other, all masses finite
    qs, qe, f = W.two_spheres(seed=3, level=1, radius=0.5, gap=1.2, approach=0.25)
    scenes["spheres"] = (qs.reshape(-1, 3), qe.reshape(-1, 3), f, np.ones(qs.size), 0.02, 0.01)
    # the start already closer than inner_eta, and a vertex in no face
    q0 = scenes["triangles"][0].copy()
    q0[3:, 2] = 0.001
    scenes["intersecting_start"] = (q0, q0, scenes["triangles"][2], scenes["triangles"][3], 0.01, 0.005)
    q0 = np.concatenate([scenes["triangles"][0], [[5.0, 5.0, 5.0]]])
    scenes["dangling"] = (q0, q0, scenes["triangles"][2], np.ones(q0.size), 0.01, 0.005)
    return scenes


def velocity_filter_fixtures(ref) -> None:
    arrays, meta = {}, {}
    for name, (q0, q1, f, mi, oe, ie) in velocity_filter_scenes().items():
        ret, qe = ref.velocity_filter(q0, q1, f, mi, oe, ie)
        for key, val in (("qstart", q0), ("qend", q1), ("faces", f), ("invmasses", mi), ("result", qe)):
            arrays[f"{name}_{key}"] = np.ascontiguousarray(val)
        meta[name] = {"outer_eta": oe, "inner_eta": ie, "return": int(ret)}
    np.savez_compressed(os.path.join(HERE, "velocity_filter.npz"), **arrays)
    with open(os.path.join(HERE, "velocity_filter.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)


def main() -> None:
    if not os.path.isdir(REF_TREE):
        sys.exit(f"reference tree not found at {REF_TREE}")
    O.build(ref=True)
    ref = O.Reference()
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "distances":
        distance_fixtures(ref)
        return
    if only == "trivial":
        trivial_fixtures(ref)
        return
    if only == "penalty":
        penalty_fixtures(ref)
        return
    if only == "history":
        history_fixtures(ref)
        return
    if only == "velocity_filter":
        velocity_filter_fixtures(ref)
        return

    kat = []
    for name, pts in KAT:
        h, t = ref.prim(name, pts, 1e-6)
        kat.append({"kind": name, "points": pts, "eta": 1e-6, "hit": h, "t": t, "t_hex": float(t).hex()})
    with open(os.path.join(HERE, "kat_testctcd.json"), "w") as fh:
        json.dump(kat, fh, indent=1)

    sizes = {W.KIND_VF: 1200, W.KIND_EE: 1200, W.KIND_VE: 600, W.KIND_VV: 600}
    out = {}
    for kind, n in sizes.items():
        x = np.concatenate([W.primitive_batch(kind, n, seed=20240 + kind), edge_cases(kind)])
        rng = np.random.default_rng(77 + kind)
        eta = np.full(x.shape[0], 1e-6)
        pick = rng.permutation(x.shape[0])
        eta[pick[: x.shape[0] // 10]] = 1e-3
        eta[pick[x.shape[0] // 10: x.shape[0] // 5]] = 0.0
        hit, t = ref.batch(kind, x, eta)
        out[f"x{kind}"] = x
        out[f"eta{kind}"] = eta
        out[f"hit{kind}"] = hit
        out[f"t{kind}"] = t
    np.savez_compressed(os.path.join(HERE, "prims.npz"), **out)

    meshes = {}
    qs, qe, f = W.two_spheres(seed=1)
    meshes["spheres"] = (qs, qe, f, 1e-6)
    v0, f0 = load_obj(os.path.join(REF_TREE, "meshes", "test1.obj"))
    v1, _ = load_obj(os.path.join(REF_TREE, "meshes", "test2.obj"))
    meshes["test12"] = (v0.ravel(), v1.ravel(), f0, 1e-6)
    v0, f0 = load_obj(os.path.join(REF_TREE, "meshes", "V0_prob3_402.obj"))
    v1, _ = load_obj(os.path.join(REF_TREE, "meshes", "V1_prob3_402.obj"))
    meshes["prob3"] = (v0.ravel(), v1.ravel(), f0, 1e-8)

    arrays, meta = {}, {}
    for name, (qs, qe, f, eta) in meshes.items():
        arrays[f"{name}_qstart"] = qs
        arrays[f"{name}_qend"] = qe
        arrays[f"{name}_faces"] = f
        fixed = np.zeros(qs.size // 3, np.uint8)
        fixed[: qs.size // 6] = 1
        arrays[f"{name}_fixed"] = fixed
        entry = {"eta": eta}
        for kind, label in ((0, "kdop"), (1, "aabb")):
            for fx_label, fx in (("", None), ("_fixed", fixed)):
                vf, ee = ref.broadphase(kind, qs, qe, f, eta, fx)
                entry[f"{label}{fx_label}"] = {"n_vf": int(vf.shape[0]), "n_ee": int(ee.shape[0]),
                                               "digest": digest(vf, ee)}
        vf, ee = ref.broadphase(0, qs, qe, f, eta)
        vh, eh = ref.narrowphase(qs, qe, vf, eta, ee, eta)
        arrays[f"{name}_hit_vf"] = vf[vh.astype(bool)]
        arrays[f"{name}_hit_ee"] = ee[eh.astype(bool)]
        entry["narrow"] = {"n_vf_hit": int(vh.sum()), "n_ee_hit": int(eh.sum()), "digest": digest(vh, eh)}
        meta[name] = entry
    np.savez_compressed(os.path.join(HERE, "meshes.npz"), **arrays)
    with open(os.path.join(HERE, "meshes.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    distance_fixtures(ref)
    trivial_fixtures(ref)
    penalty_fixtures(ref)
    history_fixtures(ref)
    velocity_filter_fixtures(ref)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
