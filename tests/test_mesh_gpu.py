"""Mesh path on the GPU through the C ABI: broad phase (k-DOP and AABB
candidate search) and the CTCD narrow phase over stencils, against the golden
fixtures (made by the reference's own sources) and the oracle.

Parity bar: candidate lists identical element for element (same stencils, same
std::set order); identical hit flags and first-hit sub-test; contact times
within 1e-12 relative."""
import hashlib
import json
import os

import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12
KINDS = {"kdop": C.BROADPHASE_KDOP13, "aabb": C.BROADPHASE_AABB}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


@pytest.fixture(scope="module")
def ctx():
    from collisiondetection_gb300 import build as B

    B.build_library()
    c = C.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def golden(golden_dir):
    meta = json.load(open(os.path.join(golden_dir, "meshes.json")))
    arrays = np.load(os.path.join(golden_dir, "meshes.npz"))
    return meta, arrays


def _scene(golden, name):
    meta, a = golden
    return (a[f"{name}_qstart"], a[f"{name}_qend"], a[f"{name}_faces"], a[f"{name}_fixed"], meta[name])


@pytest.mark.parametrize("name", ["test12", "prob3", "spheres"])
@pytest.mark.parametrize("label", ["kdop", "aabb"])
@pytest.mark.parametrize("use_fixed", [False, True])
def test_broadphase_matches_reference(ctx, golden, name, label, use_fixed):
    qs, qe, f, fixed, meta = _scene(golden, name)
    want = meta[label + ("_fixed" if use_fixed else "")]
    with C.Mesh(ctx, f, qs, qe, fixed if use_fixed else None) as m:
        vf, ee = m.broadphase(KINDS[label], meta["eta"])
        assert (vf.shape[0], ee.shape[0]) == (want["n_vf"], want["n_ee"])
        assert digest(vf, ee) == want["digest"]


@pytest.mark.parametrize("name", ["test12", "prob3", "spheres"])
@pytest.mark.parametrize("path", [C.PATH_FP64, C.PATH_CULL_REFINE])
def test_narrowphase_matches_reference(ctx, golden, oracle, name, path):
    qs, qe, f, _, meta = _scene(golden, name)
    eta = meta["eta"]
    with C.Mesh(ctx, f, qs, qe) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, eta)
        out = m.narrowphase(vf, eta, ee, eta, path=path)
        assert digest(out["vf_hit"], out["ee_hit"]) == meta["narrow"]["digest"]
        st = m.stats()
        assert (st["vf_hits"], st["ee_hits"]) == (meta["narrow"]["n_vf_hit"], meta["narrow"]["n_ee_hit"])
        ref = oracle.narrowphase(qs, qe, vf, eta, ee, eta)
        for k in ("vf", "ee"):
            np.testing.assert_array_equal(out[f"{k}_which"], ref[f"{k}_which"])
            hit = out[f"{k}_hit"] == 1
            rel = np.abs(out[f"{k}_t"][hit] - ref[f"{k}_t"][hit]) / np.maximum(np.abs(ref[f"{k}_t"][hit]), 1e-300)
            assert not hit.any() or rel.max() <= TOL
            assert np.isnan(out[f"{k}_t"][~hit]).all()


@pytest.mark.parametrize("name", ["test12", "prob3", "spheres"])
def test_detect_matches_reference(ctx, golden, oracle, name):
    qs, qe, f, _, meta = _scene(golden, name)
    _, a = golden
    eta = meta["eta"]
    with C.Mesh(ctx, f, qs, qe) as m:
        for _ in range(2):  # second step reuses every buffer
            vf, vft, ee, eet = m.detect(C.BROADPHASE_KDOP13, eta, eta)
            np.testing.assert_array_equal(vf, a[f"{name}_hit_vf"])
            np.testing.assert_array_equal(ee, a[f"{name}_hit_ee"])
        st = m.stats()
        assert (st["n_vf"], st["n_ee"]) == (meta["kdop"]["n_vf"], meta["kdop"]["n_ee"])
        ref = oracle.narrowphase(qs, qe, vf, eta, ee, eta)
        assert ref["vf_hit"].all() and ref["ee_hit"].all()
        for t, rt in ((vft, ref["vf_t"]), (eet, ref["ee_t"])):
            assert t.size == 0 or (np.abs(t - rt) / np.maximum(np.abs(rt), 1e-300)).max() <= TOL


@pytest.mark.parametrize("label", ["kdop", "aabb"])
def test_larger_scene_matches_oracle(ctx, oracle, label):
    # A 64x64 sheet dropping onto a level-3 icosphere: 4,096 + 642 vertices,
    # 7,938 + 1,280 faces; a few dozen sheet-sphere contacts.
    qs, qe, f = W.sheet_on_sphere(grid=64, level=3, seed=3, gap=-0.002, drop=0.004)
    eta = 1e-4
    fixed = np.zeros(qs.size // 3, np.uint8)
    fixed[4096:] = 1  # the sphere does not move
    with C.Mesh(ctx, f, qs, qe, fixed) as m:
        vf, ee = m.broadphase(KINDS[label], eta)
        rvf, ree = oracle.broadphase(KINDS[label], qs, qe, f, eta, fixed)
        np.testing.assert_array_equal(vf, rvf)
        np.testing.assert_array_equal(ee, ree)
        out = m.narrowphase(vf, eta, ee, eta)
        ref = oracle.narrowphase(qs, qe, vf, eta, ee, eta)
        for k in ("vf", "ee"):
            np.testing.assert_array_equal(out[f"{k}_hit"], ref[f"{k}_hit"])
            np.testing.assert_array_equal(out[f"{k}_which"], ref[f"{k}_which"])
        assert out["vf_hit"].any() and out["ee_hit"].any()


@pytest.fixture(scope="module")
def cloth():
    # The cloth-on-sphere configuration at full size: a 256 x 256 sheet
    # (65,536 vertices, 130,050 faces) over a level-6 icosphere (40,962
    # vertices, 81,920 faces), 50 seeded steps.
    return W.cloth_frames(grid=256, level=6, seed=0, steps=50)


@pytest.mark.parametrize("step", [25, 40, 49])
def test_full_size_cloth_step_matches_oracle(ctx, oracle, cloth, step):
    # steps from the first contact of sheet and sphere (about step 25) on
    import oracle as O

    faces, frames = cloth
    assert faces.shape[0] == 211_970 and frames.shape[1] == 3 * 106_498
    eta = 1e-6
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        m.set_positions(frames[step], frames[step + 1])
        col = m.detect(C.BROADPHASE_KDOP13, eta, eta)
        cand = m.candidates()
    r = O.compare_mesh_step(oracle, frames[step], frames[step + 1], faces, eta, cand, col,
                            nthreads=os.cpu_count() or 4)
    assert r["identical_candidates"] and r["identical_collisions"], r
    assert r["max_rel_t_err"] <= TOL and r["candidates"] > 10_000


def test_refitted_tree_gives_the_built_trees_results(ctx, cloth):
    # Consecutive cloth steps on one mesh: the kept tree is refitted (node
    # slabs only) instead of rebuilt, which must not change any candidate or
    # collision; a fresh build of every step is the reference.
    faces, frames = cloth
    eta = 1e-6
    steps = range(24, 36)
    got, built = [], []
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        for k in steps:
            m.set_positions(frames[k], frames[k + 1])
            got.append((m.detect(C.BROADPHASE_KDOP13, eta, eta), m.candidates()))
            built.append(m.stats()["tree_built"])
    assert built[0] == 1 and built.count(0) >= len(built) // 2
    ctx.set_option("tree_refit", 0)
    try:
        for k, (col, cand) in zip(steps, got):
            with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
                m.set_positions(frames[k], frames[k + 1])
                ref = m.detect(C.BROADPHASE_KDOP13, eta, eta)
                rcand = m.candidates()
                assert m.stats()["tree_built"] == 1
            for a, b in zip(cand + col, rcand + ref):
                np.testing.assert_array_equal(a, b)
    finally:
        ctx.set_option("tree_refit", 1)


@pytest.mark.parametrize("label", ["kdop", "aabb"])
def test_traversal_kernels_agree(ctx, cloth, label):
    # The warp-per-32-faces and four-lanes-per-face traversals perform
    # exactly the slab tests of the thread-per-face ones (each query is
    # tested only against the nodes its own traversal reaches), and all find
    # the same candidates.
    faces, frames = cloth
    k = 40
    out = {}
    for trav in (0, 1, 2, 3, 4):
        ctx.set_option("traversal", trav)
        ctx.set_option("count_slab_tests", 1)
        try:
            with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
                m.set_positions(frames[k], frames[k + 1])
                vf, ee = m.broadphase(KINDS[label], 1e-6)
                out[trav] = (vf, ee, m.stats()["slab_tests"], m.stats()["face_pairs"])
        finally:
            ctx.set_option("count_slab_tests", 0)
            ctx.set_option("traversal", 3)
    for trav in (1, 2, 3, 4):
        np.testing.assert_array_equal(out[0][0], out[trav][0])
        np.testing.assert_array_equal(out[0][1], out[trav][1])
        assert out[0][2] == out[trav][2] > 0 and out[0][3] == out[trav][3]


@pytest.mark.parametrize("label", ["kdop", "aabb"])
def test_graph_step_equals_direct_step(ctx, cloth, label):
    # Consecutive cloth steps through ccd_mesh_detect_graph: the first one
    # (and every step whose candidates outgrow the capture, as contact
    # spreads from step 25 on) runs directly and captures; the others replay
    # the captured graph.  Every step's candidates and collisions equal a
    # direct step's on a mesh of its own.
    faces, frames = cloth
    eta = 1e-6
    kind = KINDS[label]
    got, replays = [], 0
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        for k in range(20, 45):
            m.set_positions(frames[k], frames[k + 1])
            col = m.detect(kind, eta, eta, graph=True)
            got.append((col, m.candidates(), m.stats()))
            replays += m.stats()["graph_replay"]
    assert replays >= 10
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3) as m:
        for k, (col, cand, st) in zip(range(20, 45), got):
            m.set_positions(frames[k], frames[k + 1])
            ref = m.detect(kind, eta, eta)
            rcand = m.candidates()
            for a, b in zip(cand + col, rcand + ref):
                np.testing.assert_array_equal(a, b)
            assert st["n_vf"] == m.stats()["n_vf"] and st["face_pairs"] == m.stats()["face_pairs"]


def test_graph_step_on_instances_matches_oracle(ctx, oracle):
    # An instance mesh (32 instances of the uneven batch) replayed from its
    # graph on a second step, against the oracle on each instance alone.
    import oracle as O

    sizes = W.uneven_sizes(512, seed=0)
    pick = [int(i) for i in np.nonzero(sizes <= 30_000)[0][:32]]
    faces, frames, vo, fo = W.uneven_batch(512, seed=0, select=pick, steps=2)
    eta = 1e-6
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3, instances=(vo, fo)) as m:
        m.set_positions(frames[0], frames[1])
        m.detect(C.BROADPHASE_KDOP13, eta, eta, graph=True)
        m.set_positions(frames[1], frames[2])
        col = m.detect(C.BROADPHASE_KDOP13, eta, eta, graph=True)
        assert m.stats()["graph_replay"] == 1
        cand = m.candidates()
    parts = {k: [] for k in ("vf_c", "ee_c", "vf_hit", "ee_hit", "vf_t", "ee_t")}
    for i in range(32):
        a, b = 3 * vo[i], 3 * vo[i + 1]
        fi = faces[fo[i]:fo[i + 1]] - vo[i]
        vf_c, ee_c = oracle.broadphase(0, frames[1][a:b], frames[2][a:b], fi, eta)
        r = oracle.narrowphase(frames[1][a:b], frames[2][a:b], vf_c, eta, ee_c, eta, nthreads=os.cpu_count() or 4)
        parts["vf_c"].append(vf_c + vo[i])
        parts["ee_c"].append(ee_c + vo[i])
        for k in ("vf_hit", "ee_hit", "vf_t", "ee_t"):
            parts[k].append(r[k])
    cat = {k: np.concatenate(v) for k, v in parts.items()}
    r = O.compare_step_results(cat["vf_c"], cat["ee_c"], cat, cand, col)
    assert r["identical_candidates"] and r["identical_collisions"], r
    assert r["max_rel_t_err"] <= TOL


def test_graph_step_falls_back_when_not_eligible(ctx, golden):
    # With the context's tree refit off, or profiling on, the call is the
    # direct step (and says so).
    qs, qe, f, _, meta = _scene(golden, "spheres")
    with C.Mesh(ctx, f, qs, qe) as m:
        ref = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
        ctx.set_option("tree_refit", 0)
        try:
            for _ in range(3):
                got = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6, graph=True)
                assert m.stats()["graph_replay"] == 0
        finally:
            ctx.set_option("tree_refit", 1)
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)


def test_uneven_instances_match_oracle(ctx, oracle):
    # 32 instances of the 512-instance uneven batch (icospheres and sheet
    # pairs; the first 32 with at most 30,000 requested triangles, so that
    # the oracle finishes in seconds) in one instance mesh, against the
    # oracle run on each instance alone.
    import oracle as O

    sizes = W.uneven_sizes(512, seed=0)
    pick = [int(i) for i in np.nonzero(sizes <= 30_000)[0][:32]]
    faces, frames, vo, fo = W.uneven_batch(512, seed=0, select=pick)
    eta = 1e-6
    with C.Mesh(ctx, faces, nverts=frames.shape[1] // 3, instances=(vo, fo)) as m:
        m.set_positions(frames[0], frames[1])
        col = m.detect(C.BROADPHASE_KDOP13, eta, eta)
        cand = m.candidates()
    parts = {k: [] for k in ("vf_c", "ee_c", "vf_hit", "ee_hit", "vf_t", "ee_t")}
    for i in range(32):
        a, b = 3 * vo[i], 3 * vo[i + 1]
        fi = faces[fo[i]:fo[i + 1]] - vo[i]
        vf_c, ee_c = oracle.broadphase(0, frames[0][a:b], frames[1][a:b], fi, eta)
        r = oracle.narrowphase(frames[0][a:b], frames[1][a:b], vf_c, eta, ee_c, eta, nthreads=os.cpu_count() or 4)
        parts["vf_c"].append(vf_c + vo[i])
        parts["ee_c"].append(ee_c + vo[i])
        for k in ("vf_hit", "ee_hit", "vf_t", "ee_t"):
            parts[k].append(r[k])
    cat = {k: np.concatenate(v) for k, v in parts.items()}
    r = O.compare_step_results(cat["vf_c"], cat["ee_c"], cat, cand, col)
    assert r["identical_candidates"] and r["identical_collisions"], r
    assert r["max_rel_t_err"] <= TOL and r["collisions"] > 0


def test_per_stencil_eta_and_order_independence(ctx, oracle, golden):
    qs, qe, f, _, meta = _scene(golden, "spheres")
    with C.Mesh(ctx, f, qs, qe) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, 1e-3)
        rng = np.random.default_rng(5)
        vfe = 10.0 ** rng.uniform(-7, -3, vf.shape[0])
        eee = 10.0 ** rng.uniform(-7, -3, ee.shape[0])
        out = m.narrowphase(vf, vfe, ee, eee)
        ref = oracle.narrowphase(qs, qe, vf, vfe, ee, eee)
        np.testing.assert_array_equal(out["vf_hit"], ref["vf_hit"])
        np.testing.assert_array_equal(out["ee_hit"], ref["ee_hit"])
        # Unsorted, non-canonical stencils give the same per-stencil answers
        # (the reference canonicalises in the stencil constructors).
        perm = rng.permutation(vf.shape[0])
        shuffled = vf[perm][:, [0, 3, 1, 2]]
        out2 = m.narrowphase(shuffled, vfe[perm], ee[:0], 1e-6)
        np.testing.assert_array_equal(out2["vf_hit"], out["vf_hit"][perm])


def test_edge_cases(ctx):
    # No faces, one face, two faces sharing a vertex: no candidates.
    qs = np.zeros(12)
    qe = np.zeros(12)
    for faces in (np.zeros((0, 3), np.int32), np.array([[0, 1, 2]]), np.array([[0, 1, 2], [2, 3, 1]])):
        with C.Mesh(ctx, faces, qs, qe) as m:
            vf, ee = m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
            assert vf.shape == (0, 4) and ee.shape == (0, 4)
            vf, vft, ee, eet = m.detect(C.BROADPHASE_AABB, 1e-6, 1e-6)
            assert vf.shape == (0, 4) and ee.shape == (0, 4)
    # Two coincident separate triangles: 6 vertex-face and 9 edge-edge stencils.
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    pos = np.concatenate([tri, tri]).ravel()
    with C.Mesh(ctx, np.array([[0, 1, 2], [3, 4, 5]]), pos, pos) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
        assert vf.shape == (6, 4) and ee.shape == (9, 4)
        assert [tuple(r) for r in vf] == sorted(tuple(r) for r in vf)
        # All fixed: nothing is emitted.
        m.set_fixed(np.ones(6, np.uint8))
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
        assert vf.shape == (0, 4) and ee.shape == (0, 4)
    # Invalid input is rejected before any device work.
    with pytest.raises(C.CcdError):
        C.Mesh(ctx, np.array([[0, 1, 7]]), np.zeros(9), np.zeros(9))
    with C.Mesh(ctx, np.array([[0, 1, 2]]), np.zeros(9), np.zeros(9)) as m:
        with pytest.raises(C.CcdError):
            m.narrowphase(np.array([[0, 1, 2, 3]]), 1e-6, np.zeros((0, 4)), 1e-6)
        with pytest.raises(C.CcdError):
            m.narrowphase(np.array([[0, 1, 2, 0]]), [1e-6, 1e-6], np.zeros((0, 4)), 1e-6)


def _concat(scenes):
    faces, qs, qe, fixed, vo, fo = [], [], [], [], [0], [0]
    for s_qs, s_qe, s_f, s_fx in scenes:
        faces.append(np.asarray(s_f, np.int32) + vo[-1])
        qs.append(np.asarray(s_qs).ravel())
        qe.append(np.asarray(s_qe).ravel())
        fixed.append(np.asarray(s_fx, np.uint8))
        vo.append(vo[-1] + np.asarray(s_qs).size // 3)
        fo.append(fo[-1] + len(s_f))
    return (np.concatenate(faces), np.concatenate(qs), np.concatenate(qe), np.concatenate(fixed),
            np.array(vo, np.int32), np.array(fo, np.int32))


@pytest.mark.parametrize("label", ["kdop", "aabb"])
def test_instances_equal_each_instance_alone(ctx, golden, label):
    # Three reference scenes and a second copy of the two-sphere scene at the
    # same coordinates (instances overlap in space but are never paired).
    names = ["test12", "spheres", "prob3", "spheres"]
    scenes = [_scene(golden, n)[:4] for n in names]
    scenes = [(qs, qe, f, fx) for qs, qe, f, fx in scenes]
    f, qs, qe, fixed, vo, fo = _concat(scenes)
    eta = 1e-6
    with C.Mesh(ctx, f, qs, qe, instances=(vo, fo)) as m:
        for use_fixed in (False, True):
            m.set_fixed(fixed if use_fixed else None)
            vf, ee = m.broadphase(KINDS[label], eta)
            want_vf, want_ee = [], []
            for i, (s_qs, s_qe, s_f, s_fx) in enumerate(scenes):
                with C.Mesh(ctx, s_f, s_qs, s_qe, s_fx if use_fixed else None) as single:
                    a, b = single.broadphase(KINDS[label], eta)
                want_vf.append(a + vo[i])
                want_ee.append(b + vo[i])
            np.testing.assert_array_equal(vf, np.concatenate(want_vf))
            np.testing.assert_array_equal(ee, np.concatenate(want_ee))
        m.set_fixed(None)
        vf, vft, ee, eet = m.detect(KINDS[label], eta, eta)
        want = [[], [], [], []]
        for i, (s_qs, s_qe, s_f, _) in enumerate(scenes):
            with C.Mesh(ctx, s_f, s_qs, s_qe) as single:
                a, at, b, bt = single.detect(KINDS[label], eta, eta)
            want[0].append(a + vo[i])
            want[1].append(at)
            want[2].append(b + vo[i])
            want[3].append(bt)
        np.testing.assert_array_equal(vf, np.concatenate(want[0]))
        np.testing.assert_array_equal(vft, np.concatenate(want[1]))
        np.testing.assert_array_equal(ee, np.concatenate(want[2]))
        np.testing.assert_array_equal(eet, np.concatenate(want[3]))


def test_instances_reject_foreign_vertices(ctx):
    tri = np.array([[0, 1, 2], [3, 4, 5]], np.int32)
    pos = np.zeros(18)
    with pytest.raises(C.CcdError):  # face 1 of instance 0 uses instance 1's vertices
        C.Mesh(ctx, tri, pos, pos, instances=(np.array([0, 3, 6]), np.array([0, 2, 2])))
    with C.Mesh(ctx, tri, pos, pos, instances=(np.array([0, 3, 6]), np.array([0, 1, 2]))) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, 1e-6)
        assert vf.shape == (0, 4) and ee.shape == (0, 4)  # coincident, but different instances


def test_slab_test_counting_and_broadphase_timing(ctx, golden):
    qs, qe, f, _, meta = _scene(golden, "spheres")
    with C.Mesh(ctx, f, qs, qe) as m:
        vf0, ee0 = m.broadphase(C.BROADPHASE_KDOP13, meta["eta"])
        assert m.stats()["slab_tests"] == -1
        ctx.set_option("count_slab_tests", 1)
        ctx.set_profiling(True)
        vf1, ee1 = m.broadphase(C.BROADPHASE_KDOP13, meta["eta"])
        st = m.stats()
        ctx.set_profiling(False)
        ctx.set_option("count_slab_tests", 0)
        np.testing.assert_array_equal(vf0, vf1)  # counting changes nothing but the count
        np.testing.assert_array_equal(ee0, ee1)
        # at least one slab test per reported pair, at most one per (leaf, node)
        assert st["face_pairs"] <= st["slab_tests"] <= f.shape[0] * (2 * f.shape[0])
        assert 0 < st["traversal_ms"] <= st["broadphase_ms"]


# ------------------------------------------------------------------ TrivialBroadPhase
@pytest.mark.parametrize("mesh", ["test12", "prob3", "spheres"])
def test_trivial_broadphase_matches_reference(ctx, golden_dir, mesh):
    meta = json.load(open(os.path.join(golden_dir, "trivial.json")))[mesh]
    g = np.load(os.path.join(golden_dir, "meshes.npz"))
    qs, qe, f, fixed = g[f"{mesh}_qstart"], g[f"{mesh}_qend"], g[f"{mesh}_faces"], g[f"{mesh}_fixed"]
    with C.Mesh(ctx, f, qs, qe) as m:
        for label, fx in (("free", None), ("fixed", fixed)):
            m.set_fixed(fx)
            vf, ee = m.broadphase(C.BROADPHASE_TRIVIAL, 1e-6)
            exp = meta[label]
            assert (vf.shape[0], ee.shape[0]) == (exp["n_vf"], exp["n_ee"])
            assert digest(vf, ee) == exp["digest"]


@pytest.mark.parametrize("case", ["spheres", "cloth"])
def test_tree_broadphases_against_every_stencil(ctx, oracle, case):
    """The k-DOP and AABB trees against the trivial broad phase (every stencil
    of the mesh), with the narrow phase's eta equal to the padding.  Every
    collision the trees find is found with every stencil too, with the same t,
    and so is every vertex-face collision.  The reference's edge-edge test
    measures the distance between the edges' lines, so it also reports nearly
    collinear edges far apart (along a row of the wrinkled sheet: 114 such
    hits; one on the spheres); only the broad phase keeps those out, so the
    extra hits are edge-edge stencils the trees never propose.  The trivial
    result itself is the oracle's."""
    if case == "spheres":
        qs, qe, f = W.two_spheres(seed=2, level=2)
    else:
        f, frames = W.cloth_frames(grid=20, level=2, seed=4, steps=6)
        qs, qe = frames[4], frames[5]
    eta = 1e-3
    with C.Mesh(ctx, f, qs, qe) as m:
        tvf, tvft, tee, teet = m.detect(C.BROADPHASE_TRIVIAL, eta, eta)
        assert tvf.shape[0] + tee.shape[0] > 0
        cvf, cee = oracle.broadphase(2, qs, qe, f, eta)
        r = oracle.narrowphase(qs, qe, cvf, eta, cee, eta, nthreads=os.cpu_count() or 1)
        np.testing.assert_array_equal(tvf, cvf[r["vf_hit"] == 1])
        np.testing.assert_array_equal(tee, cee[r["ee_hit"] == 1])
        for kind in (C.BROADPHASE_KDOP13, C.BROADPHASE_AABB):
            vf, vft, ee, eet = m.detect(kind, eta, eta)
            cand_vf, cand_ee = m.broadphase(kind, eta)
            for got, t_got, every, t_every, cand in ((vf, vft, tvf, tvft, cand_vf), (ee, eet, tee, teet, cand_ee)):
                pos = {tuple(x): i for i, x in enumerate(every)}
                assert all(tuple(x) in pos for x in got)
                np.testing.assert_array_equal(t_got, t_every[[pos[tuple(x)] for x in got]])
                extra = set(pos) - set(map(tuple, got))
                assert not (extra & set(map(tuple, cand)))
            assert vf.shape[0] == tvf.shape[0]  # no vertex-face hit is left out in either scene


def test_trivial_broadphase_rejects_instances(ctx):
    v, f = W.icosphere(1, 0.5)
    vv = np.concatenate([v, v + 2.0])
    ff = np.concatenate([f, f + v.shape[0]]).astype(np.int32)
    with C.Mesh(ctx, ff, vv.ravel(), vv.ravel(), instances=([0, v.shape[0], vv.shape[0]],
                                                          [0, f.shape[0], ff.shape[0]])) as m:
        with pytest.raises(C.CcdError):
            m.broadphase(C.BROADPHASE_TRIVIAL, 1e-6)


# ------------------------------------------------------------------ multi-entry History
@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_multi_entry_history_matches_reference(ctx, oracle, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "history.json")))[scene]
    g = np.load(os.path.join(golden_dir, "history.npz"))
    off, tt, pp = g[f"{scene}_offsets"], g[f"{scene}_times"], g[f"{scene}_positions"]
    f, fixed, eta = g[f"{scene}_faces"], g[f"{scene}_fixed"], meta["eta"]
    with C.Mesh(ctx, f, nverts=off.size - 1) as m:
        m.set_history(off, tt, pp)
        for label in ("kdop", "aabb"):
            for fx_label, fx in (("", None), ("_fixed", fixed)):
                m.set_fixed(fx)
                vf, ee = m.broadphase(KINDS[label], eta)
                exp = meta[f"{label}{fx_label}"]
                assert (vf.shape[0], ee.shape[0]) == (exp["n_vf"], exp["n_ee"])
                assert digest(vf, ee) == exp["digest"]
        m.set_fixed(None)
        hvf, hvft, hee, heet = m.detect(C.BROADPHASE_KDOP13, eta, eta)
        np.testing.assert_array_equal(hvf, g[f"{scene}_hit_vf"])
        np.testing.assert_array_equal(hee, g[f"{scene}_hit_ee"])
        # contact times and sub-tests against the oracle
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, eta)
        out = m.narrowphase(vf, eta, ee, eta)
        ref = oracle.narrowphase_history(off, tt, pp, vf, eta, ee, eta)
        for k in ("vf", "ee"):
            np.testing.assert_array_equal(out[f"{k}_hit"], ref[f"{k}_hit"])
            np.testing.assert_array_equal(out[f"{k}_which"], ref[f"{k}_which"])
            h = ref[f"{k}_hit"] == 1
            rel = np.abs(out[f"{k}_t"][h] - ref[f"{k}_t"][h]) / np.maximum(np.abs(ref[f"{k}_t"][h]), 1e-300)
            assert not h.any() or rel.max() <= TOL


def test_two_entry_history_equals_a_step(ctx):
    """A history of two entries per vertex (t = 0 and 1) gives exactly what
    the step of ccd_mesh_set_positions gives, and set_positions afterwards
    returns to the step."""
    qs, qe, f = W.two_spheres(seed=3)
    nv = qs.size // 3
    off = np.arange(0, 2 * nv + 1, 2, dtype=np.int32)
    tt = np.tile([0.0, 1.0], nv)
    pp = np.stack([qs.reshape(-1, 3), qe.reshape(-1, 3)], axis=1).reshape(-1, 3)
    with C.Mesh(ctx, f, qs, qe) as m:
        step = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
        m.set_history(off, tt, pp)
        hist = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
        m.set_positions(qs, qe)
        again = m.detect(C.BROADPHASE_KDOP13, 1e-6, 1e-6)
    for a, b, c in zip(step, hist, again):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)
    assert step[0].shape[0] + step[2].shape[0] > 0


def test_history_rejects_bad_input(ctx):
    v, f = W.icosphere(1, 0.5)
    nv = v.shape[0]
    with C.Mesh(ctx, f, nverts=nv) as m:
        off = np.arange(0, 2 * nv + 1, 2, dtype=np.int32)
        tt = np.tile([0.0, 1.0], nv)
        pp = np.repeat(v, 2, axis=0)
        bad_t = tt.copy()
        bad_t[1] = -1.0  # decreasing
        with pytest.raises(C.CcdError):
            m.set_history(off, bad_t, pp)
        empty = off.copy()
        empty[1:] -= 2  # vertex 0 without entries
        empty[0] = 0
        with pytest.raises(C.CcdError):
            m.set_history(empty, tt[: empty[-1]], pp[: empty[-1]])


# ------------------------------------------------------------------ SeparatingPlaneNarrowPhase
@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_separating_plane_matches_reference(ctx, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "history.json")))[scene]
    g = np.load(os.path.join(golden_dir, "history.npz"))
    off, tt, pp, f, eta = g[f"{scene}_offsets"], g[f"{scene}_times"], g[f"{scene}_positions"], g[f"{scene}_faces"], \
        meta["eta"]
    with C.Mesh(ctx, f, nverts=off.size - 1) as m:
        m.set_history(off, tt, pp)
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, eta)
        out = m.narrowphase_separating_plane(vf, eta, ee, eta)
    for k in ("vf", "ee"):
        np.testing.assert_array_equal(out[f"{k}_status"], g[f"{scene}_sp_{k}_stalled"])
        ok = out[f"{k}_status"] == 0
        np.testing.assert_array_equal(out[f"{k}_hit"][ok], g[f"{scene}_sp_{k}_hit"])
        assert not out[f"{k}_hit"][~ok].any()


def test_separating_plane_on_a_step_matches_oracle(ctx, oracle):
    """Without a history set, the two-entry step is the history (eps = 1/4)."""
    qs, qe, f = W.two_spheres(seed=2)
    nv = qs.size // 3
    off = np.arange(0, 2 * nv + 1, 2, dtype=np.int32)
    tt = np.tile([0.0, 1.0], nv)
    pp = np.stack([qs.reshape(-1, 3), qe.reshape(-1, 3)], axis=1).reshape(-1, 3)
    eta = 1e-3
    with C.Mesh(ctx, f, qs, qe) as m:
        vf, ee = m.broadphase(C.BROADPHASE_KDOP13, eta)
        out = m.narrowphase_separating_plane(vf, eta, ee, eta)
    vh, eh, vs, es = oracle.separating_plane(off, tt, pp, vf, eta, ee, eta)
    np.testing.assert_array_equal(out["vf_hit"], vh)
    np.testing.assert_array_equal(out["ee_hit"], eh)
    np.testing.assert_array_equal(out["vf_status"], vs)
    np.testing.assert_array_equal(out["ee_status"], es)
    assert vh.sum() + eh.sum() > 0
