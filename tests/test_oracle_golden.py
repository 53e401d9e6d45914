"""The C restatement (oracle/) against fixtures produced by the reference's
own sources (tests/golden/make_golden.py).  CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def test_testctcd_known_answers(oracle, golden_dir):
    kat = json.load(open(os.path.join(golden_dir, "kat_testctcd.json")))
    assert len(kat) == 4
    for case in kat:
        h, t = oracle.prim(case["kind"], case["points"], case["eta"])
        assert h == case["hit"] == 1
        assert float(t).hex() == case["t_hex"]


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_primitives_bit_exact(oracle, golden_dir, kind):
    g = np.load(os.path.join(golden_dir, "prims.npz"))
    x, eta, hit, t = g[f"x{kind}"], g[f"eta{kind}"], g[f"hit{kind}"], g[f"t{kind}"]
    h2, t2 = oracle.batch(kind, x, eta)
    np.testing.assert_array_equal(h2, hit)
    same = (t2.view(np.uint64) == t.view(np.uint64)) | (np.isnan(t) & np.isnan(t2))
    assert same.all(), np.nonzero(~same)[0][:10]
    assert hit.sum() > 0 and (hit == 0).sum() > 0


@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_flop_counter_runs_the_oracle(golden_dir, kind):
    # The counting build of the primitive tests computes exactly the
    # reference's results (same operations, same rounding), so its counts are
    # those of the reference's op sequence on these rows.
    import oracle as O

    O.build()
    fc = O.FlopCounter()
    g = np.load(os.path.join(golden_dir, "prims.npz"))
    x, eta, hit, t = g[f"x{kind}"], g[f"eta{kind}"], g[f"hit{kind}"], g[f"t{kind}"]
    h2, t2, flops, tot = fc.batch(kind, x, eta, nthreads=4)
    np.testing.assert_array_equal(h2, hit)
    same = (t2.view(np.uint64) == t.view(np.uint64)) | (np.isnan(t) & np.isnan(t2))
    assert same.all()
    assert flops.min() > 0  # every test forms at least its first polynomial
    assert int(flops.astype(np.int64).sum()) == tot["add"] + tot["mul"] + tot["div"] + tot["sqrt"]
    _, _, f1, tot1 = fc.batch(kind, x, eta, nthreads=1)
    np.testing.assert_array_equal(f1, flops)
    assert tot1 == tot


def test_flop_counts_of_simple_cases():
    # Vertex-vertex rows that meet the quadratic branch with two roots: the
    # count is the reference's fixed sequence (src/CTCD.cpp:604-692) and does
    # not depend on the coordinates.
    import oracle as O

    fc = O.FlopCounter()
    rows = np.array([[0, 0, 0, 1, 0, 0, 0.5, 0, 0, 0.6, 0, 0],
                     [0, 0, 0, 2, 0, 0, 0.7, 0, 0, 1.0, 0, 0]], float)
    h, t, flops, tot = fc.batch(3, rows, 1e-3)
    assert flops[0] == flops[1] > 20 and tot["transcendental"] == 0 and tot["sqrt"] == 2


def test_threaded_batch_matches_serial(oracle, golden_dir):
    g = np.load(os.path.join(golden_dir, "prims.npz"))
    for kind in range(4):
        h1, t1 = oracle.batch(kind, g[f"x{kind}"], g[f"eta{kind}"], nthreads=1)
        h4, t4 = oracle.batch(kind, g[f"x{kind}"], g[f"eta{kind}"], nthreads=4)
        np.testing.assert_array_equal(h1, h4)
        np.testing.assert_array_equal(t1, t4)


@pytest.mark.parametrize("mesh", ["test12", "prob3", "spheres"])
def test_broadphase_candidate_sets(oracle, golden_dir, mesh):
    meta = json.load(open(os.path.join(golden_dir, "meshes.json")))[mesh]
    g = np.load(os.path.join(golden_dir, "meshes.npz"))
    qs, qe, f, fixed = g[f"{mesh}_qstart"], g[f"{mesh}_qend"], g[f"{mesh}_faces"], g[f"{mesh}_fixed"]
    for kind, label in ((0, "kdop"), (1, "aabb")):
        for fx_label, fx in (("", None), ("_fixed", fixed)):
            vf, ee = oracle.broadphase(kind, qs, qe, f, meta["eta"], fx)
            exp = meta[f"{label}{fx_label}"]
            assert (vf.shape[0], ee.shape[0]) == (exp["n_vf"], exp["n_ee"])
            assert _digest(vf, ee) == exp["digest"]


@pytest.mark.parametrize("mesh", ["test12", "prob3", "spheres"])
def test_narrowphase_colliding_set(oracle, golden_dir, mesh):
    meta = json.load(open(os.path.join(golden_dir, "meshes.json")))[mesh]
    g = np.load(os.path.join(golden_dir, "meshes.npz"))
    qs, qe, f = g[f"{mesh}_qstart"], g[f"{mesh}_qend"], g[f"{mesh}_faces"]
    eta = meta["eta"]
    vf, ee = oracle.broadphase(0, qs, qe, f, eta)
    out = oracle.narrowphase(qs, qe, vf, eta, ee, eta, nthreads=2)
    assert _digest(out["vf_hit"], out["ee_hit"]) == meta["narrow"]["digest"]
    np.testing.assert_array_equal(vf[out["vf_hit"].astype(bool)], g[f"{mesh}_hit_vf"])
    np.testing.assert_array_equal(ee[out["ee_hit"].astype(bool)], g[f"{mesh}_hit_ee"])
    # every hit reports which test in the chain fired and a time
    assert (out["vf_which"][out["vf_hit"] == 1] >= 0).all()
    assert np.isfinite(out["ee_t"][out["ee_hit"] == 1]).all()


def test_stencil_canonical_forms(oracle):
    import ctypes

    r = (ctypes.c_int32 * 4)()
    oracle.lib.oracle_vf_canon(7, 9, 3, 5, r)
    assert list(r) == [7, 3, 5, 9]
    oracle.lib.oracle_ee_canon(9, 4, 2, 8, r)
    assert list(r) == [2, 8, 4, 9]
    oracle.lib.oracle_ee_canon(1, 4, 8, 2, r)
    assert list(r) == [1, 4, 2, 8]


def _same_bits(a, b):
    """Equal bit for bit, NaN matching any NaN."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("kind", [0, 1])
def test_distance_queries_bit_exact(oracle, golden_dir, kind):
    g = np.load(os.path.join(golden_dir, "distances.npz"))
    rows = g[f"rows{kind}"]
    vec, bary = oracle.distance(kind, rows)
    assert _same_bits(vec, g[f"vec{kind}"]).all()
    assert _same_bits(bary, g[f"bary{kind}"]).all()
    less = oracle.distance_less_than(kind, rows, g[f"eta{kind}"])
    np.testing.assert_array_equal(less, g[f"less{kind}"])
    assert 0 < less.sum() < less.size


@pytest.mark.parametrize("mesh", ["spheres", "test1", "prob3", "prob11", "cloth", "one_triangle", "two_triangles",
                                  "shared_edge", "coincident_copies", "isolated_vertex", "repeated_index"])
def test_mesh_self_distance(oracle, golden_dir, mesh):
    meta = json.load(open(os.path.join(golden_dir, "distances.json")))["self_distance"][mesh]
    g = np.load(os.path.join(golden_dir, "distances.npz"))
    v, f, fixed = g[f"mesh_{mesh}_verts"], g[f"mesh_{mesh}_faces"], g[f"mesh_{mesh}_fixed"]
    for label, fx in (("free", None), ("fixed", fixed)):
        d, nvf, nee = oracle.mesh_self_distance(v, f, fx)
        exp = meta[label]
        assert float(d).hex() == exp["distance_hex"]
        assert (nvf, nee) == (exp["n_vf"], exp["n_ee"])


@pytest.mark.parametrize("mesh,label", [("test12", "free"), ("test12", "fixed"), ("prob3", "free"),
                                        ("prob3", "fixed"), ("spheres", "fixed")])
def test_trivial_broadphase(oracle, golden_dir, mesh, label):
    meta = json.load(open(os.path.join(golden_dir, "trivial.json")))[mesh][label]
    g = np.load(os.path.join(golden_dir, "meshes.npz"))
    qs, qe, f, fixed = g[f"{mesh}_qstart"], g[f"{mesh}_qend"], g[f"{mesh}_faces"], g[f"{mesh}_fixed"]
    vf, ee = oracle.broadphase(2, qs, qe, f, 1e-6, fixed if label == "fixed" else None)
    assert (vf.shape[0], ee.shape[0]) == (meta["n_vf"], meta["n_ee"])
    assert _digest(vf, ee) == meta["digest"]


@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_penalty_group_force(oracle, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "penalty.json")))
    g = np.load(os.path.join(golden_dir, "penalty.npz"))
    p = meta[scene]
    for label, use_new in (("new", True), ("old", False)):
        F, vfire, efire, used = oracle.penalty_group_force(
            g[f"{scene}_q"], g[f"{scene}_v"], g[f"{scene}_F0"], g[f"{scene}_vf"], g[f"{scene}_ee"], p["outer_eta"],
            p["inner_eta"], p["stiffness"], p["cor"], p["dt"],
            g[f"{scene}_vf_isnew"] if use_new else None, g[f"{scene}_ee_isnew"] if use_new else None)
        assert _same_bits(F, g[f"{scene}_{label}_F"]).all()
        np.testing.assert_array_equal(vfire, g[f"{scene}_{label}_vf_fired"])
        np.testing.assert_array_equal(efire, g[f"{scene}_{label}_ee_fired"])
        assert used == meta[f"{scene}_{label}"]["newused"]


@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_multi_entry_history(oracle, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "history.json")))[scene]
    g = np.load(os.path.join(golden_dir, "history.npz"))
    off, tt, pp = g[f"{scene}_offsets"], g[f"{scene}_times"], g[f"{scene}_positions"]
    f, fixed, eta = g[f"{scene}_faces"], g[f"{scene}_fixed"], meta["eta"]
    for kind, label in ((0, "kdop"), (1, "aabb")):
        for fx_label, fx in (("", None), ("_fixed", fixed)):
            vf, ee = oracle.broadphase_history(kind, off, tt, pp, f, eta, fx)
            exp = meta[f"{label}{fx_label}"]
            assert (vf.shape[0], ee.shape[0]) == (exp["n_vf"], exp["n_ee"])
            assert _digest(vf, ee) == exp["digest"]
    vf, ee = oracle.broadphase_history(0, off, tt, pp, f, eta)
    out = oracle.narrowphase_history(off, tt, pp, vf, eta, ee, eta)
    assert _digest(out["vf_hit"], out["ee_hit"]) == meta["narrow"]["digest"]
    np.testing.assert_array_equal(vf[out["vf_hit"] == 1], g[f"{scene}_hit_vf"])
    np.testing.assert_array_equal(ee[out["ee_hit"] == 1], g[f"{scene}_hit_ee"])


@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_separating_plane_narrowphase(oracle, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "history.json")))[scene]
    g = np.load(os.path.join(golden_dir, "history.npz"))
    off, tt, pp, f, eta = g[f"{scene}_offsets"], g[f"{scene}_times"], g[f"{scene}_positions"], g[f"{scene}_faces"], \
        meta["eta"]
    vf, ee = oracle.broadphase_history(0, off, tt, pp, f, eta)
    vh, eh, vs, es = oracle.separating_plane(off, tt, pp, vf, eta, ee, eta)
    np.testing.assert_array_equal(vs, g[f"{scene}_sp_vf_stalled"])
    np.testing.assert_array_equal(es, g[f"{scene}_sp_ee_stalled"])
    np.testing.assert_array_equal(vh[vs == 0], g[f"{scene}_sp_vf_hit"])
    np.testing.assert_array_equal(eh[es == 0], g[f"{scene}_sp_ee_hit"])
    assert not vh[vs == 1].any() and not eh[es == 1].any()
