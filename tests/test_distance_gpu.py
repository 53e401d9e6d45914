"""Distance queries on the GPU (ccd_distance_*, ccd_mesh_self_distance,
ccd_self_distance) against the golden fixtures (produced by the reference's
own src/Distance.cpp) and the oracle.

Parity bar: bit-identical vectors, barycentric coordinates, predicate flags
and self distances; identical stencil counts (the ones the reference prints).
At the full sheet-on-sphere size (211,970 faces) the oracle's O(V F) vertex
scan is too slow, so the three stages are checked one by one: the vertex
scan's minimum recomputed exactly on the CPU from a k-d tree's neighbour
pairs, the candidate set against the oracle's AABB broad phase at that
padding, and the least stencil distance against the oracle's closest-point
queries over those candidates."""
import json
import os

import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MESHES = ["spheres", "test1", "prob3", "prob11", "cloth", "one_triangle", "two_triangles", "shared_edge",
          "coincident_copies", "isolated_vertex", "repeated_index"]


@pytest.fixture(scope="module")
def ctx():
    from collisiondetection_gb300 import build as B

    B.build_library()
    c = C.Context(0)
    yield c
    c.close()


def _same_bits(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("kind", [C.DISTANCE_VERTEX_FACE, C.DISTANCE_EDGE_EDGE])
def test_distance_queries_match_reference(ctx, golden_dir, kind):
    g = np.load(os.path.join(golden_dir, "distances.npz"))
    rows = g[f"rows{kind}"]
    vec, bary = ctx.distance(kind, rows)
    bad = np.nonzero(~_same_bits(vec, g[f"vec{kind}"]).all(axis=1))[0]
    assert bad.size == 0, f"vectors differ at rows {bad[:10]}"
    assert _same_bits(bary, g[f"bary{kind}"]).all()
    vec2, none = ctx.distance(kind, rows, want_bary=False)
    assert none is None and _same_bits(vec2, vec).all()
    less = ctx.distance_less_than(kind, rows, g[f"eta{kind}"])
    np.testing.assert_array_equal(less, g[f"less{kind}"])
    # one shared eta is the same as that eta on every row
    np.testing.assert_array_equal(ctx.distance_less_than(kind, rows, 0.2),
                                  ctx.distance_less_than(kind, rows, np.full(rows.shape[0], 0.2)))


def test_distance_device_entry_point(ctx, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    rows = rng.uniform(-1, 1, (300_000, 12))
    for kind in (C.DISTANCE_VERTEX_FACE, C.DISTANCE_EDGE_EDGE):
        d_rows = torch.from_numpy(rows).cuda()
        d_vec = torch.empty((rows.shape[0], 3), dtype=torch.float64, device="cuda")
        d_bary = torch.empty((rows.shape[0], 3 if kind == 0 else 4), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ctx.distance_device(kind, rows.shape[0], d_rows.data_ptr(), d_vec.data_ptr(), d_bary.data_ptr())
        ctx.synchronize()
        vec, bary = oracle.distance(kind, rows)
        assert _same_bits(d_vec.cpu().numpy(), vec).all()
        assert _same_bits(d_bary.cpu().numpy(), bary).all()


@pytest.mark.parametrize("mesh", MESHES)
def test_self_distance_matches_reference(ctx, golden_dir, mesh):
    meta = json.load(open(os.path.join(golden_dir, "distances.json")))["self_distance"][mesh]
    g = np.load(os.path.join(golden_dir, "distances.npz"))
    v, f, fixed = g[f"mesh_{mesh}_verts"], g[f"mesh_{mesh}_faces"], g[f"mesh_{mesh}_fixed"]
    with C.Mesh(ctx, f, nverts=v.shape[0]) as m:
        for label, fx in (("free", None), ("fixed", fixed)):
            m.set_fixed(fx)
            d, nvf, nee = m.self_distance(v)
            exp = meta[label]
            assert float(d).hex() == exp["distance_hex"], (label, d, exp["distance"])
            assert (nvf, nee) == (exp["n_vf"], exp["n_ee"])
            vf, ee = m.candidates()
            assert vf.shape[0] == nvf and ee.shape[0] == nee
        assert float(ctx.self_distance(v, f, fixed)).hex() == meta["fixed"]["distance_hex"]


@pytest.mark.parametrize("case", ["cloth32", "spheres4"])
def test_self_distance_matches_oracle(ctx, oracle, case):
    if case == "cloth32":
        f, frames = W.cloth_frames(grid=32, level=3, seed=5, steps=3)
        v = frames[2]
    else:
        qs, _, f = W.two_spheres(seed=4, level=4)
        v = qs
    v = np.ascontiguousarray(v, np.float64).reshape(-1, 3)
    fixed = (np.arange(v.shape[0]) % 3 == 0).astype(np.uint8)
    with C.Mesh(ctx, f, nverts=v.shape[0]) as m:
        for fx in (None, fixed):
            m.set_fixed(fx)
            d, nvf, nee = m.self_distance(v)
            d_ref, nvf_ref, nee_ref = oracle.mesh_self_distance(v, f, fx)
            assert float(d).hex() == float(d_ref).hex()
            assert (nvf, nee) == (nvf_ref, nee_ref)


def test_instance_mesh_is_measured_as_one_mesh(ctx, oracle):
    a_v, a_f = W.icosphere(2, 0.5)
    b_v = a_v + np.array([1.02, 0.0, 0.0])
    v = np.concatenate([a_v, b_v])
    f = np.concatenate([a_f, a_f + a_v.shape[0]]).astype(np.int32)
    voff = np.array([0, a_v.shape[0], v.shape[0]], np.int32)
    foff = np.array([0, a_f.shape[0], f.shape[0]], np.int32)
    with C.Mesh(ctx, f, nverts=v.shape[0], instances=(voff, foff)) as m:
        d, nvf, nee = m.self_distance(v)
    d_ref, nvf_ref, nee_ref = oracle.mesh_self_distance(v, f)
    assert float(d).hex() == float(d_ref).hex() and (nvf, nee) == (nvf_ref, nee_ref)
    assert d < 0.03  # the gap between the spheres, not a sphere's own spacing


# ------------------------------------------------------------------ full size
def _vertex_scan_min_sq(v, f):
    """The minimum of Distance::meshSelfDistance's vertex scan
    (src/Distance.cpp:21-34), exactly: squared distances with the reference's
    operation order over every qualifying pair within a radius that covers
    the minimum (k-d tree neighbour pairs)."""
    spatial = pytest.importorskip("scipy.spatial")
    nv = v.shape[0]
    # incidence, padded: faces of each vertex
    fid = np.repeat(np.arange(f.shape[0]), 3)
    vert = f.ravel()
    order = np.argsort(vert, kind="stable")
    deg = np.bincount(vert, minlength=nv)
    width = int(deg.max())
    pad = np.full((nv, width), -1, np.int64)
    start = np.concatenate([[0], np.cumsum(deg)[:-1]])
    rank = np.arange(vert.size) - start[vert[order]]
    pad[vert[order], rank] = fid[order]

    def qualifying(i, j):  # some face of j misses i
        cand = pad[j]
        fv = f[np.clip(cand, 0, None)]
        return ((cand >= 0) & ~(fv == i[:, None, None]).any(-1)).any(-1)

    def sq(i, j):
        d = v[i] - v[j]
        return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]

    tree = spatial.cKDTree(v)
    _, nb = tree.query(v, k=min(9, nv))
    i = np.repeat(np.arange(nv), nb.shape[1] - 1)
    j = nb[:, 1:].ravel()
    ok = qualifying(i, j)
    upper = sq(i[ok], j[ok]).min()
    pairs = tree.query_pairs(np.sqrt(upper) * (1 + 1e-9) + 1e-300, output_type="ndarray")
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    ok = qualifying(i, j)
    return sq(i[ok], j[ok]).min()


def test_self_distance_full_size_sheet_on_sphere(ctx, oracle):
    f, frames = W.cloth_frames(grid=256, level=6, seed=0, steps=4)
    v = np.ascontiguousarray(frames[3], np.float64).reshape(-1, 3)
    with C.Mesh(ctx, f, nverts=v.shape[0]) as m:
        d, nvf, nee = m.self_distance(v)
        vf, ee = m.candidates()
    # stage 1: the vertex scan
    closest = float(np.sqrt(_vertex_scan_min_sq(v, f)))
    # stage 2: the AABB candidate set at that padding
    ovf, oee = oracle.broadphase(1, v.ravel(), v.ravel(), f, closest)
    np.testing.assert_array_equal(vf, ovf)
    np.testing.assert_array_equal(ee, oee)
    # stage 3: the least stencil distance
    vvec, _ = oracle.distance(0, v[vf].reshape(-1, 12))
    evec, _ = oracle.distance(1, v[ee].reshape(-1, 12))
    norms = [np.sqrt((x[:, 0] * x[:, 0] + x[:, 1] * x[:, 1]) + x[:, 2] * x[:, 2]) for x in (vvec, evec)]
    expect = min(n.min() for n in norms if n.size)
    assert float(d).hex() == float(expect).hex()
    assert (nvf, nee) == (vf.shape[0], ee.shape[0]) and nvf > 0
