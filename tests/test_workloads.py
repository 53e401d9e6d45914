"""The synthetic workload generators (collisiondetection_gb300/workloads.py)
build the benchmark scenes at their stated shapes, sizes and distributions.
CPU only: these are host-side inputs of the bench and the GPU tests."""
import numpy as np
import pytest

from collisiondetection_gb300 import workloads as W


def _edges(f):
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    return np.unique(e, axis=0, return_counts=True)


@pytest.mark.parametrize("level,nv,nf", [(3, 642, 1280), (6, 40962, 81920)])
def test_icosphere_sizes_and_closed_surface(level, nv, nf):
    v, f = W.icosphere(level, radius=0.4)
    assert v.shape == (nv, 3) and f.shape == (nf, 3) and f.dtype == np.int32
    assert np.allclose(np.linalg.norm(v, axis=1), 0.4, rtol=0, atol=1e-12)
    e, counts = _edges(f)
    assert np.all(counts == 2)  # every edge borders two faces: a closed 2-manifold
    assert nv - e.shape[0] + nf == 2  # Euler characteristic of a sphere


def test_grid_sheet_sizes_and_spacing():
    v, f = W.grid_sheet(256, 256)
    assert v.shape == (65536, 3) and f.shape == (130050, 3)
    e, counts = _edges(f)
    lengths = np.linalg.norm(v[e[:, 0]] - v[e[:, 1]], axis=1)
    h = 1.0 / 255
    # axis-aligned edges of length 1/255 and one diagonal per cell
    assert np.allclose(np.sort(np.unique(np.round(lengths / h, 9))), [1.0, np.round(np.sqrt(2.0), 9)])
    assert counts.max() == 2


def test_two_spheres_scene():
    q0, q1, f = W.two_spheres(seed=1)
    v0, v1 = q0.reshape(-1, 3), q1.reshape(-1, 3)
    assert v0.shape == (1284, 3) and f.shape == (2560, 3)
    assert f[:1280].max() < 642 and f[1280:].min() >= 642
    c0, c1 = v0[:642].mean(0), v0[642:].mean(0)
    assert np.allclose(c1 - c0, [2.5, 0.0, 0.0], atol=1e-12)
    d = v1 - v0
    assert np.allclose(d[:642].mean(0), [0.8, 0, 0], atol=3e-3)
    assert np.allclose(d[642:].mean(0), [-0.8, 0, 0], atol=3e-3)
    jitter = d - np.where(np.arange(1284)[:, None] < 642, [0.8, 0, 0], [-0.8, 0, 0])
    assert 0.009 < jitter.std() < 0.011
    assert np.array_equal(q1, W.two_spheres(seed=1)[1])  # seeded


def test_cloth_on_sphere_scene():
    f, frames = W.cloth_frames(grid=256, level=6, seed=0, steps=2)
    assert f.shape == (211970, 3) and frames.shape == (3, 3 * 106498)
    x = frames.reshape(3, -1, 3)
    sheet, sphere = x[:, :65536], x[:, 65536:]
    assert np.isclose(sheet[0, :, 2].min() - sphere[0, :, 2].max(), 0.05, atol=1e-12)
    assert np.array_equal(sphere[0], sphere[2])  # the sphere is static
    dz = sheet[1, :, 2] - sheet[0, :, 2]
    assert dz.min() >= -0.005 - 1e-15 and dz.max() <= 0.001 + 1e-15
    assert np.isclose(dz.mean(), -0.002, atol=5e-4)
    assert np.array_equal(sheet[1, :, :2], sheet[0, :, :2])  # only z moves


def _coplanarity(rows, kind, t):
    n = rows.shape[0]
    s, e = rows[:, :12].reshape(n, 4, 3), rows[:, 12:].reshape(n, 4, 3)
    x = s + t * (e - s)
    if kind == W.KIND_VF:
        return np.einsum("ij,ij->i", x[:, 0] - x[:, 1], np.cross(x[:, 2] - x[:, 1], x[:, 3] - x[:, 1]))
    return np.einsum("ij,ij->i", x[:, 2] - x[:, 0], np.cross(x[:, 1] - x[:, 0], x[:, 3] - x[:, 2]))


@pytest.mark.parametrize("kind", [W.KIND_VF, W.KIND_EE])
def test_primitive_batch_distribution_and_degenerate_fifth(kind):
    n = 30000
    rows = W.primitive_batch(kind, n, seed=3)
    assert rows.shape == (n, 24) and rows.dtype == np.float64 and rows.flags.c_contiguous
    assert np.array_equal(rows, W.primitive_batch(kind, n, seed=3))
    assert not np.array_equal(rows, W.primitive_batch(kind, n, seed=4))
    # coplanar and parallel rows: within 1e-8 of coplanar at both ends (2/3 of 20%)
    ts = np.array([0.0, 1 / 3, 2 / 3, 1.0])
    vals = np.stack([_coplanarity(rows, kind, t) for t in ts], 1)
    flat = (np.abs(vals[:, 0]) < 1e-8) & (np.abs(vals[:, 3]) < 1e-8)
    assert abs(int(flat.sum()) - 2 * n // 15) <= 3
    # tangential rows: the coplanarity cubic has a double root in [0, 1] (1/3 of 20%)
    co = np.linalg.solve(np.vander(ts, 4), vals.T).T
    a, b, c, d = co.T
    disc = 4 * b * b - 12 * a * c
    scale = np.abs(co).max(1)
    double = np.zeros(n, bool)
    for sgn in (-1.0, 1.0):
        with np.errstate(all="ignore"):
            tc = (-2 * b + sgn * np.sqrt(np.maximum(disc, 0))) / (6 * a)
        fv = ((a * tc + b) * tc + c) * tc + d
        double |= (disc >= 0) & (tc >= 0) & (tc <= 1) & (np.abs(fv) < 1e-9 * scale)
    assert abs(int((double & ~flat).sum()) - n // 15) <= 3
    # the other 80%: start uniform in [0,1]^3, end = start + N(0, 0.1)
    rest = rows[~flat & ~double]
    assert rest[:, :12].min() >= 0.0 and rest[:, :12].max() <= 1.0
    assert abs(np.std(rest[:, 12:] - rest[:, :12]) - 0.1) < 2e-3


def test_motion_request_moves_rigidly_by_half_to_two_edges():
    for seed in range(6):
        f, frames = W.motion_request(5000, seed=seed, steps=4)
        v = frames.reshape(5, -1, 3)
        assert f.min() >= 0 and f.max() < v.shape[1]
        edge = W._mean_edge(v[0], f)
        for k in range(4):
            step = np.linalg.norm((v[k + 1] - v[k]).mean(0))
            assert 0.45 * edge < step < 2.1 * edge


def test_pair_request_meshes_meet_halfway():
    for seed in range(6):
        f, frames = W.pair_request(4000, seed=seed, steps=10)
        v = frames.reshape(11, -1, 3)
        nf = f.shape[0]
        assert 1500 <= nf <= 20000 and f.min() >= 0 and f.max() < v.shape[1]
        half = v.shape[1] // 2
        # the second mesh closes in on the first at a constant rate
        d0 = (v[0, half:] - v[0, :half]).mean(0)
        d0 /= np.linalg.norm(d0)
        gaps = [float((v[k, half:] - v[k, :half]).mean(0) @ d0) for k in range(11)]
        steps = np.diff(gaps)
        assert np.all(steps < 0) and np.ptp(steps) < 0.2 * abs(steps.mean())


def test_uneven_batch_offsets_and_sizes():
    faces, frames, vo, fo = W.uneven_batch(n_instances=12, lo=200, hi=5000, seed=2, steps=1)
    assert vo[0] == 0 and fo[0] == 0 and np.all(np.diff(vo) > 0) and np.all(np.diff(fo) > 0)
    assert vo[-1] * 3 == frames.shape[1] and fo[-1] == faces.shape[0]
    want = W.uneven_sizes(12, 200, 5000, seed=2)
    for i in range(12):
        fi = faces[fo[i]:fo[i + 1]]
        # an icosphere of the nearest level or two sheets of about that many faces
        assert want[i] / 4.5 < fi.shape[0] < want[i] * 4.5
        assert fi.min() >= vo[i] and fi.max() < vo[i + 1]  # instances share no vertex
    # the full configuration's triangle counts: log-uniform in [200, 2e5], about 15M in total
    sizes = W.uneven_sizes(512, 200.0, 2e5, seed=0)
    assert sizes.min() >= 200 and sizes.max() <= 200000 and 12e6 < sizes.sum() < 18e6


def test_multi_entry_history_shape():
    q0 = np.random.default_rng(0).uniform(size=(50, 3))
    q1 = q0 + 0.1
    off, times, pos = W.multi_entry_history(q0, q1, seed=5)
    assert off[0] == 0 and off[-1] == times.size == pos.shape[0]
    for v in range(50):
        t = times[off[v]:off[v + 1]]
        assert t[0] == 0.0 and t[-1] == 1.0 and np.all(np.diff(t) > 0)
        assert np.array_equal(pos[off[v]], q0[v]) and np.array_equal(pos[off[v + 1] - 1], q1[v])
    assert (np.diff(off) > 2).any()
