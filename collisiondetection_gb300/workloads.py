"""Seeded synthetic workloads for the CTCD path (numpy only).

* ``primitive_batch`` -- raw swept vertex-face / edge-edge quadruples: start
  points uniform in [0,1]^3, end = start + N(0, sigma) per coordinate, with a
  fraction built near-degenerate (coplanar, parallel, tangential double root).
  Rows are laid out in the argument order of the reference's
  ``CTCD::vertexFaceCTCD`` / ``CTCD::edgeEdgeCTCD`` (include/CTCD.h:36-58):
  8 points x 3 coordinates, all start points first, then all end points.
* ``icosphere`` / ``two_spheres`` -- the two-sphere mesh scene (two level-3
  icospheres, centres 2.5 apart, moving 0.8 towards each other with jitter).
* ``grid_sheet`` -- a regular triangulated sheet.

The reference ships no benchmark inputs; these generators stand in for its
example meshes at the sizes and value distributions of the benchmark.
"""
from __future__ import annotations

import numpy as np

KIND_VF, KIND_EE, KIND_VE, KIND_VV = 0, 1, 2, 3
ROW_WIDTH = {KIND_VF: 24, KIND_EE: 24, KIND_VE: 18, KIND_VV: 12}
NPTS = {KIND_VF: 4, KIND_EE: 4, KIND_VE: 3, KIND_VV: 2}


def _unit(v):
    n = np.linalg.norm(v, axis=-1, keepdims=True)
    n[n == 0] = 1.0
    return v / n


def _rows(start, end):
    """(n, k, 3) start/end points -> (n, 6k) rows: starts then ends."""
    n = start.shape[0]
    return np.concatenate([start.reshape(n, -1), end.reshape(n, -1)], axis=1)


def _split(rows, k):
    n = rows.shape[0]
    return rows[:, : 3 * k].reshape(n, k, 3), rows[:, 3 * k:].reshape(n, k, 3)


def _coplanar_vf(s, e, rng):
    # Vertex projected into the face's plane at t=0 and t=1, then offset 1e-9.
    for pts in (s, e):
        n = _unit(np.cross(pts[:, 2] - pts[:, 1], pts[:, 3] - pts[:, 1]))
        d = np.einsum("ij,ij->i", pts[:, 0] - pts[:, 1], n)
        off = 1e-9 * rng.choice([-1.0, 1.0], size=(len(d), 1))
        pts[:, 0] = pts[:, 0] - d[:, None] * n + off * n


def _coplanar_ee(s, e, rng):
    # Second edge projected into a plane through the first edge, offset 1e-9.
    for pts in (s, e):
        e0 = pts[:, 1] - pts[:, 0]
        mid = 0.5 * (pts[:, 2] + pts[:, 3])
        n = _unit(np.cross(e0, mid - pts[:, 0]))
        off = 1e-9 * rng.choice([-1.0, 1.0], size=(len(n), 1))
        for j in (2, 3):
            d = np.einsum("ij,ij->i", pts[:, j] - pts[:, 0], n)
            pts[:, j] = pts[:, j] - d[:, None] * n + off * n


def _parallel_vf(s, e, rng):
    # Face translates rigidly; the vertex starts within 1e-9 of the plane and
    # moves parallel to it (plus 1e-9 noise).
    d = e[:, 1] - s[:, 1]
    e[:, 2] = s[:, 2] + d
    e[:, 3] = s[:, 3] + d
    n = _unit(np.cross(s[:, 2] - s[:, 1], s[:, 3] - s[:, 1]))
    h = np.einsum("ij,ij->i", s[:, 0] - s[:, 1], n)
    s[:, 0] = s[:, 0] - h[:, None] * n + 1e-9 * rng.uniform(-1, 1, size=(len(h), 1)) * n
    w = rng.normal(0.0, 0.1, size=d.shape)
    w = w - np.einsum("ij,ij->i", w, n)[:, None] * n
    e[:, 0] = s[:, 0] + d + w + 1e-9 * rng.normal(size=d.shape)


def _parallel_ee(s, e, rng):
    # Second edge direction = first edge direction + 1e-9 noise, at both ends.
    for pts in (s, e):
        pts[:, 3] = pts[:, 2] + (pts[:, 1] - pts[:, 0]) + 1e-9 * rng.normal(size=pts[:, 0].shape)


def _vf_cubic_jac(s, e, tstar):
    """Value/derivative of the exact VF coplanarity cubic at t* and their
    gradients w.r.t. (vertex start, vertex velocity)."""
    x = [s[:, j] + tstar[:, None] * (e[:, j] - s[:, j]) for j in range(4)]
    v = [e[:, j] - s[:, j] for j in range(4)]
    a, b = x[2] - x[1], x[3] - x[1]
    da, db = v[2] - v[1], v[3] - v[1]
    nrm = np.cross(a, b)
    dn = np.cross(da, b) + np.cross(a, db)
    r = x[0] - x[1]
    f = np.einsum("ij,ij->i", r, nrm)
    fp = np.einsum("ij,ij->i", v[0] - v[1], nrm) + np.einsum("ij,ij->i", r, dn)
    t = tstar[:, None]
    g_f = np.concatenate([nrm, t * nrm], axis=1)
    g_fp = np.concatenate([dn, nrm + t * dn], axis=1)
    return f, fp, g_f, g_fp


def _ee_cubic_jac(s, e, tstar):
    """Same for the EE coplanarity cubic (p0-p1).((p0-q0)x(p1-q1)) w.r.t. the
    start and velocity of q0 (argument 0), in which it is affine."""
    x = [s[:, j] + tstar[:, None] * (e[:, j] - s[:, j]) for j in range(4)]
    v = [e[:, j] - s[:, j] for j in range(4)]
    # argument order q0, p0, q1, p1
    u = x[1] - x[3]
    du = v[1] - v[3]
    w = x[3] - x[2]
    dw = v[3] - v[2]
    c = np.cross(w, u)  # d/dq0 of u.((p0-q0) x w) = -(w x u)... sign folded below
    dc = np.cross(dw, u) + np.cross(w, du)
    z = x[1] - x[0]
    dz = v[1] - v[0]
    f = np.einsum("ij,ij->i", u, np.cross(z, w))
    fp = (np.einsum("ij,ij->i", du, np.cross(z, w)) + np.einsum("ij,ij->i", u, np.cross(dz, w))
          + np.einsum("ij,ij->i", u, np.cross(z, dw)))
    # f = u.(z x w) = z.(w x u) = (p0 - q0).c  ->  df/dq0 = -c
    t = tstar[:, None]
    g_f = np.concatenate([-c, -t * c], axis=1)
    # fp = dz.c + z.dc ; dz depends on q0 velocity (-1), z on q0 position (-1)
    g_fp = np.concatenate([-dc, -c - t * dc], axis=1)
    return f, fp, g_f, g_fp


def _tangent(s, e, rng, jac, idx):
    """Least-norm change to (start, velocity) of point idx so that the
    coplanarity cubic has a double root at a random t* in (0,1)."""
    tstar = rng.uniform(0.0, 1.0, size=s.shape[0])
    for _ in range(3):
        f, fp, g_f, g_fp = jac(s, e, tstar)
        M = np.stack([g_f, g_fp], axis=1)          # (n, 2, 6)
        rhs = -np.stack([f, fp], axis=1)           # (n, 2)
        MMt = M @ np.transpose(M, (0, 2, 1))       # (n, 2, 2)
        det = MMt[:, 0, 0] * MMt[:, 1, 1] - MMt[:, 0, 1] * MMt[:, 1, 0]
        ok = np.abs(det) > 1e-300
        inv = np.zeros_like(MMt)
        inv[ok, 0, 0] = MMt[ok, 1, 1] / det[ok]
        inv[ok, 1, 1] = MMt[ok, 0, 0] / det[ok]
        inv[ok, 0, 1] = -MMt[ok, 0, 1] / det[ok]
        inv[ok, 1, 0] = -MMt[ok, 1, 0] / det[ok]
        lam = np.einsum("nij,nj->ni", inv, rhs)
        delta = np.einsum("nji,nj->ni", M, lam)    # (n, 6)
        vel = e[:, idx] - s[:, idx]
        s[:, idx] = s[:, idx] + delta[:, :3]
        e[:, idx] = s[:, idx] + vel + delta[:, 3:]


def primitive_batch(kind: int, n: int, seed: int, sigma: float = 0.1, degenerate_frac: float = 0.2) -> np.ndarray:
    """(n, ROW_WIDTH[kind]) float64 rows of seeded swept primitives."""
    rng = np.random.default_rng([seed, kind])
    k = NPTS[kind]
    s = rng.uniform(0.0, 1.0, size=(n, k, 3))
    e = s + rng.normal(0.0, sigma, size=(n, k, 3))
    n_deg = int(round(degenerate_frac * n))
    if n_deg and kind in (KIND_VF, KIND_EE):
        sel = rng.permutation(n)[:n_deg]
        parts = np.array_split(sel, 3)
        for which, ids in enumerate(parts):
            if len(ids) == 0:
                continue
            ss, ee = s[ids].copy(), e[ids].copy()
            if which == 0:
                (_coplanar_vf if kind == KIND_VF else _coplanar_ee)(ss, ee, rng)
            elif which == 1:
                (_parallel_vf if kind == KIND_VF else _parallel_ee)(ss, ee, rng)
            else:
                if kind == KIND_VF:
                    _tangent(ss, ee, rng, _vf_cubic_jac, 0)
                else:
                    _tangent(ss, ee, rng, _ee_cubic_jac, 0)
            s[ids], e[ids] = ss, ee
    elif n_deg and kind == KIND_VE:
        ids = rng.permutation(n)[:n_deg]
        # vertex on the edge's line at both ends (plus 1e-9 noise)
        for pts in (s, e):
            a = rng.uniform(-0.5, 1.5, size=(len(ids), 1))
            pts[ids, 0] = pts[ids, 1] + a * (pts[ids, 2] - pts[ids, 1]) + 1e-9 * rng.normal(size=(len(ids), 3))
    elif n_deg and kind == KIND_VV:
        ids = rng.permutation(n)[:n_deg]
        # the two vertices meet (to 1e-9) at a random time
        tstar = rng.uniform(0.0, 1.0, size=(len(ids), 1))
        meet = s[ids, 1] + tstar * (e[ids, 1] - s[ids, 1]) + 1e-9 * rng.normal(size=(len(ids), 3))
        vel = e[ids, 0] - s[ids, 0]
        s[ids, 0] = meet - tstar * vel
        e[ids, 0] = s[ids, 0] + vel
    return np.ascontiguousarray(_rows(s, e))


# ------------------------------------------------------------------ meshes
def icosphere(level: int, radius: float = 1.0):
    """Subdivided icosahedron: (V, 3) float64 vertices, (F, 3) int32 faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    F = faces
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[key] = len(V) - 1
            return cache[key]

        nf = []
        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    return radius * np.array(V, dtype=np.float64), np.array(F, dtype=np.int32)


def two_spheres(seed: int, level: int = 3, radius: float = 1.0, gap: float = 2.5, approach: float = 0.8,
                jitter: float = 0.01):
    """Two icospheres, centres `gap` apart on x, each moving `approach`
    towards the other plus N(0, jitter) per coordinate.  Returns
    (qstart (3V,), qend (3V,), faces (F, 3) int32)."""
    rng = np.random.default_rng(seed)
    v, f = icosphere(level, radius)
    nv = v.shape[0]
    a = v + np.array([-gap / 2, 0.0, 0.0])
    b = v + np.array([gap / 2, 0.0, 0.0])
    start = np.concatenate([a, b])
    faces = np.concatenate([f, f + nv]).astype(np.int32)
    move = np.concatenate([np.tile([approach, 0.0, 0.0], (nv, 1)), np.tile([-approach, 0.0, 0.0], (nv, 1))])
    end = start + move + rng.normal(0.0, jitter, size=start.shape)
    return start.ravel().copy(), end.ravel().copy(), faces


def grid_sheet(nx: int, ny: int, size: float = 1.0):
    """nx*ny vertex grid on [0,size]^2 at z=0: (V, 3) vertices, (F, 3) faces."""
    xs = np.linspace(0.0, size, nx)
    ys = np.linspace(0.0, size, ny)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    v = np.stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)], axis=1)
    idx = np.arange(nx * ny).reshape(ny, nx)
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, :-1].ravel()
    d = idx[1:, 1:].ravel()
    f = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)]).astype(np.int32)
    return v, f


def cloth_frames(grid: int = 256, level: int = 6, seed: int = 0, steps: int = 50, gap: float = 0.05,
                 drop: float = 0.002, wrinkle: float = 0.003, radius: float = 0.4):
    """Cloth-on-sphere sequence: a grid x grid vertex sheet on [0,1]^2 starting
    `gap` above the top of an icosphere (subdivision `level`, centre
    (0.5, 0.5, 0), radius `radius`), in one mesh (sheet vertices first).  Each
    step moves every sheet vertex by dz = -drop + wrinkle * sin(2 pi (kx x +
    ky y) + phase), with (kx, ky, phase) drawn per step from the seed; the
    sphere is static.  Returns (faces (F, 3) int32, frames (steps + 1, 3V)):
    step k goes from frames[k] to frames[k + 1]."""
    sv, sf = grid_sheet(grid, grid)
    cv, cf = icosphere(level, radius)
    cv = cv + np.array([0.5, 0.5, 0.0])
    sv = sv + np.array([0.0, 0.0, radius + gap])
    rng = np.random.default_rng(seed)
    x, y = sv[:, 0], sv[:, 1]
    nv = sv.shape[0] + cv.shape[0]
    frames = np.empty((steps + 1, 3 * nv))
    z = sv[:, 2].copy()
    for k in range(steps + 1):
        frames[k] = np.concatenate([np.stack([x, y, z], 1), cv]).ravel()
        if k < steps:
            kx, ky = rng.uniform(1.0, 4.0, 2)
            phase = rng.uniform(0.0, 2 * np.pi)
            z = z - drop + wrinkle * np.sin(2 * np.pi * (kx * x + ky * y) + phase)
    faces = np.concatenate([sf, cf + sv.shape[0]]).astype(np.int32)
    return faces, frames


def sheet_on_sphere(grid: int = 256, level: int = 6, seed: int = 0, step: int = 0, gap: float = 0.05,
                    drop: float = 0.002, wrinkle: float = 0.003, radius: float = 0.4):
    """Step `step` of cloth_frames(...): (qstart (3V,), qend (3V,), faces)."""
    faces, frames = cloth_frames(grid, level, seed, step + 1, gap, drop, wrinkle, radius)
    return frames[step].copy(), frames[step + 1].copy(), faces


_ICO_CACHE = {}


def _icosphere_cached(level: int):
    if level not in _ICO_CACHE:
        _ICO_CACHE[level] = icosphere(level, 1.0)
    return _ICO_CACHE[level]


def _mean_edge(v, f):
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    return float(np.linalg.norm(v[e[:, 0]] - v[e[:, 1]], axis=1).mean())


def motion_request(tris: int, seed: int, steps: int = 10):
    """One collision query of the uneven-batch / serving workloads: an
    icosphere (subdivision level nearest to `tris` triangles) or a pair of
    grid sheets two edge lengths apart, moved each step by a rigid translation
    of 0.5-2 mean edge lengths in a random direction plus N(0, 0.1 edge)
    per-vertex jitter.  Returns (faces (F, 3) int32, frames (steps + 1, 3V))."""
    rng = np.random.default_rng(seed)
    if rng.random() < 0.5:
        level = int(np.clip(np.rint(np.log(max(tris, 20) / 20.0) / np.log(4.0)), 1, 7))
        v, f = _icosphere_cached(level)
    else:
        n = int(max(3, np.rint(np.sqrt(max(tris, 8) / 4.0) + 1)))
        a, fa = grid_sheet(n, n)
        edge = 1.0 / (n - 1)
        b = a + np.array([0.3 * edge, 0.3 * edge, 2.0 * edge])
        v = np.concatenate([a, b])
        f = np.concatenate([fa, fa + a.shape[0]]).astype(np.int32)
    edge = _mean_edge(v, f)
    frames = np.empty((steps + 1, v.size))
    pos = v.copy()
    frames[0] = pos.ravel()
    for k in range(steps):
        d = rng.normal(size=3)
        d *= rng.uniform(0.5, 2.0) * edge / np.linalg.norm(d)
        pos = pos + d
        frames[k + 1] = (pos + rng.normal(0.0, 0.1 * edge, pos.shape)).ravel()
    return np.ascontiguousarray(f, dtype=np.int32), frames


def pair_request(tris: int, seed: int, steps: int = 10, contact_step: float = 0.5):
    """One collision query of the serving workload: a mesh pair -- two
    icospheres side by side, or two grid sheets one above the other -- of
    about `tris` triangles together, a gap of three mean edge lengths apart.
    Each step moves the pair by a rigid translation of 0.5-2 mean edge lengths
    in a random direction, closes the gap by a constant amount so that the
    two meshes first touch about `contact_step` of the way through the
    sequence (and then pass into each other), and adds N(0, 0.1 edge)
    per-vertex jitter.  Returns (faces (F, 3) int32, frames (steps + 1, 3V))."""
    rng = np.random.default_rng(seed)
    if rng.random() < 0.5:
        level = int(np.clip(np.rint(np.log(max(tris / 2, 20) / 20.0) / np.log(4.0)), 1, 7))
        a, fa = _icosphere_cached(level)
        edge = _mean_edge(a, fa)
        gap = 3.0 * edge
        axis = np.array([1.0, 0.0, 0.0])
        b = a + (2.0 + gap) * axis
    else:
        n = int(max(3, np.rint(np.sqrt(max(tris / 2, 8) / 2.0) + 1)))
        a, fa = grid_sheet(n, n)
        edge = 1.0 / (n - 1)
        gap = 3.0 * edge
        axis = np.array([0.0, 0.0, 1.0])
        b = a + np.array([0.3 * edge, 0.3 * edge, gap])
    v = np.concatenate([a, b])
    f = np.concatenate([fa, fa + a.shape[0]]).astype(np.int32)
    close = gap / max(contact_step * steps, 1e-9)  # gap closed per step
    frames = np.empty((steps + 1, v.size))
    pos = v.copy()
    frames[0] = pos.ravel()
    nb = b.shape[0]
    for k in range(steps):
        d = rng.normal(size=3)
        d *= rng.uniform(0.5, 2.0) * edge / np.linalg.norm(d)
        pos = pos + d
        pos[-nb:] -= close * axis
        frames[k + 1] = (pos + rng.normal(0.0, 0.1 * edge, pos.shape)).ravel()
    return np.ascontiguousarray(f, dtype=np.int32), frames


def uneven_sizes(n_instances: int = 512, lo: float = 200.0, hi: float = 2e5, seed: int = 0) -> np.ndarray:
    """Requested triangle counts of an uneven batch: log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n_instances)).astype(int)


def uneven_batch(n_instances: int = 512, lo: float = 200.0, hi: float = 2e5, seed: int = 0, steps: int = 1,
                 select=None):
    """Uneven batch of independent collision queries: `n_instances` motion
    requests (motion_request) with triangle counts log-uniform in [lo, hi],
    concatenated.  `select` (optional) keeps only the instances with those
    indices, each exactly as in the whole batch.  Returns (faces (F, 3) int32
    with global vertex indices, frames (steps + 1, 3V), vertex_offsets,
    face_offsets)."""
    sizes = uneven_sizes(n_instances, lo, hi, seed)
    faces, frames, vo, fo = [], [], [0], [0]
    for i in (range(n_instances) if select is None else select):
        f, fr = motion_request(int(sizes[i]), 100000 + seed * 10000 + i, steps=steps)
        faces.append(f + vo[-1])
        frames.append(fr.reshape(steps + 1, -1, 3))
        vo.append(vo[-1] + fr.shape[1] // 3)
        fo.append(fo[-1] + f.shape[0])
    return (np.ascontiguousarray(np.concatenate(faces), dtype=np.int32),
            np.ascontiguousarray(np.concatenate(frames, axis=1).reshape(steps + 1, -1)),
            np.array(vo, np.int32), np.array(fo, np.int32))


def multi_entry_history(q0, q1, seed: int, active: float = 0.3, max_entries: int = 6, jitter: float = 0.02,
                        pool: int = 16):
    """A History with extra entries between its start (t = 0, q0) and end
    (t = 1, q1), shaped like the ones the active-layers loop leaves: a
    fraction `active` of the vertices gets 1..max_entries intermediate
    entries at times drawn from a shared pool (so that vertices share entry
    times, as the vertices of one penalty group do), at the straight-line
    position plus N(0, jitter) noise.  Returns (offsets [V+1] int32, times [E],
    positions [E][3])."""
    rng = np.random.default_rng(seed)
    q0 = np.asarray(q0, np.float64).reshape(-1, 3)
    q1 = np.asarray(q1, np.float64).reshape(-1, 3)
    nv = q0.shape[0]
    times_pool = np.sort(rng.uniform(0.02, 0.98, pool))
    offsets = np.zeros(nv + 1, np.int32)
    times, positions = [], []
    for v in range(nv):
        ts = [0.0]
        if rng.random() < active:
            k = int(rng.integers(1, max_entries + 1))
            ts += sorted(rng.choice(times_pool, size=min(k, pool), replace=False).tolist())
        ts.append(1.0)
        for t in ts:
            p = (1.0 - t) * q0[v] + t * q1[v]
            if 0.0 < t < 1.0:
                p = p + rng.normal(0.0, jitter, 3)
            elif t == 1.0:
                p = q1[v]
            else:
                p = q0[v]
            times.append(t)
            positions.append(p)
        offsets[v + 1] = offsets[v] + len(ts)
    return offsets, np.array(times, np.float64), np.array(positions, np.float64)
