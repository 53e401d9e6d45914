"""ORACLE / TEST INFRASTRUCTURE ONLY.

ctypes loader for the C restatement (oracle/_build/libccd_oracle.so) and, where
it was built, the reference compiled from its own sources
(oracle/_ref/libccd_ref.so).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module, and only to check results.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libccd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libccd_ref.so")
FLOPS_SO = os.path.join(HERE, "_build", "libccd_flops.so")

_P = ctypes.c_void_p
_I64 = ctypes.c_int64


def build(ref: bool = False) -> None:
    """Compile the C restatement (and the reference, when asked and present)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


class _Lib:
    def __init__(self, path: str, prefix: str):
        self.lib = ctypes.CDLL(path)
        self.prefix = prefix
        L = self.lib
        for k in ("vf", "ee", "ve", "vv"):
            fn = getattr(L, f"{prefix}_{k}")
            fn.argtypes = [_P, ctypes.c_double, _P]
            fn.restype = ctypes.c_int

    def _distance_setup(self):
        L, pre = self.lib, self.prefix
        getattr(L, f"{pre}_distance_batch").argtypes = [ctypes.c_int, _I64, _P, _P, _P]
        getattr(L, f"{pre}_distance_less_than").argtypes = [ctypes.c_int, _I64, _P, _P, ctypes.c_int, _P]
        fn = getattr(L, f"{pre}_penalty_group_force")
        fn.argtypes = [ctypes.c_int, _P, _P, _I64, _P, _P, _I64, _P, _P] + [ctypes.c_double] * 5 + [_P, _P, _P]
        fn.restype = ctypes.c_int

    def penalty_group_force(self, q, v, F, vf, ee, outer_eta, inner_eta, stiffness, cor, dt, vf_isnew=None,
                            ee_isnew=None):
        """PenaltyGroup::addForce; returns (F_out, vf_fired, ee_fired, newused)."""
        q = np.ascontiguousarray(q, dtype=np.float64).ravel()
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        Fo = np.ascontiguousarray(F, dtype=np.float64).ravel().copy()
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vn = None if vf_isnew is None else np.ascontiguousarray(vf_isnew, dtype=np.uint8)
        en = None if ee_isnew is None else np.ascontiguousarray(ee_isnew, dtype=np.uint8)
        vfire = np.zeros(vf.shape[0], np.uint8)
        efire = np.zeros(ee.shape[0], np.uint8)
        fn = getattr(self.lib, f"{self.prefix}_penalty_group_force")
        used = fn(q.size // 3, _ptr(q), _ptr(v), vf.shape[0], _ptr(vf), _ptr(vn), ee.shape[0], _ptr(ee), _ptr(en),
                  outer_eta, inner_eta, stiffness, cor, dt, _ptr(Fo), _ptr(vfire), _ptr(efire))
        if used < 0:
            raise MemoryError("penalty_group_force failed")
        return Fo, vfire, efire, bool(used)

    def distance(self, kind: int, rows):
        """Distance::vertexFaceDistance (0) / edgeEdgeDistance (1) per row of
        12 doubles; returns (vec [n][3], bary [n][3|4])."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 12)
        n = rows.shape[0]
        vec = np.zeros((n, 3))
        bary = np.zeros((n, 3 if kind == 0 else 4))
        getattr(self.lib, f"{self.prefix}_distance_batch")(kind, n, _ptr(rows), _ptr(vec), _ptr(bary))
        return vec, bary

    def distance_less_than(self, kind: int, rows, eta):
        """vertexPlaneDistanceLessThan (0) / lineLineDistanceLessThan (1)."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 12)
        n = rows.shape[0]
        eta_a = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        per = 1 if eta_a.size == n and n != 1 else 0
        out = np.zeros(n, np.uint8)
        getattr(self.lib, f"{self.prefix}_distance_less_than")(kind, n, _ptr(rows), _ptr(eta_a), per, _ptr(out))
        return out

    def prim(self, kind: str, x, eta: float):
        """One primitive test; returns (hit, t or None)."""
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        t = ctypes.c_double(np.nan)
        h = getattr(self.lib, f"{self.prefix}_{kind}")(_ptr(x), eta, ctypes.byref(t))
        return int(h), (t.value if h else None)


class Oracle(_Lib):
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        super().__init__(path, "oracle")
        L = self.lib
        L.oracle_batch.argtypes = [ctypes.c_int, _I64, _P, _P, ctypes.c_int, _P, _P, ctypes.c_int]
        L.oracle_broadphase.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P, ctypes.c_double, _P,
                                        _P, _P]
        L.oracle_broadphase.restype = ctypes.c_int
        L.oracle_broadphase_get.argtypes = [_P, _P]
        L.oracle_broadphase_face_pairs.restype = ctypes.c_int64
        L.oracle_narrowphase.argtypes = [ctypes.c_int, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _P,
                                         ctypes.c_int]
        L.oracle_mesh_self_distance.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, _P, _P, _P]
        L.oracle_mesh_self_distance.restype = ctypes.c_double
        L.oracle_vertex_scan.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_int]
        L.oracle_vertex_scan.restype = ctypes.c_double
        L.oracle_broadphase_history.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P,
                                                ctypes.c_double, _P, _P, _P]
        L.oracle_broadphase_history.restype = ctypes.c_int
        L.oracle_narrowphase_history.argtypes = [ctypes.c_int, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P, _P,
                                                 _P, _P, _P]
        L.oracle_narrowphase_history.restype = ctypes.c_int
        L.oracle_separating_plane.argtypes = [ctypes.c_int, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P]
        L.oracle_separating_plane.restype = ctypes.c_int64
        L.oracle_velocity_filter.argtypes = [ctypes.c_int, _P, _P, ctypes.c_int, _P, _P] + [ctypes.c_double] * 5 + \
            [ctypes.c_int, _P]
        L.oracle_velocity_filter.restype = ctypes.c_int
        self._distance_setup()

    def broadphase_history(self, kind: int, offsets, times, positions, faces, eta: float, fixed=None):
        """The broad phase on a multi-entry history (slabs over every entry)."""
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        nvf, nee = ctypes.c_int64(), ctypes.c_int64()
        rc = self.lib.oracle_broadphase_history(kind, off.size - 1, _ptr(off), _ptr(pos), faces.shape[0],
                                                _ptr(faces), eta, _ptr(fx), ctypes.byref(nvf), ctypes.byref(nee))
        if rc != 0:
            raise MemoryError("oracle_broadphase_history failed")
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        self.lib.oracle_broadphase_get(_ptr(vf), _ptr(ee))
        return vf, ee

    def narrowphase_history(self, offsets, times, positions, vf, vf_eta, ee, ee_eta):
        """CTCDNarrowPhase on a multi-entry history: dict of hit / t / which."""
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tt = np.ascontiguousarray(times, dtype=np.float64)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        out = {"vf_hit": np.zeros(vf.shape[0], np.uint8), "ee_hit": np.zeros(ee.shape[0], np.uint8),
               "vf_t": np.full(vf.shape[0], np.nan), "ee_t": np.full(ee.shape[0], np.nan),
               "vf_which": np.zeros(vf.shape[0], np.int8), "ee_which": np.zeros(ee.shape[0], np.int8)}
        rc = self.lib.oracle_narrowphase_history(off.size - 1, _ptr(off), _ptr(tt), _ptr(pos), vf.shape[0], _ptr(vf),
                                                 _ptr(vfe), ee.shape[0], _ptr(ee), _ptr(eee), _ptr(out["vf_hit"]),
                                                 _ptr(out["ee_hit"]), _ptr(out["vf_t"]), _ptr(out["ee_t"]),
                                                 _ptr(out["vf_which"]), _ptr(out["ee_which"]))
        if rc != 0:
            raise MemoryError("oracle_narrowphase_history failed")
        return out

    def separating_plane(self, offsets, times, positions, vf, vf_eta, ee, ee_eta):
        """SeparatingPlaneNarrowPhase on a multi-entry history: (vf_hit,
        ee_hit, vf_status, ee_status); status 1 marks a stalled recursion."""
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tt = np.ascontiguousarray(times, dtype=np.float64)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        vh = np.zeros(vf.shape[0], np.uint8)
        eh = np.zeros(ee.shape[0], np.uint8)
        vs = np.zeros(vf.shape[0], np.uint8)
        es = np.zeros(ee.shape[0], np.uint8)
        self.lib.oracle_separating_plane(off.size - 1, _ptr(off), _ptr(tt), _ptr(pos), vf.shape[0], _ptr(vf),
                                         _ptr(vfe), ee.shape[0], _ptr(ee), _ptr(eee), _ptr(vh), _ptr(eh), _ptr(vs),
                                         _ptr(es))
        return vh, eh, vs, es

    def velocity_filter(self, qstart, qend, faces, invmasses, outer_eta, inner_eta, base_stiffness=1e-4,
                        base_substep=1e-4, cor=0.1, max_rollbacks=1000):
        """VelocityFilter::velocityFilter: (return value, filtered qend, events)."""
        qs = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qe = np.ascontiguousarray(qend, dtype=np.float64).ravel().copy()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        mi = np.ascontiguousarray(invmasses, dtype=np.float64).ravel()
        ev = ctypes.c_int64(0)
        r = self.lib.oracle_velocity_filter(qs.size // 3, _ptr(qs), _ptr(qe), faces.shape[0], _ptr(faces), _ptr(mi),
                                            outer_eta, inner_eta, base_stiffness, base_substep, cor, max_rollbacks,
                                            ctypes.byref(ev))
        return int(r), qe, int(ev.value)

    def vertex_scan(self, verts, faces, i0: int, i1: int) -> float:
        """meshSelfDistance's O(V F) vertex scan over vertices [i0, i1)."""
        verts = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        return float(self.lib.oracle_vertex_scan(verts.size // 3, _ptr(verts), faces.shape[0], _ptr(faces), i0, i1))

    def mesh_self_distance(self, verts, faces, fixed=None):
        """Distance::meshSelfDistance; returns (distance, n_vf, n_ee)."""
        verts = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        nvf, nee = ctypes.c_int64(), ctypes.c_int64()
        d = self.lib.oracle_mesh_self_distance(verts.size // 3, _ptr(verts), faces.shape[0], _ptr(faces), _ptr(fx),
                                               ctypes.byref(nvf), ctypes.byref(nee))
        return float(d), int(nvf.value), int(nee.value)

    def batch(self, kind: int, x, eta, nthreads: int = 1):
        """kind 0..3 (VF, EE, VE, VV); eta scalar or per-row.  Returns
        (hit uint8[n], t float64[n]) with t NaN where there is no hit."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.shape[0]
        eta_a = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        per = 1 if eta_a.size == n and n != 1 else 0
        hit = np.zeros(n, np.uint8)
        t = np.full(n, np.nan)
        self.lib.oracle_batch(kind, n, _ptr(x), _ptr(eta_a), per, _ptr(hit), _ptr(t), nthreads)
        return hit, t

    def broadphase(self, kind: int, qstart, qend, faces, eta: float, fixed=None):
        qstart = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qend = np.ascontiguousarray(qend, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        nvf, nee = ctypes.c_int64(), ctypes.c_int64()
        rc = self.lib.oracle_broadphase(kind, qstart.size // 3, _ptr(qstart), _ptr(qend), faces.shape[0], _ptr(faces),
                                        eta, _ptr(fx), ctypes.byref(nvf), ctypes.byref(nee))
        if rc != 0:
            raise MemoryError("oracle_broadphase failed")
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        self.lib.oracle_broadphase_get(_ptr(vf), _ptr(ee))
        return vf, ee

    def face_pairs(self) -> int:
        return int(self.lib.oracle_broadphase_face_pairs())

    def narrowphase(self, qstart, qend, vf, vf_eta, ee, ee_eta, nthreads: int = 1):
        qstart = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qend = np.ascontiguousarray(qend, dtype=np.float64).ravel()
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        out = {
            "vf_hit": np.zeros(vf.shape[0], np.uint8), "ee_hit": np.zeros(ee.shape[0], np.uint8),
            "vf_t": np.full(vf.shape[0], np.nan), "ee_t": np.full(ee.shape[0], np.nan),
            "vf_which": np.zeros(vf.shape[0], np.int8), "ee_which": np.zeros(ee.shape[0], np.int8),
        }
        self.lib.oracle_narrowphase(qstart.size // 3, _ptr(qstart), _ptr(qend), vf.shape[0], _ptr(vf), _ptr(vfe),
                                    ee.shape[0], _ptr(ee), _ptr(eee), _ptr(out["vf_hit"]), _ptr(out["ee_hit"]),
                                    _ptr(out["vf_t"]), _ptr(out["ee_t"]), _ptr(out["vf_which"]),
                                    _ptr(out["ee_which"]), nthreads)
        return out


class FlopCounter:
    """The oracle's primitive tests over a counting scalar (oracle/flops.cpp):
    per row, the floating-point operations the reference's op sequence
    performs for that test (src/CTCD.cpp, src/rpoly.h)."""

    CATEGORIES = ("add", "mul", "div", "sqrt", "cmp", "transcendental")

    def __init__(self, path: str = FLOPS_SO):
        self.lib = ctypes.CDLL(path)
        self.lib.oracle_flops_batch.argtypes = [ctypes.c_int, _I64, _P, _P, ctypes.c_int, _P, _P, _P, _P,
                                                ctypes.c_int]
        self.lib.oracle_flops_batch.restype = None

    def batch(self, kind: int, x, eta, nthreads: int = 1):
        """Returns (hit uint8[n], t float64[n] (NaN where no hit), flops
        uint32[n] (add + mul + div + sqrt per row), totals dict)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.shape[0]
        eta_a = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        per = 1 if eta_a.size == n and n != 1 else 0
        hit = np.zeros(n, np.uint8)
        t = np.full(n, np.nan)
        flops = np.zeros(n, np.uint32)
        totals = np.zeros(6, np.uint64)
        self.lib.oracle_flops_batch(kind, n, _ptr(x), _ptr(eta_a), per, _ptr(hit), _ptr(t), _ptr(flops),
                                    _ptr(totals), nthreads)
        return hit, t, flops, {k: int(v) for k, v in zip(self.CATEGORIES, totals)}


class Reference(_Lib):
    """The reference's own compiled sources (development container only)."""

    def __init__(self, path: str = REF_SO):
        super().__init__(path, "ref")
        L = self.lib
        L.ref_batch.argtypes = [ctypes.c_int, _I64, _P, _P, ctypes.c_int, _P, _P]
        L.ref_broadphase.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P, ctypes.c_double, _P, _P,
                                     _P]
        L.ref_broadphase_get.argtypes = [_P, _P]
        L.ref_narrowphase.argtypes = [ctypes.c_int, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P]
        L.ref_mesh_self_distance.argtypes = [ctypes.c_int, _P, ctypes.c_int, _P, _P]
        L.ref_mesh_self_distance.restype = ctypes.c_double
        L.ref_broadphase_history.argtypes = [ctypes.c_int, ctypes.c_int, _P, _P, _P, ctypes.c_int, _P,
                                             ctypes.c_double, _P, _P, _P]
        L.ref_narrowphase_history.argtypes = [ctypes.c_int, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P]
        L.ref_separating_plane.argtypes = [ctypes.c_int, _P, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _P]
        L.ref_velocity_filter.argtypes = [ctypes.c_int, _P, _P, ctypes.c_int, _P, _P] + [ctypes.c_double] * 5 + \
            [ctypes.c_int]
        L.ref_velocity_filter.restype = ctypes.c_int
        self._distance_setup()

    def broadphase_history(self, kind: int, offsets, times, positions, faces, eta: float, fixed=None):
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tt = np.ascontiguousarray(times, dtype=np.float64)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        nvf, nee = ctypes.c_int64(), ctypes.c_int64()
        self.lib.ref_broadphase_history(kind, off.size - 1, _ptr(off), _ptr(tt), _ptr(pos), faces.shape[0],
                                        _ptr(faces), eta, _ptr(fx), ctypes.byref(nvf), ctypes.byref(nee))
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        self.lib.ref_broadphase_get(_ptr(vf), _ptr(ee))
        return vf, ee

    def narrowphase_history(self, offsets, times, positions, vf, vf_eta, ee, ee_eta):
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tt = np.ascontiguousarray(times, dtype=np.float64)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        vh = np.zeros(vf.shape[0], np.uint8)
        eh = np.zeros(ee.shape[0], np.uint8)
        self.lib.ref_narrowphase_history(off.size - 1, _ptr(off), _ptr(tt), _ptr(pos), vf.shape[0], _ptr(vf),
                                         _ptr(vfe), ee.shape[0], _ptr(ee), _ptr(eee), _ptr(vh), _ptr(eh))
        return vh, eh

    def separating_plane(self, offsets, times, positions, vf, vf_eta, ee, ee_eta):
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        tt = np.ascontiguousarray(times, dtype=np.float64)
        pos = np.ascontiguousarray(positions, dtype=np.float64)
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        vh = np.zeros(vf.shape[0], np.uint8)
        eh = np.zeros(ee.shape[0], np.uint8)
        self.lib.ref_separating_plane(off.size - 1, _ptr(off), _ptr(tt), _ptr(pos), vf.shape[0], _ptr(vf), _ptr(vfe),
                                      ee.shape[0], _ptr(ee), _ptr(eee), _ptr(vh), _ptr(eh))
        return vh, eh

    def velocity_filter(self, qstart, qend, faces, invmasses, outer_eta, inner_eta, base_stiffness=1e-4,
                        base_substep=1e-4, cor=0.1, max_rollbacks=1000):
        """VelocityFilter::velocityFilter: (return value, filtered qend)."""
        qs = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qe = np.ascontiguousarray(qend, dtype=np.float64).ravel().copy()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        mi = np.ascontiguousarray(invmasses, dtype=np.float64).ravel()
        r = self.lib.ref_velocity_filter(qs.size // 3, _ptr(qs), _ptr(qe), faces.shape[0], _ptr(faces), _ptr(mi),
                                         outer_eta, inner_eta, base_stiffness, base_substep, cor, max_rollbacks)
        return int(r), qe

    def mesh_self_distance(self, verts, faces, fixed=None) -> float:
        verts = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        return float(self.lib.ref_mesh_self_distance(verts.size // 3, _ptr(verts), faces.shape[0], _ptr(faces),
                                                     _ptr(fx)))

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO)

    def batch(self, kind: int, x, eta):
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = x.shape[0]
        eta_a = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        per = 1 if eta_a.size == n and n != 1 else 0
        hit = np.zeros(n, np.uint8)
        t = np.full(n, np.nan)
        self.lib.ref_batch(kind, n, _ptr(x), _ptr(eta_a), per, _ptr(hit), _ptr(t))
        return hit, t

    def broadphase(self, kind: int, qstart, qend, faces, eta: float, fixed=None):
        qstart = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qend = np.ascontiguousarray(qend, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        nvf, nee = ctypes.c_int64(), ctypes.c_int64()
        self.lib.ref_broadphase(kind, qstart.size // 3, _ptr(qstart), _ptr(qend), faces.shape[0], _ptr(faces), eta,
                                _ptr(fx), ctypes.byref(nvf), ctypes.byref(nee))
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        self.lib.ref_broadphase_get(_ptr(vf), _ptr(ee))
        return vf, ee

    def narrowphase(self, qstart, qend, vf, vf_eta, ee, ee_eta):
        qstart = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qend = np.ascontiguousarray(qend, dtype=np.float64).ravel()
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vfe = np.ascontiguousarray(np.broadcast_to(np.asarray(vf_eta, np.float64), (vf.shape[0],)))
        eee = np.ascontiguousarray(np.broadcast_to(np.asarray(ee_eta, np.float64), (ee.shape[0],)))
        vh = np.zeros(vf.shape[0], np.uint8)
        eh = np.zeros(ee.shape[0], np.uint8)
        self.lib.ref_narrowphase(qstart.size // 3, _ptr(qstart), _ptr(qend), vf.shape[0], _ptr(vf), _ptr(vfe),
                                 ee.shape[0], _ptr(ee), _ptr(eee), _ptr(vh), _ptr(eh))
        return vh, eh


def compare_mesh_step(orc: Oracle, qs, qe, faces, eta: float, candidates, collisions, nthreads: int = 1,
                      kind: int = 0) -> dict:
    """The oracle's broad phase (kind 0 k-DOP, 1 AABB) and CTCD narrow phase
    on one step (qs -> qe), against a GPU step's candidate stencils
    (vf, ee) and colliding stencils (vf, vf_t, ee, ee_t)."""
    vf_c, ee_c = orc.broadphase(kind, qs, qe, faces, eta)
    out = orc.narrowphase(qs, qe, vf_c, eta, ee_c, eta, nthreads=nthreads)
    return compare_step_results(vf_c, ee_c, out, candidates, collisions)


def compare_step_results(vf_c, ee_c, out, candidates, collisions) -> dict:
    """The oracle's candidates (vf_c, ee_c) and narrow-phase results `out`
    against a GPU step's candidate stencils (vf, ee) and colliding stencils
    (vf, vf_t, ee, ee_t).  Candidate and colliding sets must be identical
    (same stencils, same order); contact times are compared relative to the
    oracle's."""
    g_vf_c, g_ee_c = candidates
    g_vf, g_vft, g_ee, g_eet = collisions
    vh, eh = out["vf_hit"] == 1, out["ee_hit"] == 1
    same_cand = bool(np.array_equal(vf_c, g_vf_c) and np.array_equal(ee_c, g_ee_c))
    same_col = bool(np.array_equal(vf_c[vh], g_vf) and np.array_equal(ee_c[eh], g_ee))
    err = 0.0
    if same_col:
        for ref, got in ((out["vf_t"][vh], g_vft), (out["ee_t"][eh], g_eet)):
            if ref.size:
                err = max(err, float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300))))
    return {"candidates": int(vf_c.shape[0] + ee_c.shape[0]), "collisions": int(vh.sum() + eh.sum()),
            "identical_candidates": same_cand, "identical_collisions": same_col, "max_rel_t_err": err}


def merge_checks(checks, steps=None) -> dict:
    """One summary of several compare_step_results."""
    d = {"candidates": sum(c["candidates"] for c in checks), "collisions": sum(c["collisions"] for c in checks),
         "identical_candidates": all(c["identical_candidates"] for c in checks),
         "identical_collisions": all(c["identical_collisions"] for c in checks),
         "max_rel_t_err": max([c["max_rel_t_err"] for c in checks] + [0.0])}
    if steps is not None:
        d["steps"] = list(steps)
    return d
