"""ctypes binding of the C ABI in include/ccd_gb300.h (libccd_gb300.so).

There is no CPU fallback: if the native library is missing or no CUDA device
is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from .build import LIB, ROOT

HEADER = os.path.join(ROOT, "include", "ccd_gb300.h")

CCD_OK = 0
VERTEX_FACE, EDGE_EDGE, VERTEX_EDGE, VERTEX_VERTEX = 0, 1, 2, 3
PATH_FP64, PATH_CULL_REFINE, PATH_REFINE_ALL = 0, 1, 2
BROADPHASE_KDOP13, BROADPHASE_AABB, BROADPHASE_TRIVIAL = 0, 1, 2
DISTANCE_VERTEX_FACE, DISTANCE_EDGE_EDGE = 0, 1    # ccd_distance_batch
DISTANCE_VERTEX_PLANE, DISTANCE_LINE_LINE = 0, 1   # ccd_distance_less_than_batch
ROW_WIDTH = {VERTEX_FACE: 24, EDGE_EDGE: 24, VERTEX_EDGE: 18, VERTEX_VERTEX: 12}

_P = ctypes.c_void_p
_I64 = ctypes.c_int64


class CcdError(RuntimeError):
    pass


class BatchStats(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int64), ("survivors", ctypes.c_int64), ("hits", ctypes.c_int64),
                ("status_flags", ctypes.c_int64)]


class MeshStats(ctypes.Structure):
    _fields_ = [("face_pairs", ctypes.c_int64), ("n_vf", ctypes.c_int64), ("n_ee", ctypes.c_int64),
                ("vf_hits", ctypes.c_int64), ("ee_hits", ctypes.c_int64), ("slab_tests", ctypes.c_int64),
                ("broadphase_ms", ctypes.c_float), ("traversal_ms", ctypes.c_float),
                ("self_distance_eta", ctypes.c_double), ("tree_built", ctypes.c_int32),
                ("tree_refits", ctypes.c_int32), ("graph_replay", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class VelocityFilterStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("layers", ctypes.c_int32), ("events", ctypes.c_int64),
                ("collisions", ctypes.c_int64), ("history_entries", ctypes.c_int64),
                ("start_distance", ctypes.c_double)]


class BatchTimings(ctypes.Structure):
    _fields_ = [("cull_ms", ctypes.c_float), ("refine_ms", ctypes.c_float), ("launches", ctypes.c_int32)]


class TuneResult(ctypes.Structure):
    _fields_ = [("wave_steps", ctypes.c_int32), ("pool_budget", ctypes.c_int32), ("wave_min_rows", ctypes.c_int64),
                ("candidates", ctypes.c_int32), ("mismatches", ctypes.c_int32), ("chosen", ctypes.c_int32),
                ("warp_finish", ctypes.c_int32), ("default_ms", ctypes.c_double), ("best_ms", ctypes.c_double),
                ("shift_after", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Fp64Peak(ctypes.Structure):
    _fields_ = [("ops_per_s", ctypes.c_double), ("fma_flops_per_s", ctypes.c_double), ("ms", ctypes.c_double),
                ("ops", ctypes.c_int64), ("div_per_s", ctypes.c_double), ("add_latency_cycles", ctypes.c_double),
                ("mul_latency_cycles", ctypes.c_double), ("div_latency_cycles", ctypes.c_double)]


_lib = None


def header_functions():
    """Names of the functions declared in include/ccd_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|void|const char\s*\*)\s*(ccd_\w+)\(", text, re.M)))


def load(path: str = LIB):
    """Loads libccd_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"native library {path} is missing: run collisiondetection_gb300.build.build_library() "
                          "(no CPU fallback exists)")
    L = ctypes.CDLL(path)
    L.ccd_version.restype = ctypes.c_int
    L.ccd_status_string.restype = ctypes.c_char_p
    L.ccd_status_string.argtypes = [ctypes.c_int]
    L.ccd_last_error.restype = ctypes.c_char_p
    L.ccd_last_error.argtypes = [_P]
    L.ccd_context_create.argtypes = [ctypes.c_int, ctypes.POINTER(_P)]
    L.ccd_context_destroy.argtypes = [_P]
    L.ccd_context_set_stream.argtypes = [_P, _P]
    L.ccd_context_synchronize.argtypes = [_P]
    L.ccd_last_batch_stats.argtypes = [_P, ctypes.POINTER(BatchStats)]
    L.ccd_context_set_profiling.argtypes = [_P, ctypes.c_int]
    L.ccd_last_batch_timings.argtypes = [_P, ctypes.POINTER(BatchTimings)]
    L.ccd_context_set_option.argtypes = [_P, ctypes.c_char_p, ctypes.c_int64]
    for name in ("ccd_vertex_face_ctcd", "ccd_edge_edge_ctcd", "ccd_vertex_edge_ctcd", "ccd_vertex_vertex_ctcd"):
        fn = getattr(L, name)
        fn.argtypes = [_P, _P, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.ccd_prim_batch.argtypes = [_P, ctypes.c_int, ctypes.c_int, _I64, _P, _P, _I64, _P, _P]
    L.ccd_prim_batch_device.argtypes = [_P, ctypes.c_int, ctypes.c_int, _I64, _P, _P, _I64, _P, _P, _P]
    L.ccd_autotune_prim_batch.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _I64, ctypes.c_int,
                                          ctypes.POINTER(TuneResult)]
    L.ccd_prim_cull_device.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _I64, _P, _P, ctypes.POINTER(_I64)]
    L.ccd_fp64_peak.argtypes = [_P, ctypes.c_int, ctypes.POINTER(Fp64Peak)]
    L.ccd_mesh_create.argtypes = [_P, ctypes.c_int32, ctypes.c_int32, _P, ctypes.POINTER(_P)]
    L.ccd_mesh_destroy.argtypes = [_P]
    L.ccd_mesh_create_instances.argtypes = [_P, ctypes.c_int32, _P, _P, _P, ctypes.POINTER(_P)]
    L.ccd_mesh_set_positions.argtypes = [_P, _P, _P]
    L.ccd_mesh_set_positions_device.argtypes = [_P, _P, _P]
    L.ccd_mesh_set_fixed.argtypes = [_P, _P]
    L.ccd_mesh_set_history.argtypes = [_P, _P, _P, _P]
    L.ccd_narrowphase_separating_plane.argtypes = [_P, _I64, _P, _P, _I64, _I64, _P, _P, _I64, _P, _P, _P, _P]
    L.ccd_broadphase.argtypes = [_P, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]
    L.ccd_broadphase_get.argtypes = [_P, _P, _P]
    L.ccd_narrowphase.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _I64, _I64, _P, _P, _I64, _P, _P, _P, _P, _P, _P]
    L.ccd_mesh_detect.argtypes = [_P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.POINTER(_I64), ctypes.POINTER(_I64)]
    L.ccd_mesh_get_collisions.argtypes = [_P, _P, _P, _P, _P]
    L.ccd_mesh_detect_graph.argtypes = L.ccd_mesh_detect.argtypes
    L.ccd_mesh_last_stats.argtypes = [_P, ctypes.POINTER(MeshStats)]
    L.ccd_distance_batch.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _P]
    L.ccd_distance_batch_device.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _P]
    L.ccd_distance_less_than_batch.argtypes = [_P, ctypes.c_int, _I64, _P, _P, _I64, _P]
    L.ccd_mesh_self_distance.argtypes = [_P, _P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64),
                                         ctypes.POINTER(_I64)]
    L.ccd_self_distance.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int32, _P, _P, ctypes.POINTER(ctypes.c_double)]
    L.ccd_penalty_group_force.argtypes = [_P, ctypes.c_int32, _P, _P, _I64, _P, _P, _I64, _P, _P, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P,
                                          _P, _P, ctypes.POINTER(ctypes.c_int)]
    L.ccd_penalty_group_force_device.argtypes = L.ccd_penalty_group_force.argtypes
    L.ccd_velocity_filter.argtypes = [_P, ctypes.c_int32, _P, _P, ctypes.c_int32, _P, _P, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                      ctypes.POINTER(VelocityFilterStats)]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class Context:
    """One device context (device buffers + streams) of the C ABI."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _P()
        rc = self.lib.ccd_context_create(device, ctypes.byref(h))
        if rc != CCD_OK:
            raise CcdError(f"ccd_context_create: {self.lib.ccd_status_string(rc).decode()}")
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ccd_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != CCD_OK:
            msg = self.lib.ccd_last_error(self.handle).decode()
            raise CcdError(f"{what}: {self.lib.ccd_status_string(rc).decode()}: {msg}")

    def synchronize(self):
        self._check(self.lib.ccd_context_synchronize(self.handle), "ccd_context_synchronize")

    def set_stream(self, stream_ptr: int | None):
        self._check(self.lib.ccd_context_set_stream(self.handle, stream_ptr), "ccd_context_set_stream")

    def stats(self) -> dict:
        st = BatchStats()
        self._check(self.lib.ccd_last_batch_stats(self.handle, ctypes.byref(st)), "ccd_last_batch_stats")
        return {f: getattr(st, f) for f, _ in BatchStats._fields_}

    def set_option(self, name: str, value: int):
        """Tuning option (ccd_context_set_option): "wave_steps", "wave_min_rows",
        "pool_budget", "chunk_rows", ... (include/ccd_gb300.h lists them)."""
        self._check(self.lib.ccd_context_set_option(self.handle, name.encode(), int(value)), "ccd_context_set_option")

    def set_profiling(self, on: bool):
        self._check(self.lib.ccd_context_set_profiling(self.handle, int(bool(on))), "ccd_context_set_profiling")

    def timings(self) -> dict:
        tm = BatchTimings()
        self._check(self.lib.ccd_last_batch_timings(self.handle, ctypes.byref(tm)), "ccd_last_batch_timings")
        return {f: getattr(tm, f) for f, _ in BatchTimings._fields_}

    def single(self, kind: int, points, eta: float, t_in: float = float("nan")):
        """One query through the single-call entry points; returns (hit, t)."""
        name = {VERTEX_FACE: "ccd_vertex_face_ctcd", EDGE_EDGE: "ccd_edge_edge_ctcd",
                VERTEX_EDGE: "ccd_vertex_edge_ctcd", VERTEX_VERTEX: "ccd_vertex_vertex_ctcd"}[kind]
        x = np.ascontiguousarray(points, dtype=np.float64).ravel()
        if x.size != ROW_WIDTH[kind]:
            raise ValueError("wrong number of coordinates")
        hit = ctypes.c_int(0)
        t = ctypes.c_double(t_in)
        self._check(getattr(self.lib, name)(self.handle, _ptr(x), eta, ctypes.byref(hit), ctypes.byref(t)), name)
        return hit.value, t.value

    def prim_batch(self, kind: int, rows, eta, path: int = PATH_CULL_REFINE, t=None):
        """Host-memory batch (ccd_prim_batch).  Returns (hit uint8, t float64);
        t keeps its input values (NaN by default) where hit == 0."""
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        n = rows.shape[0] if rows.ndim == 2 else rows.size // ROW_WIDTH[kind]
        eta = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        hit = np.zeros(n, np.uint8)
        t = np.full(n, np.nan) if t is None else np.ascontiguousarray(t, dtype=np.float64).copy()
        self._check(self.lib.ccd_prim_batch(self.handle, kind, path, n, _ptr(rows), _ptr(eta), eta.size, _ptr(hit),
                                            _ptr(t)), "ccd_prim_batch")
        return hit, t

    def distance(self, kind: int, rows, want_bary: bool = True):
        """Distance::vertexFaceDistance (DISTANCE_VERTEX_FACE) or
        edgeEdgeDistance (DISTANCE_EDGE_EDGE) per row of 12 doubles
        (ccd_distance_batch).  Returns (vec [n][3], bary [n][3|4] or None)."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 12)
        n = rows.shape[0]
        vec = np.zeros((n, 3))
        bary = np.zeros((n, 3 if kind == DISTANCE_VERTEX_FACE else 4)) if want_bary else None
        self._check(self.lib.ccd_distance_batch(self.handle, kind, n, _ptr(rows), _ptr(vec), _ptr(bary)),
                    "ccd_distance_batch")
        return vec, bary

    def distance_device(self, kind: int, n: int, rows_ptr: int, vec_ptr: int, bary_ptr: int | None = None):
        """Device-memory form (ccd_distance_batch_device); asynchronous."""
        self._check(self.lib.ccd_distance_batch_device(self.handle, kind, n, rows_ptr, vec_ptr, bary_ptr),
                    "ccd_distance_batch_device")

    def distance_less_than(self, kind: int, rows, eta):
        """Distance::vertexPlaneDistanceLessThan (DISTANCE_VERTEX_PLANE) or
        lineLineDistanceLessThan (DISTANCE_LINE_LINE) per row; uint8 [n]."""
        rows = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, 12)
        n = rows.shape[0]
        eta = np.ascontiguousarray(np.atleast_1d(np.asarray(eta, dtype=np.float64)))
        out = np.zeros(n, np.uint8)
        self._check(self.lib.ccd_distance_less_than_batch(self.handle, kind, n, _ptr(rows), _ptr(eta), eta.size,
                                                          _ptr(out)), "ccd_distance_less_than_batch")
        return out

    def self_distance(self, verts, faces, fixed=None) -> float:
        """Distance::meshSelfDistance(verts, faces, fixedVerts) (ccd_self_distance)."""
        verts = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        faces = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8).ravel()
        d = ctypes.c_double()
        self._check(self.lib.ccd_self_distance(self.handle, verts.size // 3, _ptr(verts), faces.shape[0], _ptr(faces),
                                               _ptr(fx), ctypes.byref(d)), "ccd_self_distance")
        return d.value

    def penalty_group_force(self, q, v, F, vf, ee, outer_eta: float, inner_eta: float, stiffness: float,
                            cor: float, dt: float, vf_isnew=None, ee_isnew=None):
        """PenaltyGroup::addForce (ccd_penalty_group_force).  Returns
        (F_out, vf_fired, ee_fired, newused); F is not modified."""
        q = np.ascontiguousarray(q, dtype=np.float64).ravel()
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        Fo = np.ascontiguousarray(F, dtype=np.float64).ravel().copy()
        vf = np.ascontiguousarray(vf, dtype=np.int32).reshape(-1, 4)
        ee = np.ascontiguousarray(ee, dtype=np.int32).reshape(-1, 4)
        vn = None if vf_isnew is None else np.ascontiguousarray(vf_isnew, dtype=np.uint8)
        en = None if ee_isnew is None else np.ascontiguousarray(ee_isnew, dtype=np.uint8)
        vfire = np.zeros(vf.shape[0], np.uint8)
        efire = np.zeros(ee.shape[0], np.uint8)
        used = ctypes.c_int(0)
        self._check(self.lib.ccd_penalty_group_force(self.handle, q.size // 3, _ptr(q), _ptr(v), vf.shape[0], _ptr(vf),
                                                     _ptr(vn), ee.shape[0], _ptr(ee), _ptr(en), outer_eta, inner_eta,
                                                     stiffness, cor, dt, _ptr(Fo), _ptr(vfire), _ptr(efire),
                                                     ctypes.byref(used)), "ccd_penalty_group_force")
        return Fo, vfire, efire, bool(used.value)

    def penalty_group_force_device(self, nverts: int, q_ptr: int, v_ptr: int, n_vf: int, vf_ptr: int, n_ee: int,
                                   ee_ptr: int, outer_eta: float, inner_eta: float, stiffness: float, cor: float,
                                   dt: float, F_ptr: int, vf_fired_ptr: int, ee_fired_ptr: int,
                                   vf_isnew_ptr: int | None = None, ee_isnew_ptr: int | None = None) -> bool:
        """Device-memory form (ccd_penalty_group_force_device); returns newused."""
        used = ctypes.c_int(0)
        self._check(self.lib.ccd_penalty_group_force_device(self.handle, nverts, q_ptr, v_ptr, n_vf, vf_ptr,
                                                            vf_isnew_ptr, n_ee, ee_ptr, ee_isnew_ptr, outer_eta,
                                                            inner_eta, stiffness, cor, dt, F_ptr, vf_fired_ptr,
                                                            ee_fired_ptr, ctypes.byref(used)),
                    "ccd_penalty_group_force_device")
        return bool(used.value)

    def velocity_filter(self, qstart, qend, faces, invmasses, outer_eta: float, inner_eta: float,
                        base_stiffness: float = 1e-4, base_substep: float = 1e-4, cor: float = 0.1,
                        max_rollbacks: int = 1000):
        """VelocityFilter::velocityFilter (ccd_velocity_filter).  Returns
        (result, qend_out, stats): result is the reference's return value;
        qend_out the filtered end positions (qend unchanged when result < 0)."""
        qs = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qe = np.ascontiguousarray(qend, dtype=np.float64).ravel().copy()
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        mi = np.ascontiguousarray(invmasses, dtype=np.float64).ravel()
        if qe.size != qs.size or mi.size != qs.size:
            raise ValueError("qstart, qend and invmasses must have the same size")
        res = ctypes.c_int32(0)
        st = VelocityFilterStats()
        self._check(self.lib.ccd_velocity_filter(self.handle, qs.size // 3, _ptr(qs), _ptr(qe), f.shape[0], _ptr(f),
                                                 _ptr(mi), outer_eta, inner_eta, base_stiffness, base_substep, cor,
                                                 max_rollbacks, ctypes.byref(res), ctypes.byref(st)),
                    "ccd_velocity_filter")
        return res.value, qe, {k: getattr(st, k) for k, _ in VelocityFilterStats._fields_}

    def prim_batch_device(self, kind: int, n: int, rows_ptr: int, eta_ptr: int, eta_count: int, hit_ptr: int,
                          t_ptr: int, status_ptr: int | None = None, path: int = PATH_CULL_REFINE):
        """Device-memory batch (ccd_prim_batch_device); pointers are raw device
        addresses (e.g. torch tensor data_ptr()).  Asynchronous."""
        self._check(self.lib.ccd_prim_batch_device(self.handle, kind, path, n, rows_ptr, eta_ptr, eta_count,
                                                   hit_ptr, t_ptr, status_ptr), "ccd_prim_batch_device")


    def prim_cull_device(self, kind: int, n: int, rows_ptr: int, eta_ptr: int, eta_count: int, hit_ptr: int,
                         survivors_ptr: int) -> int:
        """The FP32 stage alone (ccd_prim_cull_device): rejected rows get
        hit = 0, the others' indices go to survivors; returns their count."""
        cnt = _I64(0)
        self._check(self.lib.ccd_prim_cull_device(self.handle, kind, n, rows_ptr, eta_ptr, eta_count, hit_ptr,
                                                  survivors_ptr, ctypes.byref(cnt)), "ccd_prim_cull_device")
        return int(cnt.value)

    def fp64_peak(self, reps: int = 3) -> dict:
        """This device's FP64 add / multiply and fused multiply-add rates
        (ccd_fp64_peak)."""
        res = Fp64Peak()
        self._check(self.lib.ccd_fp64_peak(self.handle, reps, ctypes.byref(res)), "ccd_fp64_peak")
        return {f: getattr(res, f) for f, _ in Fp64Peak._fields_}

    def autotune_prim_batch(self, kind: int, n: int, rows_ptr: int, eta_ptr: int, eta_count: int = 1,
                            reps: int = 3) -> dict:
        """Work-split autotuner (ccd_autotune_prim_batch) on a device batch of
        vertex-face or edge-edge rows; sets the fastest split as this
        context's options and returns what it measured."""
        res = TuneResult()
        self._check(self.lib.ccd_autotune_prim_batch(self.handle, kind, n, rows_ptr, eta_ptr, eta_count, reps,
                                                     ctypes.byref(res)), "ccd_autotune_prim_batch")
        return {f: getattr(res, f) for f, _ in TuneResult._fields_ if f != "reserved"}


def _stencils(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a.reshape(-1, 4)


class Mesh:
    """A mesh resident on a context's device (ccd_mesh_*): the reference's
    Mesh faces plus a two-entry History (start, end) of vertex positions.

    broadphase() mirrors BroadPhase::findCollisionCandidates
    (src/RetrospectiveDetection.h:13) and narrowphase() mirrors
    CTCDNarrowPhase::findCollisions (src/CTCDNarrowPhase.cpp:9-24)."""

    def __init__(self, ctx: Context, faces, qstart=None, qend=None, fixed=None, nverts: int | None = None,
                 instances=None):
        """instances: optional (vertex_offsets, face_offsets) of independent
        instances making up the mesh (ccd_mesh_create_instances)."""
        self.ctx = ctx
        self.lib = ctx.lib
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        if nverts is None:
            if qstart is None:
                raise ValueError("nverts or qstart is required")
            nverts = np.asarray(qstart).size // 3
        self.nverts, self.nfaces = int(nverts), int(f.shape[0])
        h = _P()
        if instances is None:
            ctx._check(self.lib.ccd_mesh_create(ctx.handle, self.nverts, self.nfaces, _ptr(f), ctypes.byref(h)),
                       "ccd_mesh_create")
        else:
            vo = np.ascontiguousarray(instances[0], dtype=np.int32)
            fo = np.ascontiguousarray(instances[1], dtype=np.int32)
            if vo.size != fo.size or vo[-1] != self.nverts or fo[-1] != self.nfaces:
                raise ValueError("instance offsets must end at nverts and nfaces")
            ctx._check(self.lib.ccd_mesh_create_instances(ctx.handle, vo.size - 1, _ptr(vo), _ptr(fo), _ptr(f),
                                                          ctypes.byref(h)), "ccd_mesh_create_instances")
        self.handle = h
        if qstart is not None:
            self.set_positions(qstart, qend)
        if fixed is not None:
            self.set_fixed(fixed)

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ccd_mesh_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_positions(self, qstart, qend):
        qs = np.ascontiguousarray(qstart, dtype=np.float64).ravel()
        qe = np.ascontiguousarray(qend, dtype=np.float64).ravel()
        if qs.size != 3 * self.nverts or qe.size != 3 * self.nverts:
            raise ValueError("positions must hold 3 * nverts doubles")
        self.ctx._check(self.lib.ccd_mesh_set_positions(self.handle, _ptr(qs), _ptr(qe)), "ccd_mesh_set_positions")

    def set_positions_device(self, qstart_ptr: int, qend_ptr: int):
        self.ctx._check(self.lib.ccd_mesh_set_positions_device(self.handle, qstart_ptr, qend_ptr),
                        "ccd_mesh_set_positions_device")

    def set_history(self, offsets, times, positions):
        """A multi-entry History (ccd_mesh_set_history): vertex v's entries
        are offsets[v] .. offsets[v+1]-1 of times and positions ([E][3])."""
        off = np.ascontiguousarray(offsets, dtype=np.int32).ravel()
        tt = np.ascontiguousarray(times, dtype=np.float64).ravel()
        pp = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if off.size != self.nverts + 1 or tt.size != off[-1] or pp.shape[0] != off[-1]:
            raise ValueError("offsets must hold nverts + 1 values and the arrays offsets[-1] entries")
        self.ctx._check(self.lib.ccd_mesh_set_history(self.handle, _ptr(off), _ptr(tt), _ptr(pp)),
                        "ccd_mesh_set_history")

    def set_fixed(self, fixed):
        fx = None
        if fixed is not None:
            fx = np.ascontiguousarray(fixed, dtype=np.uint8).ravel()
            if fx.size != self.nverts:
                raise ValueError("fixed must hold nverts flags")
        self.ctx._check(self.lib.ccd_mesh_set_fixed(self.handle, _ptr(fx)), "ccd_mesh_set_fixed")

    def broadphase(self, kind: int = BROADPHASE_KDOP13, outer_eta: float = 1e-6):
        """Candidate stencils (vf [n][4], ee [n][4]) in the reference's set order."""
        nvf, nee = _I64(), _I64()
        self.ctx._check(self.lib.ccd_broadphase(self.handle, kind, outer_eta, ctypes.byref(nvf), ctypes.byref(nee)),
                        "ccd_broadphase")
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        self.ctx._check(self.lib.ccd_broadphase_get(self.handle, _ptr(vf), _ptr(ee)), "ccd_broadphase_get")
        return vf, ee

    def narrowphase(self, vf, vf_eta, ee, ee_eta, path: int = PATH_CULL_REFINE):
        """Per-stencil results: dict of vf_hit / ee_hit (uint8), vf_t / ee_t
        (NaN where no hit) and vf_which / ee_which (0 primitive, 1 vertex-edge,
        2 vertex-vertex, -1 miss)."""
        vf, ee = _stencils(vf), _stencils(ee)
        vfe = np.ascontiguousarray(np.atleast_1d(np.asarray(vf_eta, np.float64)))
        eee = np.ascontiguousarray(np.atleast_1d(np.asarray(ee_eta, np.float64)))
        nv, ne = vf.shape[0], ee.shape[0]
        out = {"vf_hit": np.zeros(nv, np.uint8), "ee_hit": np.zeros(ne, np.uint8),
               "vf_t": np.full(nv, np.nan), "ee_t": np.full(ne, np.nan),
               "vf_which": np.zeros(nv, np.int8), "ee_which": np.zeros(ne, np.int8)}
        self.ctx._check(self.lib.ccd_narrowphase(self.handle, path, nv, _ptr(vf), _ptr(vfe), vfe.size, ne, _ptr(ee),
                                                 _ptr(eee), eee.size, _ptr(out["vf_hit"]), _ptr(out["ee_hit"]),
                                                 _ptr(out["vf_t"]), _ptr(out["ee_t"]), _ptr(out["vf_which"]),
                                                 _ptr(out["ee_which"])), "ccd_narrowphase")
        return out

    def narrowphase_separating_plane(self, vf, vf_eta, ee, ee_eta):
        """SeparatingPlaneNarrowPhase::findCollisions per stencil
        (ccd_narrowphase_separating_plane): dict of vf_hit / ee_hit and
        vf_status / ee_status (1 where the reference's search stalls)."""
        vf, ee = _stencils(vf), _stencils(ee)
        vfe = np.ascontiguousarray(np.atleast_1d(np.asarray(vf_eta, np.float64)))
        eee = np.ascontiguousarray(np.atleast_1d(np.asarray(ee_eta, np.float64)))
        nv, ne = vf.shape[0], ee.shape[0]
        out = {"vf_hit": np.zeros(nv, np.uint8), "ee_hit": np.zeros(ne, np.uint8),
               "vf_status": np.zeros(nv, np.uint8), "ee_status": np.zeros(ne, np.uint8)}
        self.ctx._check(self.lib.ccd_narrowphase_separating_plane(
            self.handle, nv, _ptr(vf), _ptr(vfe), vfe.size, ne, _ptr(ee), _ptr(eee), eee.size, _ptr(out["vf_hit"]),
            _ptr(out["ee_hit"]), _ptr(out["vf_status"]), _ptr(out["ee_status"])), "ccd_narrowphase_separating_plane")
        return out

    def detect(self, kind: int = BROADPHASE_KDOP13, outer_eta: float = 1e-6, eta: float = 1e-6,
               path: int = PATH_CULL_REFINE, fetch: bool = True, graph: bool = False):
        """Broad phase + narrow phase on the device (ccd_mesh_detect, or with
        graph=True ccd_mesh_detect_graph: the same results, later steps
        replayed from a captured CUDA graph).  Returns the colliding
        (vf, vf_t, ee, ee_t) in set order, or the two counts if fetch is False."""
        nvf, nee = _I64(), _I64()
        fn = self.lib.ccd_mesh_detect_graph if graph else self.lib.ccd_mesh_detect
        self.ctx._check(fn(self.handle, kind, outer_eta, eta, path, ctypes.byref(nvf), ctypes.byref(nee)),
                        "ccd_mesh_detect_graph" if graph else "ccd_mesh_detect")
        if not fetch:
            return nvf.value, nee.value
        vf = np.zeros((nvf.value, 4), np.int32)
        ee = np.zeros((nee.value, 4), np.int32)
        vft = np.zeros(nvf.value)
        eet = np.zeros(nee.value)
        self.ctx._check(self.lib.ccd_mesh_get_collisions(self.handle, _ptr(vf), _ptr(vft), _ptr(ee), _ptr(eet)),
                        "ccd_mesh_get_collisions")
        return vf, vft, ee, eet

    def candidates(self):
        """The stencils of the mesh's last broad phase (also the one
        self_distance runs), without running a new one."""
        st = self.stats()
        vf = np.zeros((st["n_vf"], 4), np.int32)
        ee = np.zeros((st["n_ee"], 4), np.int32)
        self.ctx._check(self.lib.ccd_broadphase_get(self.handle, _ptr(vf), _ptr(ee)), "ccd_broadphase_get")
        return vf, ee

    def self_distance(self, verts):
        """Distance::meshSelfDistance on this mesh's faces and fixed flags at
        positions verts (ccd_mesh_self_distance; verts become the mesh's start
        and end positions).  Returns (distance, n_vf, n_ee): the stencil
        counts are the ones the reference prints."""
        v = np.ascontiguousarray(verts, dtype=np.float64).ravel()
        if v.size != 3 * self.nverts:
            raise ValueError("verts must hold nverts x 3 doubles")
        d, nvf, nee = ctypes.c_double(), _I64(), _I64()
        self.ctx._check(self.lib.ccd_mesh_self_distance(self.handle, _ptr(v), ctypes.byref(d), ctypes.byref(nvf),
                                                        ctypes.byref(nee)), "ccd_mesh_self_distance")
        return d.value, nvf.value, nee.value

    def stats(self) -> dict:
        st = MeshStats()
        self.ctx._check(self.lib.ccd_mesh_last_stats(self.handle, ctypes.byref(st)), "ccd_mesh_last_stats")
        return {f: getattr(st, f) for f, _ in MeshStats._fields_}


class Request(ctypes.Structure):
    _fields_ = [("nverts", ctypes.c_int32), ("nfaces", ctypes.c_int32), ("faces", _P), ("steps", ctypes.c_int32),
                ("frames", _P), ("fixed", _P), ("broadphase_kind", ctypes.c_int32), ("path", ctypes.c_int32),
                ("outer_eta", ctypes.c_double), ("eta", ctypes.c_double)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("steps", ctypes.c_int32),
                ("vf_hits", ctypes.POINTER(ctypes.c_int64)), ("ee_hits", ctypes.POINTER(ctypes.c_int64)),
                ("vf_offsets", ctypes.POINTER(ctypes.c_int64)), ("ee_offsets", ctypes.POINTER(ctypes.c_int64)),
                ("vf", ctypes.POINTER(ctypes.c_int32)), ("ee", ctypes.POINTER(ctypes.c_int32)),
                ("vf_t", ctypes.POINTER(ctypes.c_double)), ("ee_t", ctypes.POINTER(ctypes.c_double)),
                ("step_ms", ctypes.POINTER(ctypes.c_double)), ("queue_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("error", ctypes.c_char_p)]


def _bind_server(L):
    if getattr(L, "_server_bound", False):
        return
    L.ccd_server_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.POINTER(_P)]
    L.ccd_server_destroy.argtypes = [_P]
    L.ccd_server_submit.argtypes = [_P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]
    L.ccd_server_poll.argtypes = [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int)]
    L.ccd_server_wait.argtypes = [_P, ctypes.c_uint64, ctypes.POINTER(RequestResult)]
    L.ccd_server_release.argtypes = [_P, ctypes.c_uint64]
    L._server_bound = True


def _array(ptr, n, dtype, shape=None):
    if n == 0:
        return np.zeros(shape if shape else (0,), dtype)
    a = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
    return a.reshape(shape) if shape else a


class Server:
    """Serving engine (ccd_server_*): requests of (mesh, frames) run on
    `slots` workers with their own contexts, admitted within a device-memory
    budget; each step is one ccd_mesh_detect between consecutive frames."""

    def __init__(self, device: int = 0, slots: int = 4, memory_budget: int = 60 << 30):
        self.lib = load()
        _bind_server(self.lib)
        h = _P()
        rc = self.lib.ccd_server_create(device, slots, memory_budget, ctypes.byref(h))
        if rc != CCD_OK:
            raise CcdError(f"ccd_server_create: {self.lib.ccd_status_string(rc).decode()}")
        self.handle = h
        self._keep = {}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.ccd_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, faces, frames, fixed=None, kind: int = BROADPHASE_KDOP13, path: int = PATH_CULL_REFINE,
               outer_eta: float = 1e-6, eta: float = 1e-6) -> int:
        """frames: (steps + 1, 3V) positions; returns a ticket."""
        f = np.ascontiguousarray(faces, dtype=np.int32).reshape(-1, 3)
        fr = np.ascontiguousarray(frames, dtype=np.float64)
        steps = fr.shape[0] - 1
        nverts = fr.shape[1] // 3
        fx = None if fixed is None else np.ascontiguousarray(fixed, dtype=np.uint8)
        req = Request(nverts, f.shape[0], _ptr(f), steps, _ptr(fr), _ptr(fx), kind, path, outer_eta, eta)
        t = ctypes.c_uint64()
        rc = self.lib.ccd_server_submit(self.handle, ctypes.byref(req), ctypes.byref(t))
        if rc != CCD_OK:
            raise CcdError(f"ccd_server_submit: {self.lib.ccd_status_string(rc).decode()}")
        self._keep[t.value] = (f, fr, fx)  # frames are read until the request completes
        return t.value

    def poll(self, ticket: int) -> bool:
        d = ctypes.c_int(0)
        rc = self.lib.ccd_server_poll(self.handle, ticket, ctypes.byref(d))
        if rc != CCD_OK:
            raise CcdError("ccd_server_poll: unknown ticket")
        return bool(d.value)

    def wait(self, ticket: int, release: bool = True) -> dict:
        """Results: per step (vf, vf_t, ee, ee_t) arrays, step_ms, queue_ms,
        total_ms."""
        r = RequestResult()
        rc = self.lib.ccd_server_wait(self.handle, ticket, ctypes.byref(r))
        if rc != CCD_OK:
            raise CcdError("ccd_server_wait: unknown ticket")
        if r.status != CCD_OK:
            msg = r.error.decode() if r.error else ""
            self.lib.ccd_server_release(self.handle, ticket)
            self._keep.pop(ticket, None)
            raise CcdError(f"request failed: {self.lib.ccd_status_string(r.status).decode()}: {msg}")
        n = r.steps
        vfo = _array(r.vf_offsets, n + 1, np.int64)
        eeo = _array(r.ee_offsets, n + 1, np.int64)
        vf = _array(r.vf, 4 * int(vfo[-1]), np.int32, (int(vfo[-1]), 4))
        ee = _array(r.ee, 4 * int(eeo[-1]), np.int32, (int(eeo[-1]), 4))
        vft = _array(r.vf_t, int(vfo[-1]), np.float64)
        eet = _array(r.ee_t, int(eeo[-1]), np.float64)
        out = {"steps": [(vf[vfo[k]:vfo[k + 1]], vft[vfo[k]:vfo[k + 1]], ee[eeo[k]:eeo[k + 1]],
                          eet[eeo[k]:eeo[k + 1]]) for k in range(n)],
               "step_ms": _array(r.step_ms, n, np.float64), "queue_ms": r.queue_ms, "total_ms": r.total_ms}
        if release:
            self.lib.ccd_server_release(self.handle, ticket)
            self._keep.pop(ticket, None)
        return out
