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
PATH_FP64, PATH_CULL_REFINE = 0, 1
ROW_WIDTH = {VERTEX_FACE: 24, EDGE_EDGE: 24, VERTEX_EDGE: 18, VERTEX_VERTEX: 12}

_P = ctypes.c_void_p
_I64 = ctypes.c_int64


class CcdError(RuntimeError):
    pass


class BatchStats(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int64), ("survivors", ctypes.c_int64), ("hits", ctypes.c_int64),
                ("status_flags", ctypes.c_int64)]


class BatchTimings(ctypes.Structure):
    _fields_ = [("cull_ms", ctypes.c_float), ("refine_ms", ctypes.c_float), ("launches", ctypes.c_int32)]


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
    for name in ("ccd_vertex_face_ctcd", "ccd_edge_edge_ctcd", "ccd_vertex_edge_ctcd", "ccd_vertex_vertex_ctcd"):
        fn = getattr(L, name)
        fn.argtypes = [_P, _P, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.ccd_prim_batch.argtypes = [_P, ctypes.c_int, ctypes.c_int, _I64, _P, _P, _I64, _P, _P]
    L.ccd_prim_batch_device.argtypes = [_P, ctypes.c_int, ctypes.c_int, _I64, _P, _P, _I64, _P, _P, _P]
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

    def prim_batch_device(self, kind: int, n: int, rows_ptr: int, eta_ptr: int, eta_count: int, hit_ptr: int,
                          t_ptr: int, status_ptr: int | None = None, path: int = PATH_CULL_REFINE):
        """Device-memory batch (ccd_prim_batch_device); pointers are raw device
        addresses (e.g. torch tensor data_ptr()).  Asynchronous."""
        self._check(self.lib.ccd_prim_batch_device(self.handle, kind, path, n, rows_ptr, eta_ptr, eta_count,
                                                   hit_ptr, t_ptr, status_ptr), "ccd_prim_batch_device")
