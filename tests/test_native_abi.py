"""The C ABI library: it builds, loads and exports every symbol declared in
include/ccd_gb300.h.  No compute calls (CPU only)."""
import ctypes

import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import build as B


@pytest.fixture(scope="module")
def lib():
    B.build_library()
    return C.load()


def test_exports_every_header_symbol(lib):
    names = C.header_functions()
    assert "ccd_prim_batch" in names and "ccd_vertex_face_ctcd" in names
    for name in names:
        assert hasattr(lib, name), name


def test_version_and_status_strings(lib):
    assert lib.ccd_version() >= 100
    assert lib.ccd_status_string(0) == b"ok"
    assert lib.ccd_status_string(99) == b"unknown status"


def test_null_arguments_are_rejected(lib):
    assert lib.ccd_context_create(0, None) == 1
    assert lib.ccd_context_destroy(None) == 0
    assert lib.ccd_prim_batch(None, 0, 0, 1, None, None, 1, None, None) == 1
    assert lib.ccd_autotune_prim_batch(None, 0, 1, None, None, 1, 3, None) == 1
    assert lib.ccd_prim_cull_device(None, 0, 1, None, None, 1, None, None, None) == 1
    assert lib.ccd_fp64_peak(None, 3, None) == 1
    assert lib.ccd_prim_batch_device(None, 0, 2, 1, None, None, 1, None, None, None) == 1
    assert lib.ccd_server_create(0, 0, 1, None) == 1
    assert lib.ccd_server_destroy(None) == 0


def test_no_device_is_reported(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.ccd_context_create(0, ctypes.byref(h)) == 4  # CCD_ERR_NO_DEVICE
