"""The C ABI: the library loads, exports exactly what include/kifi_gpu.h
declares, and validates arguments without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "kifi_gpu.h")).read()
    return sorted(set(re.findall(r"^KIFI_API\s+[\w\s\*]+?\b(kifi_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("kifi_volume_create", "kifi_integrate_f32", "kifi_mesh", "kifi_radix_sort_u32"):
        assert s in syms


def test_library_exports_every_declared_symbol(kifi_lib):
    from merge_fusion_gb300 import _lib
    for name in declared_symbols():
        assert hasattr(kifi_lib, name), name
        assert name in _lib.SIGNATURES, "binding missing for " + name


def test_status_strings(kifi_lib):
    assert kifi_lib.kifi_status_string(0) == b"ok"
    assert kifi_lib.kifi_status_string(4) == b"capacity exceeded"


def test_volume_create_rejects_bad_resolution(kifi_lib):
    from merge_fusion_gb300 import _lib
    d = _lib.VolumeDesc()
    d.resolution, d.side_length_m, d.truncation_m = 100, 2.0, 0.02  # not a power of two
    h = C.c_void_p()
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 1
    d.resolution, d.key_bits = 2048, 32  # above the 10-bit fields of 32-bit keys
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 1
    d.resolution, d.key_bits = 16384, 0  # above the 13-bit fields of 64-bit keys
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 1
    d.resolution, d.key_bits = 256, 48  # key width neither 32 nor 64
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 1
    d.key_bits = 0
    d.resolution, d.truncation_m = 256, 0.0
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 1


def test_null_arguments_are_rejected(kifi_lib):
    assert kifi_lib.kifi_volume_size(None, None) == 1
    assert kifi_lib.kifi_integrate_f32(None, None, None, None) == 1
    assert kifi_lib.kifi_radix_sort_u32(None, 5) == 1
    assert kifi_lib.kifi_radix_sort_u32(None, 0) == 0  # empty sort is a no-op
    assert kifi_lib.kifi_volume_set_launch_mode(None, 0) == 1
    assert kifi_lib.kifi_batch_set_persistent(None, 1, 1) == 1


def test_no_device_is_reported_not_faked(kifi_lib):
    from merge_fusion_gb300 import _lib
    if _lib.device_count() > 0:
        pytest.skip("a GPU is visible")
    d = _lib.VolumeDesc()
    d.resolution, d.side_length_m, d.truncation_m = 256, 2.0, 0.02
    h = C.c_void_p()
    assert kifi_lib.kifi_volume_create(C.byref(d), C.byref(h)) == 7  # KIFI_ERR_NO_DEVICE
    with pytest.raises(_lib.KifiError):
        from merge_fusion_gb300 import kifi
        kifi.Volume(256, 2.0, 0.02)
