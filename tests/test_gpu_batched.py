"""Batched scenes (merge_fusion_gb300.batched): every scene's volume and
tracked pose after interleaved, concurrent execution equal the same scene
run alone."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _export(lib, pipe):
    vol = lib.kifi_pipeline_volume(pipe)
    n = C.c_size_t()
    assert lib.kifi_volume_size(vol, C.byref(n)) == 0
    k = np.zeros(n.value + 1, np.uint64)
    v = np.zeros((n.value + 1, 2), np.float32)
    got = C.c_size_t()
    assert lib.kifi_volume_export64(vol, k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                    n.value + 1, C.byref(got)) == 0
    pose = np.zeros(16, np.float32)
    assert lib.kifi_pipeline_sync(pipe, pose.ctypes.data_as(C.c_void_p)) == 0
    return k[:got.value], v[:got.value], pose


def test_batched_scenes_equal_single_runs(gpu):
    import torch
    from merge_fusion_gb300 import _lib, batched
    lib = _lib.load()
    specs = [{"seed": 11, "width": 320, "height": 240, "f": 292.5, "voxel_mm": 8, "res": 512, "frames": 9},
             {"seed": 12, "width": 512, "height": 424, "f": 365.0, "voxel_mm": 4, "res": 1024, "frames": 7},
             {"seed": 13, "width": 640, "height": 480, "f": 585.0, "voxel_mm": 2, "res": 2048, "frames": 8}]
    together = [batched.Scene(s, 6, 10, 0) for s in specs]
    while any(not s.done() for s in together):
        for s in together:
            if not s.done():
                s.step(lib, torch, True)
    alone = []
    for spec in specs:
        s = batched.Scene(spec, 6, 10, 0)
        while not s.done():
            s.step(lib, torch, False)
        alone.append(s)
    for a, b in zip(together, alone):
        ka, va, pa = _export(lib, a.pipe)
        kb, vb, pb = _export(lib, b.pipe)
        assert ka.size > 1000
        assert np.array_equal(ka, kb) and np.array_equal(va.view(np.uint32), vb.view(np.uint32))
        assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32))
        assert len(a.latencies_ms()) == a.spec["frames"]
    for s in together + alone:
        s.close(lib)
