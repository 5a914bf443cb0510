"""Failure detection without a GPU fault: every wait of the sort's decoupled
look-back is bounded.  The fault-injection hook makes the sorts skip their
first tile -- its look-back words are never published, so the waits on it
cannot end -- and lowers the poll limit.  The wait must give up, the call
must return KIFI_ERR_TIMEOUT with the context still usable, and the next
call must succeed.  A volume whose frame timed out keeps its voxels and its
occupancy bits, so the same frame fuses normally afterwards."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import assert_volume_equal, cam_params

pytestmark = pytest.mark.gpu

SPIN_LIMIT = 2000  # polls before a wait gives up (the default is 2^22)


def test_sort_wait_runs_out_then_the_next_sort_succeeds(gpu):
    from merge_fusion_gb300 import _lib
    lib = _lib.load()
    keys = np.random.default_rng(0).integers(0, 1 << 30, 100_000, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = keys.copy(), vals.copy()
    try:
        _lib.check(lib.kifi_sort_set_fault_injection(1, SPIN_LIMIT))
        st = lib.kifi_radix_sort_pairs_u32(k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p), k.size)
    finally:
        _lib.check(lib.kifi_sort_set_fault_injection(0, 0))
    assert st == _lib.KIFI_ERR_TIMEOUT, _lib.STATUS_NAMES.get(st, st)
    k, v = keys.copy(), vals.copy()
    _lib.check(lib.kifi_radix_sort_pairs_u32(k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p), k.size))
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


def test_a_timed_out_frame_leaves_the_volume_usable(gpu, oracle_cpu):
    from merge_fusion_gb300 import _lib, kifi, scenes
    lib = _lib.load()
    seq = scenes.sphere_scene(n_frames=3, seed=4)
    cam = seq.camera
    gv = kifi.Volume(512, 8.192, 0.048)
    ov = oracle_cpu.Volume(512, 8.192, 0.048)
    integ = kifi.Integrator()
    integ.Integrate(gv, seq.frames[0], cam_params(cam), seq.world_to_eye_f32(0))
    ov.integrate(seq.depth_m(0), cam, seq.world_to_eye_f32(0))
    try:
        _lib.check(lib.kifi_sort_set_fault_injection(1, SPIN_LIMIT))
        with pytest.raises(_lib.KifiError) as err:
            integ.Integrate(gv, seq.frames[1], cam_params(cam), seq.world_to_eye_f32(1))
    finally:
        _lib.check(lib.kifi_sort_set_fault_injection(0, 0))
    assert err.value.status == _lib.KIFI_ERR_TIMEOUT
    assert_volume_equal(gv, ov, "after the timed-out frame")
    for i in (1, 2):
        integ.Integrate(gv, seq.frames[i], cam_params(cam), seq.world_to_eye_f32(i))
        ov.integrate(seq.depth_m(i), cam, seq.world_to_eye_f32(i))
    assert_volume_equal(gv, ov, "frames fused after the timeout")
