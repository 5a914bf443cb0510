"""kifi::Pipeline on the GPU: fuse + track + mesh through kifi_pipeline_*,
checked against the volume/ICP entry points it composes and the oracle."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import cam_params, canon_bits

pytestmark = pytest.mark.gpu


def test_pipeline_matches_components_and_oracle(gpu, oracle_cpu):
    from merge_fusion_gb300 import _lib, kifi, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    lib = _lib.load()
    seq = scenes.room_scene(n_frames=4, seed=3)
    cam = seq.camera
    d = PipelineDesc()
    d.camera = cam_params(cam).camera()
    d.resolution, d.side_length_m, d.truncation_m = 1024, 4.096, 0.02
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = 15, 2, 1
    d.device = 0
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)))
    ov = oracle_cpu.Volume(1024, 4.096, 0.02)
    out = np.zeros(16, np.float32)
    try:
        for i in range(4):
            frame = np.ascontiguousarray(seq.frames[i])
            w2e = seq.world_to_eye_f32(i)
            check(lib.kifi_pipeline_integrate(pipe, frame.ctypes.data_as(C.c_void_p), 1,
                                              w2e.ctypes.data_as(C.c_void_p),
                                              out.ctypes.data_as(C.c_void_p)))
            ov.integrate(seq.depth_m(i), cam, w2e)
            if i > 0:
                prev = seq.eye_to_world_f32(i - 1)
                target = oracle_cpu.backproject(seq.depth_m(i - 1), cam, prev)
                o, _, n = oracle_cpu.icp_align(seq.depth_m(i), cam, prev, target, prev, 15)
                assert np.abs(out - o).max() < 1e-5, (i, np.abs(out - o).max())
            else:
                assert np.array_equal(out, seq.eye_to_world_f32(0)) or \
                    np.abs(out - seq.eye_to_world_f32(0)).max() < 1e-6
        vol = lib.kifi_pipeline_volume(pipe)
        n = C.c_size_t()
        check(lib.kifi_volume_size(vol, C.byref(n)))
        k = np.zeros(n.value, np.uint32)
        v = np.zeros((n.value, 2), np.float32)
        got = C.c_size_t()
        check(lib.kifi_volume_export(vol, k.ctypes.data_as(C.c_void_p),
                                     v.ctypes.data_as(C.c_void_p), n.value, C.byref(got)))
        assert np.array_equal(k, ov.keys)
        assert np.array_equal(canon_bits(v), canon_bits(ov.values))
        nv, ni = C.c_size_t(), C.c_size_t()
        check(lib.kifi_pipeline_mesh_counts(pipe, C.byref(nv), C.byref(ni)))
        vb, ib = ov.mesh(True)
        assert (nv.value, ni.value) == (vb.shape[0], ib.size)
        # two meshes (frames 2 and 4); the first found no buffers and was emitted again
        meshes, reemitted = C.c_longlong(), C.c_longlong()
        check(lib.kifi_pipeline_mesh_stats(pipe, C.byref(meshes), C.byref(reemitted)))
        assert meshes.value == 2 and 1 <= reemitted.value <= 2, (meshes.value, reemitted.value)
    finally:
        lib.kifi_pipeline_destroy(pipe)


def test_stage_timers_and_frame_log(gpu, golden):
    from merge_fusion_gb300 import _lib, kifi
    from merge_fusion_gb300._lib import check
    lib = _lib.load()
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    vol = kifi.Volume(256, 2.0, 0.02)
    check(lib.kifi_volume_set_profiling(vol.handle, 1))
    for i in range(3):
        kifi.Integrator().Integrate(vol, depth, cam_params(cam), view)
    ms = np.zeros(4)
    nf = C.c_int()
    check(lib.kifi_volume_stage_times(vol.handle, ms.ctypes.data_as(C.c_void_p), C.byref(nf)))
    assert nf.value == 3 and (ms > 0).all()
    n0 = np.zeros(64, np.uint64)
    ne = np.zeros(64, np.uint64)
    n1 = np.zeros(64, np.uint64)
    cnt = C.c_int()
    check(lib.kifi_volume_frame_log(vol.handle, n0.ctypes.data_as(C.c_void_p),
                                    ne.ctypes.data_as(C.c_void_p), n1.ctypes.data_as(C.c_void_p),
                                    64, C.byref(cnt)))
    assert cnt.value == 3
    assert n0[0] == 0 and n1[0] == golden["cases"][0]["voxels"]
    assert (n1[:3] == n0[:3] + ne[:3]).all() and n0[1] == n1[0]


def _run_pipeline(lib, seq, graphs, device_frames):
    import torch
    from merge_fusion_gb300._lib import PipelineDesc, check
    d = PipelineDesc()
    d.camera = cam_params(seq.camera).camera()
    d.resolution, d.side_length_m, d.truncation_m = 1024, 4.096, 0.02
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = 15, 3, 1
    d.device = 0
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)))
    check(lib.kifi_pipeline_set_graphs(pipe, 1 if graphs else 0))
    poses = []
    out = np.zeros(16, np.float32)
    try:
        pinned = [torch.from_numpy(np.ascontiguousarray(f).view(np.int16)).pin_memory() for f in seq.frames]
        dev = [p.cuda() for p in pinned]
        torch.cuda.synchronize()
        for i in range(len(seq.frames)):
            w2e = seq.world_to_eye_f32(i)
            if device_frames:
                check(lib.kifi_pipeline_integrate_device(pipe, C.c_void_p(dev[i].data_ptr()), 1,
                                                         w2e.ctypes.data_as(C.c_void_p)))
                check(lib.kifi_pipeline_sync(pipe, out.ctypes.data_as(C.c_void_p)))
            else:
                check(lib.kifi_pipeline_integrate(pipe, C.c_void_p(pinned[i].data_ptr()), 1,
                                                  w2e.ctypes.data_as(C.c_void_p),
                                                  out.ctypes.data_as(C.c_void_p)))
            poses.append(out.copy())
        vol = lib.kifi_pipeline_volume(pipe)
        n = C.c_size_t()
        check(lib.kifi_volume_size(vol, C.byref(n)))
        k = np.zeros(n.value, np.uint32)
        v = np.zeros((n.value, 2), np.float32)
        got = C.c_size_t()
        check(lib.kifi_volume_export(vol, k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                     n.value, C.byref(got)))
        nv, ni = C.c_size_t(), C.c_size_t()
        check(lib.kifi_pipeline_mesh_counts(pipe, C.byref(nv), C.byref(ni)))
        built, updated = C.c_longlong(), C.c_longlong()
        check(lib.kifi_pipeline_graph_stats(pipe, C.byref(built), C.byref(updated)))
        return k, v, poses, (nv.value, ni.value), (built.value, updated.value)
    finally:
        lib.kifi_pipeline_destroy(pipe)


@pytest.mark.parametrize("device_frames", [False, True])
def test_pipeline_graphs_match_plain_launches(gpu, device_frames):
    from merge_fusion_gb300 import _lib, scenes
    lib = _lib.load()
    seq = scenes.room_scene(n_frames=6, seed=5)
    k0, v0, p0, m0, _ = _run_pipeline(lib, seq, False, device_frames)
    k1, v1, p1, m1, (built, updated) = _run_pipeline(lib, seq, True, device_frames)
    assert np.array_equal(k0, k1)
    assert np.array_equal(canon_bits(v0), canon_bits(v1))
    for a, b in zip(p0, p1):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert m0 == m1
    # the first frame (no tracking) and the first tracked frame instantiate;
    # the rest update the instantiated graph in place
    assert built + updated == 6 and updated >= 3, (built, updated)


@pytest.mark.parametrize("size", [(640, 480, 585.0), (132, 97, 121.0)])
def test_host_fed_frames_equal_device_frames(gpu, size):
    """Frames fed from page-locked host memory (read by the upload kernel,
    poses taken from the ICP mailbox) give the volume, poses and mesh of the
    same frames fed from device memory.  132 x 97 uint16 is 25,608 bytes:
    the upload's 16-byte vectors leave 8 bytes for its tail."""
    from merge_fusion_gb300 import _lib, scenes
    lib = _lib.load()
    w, h, f = size
    seq = scenes.room_scene(n_frames=6, seed=8, width=w, height=h, f=f)
    k0, v0, p0, m0, _ = _run_pipeline(lib, seq, False, True)
    k1, v1, p1, m1, _ = _run_pipeline(lib, seq, False, False)
    assert np.array_equal(k0, k1)
    assert np.array_equal(canon_bits(v0), canon_bits(v1))
    for a, b in zip(p0[1:], p1[1:]):  # from the first tracked frame on
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert m0 == m1
