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


def _pipeline_alone(lib, spec, frames, w2e, iters):
    """The scene through kifi_pipeline (open loop, no mesh): volume and last pose."""
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    d = PipelineDesc()
    w, h, f = spec["width"], spec["height"], spec["f"]
    d.camera = Camera(w, h, f, f, w / 2.0, h / 2.0, 0.4, 4.0)
    vox = spec["voxel_mm"] * 1e-3
    d.resolution, d.side_length_m, d.truncation_m = spec["res"], spec["res"] * vox, 5 * vox
    d.icp_iterations, d.mesh_every, d.mesh_with_indices, d.device = iters, 0, 0, 0
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)))
    try:
        for i in range(len(frames)):
            check(lib.kifi_pipeline_integrate_device(pipe, C.c_void_p(frames[i].data_ptr()), 1,
                                                     w2e[i].ctypes.data_as(C.c_void_p)))
        return _export(lib, pipe)
    finally:
        lib.kifi_pipeline_destroy(pipe)


@pytest.mark.parametrize("queue_ctas", [0, 1, 2])
def test_batch_launches_equal_single_pipelines(gpu, queue_ctas):
    """kifi_batch (one launch per stage for all scenes, CTAs shared out by
    block maps; or, queue_ctas > 0, the persistent fusion launch over a device
    work queue with that many CTAs per SM): every scene's volume and tracked
    pose equal the scene run alone through kifi_pipeline -- 32- and 64-bit
    keys, three frame sizes, scenes of different lengths (a scene sits out the
    steps after its end)."""
    import torch
    from merge_fusion_gb300 import _lib, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    lib = _lib.load()
    iters = 10
    specs = [{"seed": 21, "width": 320, "height": 240, "f": 292.5, "voxel_mm": 8, "res": 512, "frames": 6},
             {"seed": 22, "width": 512, "height": 424, "f": 365.0, "voxel_mm": 4, "res": 1024, "frames": 4},
             {"seed": 23, "width": 640, "height": 480, "f": 585.0, "voxel_mm": 2, "res": 2048, "frames": 5}]
    data = []
    for s in specs:
        fr, poses = scenes.render_room_torch(s["frames"], seed=s["seed"], width=s["width"], height=s["height"],
                                             f=s["f"], device="cuda")
        data.append((fr, [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]))
    descs = (PipelineDesc * len(specs))()
    for d, s in zip(descs, specs):
        w, h, f = s["width"], s["height"], s["f"]
        d.camera = Camera(w, h, f, f, w / 2.0, h / 2.0, 0.4, 4.0)
        vox = s["voxel_mm"] * 1e-3
        d.resolution, d.side_length_m, d.truncation_m = s["res"], s["res"] * vox, 5 * vox
        d.icp_iterations, d.device = iters, 0
    b = C.c_void_p()
    check(lib.kifi_batch_create(descs, len(specs), C.byref(b)))
    try:
        check(lib.kifi_batch_set_persistent(b, 1 if queue_ctas else 0, queue_ctas))
        check(lib.kifi_batch_set_profiling(b, 1))
        steps = max(s["frames"] for s in specs)
        for t in range(steps):
            ptrs = (C.c_void_p * len(specs))()
            poses = np.zeros((len(specs), 16), np.float32)
            for i, (s, (fr, w2e)) in enumerate(zip(specs, data)):
                if t < s["frames"]:
                    ptrs[i] = fr[t].data_ptr()
                    poses[i] = w2e[t]
            check(lib.kifi_batch_step_device(b, ptrs, poses.ctypes.data_as(C.c_void_p)), "step %d" % t)
        check(lib.kifi_batch_sync(b))
        times = np.zeros(64, np.float32)
        n = C.c_int()
        check(lib.kifi_batch_step_times(b, times.ctypes.data_as(C.c_void_p), 64, C.byref(n)))
        assert n.value == steps and (times[:steps] > 0).all()
        for i, (s, (fr, w2e)) in enumerate(zip(specs, data)):
            vol = lib.kifi_batch_volume(b, i)
            nv = C.c_size_t()
            check(lib.kifi_volume_size(vol, C.byref(nv)))
            k = np.zeros(nv.value + 1, np.uint64)
            v = np.zeros((nv.value + 1, 2), np.float32)
            got = C.c_size_t()
            check(lib.kifi_volume_export64(vol, k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                           nv.value + 1, C.byref(got)))
            pose = np.zeros(16, np.float32)
            check(lib.kifi_batch_pose(b, i, pose.ctypes.data_as(C.c_void_p)))
            kb, vb, pb = _pipeline_alone(lib, s, fr, w2e, iters)
            assert got.value == kb.size and kb.size > 1000, (i, got.value, kb.size)
            assert np.array_equal(k[:got.value], kb)
            assert np.array_equal(v[:got.value].view(np.uint32), vb.view(np.uint32))
            assert np.array_equal(pose.view(np.uint32), pb.view(np.uint32)), (i, np.abs(pose - pb).max())
    finally:
        lib.kifi_batch_destroy(b)
    torch.cuda.synchronize()


def test_batch_rejects_what_it_does_not_run(gpu):
    from merge_fusion_gb300 import _lib
    from merge_fusion_gb300._lib import Camera, PipelineDesc
    lib = _lib.load()
    descs = (PipelineDesc * 2)()
    for d in descs:
        d.camera = Camera(320, 240, 292.5, 292.5, 160.0, 120.0, 0.4, 4.0)
        d.resolution, d.side_length_m, d.truncation_m = 512, 4.096, 0.04
    descs[1].mesh_every = 10
    b = C.c_void_p()
    assert lib.kifi_batch_create(descs, 2, C.byref(b)) == _lib.KIFI_ERR_UNSUPPORTED
    descs[1].mesh_every = 0
    descs[1].device = 7
    assert lib.kifi_batch_create(descs, 2, C.byref(b)) == _lib.KIFI_ERR_INVALID_ARGUMENT
