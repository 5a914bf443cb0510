"""kifi::Pipeline's tracking path (Pipeline.cpp:36-55) on the GPU: from the
second frame on, ICP aligns the frame against the Bin of the model's mesh
(1024 x 768, through EyeToClipRH * worldToEye), starting from the previous
tracked pose; the frame is fused with the tracked pose; the volume is meshed
(vertices only) and binned for the next frame.

The oracle runs the same loop on the CPU.  Fed the GPU's tracked poses, it
must produce a bit-identical volume and mesh, and its ICP from the same
target and guess must land within 1e-5 of the GPU's pose (the reference
solves Horn's problem in float, the GPU in float-float).  Run on its own
poses, its trajectory stays within a small bound of the GPU's."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import cam_params, canon_bits

pytestmark = pytest.mark.gpu

ICP_ITERS = 15
TARGET_W, TARGET_H = 1024, 768  # Pipeline.cpp:50


def make_pipeline(lib, cam, closed_loop=1, mesh_every=0):
    from merge_fusion_gb300._lib import PipelineDesc, check
    d = PipelineDesc()
    d.camera = cam_params(cam).camera()
    d.resolution, d.side_length_m, d.truncation_m = 1024, 4.096, 0.02
    d.icp_iterations, d.mesh_every, d.mesh_with_indices = ICP_ITERS, mesh_every, 1
    d.device = 0
    d.closed_loop = closed_loop
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)))
    return pipe


def export(lib, pipe):
    from merge_fusion_gb300._lib import check
    check(lib.kifi_pipeline_sync(pipe, None))
    vol = lib.kifi_pipeline_volume(pipe)
    n = C.c_size_t()
    check(lib.kifi_volume_size(vol, C.byref(n)))
    k = np.zeros(n.value + 1, np.uint32)
    v = np.zeros((n.value + 1, 2), np.float32)
    got = C.c_size_t()
    check(lib.kifi_volume_export(vol, k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                 n.value + 1, C.byref(got)))
    return k[:got.value], v[:got.value]


def oracle_target(oc, ov, cam, e2w):
    """Mesher::Mesh(verts) of the oracle volume, binned through
    EyeToClipRH * inverse(e2w) into the 1024 x 768 target."""
    verts, _ = ov.mesh(False)
    w2c = oc.mat_mul(oc.eye_to_clip(cam), oc.invert_transform(e2w))
    return oc.bin_points(verts, w2c, TARGET_W, TARGET_H)


def run_gpu(lib, seq, n):
    from merge_fusion_gb300._lib import check
    pipe = make_pipeline(lib, seq.camera)
    poses = []
    out = np.zeros(16, np.float32)
    try:
        for i in range(n):
            frame = np.ascontiguousarray(seq.frames[i])
            w2e = seq.world_to_eye_f32(i)
            check(lib.kifi_pipeline_integrate(pipe, frame.ctypes.data_as(C.c_void_p), 1,
                                              w2e.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)),
                  "frame %d" % i)
            poses.append(out.copy())
        keys, vals = export(lib, pipe)
    finally:
        lib.kifi_pipeline_destroy(pipe)
    return poses, keys, vals


def test_closed_loop_equals_oracle_stage_by_stage(gpu, oracle_cpu):
    """The oracle fed the GPU's poses: ICP within 1e-5, volume bit-exact."""
    from merge_fusion_gb300 import _lib, scenes
    lib = _lib.load()
    oc = oracle_cpu
    n = 5
    seq = scenes.room_scene(n_frames=n, seed=11)
    cam = seq.camera
    poses, keys, vals = run_gpu(lib, seq, n)
    # the first pose is the caller's
    assert np.array_equal(poses[0], oc.invert_transform(seq.world_to_eye_f32(0)))
    ov = oc.Volume(1024, 4.096, 0.02)
    worst = 0.0
    for i in range(n):
        if i > 0:
            target = oracle_target(oc, ov, cam, poses[i - 1])
            want, _, na = oc.icp_align(seq.depth_m(i), cam, poses[i - 1], target, poses[i - 1], ICP_ITERS)
            assert na > 1000, (i, na)
            err = float(np.abs(poses[i] - want).max())
            worst = max(worst, err)
            assert err < 1e-5, (i, err)
        ov.integrate(seq.depth_m(i), cam, oc.invert_transform(poses[i]))
    assert keys.size == ov.keys.size and keys.size > 100000
    assert np.array_equal(keys, ov.keys)
    assert np.array_equal(canon_bits(vals), canon_bits(ov.values))
    print("closed loop: %d voxels, worst pose difference %.2e" % (keys.size, worst))


def test_closed_loop_free_running_trajectory(gpu, oracle_cpu):
    """The oracle's own closed loop (its float poses feeding its own fusion)
    against the GPU's: the two trajectories stay close, and both track the
    ground truth the scene was rendered with."""
    from merge_fusion_gb300 import _lib, scenes
    lib = _lib.load()
    oc = oracle_cpu
    n = 5
    seq = scenes.room_scene(n_frames=n, seed=12)
    cam = seq.camera
    poses, _, _ = run_gpu(lib, seq, n)
    ov = oc.Volume(1024, 4.096, 0.02)
    e2w = oc.invert_transform(seq.world_to_eye_f32(0))
    diffs, truth = [], []
    for i in range(n):
        if i > 0:
            target = oracle_target(oc, ov, cam, e2w)
            e2w, _, _ = oc.icp_align(seq.depth_m(i), cam, e2w, target, e2w, ICP_ITERS)
        ov.integrate(seq.depth_m(i), cam, oc.invert_transform(e2w))
        diffs.append(float(np.abs(poses[i] - e2w).max()))
        truth.append(float(np.abs(poses[i] - seq.eye_to_world_f32(i)).max()))
    print("free-running pose differences GPU vs oracle:", ["%.1e" % d for d in diffs],
          "GPU vs ground truth:", ["%.1e" % t for t in truth])
    # Each frame's ICP differs by ~1e-7 (float vs float-float Horn solve);
    # the difference moves the fused TSDF, hence the mesh and the next
    # target, and grows along the loop (1.5e-6 after one frame, ~1e-4 after
    # four on this scene): the bound is on that growth, not on one step.
    assert diffs[1] < 1e-5 and max(diffs) < 1e-3, diffs
    assert max(truth) < 5e-2, truth


def test_closed_loop_rejects_graphs_and_bad_mode(gpu):
    from merge_fusion_gb300 import _lib, scenes
    from merge_fusion_gb300._lib import PipelineDesc
    lib = _lib.load()
    seq = scenes.sphere_scene(n_frames=1, seed=0)
    pipe = make_pipeline(lib, seq.camera)
    try:
        assert lib.kifi_pipeline_set_graphs(pipe, 1) == _lib.KIFI_ERR_UNSUPPORTED
        assert lib.kifi_pipeline_set_graphs(pipe, 0) == 0
    finally:
        lib.kifi_pipeline_destroy(pipe)
    d = PipelineDesc()
    d.camera = cam_params(seq.camera).camera()
    d.resolution, d.side_length_m, d.truncation_m = 512, 8.192, 0.048
    d.closed_loop = 2
    h = C.c_void_p()
    assert lib.kifi_pipeline_create(C.byref(d), C.byref(h)) == _lib.KIFI_ERR_INVALID_ARGUMENT
