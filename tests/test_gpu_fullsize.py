"""The benchmark's workload at full size: 640x480 frames of the room into a
1024^3 volume of 4 mm voxels.  After 24 frames (a few million voxels) the
GPU volume must equal the oracle's bit for bit; the size-independent
properties of the result -- sorted unique keys inside the volume, whole
weights no larger than the frame count, |TSDF| at most the truncation --
must hold, the mesh must equal the oracle's, and the pipeline (fusion +
tracking + periodic mesh) must leave the same volume as fusion alone."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import assert_volume_equal, cam_params, canon_bits

pytestmark = pytest.mark.gpu

W, H, F = 640, 480, 585.0
CAM = (W, H, F, F, W / 2.0, H / 2.0, 0.4, 4.0)
RES, SIDE, TRUNC = 1024, 4.096, 0.02
N = 24


def test_full_size_volume_and_properties(gpu, oracle_cpu):
    import torch
    from merge_fusion_gb300 import _lib, kifi, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    lib = _lib.load()
    dev, poses = scenes.render_room_torch(N, seed=77, width=W, height=H, f=F)
    host = dev.cpu().numpy().view(np.uint16)
    w2e = [scenes.kifi_matrix(np.linalg.inv(p)) for p in poses]
    gv = kifi.Volume(RES, SIDE, TRUNC)
    ov = oracle_cpu.Volume(RES, SIDE, TRUNC)
    for i in range(N):
        kifi.Integrator().Integrate(gv, host[i], cam_params(CAM), w2e[i])
        ov.integrate(host[i].astype(np.float32) * np.float32(0.001), CAM, w2e[i])
    assert_volume_equal(gv, ov, "room 640x480 x %d frames" % N)
    keys, vals = gv.export()
    assert keys.size > 2000000
    # properties that hold at any size
    assert np.all(keys[1:] > keys[:-1])
    x, y, z = keys & 1023, (keys >> 10) & 1023, keys >> 20
    assert x.max() < RES and y.max() < RES and z.max() < RES
    w = vals[:, 1]
    assert np.all(w >= 0) and np.all(w <= N) and np.all(w == np.round(w))
    upd = w > 0
    assert np.all(np.abs(vals[upd, 0] / w[upd]) <= np.float32(TRUNC) * (1 + 1e-6))
    verts, idx = kifi.Mesher().Mesh(gv, with_indices=True)
    assert verts.shape[0] > 100000 and idx.size % 3 == 0
    ovt, oid = ov.mesh(True)
    assert np.array_equal(canon_bits(verts), canon_bits(ovt)) and np.array_equal(idx, oid)
    # the pipeline fuses the same frames with their given poses
    d = PipelineDesc()
    d.camera = Camera(*CAM)
    d.resolution, d.side_length_m, d.truncation_m = RES, SIDE, TRUNC
    d.icp_iterations, d.mesh_every, d.mesh_with_indices, d.device = 15, 10, 1, 0
    pipe = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(pipe)), "pipeline")
    try:
        for i in range(N):
            check(lib.kifi_pipeline_integrate_device(pipe, C.c_void_p(dev[i].data_ptr()), 1,
                                                     w2e[i].ctypes.data_as(C.c_void_p)), "frame")
        check(lib.kifi_pipeline_sync(pipe, None), "sync")
        vol = lib.kifi_pipeline_volume(pipe)
        n = C.c_size_t()
        check(lib.kifi_volume_size(vol, C.byref(n)))
        pk = np.zeros(n.value + 1, np.uint32)
        pv = np.zeros((n.value + 1, 2), np.float32)
        got = C.c_size_t()
        check(lib.kifi_volume_export(vol, pk.ctypes.data_as(C.c_void_p), pv.ctypes.data_as(C.c_void_p),
                                     n.value + 1, C.byref(got)))
        assert np.array_equal(pk[:got.value], keys)
        assert np.array_equal(pv[:got.value].view(np.uint32), vals.view(np.uint32))
    finally:
        lib.kifi_pipeline_destroy(pipe)
