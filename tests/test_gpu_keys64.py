"""Volumes with 64-bit voxel keys on the GPU.

Up to 1024 voxels per axis a 64-bit key (b = 10) is the number the
reference's 30-bit key is, so a volume forced to 64-bit keys must equal the
pinned 30-bit oracle bit for bit.  Beyond that (2048 and 4096 voxels per
axis) the GPU is checked against the oracle's 64-bit path, which the CPU
tests tie to the 30-bit one."""
import os

import numpy as np
import pytest

from tests.helpers import assert_volume_equal, cam_params, canon_bits, posed

pytestmark = pytest.mark.gpu


def check_mesh(gv, ov, what):
    from merge_fusion_gb300 import kifi
    for wi in (False, True):
        va, ia = kifi.Mesher().Mesh(gv, with_indices=wi)
        vb, ib = ov.mesh(wi)
        assert va.shape == vb.shape, (what, wi, va.shape, vb.shape)
        assert np.array_equal(canon_bits(va), canon_bits(vb)), (what, wi)
        assert np.array_equal(ia, ib), (what, wi)


def test_forced_64bit_keys_equal_30bit_oracle(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    for res, side in ((256, 2.0), (1024, 4.096)):
        gv = kifi.Volume(res, side, 0.02, key_bits=64)
        assert (gv.key_bits, gv.bits_per_axis) == (64, 10)
        ov = oracle_cpu.Volume(res, side, 0.02)
        for i in range(3):
            pose = posed(view, (0.003 * i, -0.002 * i, 0.001))
            kifi.Integrator().Integrate(gv, depth, cam_params(cam), pose)
            ov.integrate(depth, cam, pose)
            k64, v = gv.export()
            assert k64.dtype == np.uint64
            assert np.array_equal(k64, ov.keys.astype(np.uint64)), (res, i)
            assert np.array_equal(canon_bits(v), canon_bits(ov.values)), (res, i)
            k32, _ = gv.export(key_bits=32)  # b = 10: the narrow read-back works
            assert np.array_equal(k32, ov.keys)
        check_mesh(gv, ov, "forced 64-bit res %d" % res)


@pytest.mark.parametrize("res,b", [(2048, 11), (4096, 12)])
def test_large_volume_matches_64bit_oracle(gpu, oracle_cpu, res, b):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.sphere_scene(n_frames=4, seed=3)
    side, trunc = 8.192, 5 * 8.192 / res
    gv = kifi.Volume(res, side, trunc)
    assert (gv.key_bits, gv.bits_per_axis) == (64, b)
    ov = oracle_cpu.Volume64(res, side, trunc)
    for i in range(4):
        kifi.Integrator().Integrate(gv, seq.frames[i], cam_params(seq.camera), seq.world_to_eye_f32(i))
        ov.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
        assert_volume_equal(gv, ov, "res %d frame %d" % (res, i))
    with pytest.raises(Exception):
        gv.export(key_bits=32)  # b > 10: keys do not fit 32 bits
    check_mesh(gv, ov, "res %d" % res)


def test_large_volume_room_frames(gpu, oracle_cpu):
    # 512x424 frames of the 8 x 3 x 8 m room at 2 mm (4096 voxels per axis)
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.room_scene(n_frames=2, seed=4, width=512, height=424, f=365.0, scale=2.0)
    gv = kifi.Volume(4096, 8.192, 0.01)
    ov = oracle_cpu.Volume64(4096, 8.192, 0.01)
    for i in range(2):
        kifi.Integrator().Integrate(gv, seq.frames[i], cam_params(seq.camera), seq.world_to_eye_f32(i))
        ov.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
    assert_volume_equal(gv, ov, "room 4096")
    assert ov.keys.size > 1000000


def test_radix_sort_u64(gpu):
    from merge_fusion_gb300 import kifi
    rng = np.random.default_rng(9)
    for n in (0, 1, 7, 4097, 300001):
        k = rng.integers(0, 1 << 63, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << 63)
        out = kifi.radix_sort(k)
        assert np.array_equal(out, np.sort(k))
        v = np.arange(n, dtype=np.uint32)
        ko, vo = kifi.radix_sort(k, v)
        order = np.argsort(k, kind="stable")
        assert np.array_equal(ko, k[order]) and np.array_equal(vo, v[order])
    # duplicates keep their order (stable)
    k = rng.integers(0, 16, 100000).astype(np.uint64) << 40
    ko, vo = kifi.radix_sort(k, np.arange(k.size, dtype=np.uint32))
    assert np.array_equal(vo, np.argsort(k, kind="stable").astype(np.uint32))


def test_insert_export_checkpoint_64bit(gpu, tmp_path):
    from merge_fusion_gb300 import kifi
    res, b = 4096, 12
    rng = np.random.default_rng(11)
    xyz = rng.integers(0, res, (5000, 3)).astype(np.uint64)
    keys = np.unique(xyz[:, 2] << (2 * b) | xyz[:, 1] << b | xyz[:, 0])
    vals = rng.standard_normal((keys.size, 2)).astype(np.float32)
    gv = kifi.Volume(res, 8.192, 0.01)
    gv.insert(keys, vals)
    k, v = gv.export()
    assert np.array_equal(k, keys) and np.array_equal(canon_bits(v), canon_bits(vals))
    # a second insert: resident voxels keep their value
    more = np.unique(np.concatenate([keys[::3], keys[-1:] + 1]))
    gv.insert(more, np.zeros((more.size, 2), np.float32))
    k2, v2 = gv.export()
    ref = np.union1d(keys, more)
    assert np.array_equal(k2, ref)
    pos = np.searchsorted(ref, keys)
    assert np.array_equal(canon_bits(v2[pos]), canon_bits(vals))
    # keys outside the volume are refused
    with pytest.raises(Exception):
        gv.insert(np.array([np.uint64(res) << np.uint64(2 * b)], np.uint64))
    path = os.path.join(str(tmp_path), "v64.kvol")
    gv.save(path)
    lv = kifi.Volume.load(path)
    assert (lv.key_bits, lv.bits_per_axis) == (64, b)
    k3, v3 = lv.export()
    assert np.array_equal(k3, k2) and np.array_equal(canon_bits(v3), canon_bits(v2))


def test_pipeline_with_64bit_keys(gpu):
    # the live path (fusion + ICP + periodic mesh) on a 2048-voxel cube
    import ctypes as C
    from merge_fusion_gb300 import _lib, scenes
    from merge_fusion_gb300._lib import Camera, PipelineDesc, check
    lib = _lib.load()
    seq = scenes.room_scene(n_frames=6, seed=5, width=320, height=240, f=292.5)
    d = PipelineDesc()
    d.camera = Camera(320, 240, 292.5, 292.5, 160.0, 120.0, 0.4, 4.0)
    d.resolution, d.side_length_m, d.truncation_m = 2048, 8.192, 0.02
    d.icp_iterations, d.mesh_every, d.mesh_with_indices, d.device = 5, 3, 1, 0
    p = C.c_void_p()
    check(lib.kifi_pipeline_create(C.byref(d), C.byref(p)), "pipeline")
    try:
        import torch
        for i in range(6):
            m = seq.world_to_eye_f32(i)
            fr = torch.as_tensor(seq.frames[i]).cuda()
            check(lib.kifi_pipeline_integrate_device(p, C.c_void_p(fr.data_ptr()), 1, m.ctypes.data_as(C.c_void_p)),
                  "frame")
        check(lib.kifi_pipeline_sync(p, None), "sync")
        n = C.c_size_t()
        check(lib.kifi_volume_size(lib.kifi_pipeline_volume(p), C.byref(n)))
        assert n.value > 100000
    finally:
        lib.kifi_pipeline_destroy(p)
