"""The oracle's 64-bit-key fusion path (oracle/kifi_oracle_k64.c) against
its pinned 30-bit path: with b = 10 a 64-bit key is the number the 30-bit
key is, so volumes, TSDF values and meshes must agree bit for bit.  Beyond
1024 voxels per axis (b = 11, 12) the keys must decode inside the volume
and stay sorted and unique."""
import numpy as np

from tests.helpers import canon_bits, posed


def _same_volume(v64, v32, what):
    assert v64.keys.dtype == np.uint64
    assert np.array_equal(v64.keys, v32.keys.astype(np.uint64)), what
    assert np.array_equal(canon_bits(v64.values), canon_bits(v32.values)), what


def _same_mesh(v64, v32, what):
    for wi in (False, True):
        va, ia = v64.mesh(wi)
        vb, ib = v32.mesh(wi)
        assert va.shape == vb.shape, (what, wi)
        assert np.array_equal(canon_bits(va), canon_bits(vb)), (what, wi)
        assert np.array_equal(ia, ib), (what, wi)


def test_k64_equals_k30_at_b10_golden_frame(oracle_cpu, golden):
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    for res, side in ((256, 2.0), (1024, 4.096), (32, 2.0)):
        a = oracle_cpu.Volume64(res, side, 0.02)
        b = oracle_cpu.Volume(res, side, 0.02)
        assert a.b == 10
        for i in range(2):
            pose = posed(view, (0.003 * i, -0.002 * i, 0.001))
            a.integrate(depth, cam, pose)
            b.integrate(depth, cam, pose)
            _same_volume(a, b, "res %d frame %d" % (res, i))
        _same_mesh(a, b, "res %d" % res)


def test_k64_equals_k30_sphere(oracle_cpu):
    from merge_fusion_gb300 import scenes
    seq = scenes.sphere_scene(n_frames=3, seed=0)
    a = oracle_cpu.Volume64(512, 8.192, 0.048)
    b = oracle_cpu.Volume(512, 8.192, 0.048)
    for i in range(3):
        a.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
        b.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
    _same_volume(a, b, "sphere")
    _same_mesh(a, b, "sphere")


def test_k64_primitives_at_b10(oracle_cpu):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 30, 5000).astype(np.uint32)
    s64 = oracle_cpu.radix_sort64(keys.astype(np.uint64))
    assert np.array_equal(s64, np.sort(keys).astype(np.uint64))
    u = np.unique(keys)
    u = u[(u & 0x3ff) < 1023]
    u = u[((u >> 10) & 0x3ff) < 1023]
    u = u[(u >> 20) < 1023]
    assert np.array_equal(oracle_cpu.expand64(u.astype(np.uint64), 10), oracle_cpu.expand(u).astype(np.uint64))


def test_k64_beyond_1024(oracle_cpu):
    from merge_fusion_gb300 import scenes
    seq = scenes.sphere_scene(n_frames=2, seed=1)
    for res, b in ((2048, 11), (4096, 12)):
        v = oracle_cpu.Volume64(res, 8.192, 0.012)
        assert v.b == b
        for i in range(2):
            v.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
        k = v.keys
        assert k.size > 10000
        assert np.all(k[1:] > k[:-1])
        m = (1 << b) - 1
        for f in (k & m, (k >> b) & m, k >> (2 * b)):
            assert f.max() < res
        # the splat's keys are a subset of the volume
        sp = np.unique(oracle_cpu.splat64(res, 8.192, 0.012, seq.depth_m(1), seq.camera, seq.world_to_eye_f32(1)))
        assert np.isin(sp, k).all()
        verts, idx = v.mesh(True)
        assert verts.shape[0] > 1000 and idx.size % 3 == 0
