"""Integrator::Integrate on the GPU against the oracle (bit-exact keys and
TSDF values) and against the reference's golden digests."""
import numpy as np
import pytest

from tests.helpers import assert_volume_equal, cam_params, canon_bits, digest, posed

pytestmark = pytest.mark.gpu


def test_imrod_matches_golden_and_oracle(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    integ = kifi.Integrator()
    vols = {}
    for case in sorted(golden["cases"], key=lambda c: (tuple(c["volume"]), c["frames"])):
        key = tuple(case["volume"])
        if key not in vols:
            vols[key] = (kifi.Volume(*key), oracle_cpu.Volume(*key))
        gv, ov = vols[key]
        pose = posed(view, golden["offsets"][case["frames"] - 1])
        integ.Integrate(gv, depth, cam_params(cam), pose)
        ov.integrate(depth, cam, pose)
        keys, vals = gv.export()
        assert keys.size == case["voxels"]
        assert digest(keys) == case["keys_sha256"]
        assert digest(vals) == case["values_sha256"]
        assert_volume_equal(gv, ov, str(case["volume"]))


def test_sphere_scene_u16_matches_oracle(gpu, oracle_cpu):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.sphere_scene(n_frames=10, seed=0)
    cam = seq.camera
    for res, side, trunc in ((1024, 8.192, 0.024), (512, 8.192, 0.048), (64, 8.192, 0.4)):
        gv = kifi.Volume(res, side, trunc)
        ov = oracle_cpu.Volume(res, side, trunc)
        for i in range(len(seq.frames)):
            kifi.Integrator().Integrate(gv, seq.frames[i], cam_params(cam), seq.world_to_eye_f32(i))
            ov.integrate(seq.depth_m(i), cam, seq.world_to_eye_f32(i))
            assert_volume_equal(gv, ov, "sphere res %d frame %d" % (res, i))


def test_room_scene_matches_oracle(gpu, oracle_cpu):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.room_scene(n_frames=3, seed=1)
    cam = seq.camera
    gv = kifi.Volume(1024, 4.096, 0.02)
    ov = oracle_cpu.Volume(1024, 4.096, 0.02)
    for i in range(3):
        kifi.Integrator().Integrate(gv, seq.frames[i], cam_params(cam), seq.world_to_eye_f32(i))
        ov.integrate(seq.depth_m(i), cam, seq.world_to_eye_f32(i))
        assert_volume_equal(gv, ov, "room frame %d" % i)
    assert ov.keys.size > 500000


def test_empty_and_invalid_frames(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    gv = kifi.Volume(256, 2.0, 0.02)
    ov = oracle_cpu.Volume(256, 2.0, 0.02)
    weird = depth.copy()
    weird[::7, ::5] = np.nan
    weird[1::9, ::3] = np.inf
    weird[2::11, 1::4] = -1.0
    frames = [np.zeros_like(depth), depth, np.zeros_like(depth), weird,
              np.full_like(depth, np.nan), depth]
    for i, f in enumerate(frames):
        pose = posed(view, (0.001 * i, 0.0, -0.001 * i))
        kifi.Integrator().Integrate(gv, f, cam_params(cam), pose)
        ov.integrate(f, cam, pose)
        assert_volume_equal(gv, ov, "frame %d" % i)


def test_volume_border_and_tiny_resolutions(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    # small cubes clip the scan: splats land on / beyond every face
    for res, side in ((2, 1.0), (4, 1.0), (16, 1.2), (128, 1.0), (1024, 1.1)):
        gv = kifi.Volume(res, side, 0.02)
        ov = oracle_cpu.Volume(res, side, 0.02)
        for i in range(2):
            pose = posed(view, (0.0, 0.0, 0.3 * i))
            kifi.Integrator().Integrate(gv, depth, cam_params(cam), pose)
            ov.integrate(depth, cam, pose)
            assert_volume_equal(gv, ov, "res %d side %g" % (res, side))


def test_tail_rule_all_residues(gpu, oracle_cpu, golden):
    # The update skips the last n % 4 voxels; exercise every residue by
    # inserting 0..3 extra far-away voxels before integrating.
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    seen = set()
    for extra in range(4):
        gv = kifi.Volume(256, 2.0, 0.02)
        ov = oracle_cpu.Volume(256, 2.0, 0.02)
        keys = np.array([(255 << 20) | (255 << 10) | x for x in range(extra)], np.uint32)
        if extra:
            vals = np.tile(np.array([[0.5, 1.0]], np.float32), (extra, 1))
            gv.insert(keys, vals)
            ov.keys, ov.values = keys, vals
        kifi.Integrator().Integrate(gv, depth, cam_params(cam), view)
        ov.integrate(depth, cam, view)
        assert_volume_equal(gv, ov, "extra %d" % extra)
        seen.add(ov.keys.size % 4)
    assert seen == {0, 1, 2, 3}


def test_insert_keeps_resident_values(gpu):
    # UnitTests/util/flat_map.cpp:35-84 on the volume's map
    from merge_fusion_gb300 import kifi
    v = kifi.Volume(128, 2.0, 0.02)
    v.insert(np.array([7], np.uint32), np.array([[117, 1]], np.float32))
    v.insert(np.array([3, 7, 55], np.uint32), np.array([[449, 1], [551, 1], [666, 1]], np.float32))
    k, vals = v.export()
    assert list(k) == [3, 7, 55]
    assert list(vals[:, 0]) == [449, 117, 666]
    v.insert(np.array([7], np.uint32))
    assert v.size() == 3
    v.clear()
    assert v.size() == 0
    with pytest.raises(kifi.KifiError):
        v.insert(np.array([5, 3], np.uint32))  # not sorted
    with pytest.raises(kifi.KifiError):
        v.insert(np.array([200], np.uint32))  # x beyond the resolution


def test_capacity_growth(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    gv = kifi.Volume(1024, 4.096, 0.02, capacity=1000)
    ov = oracle_cpu.Volume(1024, 4.096, 0.02)
    for i in range(3):
        pose = posed(view, (0.004 * i, 0.0, 0.0))
        kifi.Integrator().Integrate(gv, depth, cam_params(cam), pose)
        ov.integrate(depth, cam, pose)
    assert_volume_equal(gv, ov, "grown")
