"""Pins the C restatement (oracle/kifi_oracle.c) to the reference.

* against the committed golden digests (tests/golden, made from the
  reference by tests/golden/make_golden.py) -- runs everywhere;
* against the reference's own code compiled by oracle/build_ref.py -- runs
  where that build exists (skipped otherwise).
"""
import numpy as np
import pytest

from tests.helpers import canon_bits, digest, posed


def test_oracle_matches_golden_integration_and_mesh(oracle_cpu, golden):
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    by_vol = {}
    for case in golden["cases"]:
        by_vol.setdefault(tuple(case["volume"]), []).append(case)
    for (res, side, trunc), cases in by_vol.items():
        vol = oracle_cpu.Volume(res, side, trunc)
        for case in sorted(cases, key=lambda c: c["frames"]):
            vol.integrate(depth, cam, posed(view, golden["offsets"][case["frames"] - 1]))
            assert vol.keys.size == case["voxels"], (res, case["frames"])
            assert digest(vol.keys) == case["keys_sha256"]
            assert digest(vol.values) == case["values_sha256"]
            if "mesh_verts" in case:
                v0, _ = vol.mesh(False)
                v1, i1 = vol.mesh(True)
                assert v0.shape[0] == case["mesh_verts_only"]
                assert digest(v0) == case["mesh_verts_only_sha256"]
                assert v1.shape[0] == case["mesh_verts"] and i1.size == case["mesh_indices"]
                assert digest(v1) == case["mesh_verts_sha256"]
                assert digest(i1) == case["mesh_indices_sha256"]


def test_survey_cross_check_counts(golden):
    # Volume(256, 2, 0.02) + KinectParams(640x480, Far) + one imrod frame
    c = golden["cases"][0]
    assert (c["voxels"], c["mesh_verts"], c["mesh_indices"] // 3) == (76013, 38780, 51768)


def test_oracle_icp_matches_golden(oracle_cpu, golden):
    from tests.golden.make_golden import backproject
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    e2w = oracle_cpu.invert_transform(view)
    synth = backproject(depth, view, cam)
    for case in golden["icp"]:
        guess = e2w.copy()
        guess[12:15] += np.asarray(case["guess_offset"], np.float32)
        pose, pose_d, n = oracle_cpu.icp_align(depth, cam, guess, synth, e2w, case["iterations"])
        ref = np.asarray(case["pose"], np.float32)
        # float Horn solve in the reference vs double Jacobi here: 1e-5 m / rad
        assert np.abs(pose - ref).max() < 1e-5
        assert n > 1000
        # the FP64 reference solution (double sums and N) stays within the
        # same budget of the reference's float result
        pose64, _, n64 = oracle_cpu.icp_align(depth, cam, guess, synth, e2w, case["iterations"], fp64=True)
        assert np.abs(pose64 - ref).max() < 1e-5
        assert abs(n64 - n) <= max(3, n // 1000)


def test_oracle_matches_reference_stagewise(oracle_cpu, oracle_ref, golden):
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    rng = np.random.default_rng(7)
    for res, side in ((128, 2.0), (256, 2.0), (1024, 4.096)):
        rv = oracle_ref.Volume(res, side, 0.02)
        ov = oracle_cpu.Volume(res, side, 0.02)
        for f in range(3):
            v = posed(view, rng.normal(0, 0.004, 3)) if f else view
            k1 = rv.splat(depth, cam, v)
            k2 = oracle_cpu.splat(res, side, 0.02, depth, cam, v)
            assert np.array_equal(k1, k2)
            e1 = oracle_ref.sort_unique_expand(k1)
            e2 = oracle_cpu.expand(oracle_cpu.unique(oracle_cpu.radix_sort(k2)))
            assert np.array_equal(e1, e2)
            rv.integrate(depth, cam, v)
            ov.integrate(depth, cam, v)
            rk, rvals = rv.export()
            assert np.array_equal(rk, ov.keys)
            assert np.array_equal(canon_bits(rvals), canon_bits(ov.values))
        for wi in (False, True):
            va, ia = rv.mesh(wi)
            vb, ib = ov.mesh(wi)
            assert np.array_equal(canon_bits(va), canon_bits(vb))
            assert np.array_equal(ia, ib)


def test_oracle_matches_reference_primitives(oracle_cpu, oracle_ref):
    rng = np.random.default_rng(11)
    keys = rng.integers(0, 2**32, 20000, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(oracle_cpu.radix_sort(keys), oracle_ref.radix_sort(keys))
    vals = np.arange(keys.size, dtype=np.uint32)
    small = (keys % 97).astype(np.uint32)
    a = oracle_cpu.radix_sort_pairs(small, vals)
    b = oracle_ref.radix_sort_pairs(small, vals)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    x = rng.normal(size=1000).astype(np.float32)
    assert oracle_cpu.kahan_sum(x) == oracle_ref.kahan_sum(x)
    assert list(oracle_ref.partial_sum_exclusive([1, 3, 3, 7, 0])) == [0, 1, 4, 7, 14]
    k1 = np.unique(rng.integers(0, 200, 50)).astype(np.int32)
    k2 = np.unique(rng.integers(0, 200, 70)).astype(np.int32)
    v1 = rng.integers(-9, 9, k1.size).astype(np.int32)
    v2 = rng.integers(-9, 9, k2.size).astype(np.int32)
    a = oracle_cpu.set_union(k1, v1, k2, v2)
    b = oracle_ref.set_union(k1, v1, k2, v2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_oracle_matches_reference_synthetic_scenes(oracle_cpu, oracle_ref):
    from merge_fusion_gb300 import scenes
    seq = scenes.sphere_scene(n_frames=4, seed=3)
    cam = seq.camera
    for res, side, trunc in ((1024, 8.192, 0.024), (256, 8.192, 0.064)):
        rv = oracle_ref.Volume(res, side, trunc)
        ov = oracle_cpu.Volume(res, side, trunc)
        for i in range(4):
            rv.integrate(seq.depth_m(i), cam, seq.world_to_eye_f32(i))
            ov.integrate(seq.depth_m(i), cam, seq.world_to_eye_f32(i))
        rk, rvals = rv.export()
        assert np.array_equal(rk, ov.keys)
        assert np.array_equal(canon_bits(rvals), canon_bits(ov.values))
        va, ia = rv.mesh(True)
        vb, ib = ov.mesh(True)
        assert np.array_equal(canon_bits(va), canon_bits(vb)) and np.array_equal(ia, ib)


def test_oracle_icp_matches_reference_on_sphere(oracle_cpu, oracle_ref):
    from merge_fusion_gb300 import scenes
    from tests.golden.make_golden import backproject
    seq = scenes.sphere_scene(n_frames=3, seed=5, width=640, height=480)
    cam = seq.camera
    target = backproject(seq.depth_m(0), seq.world_to_eye_f32(0), cam)
    guess = seq.eye_to_world_f32(0)  # previous pose as the initial guess
    r = oracle_ref.icp_align(seq.depth_m(1), cam, guess, target, seq.eye_to_world_f32(0), 10)
    o, od, n = oracle_cpu.icp_align(seq.depth_m(1), cam, guess, target, seq.eye_to_world_f32(0), 10)
    assert n > 100
    assert np.abs(r - o).max() < 1e-5


def test_oracle_bin_matches_reference(oracle_cpu, oracle_ref, golden):
    # Renderer::Bin of the fixture's mesh vertices through the frame's camera,
    # into the 1024x768 buffer Pipeline uses (Pipeline.cpp:48-52)
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    vol = oracle_cpu.Volume(256, 2.0, 0.02)
    vol.integrate(depth, cam, view)
    verts, _ = vol.mesh(False)
    w2c = oracle_cpu.mat_mul(oracle_cpu.eye_to_clip(cam), view)
    for w, h in ((1024, 768), (640, 480), (97, 61)):
        a = oracle_cpu.bin_points(verts, w2c, w, h)
        b = oracle_ref.bin_points(verts, w2c, w, h)
        assert np.array_equal(canon_bits(a), canon_bits(b))
        assert (a != 0).any()


def test_oracle_icp_on_bin_target_matches_reference(oracle_cpu, oracle_ref, golden):
    # the reference's intended pipeline (Pipeline.cpp:36-55): mesh -> Bin -> ICP
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    vol = oracle_cpu.Volume(256, 2.0, 0.02)
    vol.integrate(depth, cam, view)
    verts, _ = vol.mesh(False)
    w2c = oracle_cpu.mat_mul(oracle_cpu.eye_to_clip(cam), view)
    target = oracle_cpu.bin_points(verts, w2c, 1024, 768)
    e2w = oracle_cpu.invert_transform(view)
    guess = posed(e2w, (0.004, -0.003, 0.002))
    r = oracle_ref.icp_align(depth, cam, guess, target, e2w, 5)
    o, od, n = oracle_cpu.icp_align(depth, cam, guess, target, e2w, 5)
    assert n > 100
    assert np.abs(r - o).max() < 1e-5
