"""ICP::Align, the target back-projection and Renderer::Bin on the GPU
against the oracle and the reference's golden poses.

ICP tolerance: poses within 1e-5 (rotation entries ~ rad, translation m) --
association and the Horn sums follow the reference's float arithmetic, the
centroid / cross-covariance reductions run in a different (compensated,
FP64-finished) order and the eigen-solve is a double Jacobi instead of the
reference's float tred2/tqli."""
import numpy as np
import pytest

from tests.helpers import cam_params, canon_bits, posed

pytestmark = pytest.mark.gpu

POSE_TOL = 1e-5


def test_backprojection_is_bit_exact(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    from merge_fusion_gb300 import _lib
    import ctypes as C
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    e2w = oracle_cpu.invert_transform(view)
    icp = kifi.ICP()
    icp.SetTargetFromDepth(depth, cam_params(cam), e2w)
    # read the target back through an alignment-free path: align 0 iterations
    want = oracle_cpu.backproject(depth, cam, e2w)
    # round-trip check via a 1-iteration ICP on identical data must associate
    # every 4th-column pixel with itself (distance 0 < 0.01)
    pose = icp.AlignToTarget(depth, e2w, cam_params(cam), iterations=1)
    _, _, na, rms = icp.Result()
    n_src = int((depth[:, ::4] > 0).sum())
    assert na[0] == n_src
    assert rms[0] == 0.0
    assert np.abs(pose - e2w).max() < 1e-6


def test_icp_matches_golden_and_oracle(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    e2w = oracle_cpu.invert_transform(view)
    target = oracle_cpu.backproject(depth, cam, e2w)
    icp = kifi.ICP()
    for case in golden["icp"]:
        guess = posed(e2w, case["guess_offset"])
        pose = icp.Align(depth, guess, target, e2w, cam_params(cam), case["iterations"])
        ref = np.asarray(case["pose"], np.float32)
        o, od, n = oracle_cpu.icp_align(depth, cam, guess, target, e2w, case["iterations"])
        assert np.abs(pose - ref).max() < POSE_TOL, np.abs(pose - ref).max()
        assert np.abs(pose - o).max() < POSE_TOL, np.abs(pose - o).max()
        _, pd, na, rms = icp.Result()
        assert len(na) == case["iterations"] and abs(int(na[-1]) - n) <= max(3, n // 1000)


def test_icp_consecutive_frames_sphere(gpu, oracle_cpu):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.sphere_scene(n_frames=6, seed=4)
    cam = seq.camera
    icp = kifi.ICP()
    for i in range(1, 6):
        prev_e2w = seq.eye_to_world_f32(i - 1)
        icp.SetTargetFromDepth(seq.frames[i - 1], cam_params(cam), prev_e2w)
        target = oracle_cpu.backproject(seq.depth_m(i - 1), cam, prev_e2w)
        pose = icp.AlignToTarget(seq.depth_m(i), prev_e2w, cam_params(cam), iterations=10)
        o, od, n = oracle_cpu.icp_align(seq.depth_m(i), cam, prev_e2w, target, prev_e2w, 10)
        assert n > 100
        assert np.abs(pose - o).max() < POSE_TOL, (i, np.abs(pose - o).max())


def test_icp_room_frames(gpu, oracle_cpu):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.room_scene(n_frames=3, seed=2)
    cam = seq.camera
    icp = kifi.ICP()
    for i in (1, 2):
        prev = seq.eye_to_world_f32(i - 1)
        icp.SetTargetFromDepth(seq.frames[i - 1], cam_params(cam), prev)
        target = oracle_cpu.backproject(seq.depth_m(i - 1), cam, prev)
        pose = icp.AlignToTarget(seq.depth_m(i), prev, cam_params(cam), iterations=15)
        o, od, n = oracle_cpu.icp_align(seq.depth_m(i), cam, prev, target, prev, 15)
        assert n > 1000
        assert np.abs(pose - o).max() < POSE_TOL, (i, np.abs(pose - o).max())


def test_bin_is_bit_exact(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    vol = oracle_cpu.Volume(256, 2.0, 0.02)
    vol.integrate(depth, cam, view)
    verts, _ = vol.mesh(False)
    w2c = oracle_cpu.mat_mul(oracle_cpu.eye_to_clip(cam), view)
    for w, h in ((1024, 768), (640, 480), (97, 61)):
        a = kifi.Renderer().Bin(verts, w2c, w, h)
        b = oracle_cpu.bin_points(verts, w2c, w, h)
        assert np.array_equal(canon_bits(a), canon_bits(b)), (w, h)
    # duplicate points: the first one in input order wins a pixel
    pts = np.repeat(verts[:50], 3, axis=0)
    pts[1::3] += np.float32(1e-7)
    a = kifi.Renderer().Bin(pts, w2c, 640, 480)
    b = oracle_cpu.bin_points(pts, w2c, 640, 480)
    assert np.array_equal(canon_bits(a), canon_bits(b))


def test_icp_on_bin_target(gpu, oracle_cpu, golden):
    # Pipeline's intended tracking loop (Pipeline.cpp:36-55): mesh -> Bin -> ICP
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    vol = oracle_cpu.Volume(256, 2.0, 0.02)
    vol.integrate(depth, cam, view)
    verts, _ = vol.mesh(False)
    w2c = oracle_cpu.mat_mul(oracle_cpu.eye_to_clip(cam), view)
    target = kifi.Renderer().Bin(verts, w2c, 1024, 768)
    e2w = oracle_cpu.invert_transform(view)
    guess = posed(e2w, (0.004, -0.003, 0.002))
    pose = kifi.ICP().Align(depth, guess, target, e2w, cam_params(cam), 5)
    o, od, n = oracle_cpu.icp_align(depth, cam, guess, target, e2w, 5)
    assert np.abs(pose - o).max() < POSE_TOL


def test_icp_error_vs_fp64_oracle(gpu, oracle_cpu, golden):
    # The float-float Horn solve and pose accumulation against the FP64
    # reference solution of the same associations (double sums, two-pass
    # cross-covariance, double Jacobi, double pose).
    from merge_fusion_gb300 import kifi, scenes
    worst = 0.0
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    e2w = oracle_cpu.invert_transform(view)
    target = oracle_cpu.backproject(depth, cam, e2w)
    icp = kifi.ICP()
    for case in golden["icp"]:
        guess = posed(e2w, case["guess_offset"])
        icp.Align(depth, guess, target, e2w, cam_params(cam), case["iterations"])
        _, pd, _, _ = icp.Result()
        _, od, _ = oracle_cpu.icp_align(depth, cam, guess, target, e2w, case["iterations"], fp64=True)
        worst = max(worst, float(np.abs(pd - od).max()))
    seq = scenes.room_scene(n_frames=3, seed=2)
    rc = seq.camera
    for i in (1, 2):
        prev = seq.eye_to_world_f32(i - 1)
        icp.SetTargetFromDepth(seq.frames[i - 1], cam_params(rc), prev)
        tgt = oracle_cpu.backproject(seq.depth_m(i - 1), rc, prev)
        icp.AlignToTarget(seq.depth_m(i), prev, cam_params(rc), iterations=15)
        _, pd, _, _ = icp.Result()
        _, od, _ = oracle_cpu.icp_align(seq.depth_m(i), rc, prev, tgt, prev, 15, fp64=True)
        worst = max(worst, float(np.abs(pd - od).max()))
    assert worst < POSE_TOL, worst


def test_association_is_exact(gpu, oracle_cpu, golden):
    # The association of the first iteration (pose = the guess, identical on
    # both sides) must be the reference's pair for pair: same winner (first
    # strict minimum in scan order), same len^2 bits, for 640x480 targets
    # and for 512x424 ones, whose 640x480 window clamp wraps into the next
    # target row.
    from merge_fusion_gb300 import kifi, scenes
    icp = kifi.ICP()
    icp.RecordAssociations(True)
    cases = []
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    e2w = oracle_cpu.invert_transform(view)
    target = oracle_cpu.backproject(depth, cam, e2w)
    for off in ((0.0, 0.0, 0.0), (0.01, -0.006, 0.004), (-0.03, 0.02, 0.01)):
        cases.append((depth, cam, posed(e2w, off), target, e2w))
    for seq in (scenes.room_scene(n_frames=3, seed=6), scenes.sphere_scene(n_frames=3, seed=6),
                scenes.room_scene(n_frames=2, seed=7, width=512, height=424, f=365.0, scale=2.0)):
        rc = seq.camera
        for i in (1, 2):
            if i >= len(seq.frames):
                continue
            prev = seq.eye_to_world_f32(i - 1)
            tgt = oracle_cpu.backproject(seq.depth_m(i - 1), rc, prev)
            cases.append((seq.depth_m(i), rc, prev, tgt, prev))
            cases.append((seq.depth_m(i), rc, seq.eye_to_world_f32(i), tgt, prev))
    for n, (d, c, guess, tgt, se2w) in enumerate(cases):
        icp.Align(d, guess, tgt, se2w, cam_params(c), 1)
        gi, gl = icp.Associations()
        oi, ol = oracle_cpu.icp_associate(d, c, guess, tgt, se2w)
        assert gi.size == oi.size, n
        bad = np.nonzero(gi != oi)[0]
        assert bad.size == 0, (n, bad[:5], gi[bad[:5]], oi[bad[:5]], gl[bad[:5]], ol[bad[:5]])
        assert np.array_equal(gl.view(np.uint32), ol.view(np.uint32)), n
        assert (gi >= 0).sum() > 1000, n
