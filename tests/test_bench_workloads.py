"""The workloads the bench measures, checked on the CPU: the batched scene mix
(frame sizes, voxel sizes, truncation, trajectory lengths), its playback
order, the single-scene playback, and that both bench arms name the same
workload."""
import numpy as np

import bench
from merge_fusion_gb300 import batched


def test_batched_scene_mix():
    specs = batched.scene_specs(64, 7)
    assert len(specs) == 64
    sizes = {(w, h) for w, h, _ in batched.SIZES}
    assert sizes == {(320, 240), (512, 424), (640, 480), (1024, 848)}
    for s in specs:
        assert (s["width"], s["height"]) in sizes
        assert s["voxel_mm"] in (2, 4, 8)
        # a 4.096 m cube at every voxel size
        assert s["res"] * s["voxel_mm"] == 4096
        assert 50 <= s["frames"] <= 300
    # every size and voxel size occurs, and the draw is seeded
    assert {(s["width"], s["height"]) for s in specs} == sizes
    assert {s["voxel_mm"] for s in specs} == {2, 4, 8}
    assert specs == batched.scene_specs(64, 7)
    assert specs != batched.scene_specs(64, 8)
    # seeds are distinct per scene
    assert len({s["seed"] for s in specs}) == 64


def test_batched_descriptions_truncate_at_five_voxels():
    for s in batched.scene_specs(16, 3):
        d = batched._desc(s, 15, 0)
        vox = s["voxel_mm"] * 1e-3
        assert np.isclose(d.truncation_m, 5 * vox) and np.isclose(d.side_length_m, s["res"] * vox)
        assert d.camera.width == s["width"] and d.camera.height == s["height"]
        assert d.icp_iterations == 15 and d.mesh_every == 0


def test_frame_order_plays_forward_and_back():
    assert batched.frame_order(4, 10) == [0, 1, 2, 3, 2, 1, 0, 1, 2, 3]
    assert batched.frame_order(1, 3) == [0, 0, 0]
    order = batched.frame_order(40, 300)
    assert len(order) == 300 and max(order) == 39 and min(order) == 0


def test_bench_playback_and_config():
    seq = [bench.playback(t) for t in range(700)]
    assert seq[:300] == list(range(300))
    assert seq[300:598] == list(range(298, 0, -1))
    assert seq[598] == 0 and seq[599] == 1
    cfg = bench.workload_config(100, bench.FRAMES_PER_STEP)
    assert cfg["workload"] == bench.WORKLOAD and cfg["prefill_frames"] == 100
    assert cfg["frames_per_step"] == bench.MESH_EVERY
    # kernels per frame and per mesh that the bench counts as gpu_launches
    assert bench.LAUNCHES_FUSION == 7 and bench.LAUNCHES_MESH == 8
    assert bench.LAUNCHES_TRACKING == bench.ICP_ITERS + 2
