"""A short run of the large-volume precision study (tests/precision_study.py):
64-bit-key fusion equal to the oracle bit for bit, and the GPU's ICP within
FP64-class error of the oracle's FP64 run, frame by frame and along the
tracking chain."""
import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_short(gpu, oracle_cpu):
    from tests import precision_study
    r = precision_study.run(frames=5, tsdf_frames=3, chain_frames=5, workers=2)
    t = r["tsdf_vs_oracle64"]
    assert t["keys_equal"] and t["values_bit_different"] == 0, t
    assert t["voxels_gpu"] > 1000000
    icp = r["icp_per_frame_vs_fp64"]
    assert icp["frames"] == 4
    assert icp["max_abs_pose_element"] < 1e-9, icp
    assert icp["float_pose_vs_reference_float_max_abs"] < 1e-5, icp
    last = r["drift"][-1]
    assert last["frame"] == 5
    assert last["gpu_vs_fp64_m"] < 1e-6 and last["gpu_vs_fp64_deg"] < 1e-5, last
