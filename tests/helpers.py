"""Shared helpers of the parity tests."""
import numpy as np


def posed(view, off):
    """kifi matrix (16,) with its translation column offset by `off`."""
    v = np.asarray(view, np.float32).copy()
    v[12:15] += np.asarray(off, np.float32)
    return v


def cam_params(cam):
    from merge_fusion_gb300.kifi import DepthSensorParams
    w, h, fx, fy, cx, cy, zn, zf = cam
    return DepthSensorParams((w, h), (fx, fy), (cx, cy), (zn, zf))


def assert_volume_equal(gpu_vol, ovol, what=""):
    k, v = gpu_vol.export()
    assert k.size == ovol.keys.size, (what, k.size, ovol.keys.size)
    assert np.array_equal(k, ovol.keys), what
    # TSDF sums and weights: bit-exact
    bad = np.nonzero(v.view(np.uint32) != ovol.values.view(np.uint32))[0]
    assert bad.size == 0, (what, bad[:8], v[bad[:4]], ovol.values[bad[:4]])
