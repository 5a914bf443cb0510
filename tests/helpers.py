"""Shared helpers of the parity tests."""
import numpy as np


def canon_bits(a):
    """uint32 view of a float32 array with every NaN replaced by 0x7FC00000.

    NaN payloads are platform detail (x86 SSE returns 0xFFC00000 for 0/0, Arm
    0x7FC00000, the GPU 0x7FFFFFFF); parity is on the position of NaNs and
    on every other bit."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).copy()
    b[np.isnan(a)] = 0x7FC00000
    return b


def digest(a):
    import hashlib
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = canon_bits(a)
    return hashlib.sha256(a.tobytes()).hexdigest()


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
    bad = np.nonzero((canon_bits(v) != canon_bits(ovol.values)).any(1))[0]
    assert bad.size == 0, (what, bad[:8], v[bad[:4]], ovol.values[bad[:4]])
