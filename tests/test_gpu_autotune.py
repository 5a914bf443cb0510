"""kifi_volume_autotune: tuning leaves the volume untouched, every tuned
launch shape gives bit-identical results, and choices are cached.
kifi_volume_set_launch_mode: both launch shapes (and merge builds) give
bit-identical volumes."""
import os

import numpy as np
import pytest

from tests.helpers import cam_params

pytestmark = pytest.mark.gpu


def test_autotune_is_invisible_and_cached(gpu, golden, tmp_path):
    import torch
    from merge_fusion_gb300 import kifi
    cache = tmp_path / "autotune.txt"
    os.environ["KIFI_AUTOTUNE_CACHE"] = str(cache)
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    params = cam_params(cam)
    a = kifi.Volume(256, 2.0, 0.02)
    b = kifi.Volume(256, 2.0, 0.02)
    for v in (a, b):
        kifi.Integrator().Integrate(v, depth, params, view)
    shifted = view.copy()
    shifted[12] += np.float32(0.013)
    d = torch.from_numpy(np.ascontiguousarray(depth, np.float32)).cuda()
    torch.cuda.synchronize()
    k0, v0 = a.export()
    shape = a.autotune(d.data_ptr(), False, params, shifted, force=True)
    assert min(shape.values()) > 0
    k1, v1 = a.export()
    assert np.array_equal(k0, k1) and np.array_equal(v0.view(np.uint32), v1.view(np.uint32))
    for v in (a, b):
        kifi.Integrator().Integrate(v, depth, params, shifted)
    ka, va = a.export()
    kb, vb = b.export()
    assert np.array_equal(ka, kb) and np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    # cached: the same choice without measuring, and written to the file
    assert b.autotune(d.data_ptr(), False, params, shifted) == shape
    assert cache.exists() and len(cache.read_text().split()) == 5


def test_launch_modes_give_identical_volumes(gpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    params = cam_params(cam)
    shifted = view.copy()
    shifted[12] += np.float32(0.013)
    vols = [kifi.Volume(256, 2.0, 0.02) for _ in range(2)]
    vols[0].set_launch_mode(True)
    vols[1].set_launch_mode(False)
    for v in vols:
        for w2e in (view, shifted, view):
            kifi.Integrator().Integrate(v, depth, params, w2e)
    ka, va = vols[0].export()
    kb, vb = vols[1].export()
    assert ka.size > 0
    assert np.array_equal(ka, kb) and np.array_equal(va.view(np.uint32), vb.view(np.uint32))
