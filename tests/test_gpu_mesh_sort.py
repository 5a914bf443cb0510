"""Mesher::Mesh and util::radix_sort on the GPU against the oracle."""
import numpy as np
import pytest

from tests.helpers import cam_params, canon_bits, digest, posed

pytestmark = pytest.mark.gpu


def check_mesh(gv, ov, what):
    from merge_fusion_gb300 import kifi
    for wi in (False, True):
        va, ia = kifi.Mesher().Mesh(gv, with_indices=wi)
        vb, ib = ov.mesh(wi)
        assert va.shape == vb.shape, (what, wi, va.shape, vb.shape)
        assert np.array_equal(canon_bits(va), canon_bits(vb)), (what, wi)
        assert np.array_equal(ia, ib), (what, wi)


def test_mesh_matches_golden(gpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    for case in golden["cases"]:
        if "mesh_verts" not in case or case["frames"] != 1:
            continue
        gv = kifi.Volume(*case["volume"])
        kifi.Integrator().Integrate(gv, depth, cam_params(cam), view)
        v0, _ = kifi.Mesher().Mesh(gv, with_indices=False)
        v1, i1 = kifi.Mesher().Mesh(gv, with_indices=True)
        assert v0.shape[0] == case["mesh_verts_only"]
        assert digest(v0) == case["mesh_verts_only_sha256"]
        assert (v1.shape[0], i1.size) == (case["mesh_verts"], case["mesh_indices"])
        assert digest(v1) == case["mesh_verts_sha256"]
        assert digest(i1) == case["mesh_indices_sha256"]


def test_mesh_matches_oracle_multiframe(gpu, oracle_cpu, golden):
    from merge_fusion_gb300 import kifi
    depth, view, cam = golden["depth"], golden["view"], golden["camera"]
    for res, side in ((256, 2.0), (1024, 4.096), (32, 2.0)):
        gv = kifi.Volume(res, side, 0.02)
        ov = oracle_cpu.Volume(res, side, 0.02)
        for i in range(3):
            pose = posed(view, (0.003 * i, -0.002 * i, 0.001))
            kifi.Integrator().Integrate(gv, depth, cam_params(cam), pose)
            ov.integrate(depth, cam, pose)
        check_mesh(gv, ov, "res %d" % res)


def test_mesh_sphere_and_edge_cases(gpu, oracle_cpu):
    from merge_fusion_gb300 import kifi, scenes
    seq = scenes.sphere_scene(n_frames=6, seed=2)
    gv = kifi.Volume(1024, 8.192, 0.024)
    ov = oracle_cpu.Volume(1024, 8.192, 0.024)
    for i in range(6):
        kifi.Integrator().Integrate(gv, seq.frames[i], cam_params(seq.camera), seq.world_to_eye_f32(i))
        ov.integrate(seq.depth_m(i), seq.camera, seq.world_to_eye_f32(i))
    check_mesh(gv, ov, "sphere")
    # empty and single-voxel volumes produce nothing
    e = kifi.Volume(64, 1.0, 0.02)
    va, ia = kifi.Mesher().Mesh(e)
    assert va.shape == (0, 3) and ia.size == 0
    e.insert(np.array([5], np.uint32), np.array([[-0.1, 1.0]], np.float32))
    va, ia = kifi.Mesher().Mesh(e)
    assert va.shape == (0, 3)


def test_mesh_hand_built_cubes(gpu, oracle_cpu):
    # A handful of hand-placed voxels around a sign change, including the
    # volume's largest key and cubes touching the last voxel.
    from merge_fusion_gb300 import kifi
    rng = np.random.default_rng(5)

    def pack(x, y, z):
        return z << 20 | y << 10 | x
    for trial in range(20):
        pts = set()
        base = rng.integers(0, 6, 3)
        for dx in range(3):
            for dy in range(3):
                for dz in range(3):
                    if rng.random() < 0.85:
                        pts.add(pack(*(base + (dx, dy, dz))))
        keys = np.array(sorted(pts), np.uint32)
        vals = np.stack([rng.normal(0, 0.01, keys.size), rng.integers(0, 3, keys.size)], 1)
        vals = vals.astype(np.float32)
        gv = kifi.Volume(16, 1.0, 0.02)
        gv.insert(keys, vals)
        ov = oracle_cpu.Volume(16, 1.0, 0.02)
        ov.keys, ov.values = keys, vals
        check_mesh(gv, ov, "trial %d" % trial)


@pytest.mark.parametrize("n", [1, 2, 100, 2047, 2048, 2049, 100000, 3000000])
def test_radix_sort_matches_oracle(gpu, oracle_cpu, n):
    from merge_fusion_gb300 import kifi
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(kifi.radix_sort(keys), oracle_cpu.radix_sort(keys))
    small = (keys % 37).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    a = kifi.radix_sort(small, vals)
    b = oracle_cpu.radix_sort_pairs(small, vals)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
