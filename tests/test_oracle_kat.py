"""Known-answer tests of the oracle, ported from the reference's own unit
tests (KinectFission/UnitTests), plus the C restatement's primitives."""
import numpy as np
import pytest


def test_set_union_kat(oracle_cpu):
    # UnitTests/util/algorithm.cpp:47-125
    k, v = oracle_cpu.set_union([0], [-1], [1], [7])
    assert list(k) == [0, 1] and list(v) == [-1, 7]
    k, v = oracle_cpu.set_union([7], [-1], [7], [3])
    assert list(k) == [7] and list(v) == [-1]
    k, v = oracle_cpu.set_union([0, 1, 3, 55], [4, 9, 0, 27], [0, 5, 27, 55, 88], [3, 1, 17, 0, 7])
    assert list(k) == [0, 1, 3, 5, 27, 55, 88]
    assert list(v) == [4, 9, 0, 1, 17, 27, 7]


def test_radix_sort_kat(oracle_cpu):
    # UnitTests/util/algorithm.cpp:15-45: 100 random keys sort ascending, pairs follow
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 2**31, 100, dtype=np.uint32)
    s = oracle_cpu.radix_sort(keys)
    assert np.array_equal(s, np.sort(keys))
    k, v = oracle_cpu.radix_sort_pairs(keys, keys)
    assert np.array_equal(k, v) and np.array_equal(k, np.sort(keys))


def test_radix_sort_pairs_is_stable(oracle_cpu):
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 16, 5000, dtype=np.uint32)
    k, v = oracle_cpu.radix_sort_pairs(keys, np.arange(keys.size, dtype=np.uint32))
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(v, order)


def test_kahan_sum_kat(oracle_cpu):
    # UnitTests/util/numeric.cpp:12-43: 1e5 x 1e-9 within 0.01%
    x = np.full(100000, 1e-9, np.float32)
    assert abs(oracle_cpu.kahan_sum(x) - 1e-4) / 1e-4 < 1e-4


def test_volume_geometry_kat(oracle_cpu):
    # UnitTests/Volume.cpp:13-39: res 128 over 2 m; voxel (33,21,92) center -> index +0.5
    g = oracle_cpu.geom(128, 2.0, 0.02)
    assert np.float32(g.vlen) == np.float32(2.0) / np.float32(128)
    for i in (33, 21, 92):
        c = np.float32(i) * np.float32(g.vlen) + np.float32(g.center_off)
        idx = c * np.float32(g.vlen_inv) + np.float32(g.index_off)
        assert abs(idx - (i + 0.5)) < 1e-3 * (i + 0.5)


def test_voxel_update_kat():
    # UnitTests/Voxel.cpp:11-40: 1.0 + 3 x 0.333 over 4 updates averages ~0.5
    d, w = np.float32(0), np.float32(0)
    for x in (1.0, 0.333, 0.333, 0.333):
        d, w = d + np.float32(x), w + np.float32(1)
    assert w == 4 and abs(d / w - 0.5) / 0.5 < 1e-3


def test_expand_drops_last_successor(oracle_cpu):
    # Integrator.cpp:186-250: z and y unions, then +x for all but the last key
    def pack(x, y, z):
        return z << 20 | y << 10 | x
    u = np.array([pack(5, 5, 5)], np.uint32)
    e = oracle_cpu.expand(u)
    want = sorted({pack(5 + dx, 5 + dy, 5 + dz) for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)}
                  - {pack(6, 6, 6)})
    assert list(e) == want


def test_icp_jacobi_recovers_rotation(oracle_cpu):
    # Horn's method on exact correspondences: the eigen solve must return the
    # rotation that maps src onto dst.
    import ctypes as C
    rng = np.random.default_rng(3)
    a = rng.normal(size=(4, 4))
    a = a + a.T
    ev_ref = np.linalg.eigvalsh(a)
    aa = np.ascontiguousarray(a, np.float64).copy()
    ev = np.zeros(4)
    V = np.zeros(16)
    oracle_cpu.lib().or_jacobi4(aa.ctypes.data_as(C.c_void_p), ev.ctypes.data_as(C.c_void_p),
                                V.ctypes.data_as(C.c_void_p))
    assert np.allclose(np.sort(ev), ev_ref, atol=1e-12)
    V = V.reshape(4, 4)
    assert np.allclose(a @ V, V * ev, atol=1e-10)
