"""kifi_radix_sort_pairs_u32_static (the radix sort on a static scratch area,
no device allocation) against the allocating entry point
kifi_radix_sort_pairs_u32, through the C ABI.  Sorting is integer work: the
results must be identical.  Named to be collected last, after every other
test has used the library; it also passes alone in a fresh process."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STATIC_MAX = 1 << 20


def _sorted_by_existing(lib, keys, values):
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(values, np.uint32).copy()
    rc = lib.kifi_radix_sort_pairs_u32(k.ctypes.data_as(C.c_void_p), v.ctypes.data_as(C.c_void_p),
                                       C.c_size_t(k.size))
    assert rc == 0, lib.kifi_last_error()
    return k, v


def _sorted_by_static(lib, keys, values):
    import torch
    dk = torch.from_numpy(np.ascontiguousarray(keys, np.uint32).view(np.int32)).cuda()
    dv = None if values is None else torch.from_numpy(np.ascontiguousarray(values, np.uint32).view(np.int32)).cuda()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    rc = lib.kifi_radix_sort_pairs_u32_static(C.c_void_p(dk.data_ptr()),
                                             None if dv is None else C.c_void_p(dv.data_ptr()),
                                             C.c_size_t(dk.numel()), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.kifi_last_error()
    k = dk.cpu().numpy().view(np.uint32)
    return k, (None if dv is None else dv.cpu().numpy().view(np.uint32))


def test_static_sort_equals_existing_two_calls_in_a_row(gpu):
    lib = gpu
    rng = np.random.default_rng(11)
    for n, span in ((300_001, 1 << 30), (STATIC_MAX, 1 << 16)):
        keys = rng.integers(0, span, n, dtype=np.uint32)  # span 2^16: many equal keys
        values = np.arange(n, dtype=np.uint32)
        want_k, want_v = _sorted_by_existing(lib, keys, values)
        for _ in range(2):  # two calls in a row on the same scratch
            got_k, got_v = _sorted_by_static(lib, keys, values)
            assert np.array_equal(got_k, want_k)
            assert np.array_equal(got_v, want_v)  # stable, like the existing sort
    keys = rng.integers(0, 1 << 30, 4097, dtype=np.uint32)
    got_k, _ = _sorted_by_static(lib, keys, None)
    assert np.array_equal(got_k, np.sort(keys))


def test_static_sort_rejects_more_than_its_scratch(gpu):
    lib = gpu
    assert lib.kifi_radix_sort_pairs_u32_static(C.c_void_p(16), None, C.c_size_t(STATIC_MAX + 1), None) == 1
    msg = lib.kifi_last_error()
    msg = msg.decode() if isinstance(msg, bytes) else msg
    assert "exceeds the static scratch limit" in msg
    assert lib.kifi_radix_sort_pairs_u32_static(C.c_void_p(16), None, C.c_size_t(0), None) == 0


def test_static_sort_in_a_fresh_process(gpu):
    # first call of the process: the per-device set-up runs inside the call
    code = ("import sys, ctypes as C, numpy as np, torch\n"
            "sys.path.insert(0, %r)\n"
            "from merge_fusion_gb300 import _lib\n"
            "lib = _lib.load()\n"
            "rng = np.random.default_rng(5)\n"
            "keys = rng.integers(0, 1 << 30, 100000, dtype=np.uint32)\n"
            "d = torch.from_numpy(keys.view(np.int32)).cuda()\n"
            "torch.cuda.synchronize()\n"
            "for _ in range(2):\n"
            "    assert lib.kifi_radix_sort_pairs_u32_static(C.c_void_p(d.data_ptr()), None, 100000, None) == 0\n"
            "    assert np.array_equal(d.cpu().numpy().view(np.uint32), np.sort(keys))\n"
            "    d.copy_(torch.from_numpy(keys.view(np.int32)))\n"
            "# keys with values, the last tile partial (n not a multiple of 2048)\n"
            "n = 77777\n"
            "keys = rng.integers(0, 1 << 12, n, dtype=np.uint32)\n"
            "vals = np.arange(n, dtype=np.uint32)\n"
            "wk, wv = keys.copy(), vals.copy()\n"
            "assert lib.kifi_radix_sort_pairs_u32(wk.ctypes.data_as(C.c_void_p), wv.ctypes.data_as(C.c_void_p), n) == 0\n"
            "for _ in range(2):\n"
            "    dk = torch.from_numpy(keys.view(np.int32)).cuda()\n"
            "    dv = torch.from_numpy(vals.view(np.int32)).cuda()\n"
            "    torch.cuda.synchronize()\n"
            "    assert lib.kifi_radix_sort_pairs_u32_static(C.c_void_p(dk.data_ptr()), C.c_void_p(dv.data_ptr()), n, None) == 0\n"
            "    assert np.array_equal(dk.cpu().numpy().view(np.uint32), wk)\n"
            "    assert np.array_equal(dv.cpu().numpy().view(np.uint32), wv)\n"
            "print('ok')\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr[-2000:]
