"""The pose proposer's tcgen05 BF16 GEMM (FP32 accumulation in TMEM) against
a float64 product of the same BF16-rounded operands."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# M, N, K, k_split: the proposer's layer shapes at batch 256 (forward, both
# backward products) plus ragged edges
SHAPES = [(128, 16, 16, 0), (300, 32, 32, 0), (1000, 64, 288, 0), (5120, 128, 576, 0),
          (256, 64, 128, 0), (256, 16, 64, 0), (77, 200, 40, 0), (64, 576, 76800, 4096)]


def _bf16(x):
    import torch
    return torch.from_numpy(x).to(torch.bfloat16)


@pytest.mark.parametrize("m,n,k,split", SHAPES)
def test_gemm_matches_float64(gpu, m, n, k, split):
    import torch
    lib = gpu
    rng = np.random.default_rng(m + n + k)
    a = _bf16(rng.normal(size=(m, k)).astype(np.float32))
    b = _bf16(rng.normal(size=(n, k)).astype(np.float32))
    ref = a.double().numpy() @ b.double().numpy().T
    da, db = a.cuda(), b.cuda()
    dc = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.kifi_gemm_bf16(C.c_void_p(da.data_ptr()), C.c_void_p(db.data_ptr()), C.c_void_p(dc.data_ptr()),
                            m, n, k, k, k, n, split, 1 if split else 0, None)
    assert rc == 0, lib.kifi_last_error()
    got = dc.cpu().numpy().astype(np.float64)
    bound = 2e-6 * (np.abs(a.double().numpy()) @ np.abs(b.double().numpy()).T) + 1e-6
    assert (np.abs(got - ref) <= bound).all(), float(np.abs(got - ref).max())


def test_gemm_accumulates(gpu):
    import torch
    lib = gpu
    rng = np.random.default_rng(1)
    a = _bf16(rng.normal(size=(200, 96)).astype(np.float32))
    b = _bf16(rng.normal(size=(48, 96)).astype(np.float32))
    c0 = rng.normal(size=(200, 48)).astype(np.float32)
    dc = torch.from_numpy(c0.copy()).cuda()
    da, db = a.cuda(), b.cuda()
    torch.cuda.synchronize()
    assert lib.kifi_gemm_bf16(C.c_void_p(da.data_ptr()), C.c_void_p(db.data_ptr()), C.c_void_p(dc.data_ptr()),
                              200, 48, 96, 96, 96, 48, 0, 1, None) == 0
    ref = c0 + a.double().numpy() @ b.double().numpy().T
    assert np.abs(dc.cpu().numpy() - ref).max() < 1e-4
