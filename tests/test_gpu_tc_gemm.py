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


# larger shapes: several tiles per persistent CTA (both TMEM accumulators in
# turn), and a K split that is not a multiple of the 64-deep chunk
@pytest.mark.parametrize("m,n,k,split", [(76800, 64, 288, 0), (20480, 128, 576, 0), (64, 288, 20000, 1000)])
def test_gemm_many_tiles(gpu, m, n, k, split):
    test_gemm_matches_float64(gpu, m, n, k, split)


def _im2col(x, kp):
    """col[(b, oy, ox)][(ky * 3 + kx) * C + c] of a 3x3 / stride 2 / pad 1
    convolution, zero-padded to kp columns (float64)."""
    b, h, w, c = x.shape
    ho, wo = (h + 1) // 2, (w + 1) // 2
    xp = np.zeros((b, h + 2, w + 2, c))
    xp[:, 1:h + 1, 1:w + 1] = x
    col = np.zeros((b, ho, wo, kp))
    for ky in range(3):
        for kx in range(3):
            tap = ky * 3 + kx
            col[..., tap * c:(tap + 1) * c] = xp[:, ky:ky + 2 * ho:2, kx:kx + 2 * wo:2]
    return col.reshape(b * ho * wo, kp)


# the proposer's convolutions 2-4 (input 30x40x32, 15x20x64, 8x10x64) and
# odd sizes; batches that leave partial tiles
@pytest.mark.parametrize("b,h,w,cin,cout", [(24, 30, 40, 32, 64), (19, 15, 20, 64, 64), (13, 8, 10, 64, 128),
                                            (3, 9, 7, 32, 128), (5, 21, 33, 64, 64)])
def test_implicit_conv_matches_im2col_product(gpu, b, h, w, cin, cout):
    import torch
    lib = gpu
    rng = np.random.default_rng(b * h + w)
    kp = 9 * cin
    x = _bf16(rng.normal(size=(b, h, w, cin)).astype(np.float32))
    wt = _bf16((rng.normal(size=(cout, kp)) / np.sqrt(kp)).astype(np.float32))
    bias = rng.normal(size=cout).astype(np.float32)
    ho, wo = (h + 1) // 2, (w + 1) // 2
    col = _im2col(x.double().numpy(), kp)
    pre = col @ wt.double().numpy().T + bias[None, :].astype(np.float64)
    for relu in (1, 0):
        out = torch.empty((b, ho, wo, cout), dtype=torch.bfloat16, device="cuda")
        dx, dw, db = x.cuda(), wt.cuda(), torch.from_numpy(bias).cuda()
        torch.cuda.synchronize()
        rc = lib.kifi_conv3x3s2_bf16(C.c_void_p(dx.data_ptr()), b, h, w, cin, C.c_void_p(dw.data_ptr()), cout, kp,
                                     C.c_void_p(db.data_ptr()), relu, C.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.kifi_last_error()
        got = out.float().cpu().numpy().reshape(-1, cout).astype(np.float64)
        want = np.maximum(pre, 0) if relu else pre
        # FP32 accumulation, then one BF16 rounding (relative 2^-8)
        bound = 2 ** -8 * np.abs(want) + 2e-6 * (np.abs(col) @ np.abs(wt.double().numpy()).T) + 1e-6
        assert (np.abs(got - want) <= bound).all(), float(np.abs(got - want).max())
