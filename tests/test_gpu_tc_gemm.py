"""The tcgen05 GEMM (C = A . B^T, bf16 in, fp32 out) against a PyTorch fp32
reference of the same bf16 operands, through the C ABI.  Tolerance: fp32
accumulation-order differences only (products of bf16 are exact in fp32):
|C - ref| <= 1e-4 |ref| + 2e-6 sqrt(K) max|a||b|.  The three-section hi/lo
split must reproduce a binary64 product to ~2^-17 relative."""
import ctypes
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def gemm(A, B, M, N, K, ldc=None):
    from ad_afqmc_prototype_gb300 import _lib, engine
    ldc = ldc or N
    C = torch.full((M, ldc), float("nan"), dtype=torch.float32, device=A.device)
    err = torch.zeros((1,), dtype=torch.int32, device=A.device)
    _lib.call("afq_lowp_gemm_tn", M, N, K, ctypes.c_void_p(A.data_ptr()), A.shape[1], ctypes.c_void_p(B.data_ptr()),
              B.shape[1], ctypes.c_void_p(C.data_ptr()), ldc, ctypes.c_void_p(err.data_ptr()), engine.stream_ptr())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C


@pytest.mark.parametrize("M,N,K,padk,ldc_pad", [(128, 256, 64, 0, 0), (300, 1000, 192, 8, 0), (129, 257, 128, 0, 3),
                                                 (1, 16, 64, 0, 0), (2048, 4096, 1024, 0, 0)])
def test_tc_gemm_matches_fp32(cuda, M, N, K, padk, ldc_pad):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn((M, K + padk), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K + padk), generator=g, device="cuda").to(torch.bfloat16)
    C = gemm(A, B, M, N, K, ldc=N + ldc_pad)
    ref = A[:, :K].float() @ B[:, :K].float().T
    got = C[:, :N]
    assert not torch.isnan(got).any()
    tol = 1e-4 * ref.abs() + 2e-6 * math.sqrt(K) * 16.0
    assert bool(((got - ref).abs() <= tol).all()), float((got - ref).abs().max())
    if ldc_pad:  # the padding columns are never written
        assert torch.isnan(C[:, N:]).all()


def split3(x, left: bool, K: int):
    """bf16 sections along K: left operand [hi hi lo], right operand [hi lo hi]."""
    hi = x.to(torch.bfloat16)
    lo = (x - hi.double()).to(torch.bfloat16)
    out = torch.zeros((x.shape[0], 3 * K), dtype=torch.bfloat16, device=x.device)
    secs = (hi, hi, lo) if left else (hi, lo, hi)
    for s, t in enumerate(secs):
        out[:, s * K:s * K + x.shape[1]] = t
    return out


def test_split_product_accuracy(cuda):
    M, N, Kr, K = 256, 512, 1000, 1024
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.randn((M, Kr), generator=g, device="cuda", dtype=torch.float64)
    b = torch.randn((N, Kr), generator=g, device="cuda", dtype=torch.float64) * torch.exp(
        -torch.arange(Kr, device="cuda", dtype=torch.float64) / 250.0)
    C = gemm(split3(a, True, K), split3(b, False, K), M, N, 3 * K)
    ref = a @ b.T
    rel = float(((C.double() - ref).abs().max() / ref.abs().max()).item())
    assert rel < 3e-5, rel
