"""The tcgen05 GEMM (C = A . B^T, bf16 in, fp32 out) against a PyTorch fp32
reference of the same bf16 operands, through the C ABI, in both accumulation
modes.  Tolerance: fp32 accumulation-order differences only (products of
bf16 are exact in fp32): |C - ref| <= 1e-4 |ref| + 2e-6 sqrt(K) max|a||b|.
The six-section split must reproduce a binary64 product to ~2^-22; the
drained mode must not drift on long sums of positive terms (the tensor
cores' own fp32 accumulation truncates and drifts low)."""
import ctypes
import math

import pytest
import torch

pytestmark = pytest.mark.gpu


def gemm(A, B, M, N, K, ldc=None, accumulate=1):
    from ad_afqmc_prototype_gb300 import _lib, engine
    ldc = ldc or N
    C = torch.full((M, ldc), float("nan"), dtype=torch.float32, device=A.device)
    err = torch.zeros((1,), dtype=torch.int32, device=A.device)
    _lib.call("afq_lowp_gemm_tn", M, N, K, ctypes.c_void_p(A.data_ptr()), A.shape[1], ctypes.c_void_p(B.data_ptr()),
              B.shape[1], ctypes.c_void_p(C.data_ptr()), ldc, ctypes.c_void_p(err.data_ptr()), accumulate,
              engine.stream_ptr())
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return C


@pytest.mark.parametrize("accumulate", [0, 1, 3])
@pytest.mark.parametrize("M,N,K,padk,ldc_pad", [(128, 256, 64, 0, 0), (300, 1000, 192, 8, 0), (129, 257, 128, 0, 3),
                                                 (1, 16, 64, 0, 0), (2048, 4096, 1024, 0, 0)])
def test_tc_gemm_matches_fp32(cuda, M, N, K, padk, ldc_pad, accumulate):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N)
    A = torch.randn((M, K + padk), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K + padk), generator=g, device="cuda").to(torch.bfloat16)
    C = gemm(A, B, M, N, K, ldc=N + ldc_pad, accumulate=accumulate)
    ref = A[:, :K].float() @ B[:, :K].float().T
    got = C[:, :N]
    assert not torch.isnan(got).any()
    tol = 1e-4 * ref.abs() + 2e-6 * math.sqrt(K) * 16.0
    assert bool(((got - ref).abs() <= tol).all()), float((got - ref).abs().max())
    if ldc_pad:  # the padding columns are never written
        assert torch.isnan(C[:, N:]).all()


def split6(x, left: bool, S: int):
    """bf16 pieces h, m, l of x in six sections: left [h h m h l m], right
    [h m h l h m] (the layout the mixed-precision kernels write)."""
    h = x.to(torch.bfloat16)
    r = x - h.double()
    m = r.to(torch.bfloat16)
    l_ = (r - m.double()).to(torch.bfloat16)
    secs = (h, h, m, h, l_, m) if left else (h, m, h, l_, h, m)
    Kt = (6 * S + 63) // 64 * 64
    out = torch.zeros((x.shape[0], Kt), dtype=torch.bfloat16, device=x.device)
    for s, t in enumerate(secs):
        out[:, s * S:s * S + x.shape[1]] = t
    return out


def test_split_product_accuracy(cuda):
    M, N, S = 256, 512, 1000
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.randn((M, S), generator=g, device="cuda", dtype=torch.float64)
    b = torch.randn((N, S), generator=g, device="cuda", dtype=torch.float64) * torch.exp(
        -torch.arange(S, device="cuda", dtype=torch.float64) / 250.0)
    A, B = split6(a, True, S), split6(b, False, S)
    C = gemm(A, B, M, N, A.shape[1], accumulate=1)
    ref = a @ b.T
    rel = float(((C.double() - ref).abs().max() / ref.abs().max()).item())
    assert rel < 2e-6, rel


def test_drained_accumulation_does_not_drift(cuda):
    """Sum of K positive terms spread over seven binades: the drained mode stays
    within fp32 round-to-nearest error, the tensor-core accumulation drifts low."""
    M, N, K = 128, 256, 16384
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.ones((M, K), device="cuda", dtype=torch.bfloat16)
    B = torch.exp(-7.0 * torch.rand((N, K), generator=g, device="cuda")).to(torch.bfloat16)
    exact = B.double().sum(1)
    drained = gemm(A, B, M, N, K, accumulate=1)[0].double()
    plain = gemm(A, B, M, N, K, accumulate=0)[0].double()
    rel_d = ((drained - exact) / exact)
    rel_p = ((plain - exact) / exact)
    assert float(rel_d.abs().max()) < 2e-6, float(rel_d.abs().max())
    assert float(rel_d.mean().abs()) < 3e-7, float(rel_d.mean())
    assert float(rel_p.mean()) < -3e-6  # the truncating accumulator, for the record
