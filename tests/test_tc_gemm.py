"""The tensor-core GEMM (TMA-fed operand pieces, tcgen05 TF32 or BF16 MMAs, FP32
accumulation in tensor memory) against an FP64 product of the same operands,
through the C ABI. Tolerances, as a fraction of sum_k |A_ik| |B_kj| (the scale of
the accumulated products): split TF32 (three products per step) and split BF16
(three pieces, six products) 2e-6; plain TF32 2e-3 (11-bit mantissa products);
the double-float CUDA-core tiles of the mixed solves' residual updates (terms = 2)
3e-14 (FP32 pairs: operands to ~2^-47, error-free products, TwoSum sums)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

xg = pytest.importorskip("xerus_gb300")
torch = pytest.importorskip("torch")
from xerus_gb300 import _lib as L  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    from xerus_gb300 import build
    build.build()
    return xg.Context(0)


def run(ctx, A, B, terms, C=None):
    m, k = A.shape
    n = B.shape[1]
    if C is None:
        C = torch.full((m, n), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = ctx.lib.xtt_gemm_tc(ctx.handle, m, n, k, ctypes.c_void_p(A.data_ptr()), A.stride(0),
                             ctypes.c_void_p(B.data_ptr()), B.stride(0), ctypes.c_void_p(C.data_ptr()), C.stride(0),
                             terms)
    L.check(rc)
    ctx.synchronize()
    return C


@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (128, 64, 256), (300, 200, 100), (7, 5, 3), (1024, 96, 24),
                                   (64, 512, 1000), (256, 130, 8)])
@pytest.mark.parametrize("terms,tol", [(3, 2e-6), (6, 2e-6), (1, 2e-3)])
def test_gemm_tc_matches_fp64(ctx, m, n, k, terms, tol):
    g = torch.Generator(device="cpu").manual_seed(m * 7919 + n * 31 + k)
    A = torch.randn(m, k, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(k, n, generator=g, dtype=torch.float64).cuda()
    C = run(ctx, A, B, terms)
    ref = A @ B
    scale = A.abs() @ B.abs()
    err = ((C - ref).abs() / scale).max().item()
    assert err < tol, err


def test_gemm_tc_strided_operands(ctx):
    """Leading dimensions larger than the rows (sub-matrices of larger buffers)."""
    g = torch.Generator(device="cpu").manual_seed(5)
    Abig = torch.randn(200, 150, generator=g, dtype=torch.float64).cuda()
    Bbig = torch.randn(150, 300, generator=g, dtype=torch.float64).cuda()
    A, B = Abig[:130, :70], Bbig[:70, 10:210]
    Cbig = torch.zeros(140, 260, dtype=torch.float64, device="cuda")
    C = run(ctx, A, B, 3, Cbig[:130, 30:230])
    ref = A @ B
    assert ((C - ref).abs() / (A.abs() @ B.abs())).max().item() < 2e-6
    # nothing outside the output window was written
    assert Cbig[:, :30].abs().max().item() == 0 and Cbig[:, 230:].abs().max().item() == 0
    assert Cbig[130:].abs().max().item() == 0


@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (300, 200, 100), (7, 5, 3), (1024, 128, 384), (64, 512, 1000),
                                   (256, 130, 8), (384, 128, 1024), (100, 60, 333)])
def test_gemm_double_float_matches_fp64(ctx, m, n, k):
    """K is split across CTAs (parts summed in order) where the tiles leave SMs idle:
    (64, 512, 1000), (384, 128, 1024) and (100, 60, 333)."""
    g = torch.Generator(device="cpu").manual_seed(m * 131 + n * 17 + k)
    A = torch.randn(m, k, generator=g, dtype=torch.float64).cuda()
    B = torch.randn(k, n, generator=g, dtype=torch.float64).cuda()
    C = run(ctx, A, B, 2)
    err = ((C - A @ B).abs() / (A.abs() @ B.abs())).max().item()
    assert err < 3e-14, err


def test_gemm_double_float_exponent_range(ctx):
    """Rows of A spread over 2^-50 .. 2^70 (the split's integer path), exact zeros
    and a row below 2^-74 (carried at FP32 precision: such magnitudes have no FP32
    low part), on the same operands as an FP64 product."""
    m, n, k = 96, 80, 200
    g = torch.Generator(device="cpu").manual_seed(11)
    A = torch.randn(m, k, generator=g, dtype=torch.float64)
    A *= torch.pow(2.0, torch.linspace(-50, 70, m, dtype=torch.float64))[:, None]
    A[3, ::3] = 0.0
    A[5] = torch.randn(k, generator=g, dtype=torch.float64) * 1e-30
    B = torch.randn(k, n, generator=g, dtype=torch.float64)
    A, B = A.cuda(), B.cuda()
    C = run(ctx, A, B, 2)
    rel = (C - A @ B).abs() / (A.abs() @ B.abs())
    keep = torch.ones(m, dtype=torch.bool)
    keep[5] = False
    assert rel[keep].max().item() < 3e-14
    assert rel[5].max().item() < 1e-6
