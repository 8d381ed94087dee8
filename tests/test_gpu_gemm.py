"""The BF16 tcgen05 GEMM (wp_dev_gemm_bf16) against a PyTorch FP32
reference of the same product: C = act(A . B^T + bias) with BF16 inputs.

Tolerance: FP32 output within 1e-4 relative of the FP32 reference (only the
summation order differs); BF16 output within one BF16 rounding (2^-8
relative) plus that."""
import math

import pytest

from whatprot_gb300 import capi

pytestmark = pytest.mark.gpu

SHAPES = [(128, 256, 64), (256, 512, 128), (200, 300, 192), (512, 1024, 1024), (384, 20000 // 16, 64),
          (1024, 1024, 256)]


def _ref(A, B, bias, act):
    import torch
    C = A.float() @ B.float().T
    if bias is not None:
        C = C + bias
    Z = C
    if act == 1:
        C = 0.5 * C * (1.0 + torch.erf(C / math.sqrt(2.0)))
    return C, Z


@pytest.mark.parametrize("shape", SHAPES, ids=[f"{m}x{n}x{k}" for m, n, k in SHAPES])
@pytest.mark.parametrize("act", [0, 1])
def test_gemm_fp32_out(shape, act):
    import torch
    M, N, K = shape
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g) if act else None
    C = capi.gemm_bf16(A, B, bias, act, out_fp32=True)
    ref, _ = _ref(A, B, bias, act)
    scale = math.sqrt(K)
    err = (C - ref).abs().max().item()
    assert err <= 1e-4 * scale + 1e-4 * ref.abs().max().item(), err


def test_gemm_bf16_out_and_preactivation():
    import torch
    M, N, K = 256, 512, 192
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = (torch.randn(N, K, device="cuda", generator=g) * 0.1).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    C, Z = capi.gemm_bf16(A, B, bias, 1, out_fp32=False, want_z=True)
    ref, zref = _ref(A, B, bias, 1)
    assert torch.allclose(C.float(), ref, rtol=2 ** -7, atol=1e-3)
    assert torch.allclose(Z.float(), zref, rtol=2 ** -7, atol=1e-3)


def test_gemm_rejects_bad_shapes():
    import torch
    A = torch.zeros(128, 48, device="cuda", dtype=torch.bfloat16)
    B = torch.zeros(128, 48, device="cuda", dtype=torch.bfloat16)
    with pytest.raises(capi.WpError):
        capi.gemm_bf16(A, B)  # K must be a multiple of 64
