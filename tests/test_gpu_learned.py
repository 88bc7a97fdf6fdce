"""Tensor-core (tcgen05) kernels of the learned warm start against fp32 references of the same
bf16 inputs.  Tolerances: fp32 accumulation in a different order, relative 1e-5 of the
largest |C|."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _gemm(E, A, B):
    import torch
    M, K = A.shape
    N = B.shape[0]
    out = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    s = E.lib().impec_gemm_bf16(C.c_void_p(A.data_ptr()), A.stride(0), C.c_void_p(B.data_ptr()), B.stride(0),
                                C.c_void_p(out.data_ptr()), out.stride(0), M, N, K, None)
    assert s == 0, E.last_error()
    return out


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (128, 128, 256), (300, 200, 192), (1024, 256, 576)])
def test_gemm_bf16_matches_fp32_reference(engine, M, N, K):
    import torch
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16)
    got = _gemm(engine, A, B)
    ref = A.float() @ B.float().T
    assert torch.isfinite(got).all()
    assert (got - ref).abs().max().item() <= 1e-5 * ref.abs().max().item() + 1e-6
