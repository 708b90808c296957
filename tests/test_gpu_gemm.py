"""The tcgen05 BF16 GEMM (splat_gemm_bf16) against an fp32 product of the
same bf16 operands: full and partial tiles, K not a multiple of the K tile,
strided operands, accumulation."""

import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _gemm(A, B, Cm, accumulate=False, lda=None, ldb=None):
    import torch

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300._ops import _status_word

    lib = _lib.load()
    M, K = A.shape[0], A.shape[1]
    N = B.shape[0]
    st = _status_word(A.device)
    rc = lib.splat_gemm_bf16(C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()),
                             C.c_void_p(Cm.data_ptr()), M, N, K, lda or A.stride(0),
                             ldb or B.stride(0), Cm.stride(0), int(accumulate),
                             C.c_void_p(st.data_ptr()),
                             C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "gemm_bf16")
    torch.cuda.synchronize()
    assert int(st.item()) == 0


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 192), (300, 200, 72),
                                   (1000, 32, 8), (77, 256, 1152)])
def test_gemm_matches_fp32_product(M, N, K):
    import torch

    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).bfloat16()
    B = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    Cm = torch.full((M, N), float("nan"), device="cuda")
    _gemm(A, B, Cm)
    ref = A.float() @ B.float().T
    err = (Cm - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()) * max(1.0, K / 64), err


def test_gemm_strided_and_accumulate():
    import torch

    g = torch.Generator(device="cuda").manual_seed(5)
    Abig = torch.randn(200, 96, device="cuda", generator=g).bfloat16()
    Bbig = torch.randn(130, 80, device="cuda", generator=g).bfloat16()
    A, B = Abig[:, :64], Bbig[:, :64]  # leading dimensions 96 and 80
    C0 = torch.randn(200, 130, device="cuda", generator=g)
    Cm = C0.clone()
    _gemm(A, B, Cm, accumulate=True)
    ref = C0 + A.float() @ B.float().T
    assert (Cm - ref).abs().max().item() <= 1e-3
