"""The tcgen05 BF16 GEMM (splat_gemm_bf16, TMA-fed) against an fp32 product of
the same bf16 operands: full and partial tiles, narrow N (the 32- and
64-column tiles), K not a multiple of the K tile, strided operands,
accumulation, split K; MN-major (transposed) operands (splat_gemm_bf16_mn);
and its fused bias + ReLU epilogue (splat_gemm_bf16_bias_act) to bf16 and
fp32.  Output row strides that are 16-byte multiples take the tensor-store
epilogue (tensor reduce-adds for split K and accumulation), others the
register stores; both are covered."""

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
                                   (1000, 32, 8), (77, 256, 1152), (520, 64, 288),
                                   (4100, 48, 40), (64, 288, 2048)])
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


@pytest.mark.parametrize("M,N,K,relu,bf16", [(1000, 32, 32, True, True), (333, 64, 288, True, True),
                                             (257, 128, 576, True, True),
                                             (300, 224, 256, False, False)])
def test_gemm_bias_act_epilogue(M, N, K, relu, bf16):
    import torch

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300._ops import _status_word

    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).bfloat16()
    B = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    bias = torch.randn(N, device="cuda", generator=g)
    y = torch.full((M, N), float("nan"), device="cuda",
                   dtype=torch.bfloat16 if bf16 else torch.float32)
    st = _status_word(A.device)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    rc = lib.splat_gemm_bf16_bias_act(p(A), p(B), p(bias), p(y) if bf16 else None,
                                      None if bf16 else p(y), M, N, K, K, K, N, int(relu), p(st),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "gemm_bf16_bias_act")
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float() @ B.float().T + bias
    if relu:
        ref = ref.clamp_min(0)
    if bf16:
        # the fp32 sum rounded once to bf16: within one bf16 ulp of the
        # rounded reference
        err = (y.float() - ref.bfloat16().float()).abs()
        assert bool((err <= ref.abs() * 2 ** -7 + 1e-3 * max(1.0, K / 64)).all())
    else:
        assert (y - ref).abs().max().item() <= 1e-4 * max(1.0, ref.abs().max().item()) * max(1.0, K / 64)


def _gemm_mn(A, a_mn, B, b_mn, Cm, M, N, K, accumulate=False):
    import torch

    from jaxsplat_gb300 import _lib
    from jaxsplat_gb300._ops import _status_word

    lib = _lib.load()
    st = _status_word(A.device)
    rc = lib.splat_gemm_bf16_mn(C.c_void_p(A.data_ptr()), int(a_mn), C.c_void_p(B.data_ptr()),
                                int(b_mn), C.c_void_p(Cm.data_ptr()), M, N, K, A.stride(0),
                                B.stride(0), Cm.stride(0), int(accumulate),
                                C.c_void_p(st.data_ptr()),
                                C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc, "gemm_bf16_mn")
    torch.cuda.synchronize()
    assert int(st.item()) == 0


@pytest.mark.parametrize("a_mn,b_mn", [(True, True), (False, True), (True, False),
                                       (False, False)])
@pytest.mark.parametrize("M,N,K", [(32, 32, 4096), (64, 288, 2048), (224, 256, 1024),
                                   (300, 200, 72), (1000, 64, 128), (128, 1152, 256),
                                   (77, 40, 200)])
def test_gemm_mn_major_operands(a_mn, b_mn, M, N, K):
    """op(A) op(B)^T with A stored [K, M] and/or B stored [K, N]: the
    network's weight-gradient shapes (M = output channels, N = im2col
    columns, K = pixels: split K with tensor reduce-adds) and data-gradient
    shapes, edges in every dimension."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(M * 5 + N * 3 + K + 7 * a_mn + 11 * b_mn)
    A = torch.randn(M, K, device="cuda", generator=g).bfloat16()
    B = torch.randn(N, K, device="cuda", generator=g).bfloat16()
    def stored(X, mn):
        # MN-major: [K, rows] with the row stride padded to 8 elements
        if not mn:
            return X
        S = torch.zeros(K, (X.shape[0] + 7) // 8 * 8, device="cuda", dtype=X.dtype)
        S[:, :X.shape[0]] = X.T
        return S

    As, Bs = stored(A, a_mn), stored(B, b_mn)
    Cm = torch.full((M, N), float("nan"), device="cuda")
    _gemm_mn(As, a_mn, Bs, b_mn, Cm, M, N, K)
    ref = A.float() @ B.float().T
    err = (Cm - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()) * max(1.0, K / 64), err


def test_gemm_mn_accumulate_takes_the_reduce_add():
    """accumulate = 1 with a 16-byte-aligned output stride: C += op(A) op(B)^T
    through the tensor reduce-add."""
    import torch

    g = torch.Generator(device="cuda").manual_seed(11)
    M, N, K = 96, 160, 320
    A = torch.randn(K, M, device="cuda", generator=g).bfloat16()
    B = torch.randn(K, N, device="cuda", generator=g).bfloat16()
    C0 = torch.randn(M, N, device="cuda", generator=g)
    Cm = C0.clone()
    _gemm_mn(A, True, B, True, Cm, M, N, K, accumulate=True)
    ref = C0 + A.float().T @ B.float()
    assert (Cm - ref).abs().max().item() <= 1e-3


def test_gemm_mn_rejects_short_leading_dimension():
    import torch

    from jaxsplat_gb300 import _lib

    lib = _lib.load()
    A = torch.zeros(64, 32, device="cuda", dtype=torch.bfloat16)  # stored [K=64, M=32]
    B = torch.zeros(64, 64, device="cuda", dtype=torch.bfloat16)
    Cm = torch.zeros(48, 64, device="cuda")
    # M = 48 does not fit the stored rows of 32 elements
    rc = lib.splat_gemm_bf16_mn(C.c_void_p(A.data_ptr()), 1, C.c_void_p(B.data_ptr()), 1,
                                C.c_void_p(Cm.data_ptr()), 48, 64, 64, 32, 64, 64, 0, None,
                                C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc != 0
