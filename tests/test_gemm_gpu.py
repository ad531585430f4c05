"""The tcgen05 BF16 GEMM (pvvc_gemm_bf16) against a torch FP32 matmul of the
same bf16 operands.  Tolerances: FP32 accumulation in a different order
(relative 1e-4 of the row scale) for FP32 outputs; one bf16 rounding
(2^-8 relative) on top of that for bf16 outputs."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RELU, F32, ACC, MASK = 0, 1, 2, 3


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available(), "GPU tests need a CUDA device"
    return t


def _gemm(pvvc_lib, torch, M, N, K, epi, splits=1, bias=True, lda=None, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    lda = lda or K
    A_full = torch.randn(M, lda, generator=g).to(torch.bfloat16).cuda()
    A = A_full[:, :K]
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(N, generator=g).cuda() if bias else None
    aux = torch.randn(M, N, generator=g).to(torch.bfloat16).cuda()
    ref = A.float() @ B.float().T
    if epi == RELU:
        C_ = torch.full((M, N), 7.0, dtype=torch.bfloat16, device="cuda")
        want = torch.clamp(ref + (b if bias else 0), min=0)
    elif epi == F32:
        C_ = torch.full((M, N), 7.0, dtype=torch.float32, device="cuda")
        want = ref + (b if bias else 0)
    elif epi == ACC:
        C_ = torch.full((M, N), 0.5, dtype=torch.float32, device="cuda")
        want = ref + 0.5
    else:
        C_ = torch.full((M, N), 7.0, dtype=torch.bfloat16, device="cuda")
        want = torch.where(aux.float() > 0, ref, torch.zeros_like(ref))
    rc = pvvc_lib.lib().pvvc_gemm_bf16(M, N, K, A_full.data_ptr(), lda, B.data_ptr(), K, C_.data_ptr(), N,
                                       b.data_ptr() if (bias and epi in (RELU, F32)) else None,
                                       aux.data_ptr(), N, epi, splits, torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    code = C.c_int32(-1)
    assert pvvc_lib.lib().pvvc_device_error_take(C.byref(code)) == 0 and code.value == 0
    got = C_.float()
    scale = (A.float().abs() @ B.float().abs().T) + 1e-3
    tol = (1e-4 if epi in (F32, ACC) else 2 ** -7) * scale + (2 ** -7) * want.abs()
    err = (got - want).abs()
    assert bool((err <= tol).all()), float((err / tol).max())
    return got


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (300, 128, 128), (1000, 256, 64), (513, 256, 512), (77, 64, 256)])
def test_gemm_bias_relu(pvvc_lib, torch, M, N, K):
    _gemm(pvvc_lib, torch, M, N, K, RELU)


@pytest.mark.parametrize("M,N,K", [(256, 128, 128), (129, 192, 64)])
def test_gemm_f32_bias(pvvc_lib, torch, M, N, K):
    _gemm(pvvc_lib, torch, M, N, K, F32)


@pytest.mark.parametrize("M,N,K,splits", [(256, 128, 4096, 7), (128, 256, 1024, 16), (200, 64, 640, 3)])
def test_gemm_split_k_accumulate(pvvc_lib, torch, M, N, K, splits):
    _gemm(pvvc_lib, torch, M, N, K, ACC, splits=splits, bias=False)


def test_gemm_mask_and_strided_a(pvvc_lib, torch):
    _gemm(pvvc_lib, torch, 384, 128, 128, MASK, bias=False)
    _gemm(pvvc_lib, torch, 260, 64, 128, RELU, lda=200)


def test_gemm_rejects_bad_shapes(pvvc_lib, torch):
    L = pvvc_lib.lib()
    x = torch.zeros(1 << 16, dtype=torch.bfloat16, device="cuda")
    p = x.data_ptr()
    assert L.pvvc_gemm_bf16(128, 64, 60, p, 64, p, 64, p, 64, None, None, 0, RELU, 1, None) == 1   # K % 64
    assert L.pvvc_gemm_bf16(128, 48, 64, p, 64, p, 64, p, 64, None, None, 0, RELU, 1, None) == 1   # N % 64
    assert L.pvvc_gemm_bf16(128, 64, 64, p, 60, p, 64, p, 64, None, None, 0, RELU, 1, None) == 1   # lda
    assert L.pvvc_gemm_bf16(128, 64, 64, p, 64, p, 64, p, 64, None, None, 0, RELU, 2, None) == 1   # splits
