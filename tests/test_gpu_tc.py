"""GPU: the tcgen05 tensor-core GEMM (TMEM accumulators, shared-memory
operand descriptors) against an FP32 product of the same BF16 inputs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (128, 64, 32), (200, 112, 64), (256, 240, 1600), (77, 256, 48)])
def test_tc_gemm_matches_fp32(cuda, M, N, K):
    import torch
    from dpgb import _lib

    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(cuda)
    Bt = torch.randn(N, K, generator=g).to(torch.bfloat16).to(cuda)
    D = torch.empty(M, N, dtype=torch.float32, device=cuda)
    _lib.call("dpgb_tc_gemm_bf16", ctypes.c_void_p(D.data_ptr()), ctypes.c_void_p(A.data_ptr()),
              ctypes.c_void_p(Bt.data_ptr()), M, N, K, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    ref = A.double() @ Bt.double().T
    err = (D.double() - ref).abs().max().item()
    assert err <= 1e-4 * max(1.0, ref.abs().max().item()), err
