"""tcgen05 BF16 GEMM (ffmpm_tc_gemm_bf16) against an FP64 product of the same bf16 values."""
import ctypes

import pytest
import torch

from femflow_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _gemm(A, B, split=1, out=None):
    M, K = A.shape
    n = B.shape[0]
    D = torch.zeros((M, n), dtype=torch.float32, device="cuda") if out is None else out
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.call("ffmpm_tc_gemm_bf16", ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
           ctypes.c_void_p(D.data_ptr()), M, n, K, split, ctypes.c_void_p(st.data_ptr()),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return D


@pytest.mark.parametrize("M,Nn,K,split", [(128, 16, 64, 1), (256, 64, 128, 1), (256, 48, 192, 1),
                                          (384, 256, 64, 1), (128, 128, 256, 4), (256, 112, 128, 2),
                                          (1024, 64, 1024, 8)])
def test_tc_gemm_matches_fp64_product(M, Nn, K, split):
    g = torch.Generator().manual_seed(M + Nn + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(Nn, K, generator=g).to(torch.bfloat16).cuda()
    D = _gemm(A, B, split)
    ref = A.double() @ B.double().T
    err = float((D.double() - ref).abs().max() / ref.abs().max())
    assert err < 2e-6, err


def test_tc_gemm_rejects_bad_shapes():
    A = torch.zeros(100, 64, dtype=torch.bfloat16, device="cuda")
    B = torch.zeros(16, 64, dtype=torch.bfloat16, device="cuda")
    D = torch.zeros(100, 16, device="cuda")
    with pytest.raises(RuntimeError):
        N.call("ffmpm_tc_gemm_bf16", ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
               ctypes.c_void_p(D.data_ptr()), 100, 16, 64, 1, None, None)
