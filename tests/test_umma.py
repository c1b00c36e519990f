"""tcgen05 building blocks (TMEM, SW128 descriptors, BF16 MMA, TMEM loads)
against a torch FP32 matmul of the same BF16 operands.  Tolerance: 1e-5
relative to the sum of |products| (FP32 accumulation of exact BF16 products)."""
import ctypes

import pytest
import torch

from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('N_,K', [(16, 64), (64, 128), (144, 128), (256, 128), (80, 256)])
def test_umma_gemm_matches_torch(N_, K):
    g = torch.Generator().manual_seed(N_ * 1000 + K)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N_, K, generator=g).to(torch.bfloat16).cuda()
    D = torch.full((128, N_), float('nan'), dtype=torch.float32, device='cuda')
    st = torch.zeros(1, dtype=torch.int32, device='cuda')
    N.check(N.load().vg_probe_umma_gemm(N.ptr(A), N.ptr(B), N.ptr(D), N_, K, N.ptr(st),
                                         N.stream_ptr()))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float() @ B.float().t()
    scale = A.float().abs() @ B.float().abs().t()
    err = ((D - ref).abs() / scale).max().item()
    assert err < 1e-5, err
