"""tcgen05 building blocks (TMEM, SW128 descriptors for K-major and MN-major
operands, BF16 MMA, TMEM loads) against a torch FP32 matmul of the same BF16
operands.  Tolerance: 1e-5 relative to the sum of |products| (FP32
accumulation of exact BF16 products)."""
import pytest
import torch

from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('N_,K,a_mn,b_mn', [(16, 64, 0, 0), (64, 128, 0, 0), (144, 128, 0, 0),
                                            (256, 128, 0, 0), (80, 256, 0, 0), (128, 128, 1, 0),
                                            (128, 128, 0, 1), (128, 128, 1, 1), (64, 256, 1, 1),
                                            (256, 64, 1, 1)])
def test_umma_gemm_matches_torch(N_, K, a_mn, b_mn):
    g = torch.Generator().manual_seed(N_ * 1000 + K + 7 * a_mn + 13 * b_mn)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N_, K, generator=g).to(torch.bfloat16).cuda()
    Ain = A.t().contiguous() if a_mn else A
    Bin = B.t().contiguous() if b_mn else B
    D = torch.full((128, N_), float('nan'), dtype=torch.float32, device='cuda')
    st = torch.zeros(1, dtype=torch.int32, device='cuda')
    N.check(N.load().vg_probe_umma_gemm(N.ptr(Ain), N.ptr(Bin), N.ptr(D), N_, K, a_mn, b_mn,
                                         N.ptr(st), N.stream_ptr()))
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float() @ B.float().t()
    scale = A.float().abs() @ B.float().abs().t()
    err = ((D - ref).abs() / scale).max().item()
    assert err < 1e-5, err
