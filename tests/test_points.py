"""Built-in integrands at given points (vg_eval_points, the FP32 evaluation the
fused kernels share) against their FP64 torch formulas.  FP32 tolerance:
3e-5 relative to the largest value of the batch for the ridge (sums of up
to 1000 exponentials; its FP32 decomposition |x - c 1|^2 = R + dim (m - c)^2
loses a little more with the dimension), 2e-5 for the others.  The ridge evaluates only the terms that can be nonzero in
FP32; points near and far from its diagonal check that nothing is lost."""
import ctypes

import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _eval_points(f, dim, x):
    L = N.load()
    p = f.params(dim)
    out = torch.empty(x.shape[0], dtype=torch.float32, device='cuda')
    xf = x.to(torch.float32).contiguous()
    N.check(L.vg_eval_points(int(f.kind), N.dbl_array(p), len(p), dim, x.shape[0], N.ptr(xf),
                             N.dbl_array([0.0] * dim), N.dbl_array([1.0] * dim), None, None,
                             N.ptr(out), N.stream_ptr()))
    torch.cuda.synchronize()
    return out


def _points(dim, n, seed):
    g = torch.Generator().manual_seed(seed)
    u = torch.rand(n, dim, generator=g, dtype=torch.float64)
    t = torch.rand(n, 1, generator=g, dtype=torch.float64)
    near = t + 0.004 * (u - 0.5)            # close to the diagonal
    return torch.cat([u, near.clamp(0, 1)], dim=0).cuda()


@pytest.mark.parametrize('dim', [2, 4, 7])
def test_ridge_points_vs_fp64(dim):
    f = vg.Ridge(M=1000, s=0.01)
    x = _points(dim, 4000, dim)
    got = _eval_points(f, dim, x).double()
    ref = f(x.double())
    scale = float(ref.abs().max())
    assert float((got - ref).abs().max()) <= 3e-5 * scale
    # where the FP32 value is exactly zero (every term flushed), the FP64
    # value is below the FP32 range relative to the batch's scale
    zero = got == 0
    if bool(zero.any()):
        assert float(ref[zero].abs().max()) <= 1e-25 * scale


@pytest.mark.parametrize('kind', ['gauss', 'lorentz', 'mixture', 'lattice'])
def test_other_points_vs_fp64(kind):
    dim = 5
    rng = np.random.default_rng(1)
    if kind == 'gauss':
        f = vg.Gaussian(a=30.0, c=0.4, dim=dim)
    elif kind == 'lorentz':
        f = vg.LorentzianProduct(rng.uniform(0.2, 0.8, dim), np.exp(rng.uniform(-4.6, -2.3, dim)))
    elif kind == 'mixture':
        f = vg.GaussianMixture(rng.uniform(0.2, 0.8, (3, dim)), sigma=0.1)
    else:
        f = vg.LatticeAction(0.5, 0.2)
    x = _points(dim, 3000, 7)
    got = _eval_points(f, dim, x).double()
    ref = f(x.double())
    assert float((got - ref).abs().max()) <= 2e-5 * float(ref.abs().max())
