"""Coupling-layer flow: the FP64 oracle on its own (CPU) and the GPU kernels
against it (GPU).

Tolerances of the GPU kernels (BF16 operands with FP32 accumulation in the
two dense layers, FP32 spline), against the oracle run with the same BF16
rounding of activations and weights:
  sampling / density outputs z:      |dz| <= 2e-3 absolute
  logdet:                            |d logdet| <= 2e-2 absolute (6 layers)
  round trip density(sample(zhat)):  |d zhat| <= 2e-3
  gradient of the training loss:     relative L2 error <= 2u overall and
                                     <= 4u in every parameter block (W1,
                                     b1, W2, b2, W3, b3 of each layer),
                                     u = 2^-9 the BF16 unit roundoff
(the backward rounds dL/dout, dL/dh2', dL/dh1' and the activations to
BF16 for the tensor-core weight-gradient GEMMs -- one BF16
rounding of each operand, which the oracle does not emulate -- so each
block carries a relative error of order u; measured: at most 3u per block
and 1.3u overall on these cases).
"""
import ctypes

import numpy as np
import pytest
import torch

import flow_oracle as F
from vegas_gb300 import _native as N


def _theta(dim, nlayers=6, K=32, hidden=128, seed=1, out_scale=0.5):
    return F.init_theta(dim, nlayers, K, hidden, seed=seed, out_scale=out_scale)


# ------------------------------------------------------------------ oracle
def test_oracle_identity_at_zero_output_layer():
    x = torch.rand(100, 4, dtype=torch.float64)
    th = torch.tensor(F.init_theta(4, out_scale=0.0), dtype=torch.float64)
    z, ld = F.density_pass(th, x, 4)
    assert torch.allclose(z, x, atol=1e-12)
    assert float(ld.abs().max()) < 1e-12


@pytest.mark.parametrize('dim', [1, 3, 4])
def test_oracle_inverse_and_logdet(dim):
    torch.manual_seed(0)
    th = torch.tensor(_theta(dim, K=8, hidden=16), dtype=torch.float64)
    xhat = torch.rand(200, dim, dtype=torch.float64)
    x, ld_s = F.sample_pass(th, xhat, dim, K=8, hidden=16)
    xb, ld_d = F.density_pass(th, x, dim, K=8, hidden=16)
    assert float((xb - xhat).abs().max()) < 1e-10
    assert float((ld_s - ld_d).abs().max()) < 1e-9


def test_oracle_logdet_is_log_jacobian():
    """logdet(x) = log |det d xhat / d x| (autograd Jacobian)."""
    dim = 3
    th = torch.tensor(_theta(dim, K=6, hidden=8), dtype=torch.float64)
    x = torch.rand(5, dim, dtype=torch.float64)
    _, ld = F.density_pass(th, x, dim, K=6, hidden=8)
    for i in range(5):
        J = torch.autograd.functional.jacobian(
            lambda v: F.density_pass(th, v.unsqueeze(0), dim, K=6, hidden=8)[0][0], x[i])
        assert abs(float(torch.logdet(J)) - float(ld[i])) < 1e-9


def test_oracle_density_normalised():
    """q_flow integrates to 1 on the unit cube (midpoint rule, dim 2)."""
    dim = 2
    th = torch.tensor(_theta(dim, K=8, hidden=16), dtype=torch.float64)
    m = 400
    g = (torch.arange(m, dtype=torch.float64) + 0.5) / m
    x = torch.stack(torch.meshgrid(g, g, indexing='ij'), -1).reshape(-1, 2)
    _, ld = F.density_pass(th, x, dim, K=8, hidden=16)
    assert abs(float(torch.exp(ld).mean()) - 1.0) < 1e-3


def test_oracle_gradient_finite_difference():
    dim = 3
    theta = _theta(dim, nlayers=2, K=4, hidden=8).astype(np.float64)
    rng = np.random.default_rng(0)
    x = rng.random((50, dim))
    w = rng.random(50) + 0.1
    loss, g = F.loss_and_grad(theta, x, w, dim, nlayers=2, K=4, hidden=8)
    for i in rng.choice(len(theta), 20, replace=False):
        e = np.zeros_like(theta)
        e[i] = 1e-6
        lp, _ = F.loss_and_grad(theta + e, x, w, dim, nlayers=2, K=4, hidden=8)
        lm, _ = F.loss_and_grad(theta - e, x, w, dim, nlayers=2, K=4, hidden=8)
        assert abs((lp - lm) / 2e-6 - g[i]) < 1e-6 * max(1.0, abs(g[i]))


def test_library_layout_matches_oracle():
    L = N.load()
    for dim in (1, 2, 3, 4, 8, 16):
        for K in (8, 32, 48):
            assert L.vg_flow_nparams(dim, 6, K, 128) == F.nparams(dim, 6, K, 128)
    assert L.vg_flow_nparams(17, 6, 32, 128) == -1
    assert L.vg_flow_nparams(4, 6, 32, 64) == -1


# --------------------------------------------------------------------- GPU
def _gpu_flow(dim, theta, K=32):
    from vegas_gb300.flow import Flow
    fl = Flow(dim, nlayers=6, K=K, hidden=128)
    fl.set_theta(theta)
    return fl


def _oracle_bf16(fn, *args, **kw):
    F.BF16 = True
    try:
        return fn(*args, **kw)
    finally:
        F.BF16 = False


@pytest.fixture(params=['tcgen05', 'mma.sync'])
def flow_path(request):
    L = N.load()
    L.vg_flow_set_path(1 if request.param == 'mma.sync' else 0)
    st = ctypes.c_int(0)
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    yield request.param
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    L.vg_flow_set_path(0)
    assert st.value == 0, 'a bounded wait of the tensor-core pass gave up'


@pytest.mark.gpu
@pytest.mark.parametrize('dim,K', [(1, 32), (3, 32), (4, 32), (8, 32), (16, 32), (4, 16), (9, 16)])
def test_gpu_flow_passes_vs_oracle(dim, K, flow_path):
    theta = _theta(dim, K=K)
    fl = _gpu_flow(dim, theta, K=K)
    torch.manual_seed(dim)
    n = 1000
    u = torch.rand(n, dim, dtype=torch.float32)
    th64 = torch.tensor(theta, dtype=torch.float64)
    # sampling direction
    z, ld = fl.sample(u.cuda())
    zo, ldo = _oracle_bf16(F.sample_pass, th64, u.double(), dim, K=K)
    assert float((z.cpu().double() - zo).abs().max()) <= 2e-3
    assert float((ld.cpu().double() - ldo).abs().max()) <= 2e-2
    # density direction at the oracle's points
    zh, ld2 = fl.density(zo.float().cuda())
    zho, ld2o = _oracle_bf16(F.density_pass, th64, zo, dim, K=K)
    assert float((zh.cpu().double() - zho).abs().max()) <= 2e-3
    assert float((ld2.cpu().double() - ld2o).abs().max()) <= 2e-2
    # round trip on the GPU
    zh2, ld3 = fl.density(z)
    assert float((zh2 - u.cuda()).abs().max()) <= 2e-3
    assert float((ld3 - ld).abs().max()) <= 2e-2


@pytest.mark.gpu
def test_gpu_flow_large_batch_paths_agree():
    """Ragged batch over many super-tiles: the tcgen05 and mma.sync passes agree."""
    dim = 8
    fl = _gpu_flow(dim, _theta(dim))
    L = N.load()
    u = torch.rand(300001, dim, device='cuda', generator=torch.Generator(device='cuda').manual_seed(5))
    st = ctypes.c_int(0)
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    z1, ld1 = fl.sample(u)
    L.vg_flow_set_path(1)
    try:
        z2, ld2 = fl.sample(u)
    finally:
        L.vg_flow_set_path(0)
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    assert st.value == 0
    # the passes round differently (FP32 order, BF16 rounding of H1/H2 can
    # flip between them and the flip propagates through later layers): rows
    # agree to ~1e-6; rare rows differ by a few 1e-2 in logdet
    dz = (z1 - z2).abs().max(dim=1).values
    dl = (ld1 - ld2).abs()
    assert float(dz.max()) <= 5e-3
    assert float(dl.median()) <= 1e-5
    assert float(torch.quantile(dl[:100000], 0.9999)) <= 2e-2
    assert float(dl.max()) <= 0.1


@pytest.mark.gpu
@pytest.mark.parametrize('dim', [1, 3, 4, 8, 16])
def test_gpu_flow_gradient_vs_oracle(dim, flow_path):
    theta = _theta(dim, seed=2, out_scale=0.3)
    fl = _gpu_flow(dim, theta)
    rng = np.random.default_rng(dim)
    n = 777   # ragged: not a multiple of the 128-row tile
    x = rng.random((n, dim)).astype(np.float32)
    w = (rng.random(n) ** 3 + 0.01).astype(np.float32)
    fl.grad.zero_()
    fl.loss.zero_()
    fl.accumulate_grad(torch.from_numpy(x).cuda(), torch.from_numpy(w).cuda())
    g = fl.grad.cpu().double().numpy() / w.astype(np.float64).sum()
    loss = float(fl.loss.item()) / w.astype(np.float64).sum()
    lo, go = _oracle_bf16(F.loss_and_grad, theta, x.astype(np.float64), w.astype(np.float64), dim)
    assert abs(loss - lo) <= 1e-3 * max(1.0, abs(lo))
    u = 2.0 ** -9                      # BF16 unit roundoff
    err = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert err <= 2 * u, err
    o = 0
    for li, sz in enumerate(F.layer_sizes(dim, 6, 32, 128)):
        for name in ('W1', 'b1', 'W2', 'b2', 'W3', 'b3'):
            a, b = g[o:o + sz[name]], go[o:o + sz[name]]
            o += sz[name]
            eb = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert eb <= 4 * u, (li, name, eb)
    assert o == len(go)


@pytest.mark.gpu
@pytest.mark.parametrize('dim,K', [(8, 32), (4, 16), (3, 32), (16, 32), (9, 16), (1, 32), (2, 16)])
def test_gpu_flow_backward_paths_agree(dim, K):
    """40000 rows (313 tiles: several per CTA of the tcgen05 backward, so its
    dW1 accumulator carries across tiles, and a multi-stage weight-gradient
    pipeline; dim 16 and 9 have layers of 8 and 5 transformed coordinates,
    two coordinate groups with the W3 rows streamed per group): the tcgen05
    backward against the mma.sync backward.  Both
    round the same operands to BF16; they differ in summation order and in
    rare BF16 rounding flips.  Each path is within 2u of the oracle overall
    and 4u per block (test above), so the two agree within the same bounds
    (measured: 0.6-1.4u overall)."""
    theta = _theta(dim, K=K, seed=5, out_scale=0.3)
    fl = _gpu_flow(dim, theta, K=K)
    gen = torch.Generator(device='cuda').manual_seed(dim * 100 + K)
    n = 40000
    x = torch.rand(n, dim, device='cuda', generator=gen)
    w = torch.rand(n, device='cuda', generator=gen) ** 3 + 0.01
    L = N.load()
    st = ctypes.c_int(0)
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    out = []
    for legacy in (0, 1):
        L.vg_flow_set_path(legacy)
        try:
            fl.grad.zero_()
            fl.loss.zero_()
            fl.accumulate_grad(x, w)
            out.append((fl.grad.cpu().double().numpy(), float(fl.loss.item())))
        finally:
            L.vg_flow_set_path(0)
    N.check(L.vg_flow_status(ctypes.byref(st), 1))
    assert st.value == 0, 'a bounded wait of the tensor-core backward gave up'
    (g0, l0), (g1, l1) = out
    u = 2.0 ** -9
    assert np.all(np.isfinite(g0))
    # the loss sums 2.4e5 FP32 log-pdf terms of two forward passes that round differently
    assert abs(l0 - l1) <= 1e-4 * abs(l1)
    assert np.linalg.norm(g0 - g1) / np.linalg.norm(g1) <= 2 * u
    o = 0
    for li, sz in enumerate(F.layer_sizes(dim, 6, K, 128)):
        for name in ('W1', 'b1', 'W2', 'b2', 'W3', 'b3'):
            a, b = g0[o:o + sz[name]], g1[o:o + sz[name]]
            o += sz[name]
            assert np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30) <= 4 * u, (li, name)


@pytest.mark.gpu
@pytest.mark.parametrize('n', [1, 5, 129])
def test_gpu_flow_gradient_tiny_batches(n):
    """Batches of 1, 5 and 129 rows (one tile of padding rows, and one row
    into a second tile): the tcgen05 and mma.sync backwards agree and the
    padding rows contribute nothing."""
    dim = 8
    fl = _gpu_flow(dim, _theta(dim, seed=7, out_scale=0.3))
    gen = torch.Generator(device='cuda').manual_seed(n)
    x = torch.rand(n, dim, device='cuda', generator=gen)
    w = torch.rand(n, device='cuda', generator=gen) + 0.1
    L = N.load()
    out = []
    for legacy in (0, 1):
        L.vg_flow_set_path(legacy)
        try:
            fl.grad.zero_()
            fl.loss.zero_()
            fl.accumulate_grad(x, w)
            out.append((fl.grad.cpu().double().numpy(), float(fl.loss.item())))
        finally:
            L.vg_flow_set_path(0)
    (g0, l0), (g1, l1) = out
    assert np.all(np.isfinite(g0))
    assert abs(l0 - l1) <= 1e-5 * abs(l1)
    assert np.linalg.norm(g0 - g1) <= 2 * 2.0 ** -9 * np.linalg.norm(g1)


@pytest.mark.gpu
def test_gpu_flow_training_learns_a_bump():
    """Adam steps on samples of a narrow off-diagonal 2-bump target reduce
    the variance of f/q by a large factor."""
    from vegas_gb300.flow import Flow
    dim = 4
    dev = torch.device('cuda')
    c = torch.tensor([[0.3, 0.7, 0.4, 0.6], [0.7, 0.3, 0.6, 0.4]], device=dev)

    def f(x):
        d2 = ((x.unsqueeze(1) - c) ** 2).sum(-1)
        return torch.exp(-d2 / (2 * 0.05 ** 2)).sum(1)

    fl = Flow(dim, lr=3e-3, seed=3)
    gen = torch.Generator(device=dev).manual_seed(0)

    def var_per_eval(n=1 << 16):
        u = torch.rand(n, dim, device=dev, generator=gen)
        z, ld = fl.sample(u)
        r = f(z) * torch.exp(-ld)
        return float(r.var() / r.mean() ** 2)

    v0 = var_per_eval()
    for it in range(300):
        u = torch.rand(4096, dim, device=dev, generator=gen)
        with torch.no_grad():
            z, ld = fl.sample(u)
            w = (f(z) * torch.exp(-ld)) ** 2    # (f/q)^2 with q(z) = exp(logdet(z))
        fl.train_step(z, w)
    v1 = var_per_eval()
    assert v1 < v0 / 5, (v0, v1)
