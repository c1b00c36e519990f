"""The public sampling API -- Integrator.random_batch / random / sample
(pyx:1601-1634, 1770-1814, 1816-1863) -- against the oracle's points.

The integrator is put in the oracle's state after two adapting iterations
of a peaked integrand (non-uniform grid, non-uniform sigf), so the points
come from a real vegas+ allocation.  FP64: y and hypercube ids bit-exact,
x and weights <= 1e-15 relative (the tolerances of the other FP64 parity
tests); neval_h bit-exact against the oracle's allocation from the same
sigf."""
import numpy as np
import pytest
import torch

import oracle as O
import vegas_gb300 as vg

pytestmark = pytest.mark.gpu
SEED = 808


def _adapted(neval=5000, dim=3):
    f = vg.Gaussian(a=30.0, c=0.4, dim=dim)
    st = O.State(dim * [[0, 1]], neval)
    for itn in range(1, 3):
        st.iterate(f.kind, f.params(dim), seed=SEED, stream=0, itn=itn)
    I = vg.Integrator(dim * [[0, 1]], neval=neval, precision='fp64', seed=SEED)
    g = torch.from_numpy(np.nan_to_num(st.grid)).to(I.device)
    I.map._grid.copy_(g)
    I.map._inc.copy_(torch.diff(g, dim=1))
    I._sigf.copy_(torch.from_numpy(st.sigf).to(I.device))
    I.sum_sigf = float(st.sum_sigf)
    return I, st


def _oracle_points(st, itn):
    nsf = st.neval_frac * st.neval / st.sum_sigf
    nh, rng, tot = O.alloc(st.sigf, nsf, True, st.min_neval_hcube, st.max_neval_hcube,
                           int(float(st.neval) / float(st.H)))
    y, x, w, hc = O.points(st.nstrat, st.grid, st.inc, st.ninc, nh, seed=SEED, stream=0, itn=itn)
    return nh, rng, y, x, w, hc


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_random_batch_matches_oracle_points():
    I, st = _adapted()
    I.min_neval_batch = 1000            # several batches
    itn = I._itn + 1
    batches = list(I.random_batch(yield_hcube=True, yield_y=True))
    assert len(batches) > 1
    x = torch.cat([b[0] for b in batches]).cpu().numpy()
    y = torch.cat([b[1] for b in batches]).cpu().numpy()
    w = torch.cat([b[2] for b in batches]).cpu().numpy()
    hc = torch.cat([b[3] for b in batches]).cpu().numpy()
    nh, rng, yo, xo, wo, hco = _oracle_points(st, itn)
    assert np.array_equal(I._neval_h_host(), nh)
    assert list(I.neval_hcube_range) == list(rng)
    assert I.last_neval == len(wo) == len(w)
    assert np.array_equal(y, yo)
    assert np.array_equal(hc, hco)
    assert _rel(x, xo) <= 1e-15
    assert _rel(w, wo) <= 1e-15
    # the batches follow min_neval_batch
    assert all(b[0].shape[0] == 1000 for b in batches[:-1])


def test_random_matches_random_batch():
    I1, _ = _adapted()
    I2, _ = _adapted()
    pts = []
    for k, p in enumerate(I1.random(yield_hcube=True, yield_y=True)):
        pts.append(p)
        if k == 99:
            break
    b = next(iter(I2.random_batch(yield_hcube=True, yield_y=True)))
    for i, (x, y, w, hc) in enumerate(pts):
        assert torch.equal(x, b[0][i]) and torch.equal(y, b[1][i])
        assert float(w) == float(b[2][i]) and int(hc) == int(b[3][i])


def test_sample_matches_oracle_and_estimates_integral():
    I, st = _adapted()
    itn = I._itn + 1
    w, x = I.sample(mode='rbatch')
    assert x.shape[0] == 3                      # rbatch: [dim, n]
    nh, rng, yo, xo, wo, hco = _oracle_points(st, itn)
    assert _rel(x.t().cpu().numpy(), xo) <= 1e-15
    assert _rel(w.cpu().numpy(), wo) <= 1e-15
    # sum(wgt * f(x)) estimates the integral (pyx:1816-1863)
    f = vg.Gaussian(a=30.0, c=0.4, dim=3)
    est = float((w * f(x.t())).sum())
    assert abs(est - f.exact(3)) < 0.05 * f.exact(3)
    # nbatch above neval: several passes, weights divided by their number
    w2, x2 = I.sample(nbatch=2 * I.last_neval, mode='lbatch')
    assert x2.shape[1] == 3 and x2.shape[0] == w2.shape[0]
    # sum(wgt) estimates the unit volume (exactly 1 only on a uniform map)
    assert abs(float(w2.sum()) - 1.0) < 0.05
