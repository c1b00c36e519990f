"""Array-valued integrands (reference fcn_size s > 1, _vegas.pyx:2136-2197).

GPU: the per-hypercube (co)variance kernel against a numpy restatement of
the reference loops on the same samples, FP64 (1e-12 relative); an
Integrator run returning an RAvgArray of the integrand's shape whose
components agree with their exact values (5 sigma), correlated and not; and
the same integrator, on the reference's injected uniforms, against the
compiled reference's own results (tests/golden/ref_array.npz): means and
covariance matrices per iteration and of the average, chi2 and Q."""
import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300 import _gvar as gv
from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu
EPSILON = 2.220446049250313e-16 * 1e4   # _vegas.pyx:36


def _ref_array_reduce(wgt, fx, hc, correlate):
    """pyx:2140-2193 restated in numpy (per hypercube, sample order)."""
    s = fx.shape[1]
    mean = np.zeros(s)
    var = np.zeros((s, s))
    for h in np.unique(hc):
        idx = np.nonzero(hc == h)[0]
        n = len(idx)
        wf = wgt[idx, None] * fx[idx]
        sum_wf = wf.sum(axis=0)
        m = sum_wf / n
        sum_dwf = np.zeros(s)
        sum_dwf2 = np.zeros((s, s))
        for j in range(n):
            dwf = wf[j] - m
            for c in range(s):
                if abs(dwf[c]) < EPSILON * abs(m[c]):
                    sum_dwf2[c, c] += (EPSILON * abs(m[c])) ** 2
                    dwf[c] = 0.0
                else:
                    sum_dwf2[c, c] += dwf[c] ** 2
                sum_dwf[c] += dwf[c]
                if correlate:
                    for t in range(c):
                        sum_dwf2[c, t] += dwf[c] * dwf[t]
        mean += sum_wf + sum_dwf
        for c in range(s):
            for t in range(c + 1 if correlate else 1):
                tt = t if correlate else c
                var[c, tt] += (n * sum_dwf2[c, tt] - sum_dwf[c] * sum_dwf[tt]) / (n - 1.)
    if correlate:
        var = np.tril(var) + np.tril(var, -1).T
    return mean, var


@vg.lbatchintegrand
def _f3(x):
    g = torch.exp(-20.0 * ((x - 0.45) ** 2).sum(dim=1))
    return torch.stack([g, x[:, 0] * g, x[:, 1] * x[:, 2] * g], dim=1)


@pytest.mark.parametrize('correlate', [True, False])
def test_array_reduction_matches_reference_loops(correlate):
    I = vg.Integrator(3 * [[0, 1]], neval=3000, precision='fp64', seed=5,
                      correlate_integrals=correlate)
    it, ncap = I._struct()
    I._allocate(it)
    n = int(I._read_stats().neval)
    x, _, w, hc = I._points(it, ncap, 1, None, want_hc=True)
    f = _f3(x[:n])
    fbuf = torch.zeros((ncap, 3), dtype=torch.float64, device=x.device)
    fbuf[:n] = f
    mean, var = I._reduce_array(it, fbuf, N.VG_F64, w)
    rm, rv = _ref_array_reduce(w[:n].cpu().numpy(), f.cpu().numpy(), hc[:n].cpu().numpy(), correlate)
    np.testing.assert_allclose(mean, rm, rtol=1e-12)
    np.testing.assert_allclose(var, rv, rtol=1e-11, atol=1e-300)


def test_array_reduction_many_uncorrelated_components():
    """More than 16 uncorrelated components: reduced 16 columns at a time."""
    I = vg.Integrator(3 * [[0, 1]], neval=3000, precision='fp64', seed=6,
                      correlate_integrals=False)
    it, ncap = I._struct()
    I._allocate(it)
    n = int(I._read_stats().neval)
    x, _, w, hc = I._points(it, ncap, 1, None, want_hc=True)
    base = _f3(x[:n])
    cols = [base[:, k % 3] * (1.0 + 0.1 * k) * (x[:n, k % 3] if k >= 3 else 1.0) for k in range(37)]
    f = torch.stack(cols, dim=1)
    fbuf = torch.zeros((ncap, 37), dtype=torch.float64, device=x.device)
    fbuf[:n] = f
    mean, var = I._reduce_array(it, fbuf, N.VG_F64, w)
    rm, rv = _ref_array_reduce(w[:n].cpu().numpy(), f.cpu().numpy(), hc[:n].cpu().numpy(), False)
    np.testing.assert_allclose(mean, rm, rtol=1e-12)
    np.testing.assert_allclose(var, rv, rtol=1e-11, atol=1e-300)


class _Draws(object):
    """The fixture's injected uniforms: u = k / 2^24, k from default_rng(seed)."""

    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)

    def __call__(self, size):
        return self.rng.integers(0, 2 ** 24, size=size, dtype=np.uint32).astype(np.float64) * 2.0 ** -24


@pytest.mark.parametrize('c,corr', [(0, True), (1, False)])
def test_array_integrand_matches_reference_golden(c, corr):
    """Three-component integrand against the compiled reference
    (tests/golden/ref_array.npz, make_golden.py array), injected uniforms,
    FP64: per-iteration means and covariance matrices, and the RAvgArray
    average, chi2 and Q."""
    import os
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'ref_array.npz')))
    p = 'c%d_' % c

    @vg.lbatchintegrand
    def f(x):
        gg = torch.exp(-20.0 * ((x - 0.45) ** 2).sum(dim=1))
        return torch.stack([gg, x[:, 0] * gg, x[:, 1] * x[:, 2] * gg], dim=1)

    I = vg.Integrator(3 * [[0, 1]], neval=3000, precision='fp64', ran_array_generator=_Draws(40 + c),
                      correlate_integrals=corr)
    r = I(f, nitn=3)
    for k, res in enumerate(r.itn_results):
        np.testing.assert_allclose([x.mean for x in res], g[p + 'itn_mean'][k], rtol=1e-10)
        cov = gv.evalcov(list(res))
        ref = g[p + 'itn_cov'][k]
        assert np.max(np.abs(cov - ref)) <= 1e-9 * np.max(np.abs(ref))
    np.testing.assert_allclose([x.mean for x in r], g[p + 'mean'], rtol=1e-10)
    cov = gv.evalcov(list(r))
    assert np.max(np.abs(cov - g[p + 'cov'])) <= 1e-9 * np.max(np.abs(g[p + 'cov']))
    assert abs(r.chi2 - float(g[p + 'chi2'])) <= 1e-8 * max(1.0, abs(float(g[p + 'chi2'])))
    assert abs(r.Q - float(g[p + 'Q'])) <= 1e-8


def test_array_integrand_results():
    for correlate in (True, False):
        I = vg.Integrator(3 * [[0, 1]], neval=20000, seed=9, correlate_integrals=correlate)
        I(_f3, nitn=6)
        r = I(_f3, nitn=8)
        assert isinstance(r, vg.RAvgArray) and r.shape == (3,)
        # exact values by a fine FP64 tensor-product midpoint rule
        m = 200
        g1 = (np.arange(m) + 0.5) / m
        e1 = np.exp(-20.0 * (g1 - 0.45) ** 2) / m
        ex = np.array([e1.sum() ** 3, (g1 * e1).sum() * e1.sum() ** 2, (g1 * e1).sum() ** 2 * e1.sum()])
        for k in range(3):
            assert abs(r[k].mean - ex[k]) < 5 * r[k].sdev, (k, r[k], ex[k])
        if correlate:
            c = vg._gvar.corr(r[0], r[1])
            assert 0.0 < c <= 1.0


def test_uses_jac_matches_reference_golden():
    """uses_jac=True on a map adapted to a peak, against the compiled
    reference on the same injected uniforms (tests/golden/ref_uses_jac.npz,
    make_golden.py uses_jac): the integrand gets dx/dy per direction."""
    import os
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'ref_uses_jac.npz')))

    @vg.lbatchintegrand
    def peak2(x):
        return torch.exp(-50.0 * (x[:, 0] - 0.3) ** 2) * (1.0 + x[:, 1] ** 2)

    @vg.lbatchintegrand
    def jac_f(x, jac):
        return torch.exp(-x[:, 0]) * jac[:, 0] / (1.0 + jac[:, 1])

    I = vg.Integrator(2 * [[0, 1]], neval=2000, precision='fp64', ran_array_generator=_Draws(60))
    I(peak2, nitn=3)
    r = I(jac_f, nitn=2, uses_jac=True)
    np.testing.assert_allclose([x.mean for x in r.itn_results], g['itn_mean'], rtol=1e-10)
    np.testing.assert_allclose([x.sdev for x in r.itn_results], g['itn_sdev'], rtol=1e-9)
    np.testing.assert_allclose([r.mean, r.sdev], [g['mean'], g['sdev']], rtol=1e-9)


def test_uses_jac_like_reference():
    """uses_jac=True: the integrand receives dx/dy per direction (reference
    test_vegas.py test_uses_jac: the integral of 1/prod(jac) over the map's
    range is 1 for any map), for scalar, lbatch and rbatch integrands and
    scalar / array results."""
    import numpy as np
    integ = vg.Integrator(2 * [[0, 2.]], precision='fp64', seed=3)

    def check(f, array=False):
        r = integ(f, nitn=1, neval=10, uses_jac=True)
        ans = r[0, 0] if array else r
        assert abs(ans.mean - 1.0) < 1e-10, ans

    check(lambda x, jac: 1. / np.prod(jac))
    check(lambda x, jac: [[1. / np.prod(jac)]], array=True)

    @vg.rbatchintegrand
    def fr(x, jac):
        return 1. / torch.prod(jac, dim=0)
    check(fr)

    @vg.rbatchintegrand
    def fr2(x, jac):
        return (1. / torch.prod(jac, dim=0))[None, None, :]
    check(fr2, array=True)

    @vg.lbatchintegrand
    def fl(x, jac):
        return 1. / torch.prod(jac, dim=-1)
    check(fl)

    @vg.lbatchintegrand
    def fl2(x, jac):
        return (1. / torch.prod(jac, dim=-1))[:, None, None]
    check(fl2, array=True)


def test_dict_integrands_and_uses_jac():
    """Dictionary-valued integrands give an RAvgDict keyed like the integrand
    (reference RAvgDict, pyx:2453); uses_jac dict variants of the reference's
    test_uses_jac."""
    import numpy as np
    integ = vg.Integrator(2 * [[0, 2.]], precision='fp64', seed=4)
    r = integ(lambda x, jac: dict(a=1. / np.prod(jac)), nitn=1, neval=10, uses_jac=True)
    assert isinstance(r, vg.RAvgDict) and abs(r['a'].mean - 1.0) < 1e-10

    @vg.rbatchintegrand
    def fr(x, jac):
        return dict(a=1. / torch.prod(jac, dim=0))
    r = integ(fr, nitn=1, neval=10, uses_jac=True)
    assert abs(r['a'].mean - 1.0) < 1e-10

    @vg.lbatchintegrand
    def fl(x, jac):
        return dict(a=1. / torch.prod(jac, dim=-1))
    r = integ(fl, nitn=1, neval=10, uses_jac=True)
    assert abs(r['a'].mean - 1.0) < 1e-10

    # several keys, scalar and array valued, against exact values
    @vg.lbatchintegrand
    def fd(x):
        g = torch.exp(-5.0 * ((x - 0.5) ** 2).sum(dim=1))
        return dict(g=g, moments=torch.stack([x[:, 0] * g, x[:, 1] * g], dim=1))
    I2 = vg.Integrator(2 * [[0, 1]], neval=20000, seed=6)
    I2(fd, nitn=5)
    r = I2(fd, nitn=6)
    m = 400
    t = (np.arange(m) + 0.5) / m
    e1 = np.exp(-5.0 * (t - 0.5) ** 2) / m
    g_ex = e1.sum() ** 2
    mom_ex = (t * e1).sum() * e1.sum()
    assert set(r.keys()) == {'g', 'moments'} and r['moments'].shape == (2,)
    assert abs(r['g'].mean - g_ex) < 5 * r['g'].sdev
    for k in range(2):
        assert abs(r['moments'][k].mean - mom_ex) < 5 * r['moments'][k].sdev
