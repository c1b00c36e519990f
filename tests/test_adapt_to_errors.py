"""adapt_to_errors=True on the GPU (Integrator.adapt_to_errors, pyx:1092-1101).

In this mode the map has one increment per stratum, every hypercube gets
int(neval / nhcube) evaluations, no sigf is kept, and after each hypercube's
reduction its |variance| is added to the training histogram at the y of the
hypercube's last sample (pyx:1372, 1662, 1675, 2181-2196, 2209).

* injected-sample replay of a trace recorded from the compiled reference:
  allocation bit-exact, mean / sdev, training histogram and adapted grid
  <= 1e-12 relative (FP64);
* fused FP64 iterations with Philox draws against the oracle on the same
  draws (1e-12), including hypercubes that cross tile boundaries (their
  last sample is regenerated by the finalize kernel);
* FP32: the integral within 3 sigma of the exact value.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

import oracle as O
import vegas_gb300 as vg
from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
RTOL = 1e-12


def rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def set_grid(I, grid):
    g = torch.from_numpy(np.nan_to_num(grid)).to(I.device)
    I.map._grid.copy_(g)
    I.map._inc.copy_(torch.diff(g, dim=1))


def test_replay_ate_reference_trace():
    tr = dict(np.load(os.path.join(GOLD, 'ref_ate_injected.npz')))
    I = vg.Integrator(2 * [[0, 1]], neval=int(tr['neval']), precision='fp64', seed=1, alpha=0.5,
                      adapt_to_errors=True)
    assert list(I.nstrat) == list(tr['nstrat']) and list(I.map.ninc) == list(tr['ninc'])
    H = I.nhcube
    ninc = tr['ninc']
    L = N.load()
    stream = N.stream_ptr(I.device)
    grid = tr['grid_init']
    for k in range(int(tr['nitn'])):
        set_grid(I, grid)
        it, ncap = I._struct()
        I._allocate(it)
        st = I._read_stats()
        assert st.neval == int(tr['last_neval%d' % k])
        assert [st.range_lo, st.range_hi] == list(tr['range%d' % k])
        nh = I._neval_h_host()
        assert np.all(nh == int(int(tr['neval']) / H))
        u_np = tr['u%d' % k].astype(np.float64) * 2.0 ** -24
        u = torch.from_numpy(u_np).to(I.device)
        x, y, w, hc = I._points(it, ncap, 1, u, want_y=True, want_hc=True)
        n = st.neval
        f = torch.zeros(ncap, dtype=torch.float64, device=I.device)
        f[:n] = torch.from_numpy(tr['f%d' % k]).to(I.device)
        I.map.sum_f.zero_()
        I.map.n_f.zero_()
        N.check(L.vg_reduce(ctypes.byref(it), 1, N.ptr(u), N.ptr(f), N.VG_F64, stream))
        st = I._read_stats()
        assert st.status == 0 and not st.nan_seen
        assert rel(st.mean, tr['mean%d' % k]) <= RTOL
        assert rel(st.var ** 0.5, tr['sdev%d' % k]) <= RTOL
        # training histogram: each hypercube's |variance| at its last sample
        g0 = np.nan_to_num(grid)
        yo, xo, wo, hco = O.points(tr['nstrat'], g0, np.diff(g0, axis=1), ninc, nh, u=u_np)
        _, _, _, _, _, hv = O.reduce(nh, wo, tr['f%d' % k], adaptive=False, hc_var=True)
        last = np.cumsum(nh) - 1
        sf_o, nf_o = O.add_training_data(ninc, I.map.inc_tensor.shape[1], yo[last], hv)
        sf = I.map.sum_f.cpu().numpy()
        nf = I.map.n_f.cpu().numpy()
        assert np.array_equal(nf.astype(float) + O.TINY, nf_o)
        assert rel(sf[sf_o > 0], sf_o[sf_o > 0]) <= RTOL
        N.check(L.vg_end_iteration(ctypes.byref(it), stream))
        gnew = I.map.grid
        want = tr['grid%d' % k]
        ok = ~np.isnan(want)
        assert np.max(np.abs(gnew[ok] - want[ok])) <= RTOL * np.max(np.abs(want[ok]))
        grid = want


@pytest.mark.parametrize('neval,nstrat', [(4000, None), (7500, [50, 50])])
def test_fused_fp64_ate_matches_oracle_philox(neval, nstrat):
    # nstrat 50x50 at neval 7500: 3 evaluations per hypercube, so tile
    # boundaries cut hypercubes and the finalize kernel trains those
    f = vg.Gaussian(a=50.0, c=0.3, dim=2)
    seed = 5
    kw = {} if nstrat is None else {'nstrat': nstrat}
    I = vg.Integrator(2 * [[0, 1]], neval=neval, precision='fp64', seed=seed, adapt_to_errors=True, **kw)
    st = O.State(2 * [[0, 1]], neval, adapt_to_errors=True, nstrat=nstrat)
    if nstrat is not None:
        assert int(neval / I.nhcube) == 3
    assert list(I.nstrat) == list(st.nstrat) and list(I.map.ninc) == list(st.ninc)
    for itn in range(1, 4):
        set_grid(I, st.grid)
        r = I(f, nitn=1)
        out = st.iterate(f.kind, f.params(2), seed=seed, stream=0, itn=itn)
        assert I.last_neval == out['neval']
        assert rel(r.itn_results[0].mean, out['mean']) <= RTOL
        assert rel(r.itn_results[0].var, out['var']) <= RTOL
        g = I.map.grid
        for d in range(2):
            K = st.ninc[d]
            assert np.max(np.abs(g[d, :K + 1] - st.grid[d, :K + 1])) <= RTOL


def test_fp32_ate_statistics():
    f = vg.Gaussian(a=50.0, c=0.3, dim=2)
    exact = f.exact(2)
    I = vg.Integrator(2 * [[0, 1]], neval=20000, seed=8, adapt_to_errors=True)
    I(f, nitn=10)
    r = I(f, nitn=10)
    assert abs(r.mean - exact) < 3 * r.sdev, (r.mean, r.sdev, exact)
    assert r.Q > 1e-3
