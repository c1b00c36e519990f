"""GPU parity tests: CUDA kernels (through the C ABI) against the oracle and
the reference's golden traces.

Tolerances (FP64 paths): points (y, hypercube ids, allocation) bit-exact;
x, weights <= 1e-15 relative; per-iteration mean / sdev, sigf, sum_sigf,
training histogram and adapted grid <= 1e-12 relative.  FP32 paths: final
integrals within 3 combined standard deviations of the exact value.
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


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def set_state(I, grid, sigf, sum_sigf):
    g = torch.from_numpy(np.nan_to_num(grid)).to(I.device)
    I.map._grid.copy_(g)
    I.map._inc.copy_(torch.diff(g, dim=1))
    I._sigf.copy_(torch.from_numpy(np.asarray(sigf, float)).to(I.device))
    I.sum_sigf = float(sum_sigf)


def replay_on_gpu(tr, alpha=0.5, beta=0.75):
    dim = len(tr['nstrat'])
    I = vg.Integrator(dim * [[0, 1]], neval=int(tr['neval']), precision='fp64', seed=1,
                      alpha=alpha, beta=beta)
    assert list(I.nstrat) == list(tr['nstrat'])
    assert list(I.map.ninc) == list(tr['ninc'])
    assert I.min_neval_hcube == int(tr['min_neval_hcube'])
    H = I.nhcube
    grid = tr['grid_init']
    sigf = tr['sigf_init'] if len(tr['sigf_init']) else np.ones(H)
    sum_sigf = float(tr['sum_sigf_init'])
    L = N.load()
    stream = N.stream_ptr(I.device)
    for k in range(int(tr['nitn'])):
        set_state(I, grid, sigf, sum_sigf)
        it, ncap = I._struct()
        I._allocate(it)
        st = I._read_stats()
        assert st.neval == int(tr['last_neval%d' % k])
        assert [st.range_lo, st.range_hi] == list(tr['range%d' % k])
        # allocation: bit-exact against the oracle from the same sigf
        nsf = float(tr['neval_frac']) * int(tr['neval']) / sum_sigf if sum_sigf > 0 else 0.0
        nh_o, _, _ = O.alloc(sigf, nsf, beta > 0 and H > 1, I.min_neval_hcube,
                             I.max_neval_hcube, int(int(tr['neval']) / H))
        assert np.array_equal(I._neval_h_host(), nh_o)
        # points with the reference's injected uniforms
        u_np = tr['u%d' % k].astype(np.float64) * 2.0 ** -24
        u = torch.from_numpy(u_np).to(I.device)
        x, y, w, hc = I._points(it, ncap, 1, u, want_y=True, want_hc=True)
        n = st.neval
        g0 = np.nan_to_num(grid)
        yo, xo, wo, hco = O.points(tr['nstrat'], g0, np.diff(g0, axis=1), tr['ninc'], nh_o, u=u_np)
        assert np.array_equal(y[:n].cpu().numpy(), yo)
        assert np.array_equal(hc[:n].cpu().numpy(), hco)
        assert rel(x[:n].cpu().numpy(), xo) <= 1e-15
        assert rel(w[:n].cpu().numpy(), wo) <= 1e-15
        # reduction of the reference's own integrand values
        f = torch.zeros(ncap, dtype=torch.float64, device=I.device)
        f[:n] = torch.from_numpy(tr['f%d' % k]).to(I.device)
        I.map.sum_f.zero_()
        I.map.n_f.zero_()
        N.check(L.vg_reduce(ctypes.byref(it), 1, N.ptr(u), N.ptr(f), N.VG_F64, stream))
        st = I._read_stats()
        assert st.status == 0 and not st.nan_seen
        assert rel(st.mean, tr['mean%d' % k]) <= RTOL
        assert rel(st.var ** 0.5, tr['sdev%d' % k]) <= RTOL
        new_sigf = I.sigf
        assert rel(new_sigf, tr['sigf%d' % k]) <= RTOL
        assert rel(st.sum_sigf, tr['sum_sigf%d' % k]) <= RTOL
        # training histogram against the oracle on the same fdv2
        _, _, _, _, fdv2 = O.reduce(nh_o, wo, tr['f%d' % k], beta=beta, sigf=sigf)
        sf_o, nf_o = O.add_training_data(tr['ninc'], I.map.inc_tensor.shape[1], yo, fdv2)
        sf = I.map.sum_f.cpu().numpy()
        nf = I.map.n_f.cpu().numpy()
        assert np.array_equal(nf.astype(float) + O.TINY, nf_o)
        assert rel(sf[sf_o > 0], sf_o[sf_o > 0]) <= RTOL
        # adapt on the device
        N.check(L.vg_end_iteration(ctypes.byref(it), stream))
        gnew = I.map.grid
        want = tr['grid%d' % k]
        ok = ~np.isnan(want)
        assert np.max(np.abs(gnew[ok] - want[ok])) <= RTOL * np.max(np.abs(want[ok]))
        grid, sigf, sum_sigf = want, tr['sigf%d' % k], float(tr['sum_sigf%d' % k])


def test_replay_gauss4_reference_trace():
    replay_on_gpu(load('ref_gauss4_injected.npz'))


def test_replay_ridge_reference_trace():
    replay_on_gpu(load('ref_ridge_injected.npz'))


def test_map_kernel_edges_golden():
    c = load('ref_map_adapt.npz')
    g = np.nan_to_num(c['map_grid'])
    m = vg.AdaptiveMap([list(g[d, :c['map_ninc'][d] + 1]) for d in range(2)])
    y = torch.from_numpy(c['map_y']).cuda()
    x = torch.empty_like(y)
    jac = torch.empty(y.shape[0], dtype=torch.float64, device='cuda')
    m.map(y, x, jac)
    assert np.array_equal(x.cpu().numpy(), c['map_x'])
    assert np.array_equal(jac.cpu().numpy(), c['map_jac'])


def test_adapt_kernel_golden():
    c = load('ref_map_adapt.npz')
    for k in range(int(c['n_adapt'])):
        p = 'adapt%d_' % k
        ninc = c[p + 'ninc_in']
        g = np.nan_to_num(c[p + 'grid_in'])
        m = vg.AdaptiveMap([list(g[d, :ninc[d] + 1]) for d in range(len(ninc))])
        if bool(c[p + 'train']):
            m.add_training_data(c[p + 'y'], c[p + 'f'])
            sf, nf = m.training_data()
            assert rel(sf[c[p + 'sum_f'] > 0], c[p + 'sum_f'][c[p + 'sum_f'] > 0]) <= RTOL
            assert np.array_equal(nf, c[p + 'n_f'])
        m.adapt(alpha=float(c[p + 'alpha']), ninc=c[p + 'new_ninc'])
        want = c[p + 'grid_out']
        ok = ~np.isnan(want)
        got = m.grid
        assert np.max(np.abs(got[ok] - want[ok])) <= RTOL * np.max(np.abs(want[ok])), k


def test_fused_fp64_matches_oracle_philox():
    """Fused FP64 iterations (Philox draws) == oracle on the same draws.

    Each iteration starts the GPU from the oracle's state (grid, sigf,
    sum_sigf), so single-iteration outputs are compared at 1e-12; a second
    loop lets both run freely and checks the looser agreement that results
    from grid differences at the 1e-16 level being amplified."""
    for f in (vg.Gaussian(a=100.0, c=0.5, dim=4), vg.Ridge(M=50, s=0.05)):
        seed = 99
        I = vg.Integrator(4 * [[0, 1]], neval=6000, precision='fp64', seed=seed)
        st = O.State(4 * [[0, 1]], 6000)
        for itn in range(1, 4):
            set_state(I, st.grid, st.sigf, st.sum_sigf)
            r = I(f, nitn=1)
            out = st.iterate(f.kind, f.params(4), seed=seed, stream=0, itn=itn)
            assert I.last_neval == out['neval']
            assert rel(r.itn_results[0].mean, out['mean']) <= RTOL
            assert rel(r.itn_results[0].var, out['var']) <= RTOL
            assert rel(I.sigf, st.sigf) <= RTOL
            g = I.map.grid
            for d in range(4):
                K = st.ninc[d]
                assert np.max(np.abs(g[d, :K + 1] - st.grid[d, :K + 1])) <= RTOL
        # free-running: same draws, independent state
        I = vg.Integrator(4 * [[0, 1]], neval=6000, precision='fp64', seed=seed)
        st = O.State(4 * [[0, 1]], 6000)
        for itn in range(1, 6):
            r = I(f, nitn=1)
            out = st.iterate(f.kind, f.params(4), seed=seed, stream=0, itn=itn)
            assert I.last_neval == out['neval']
            assert rel(r.itn_results[0].mean, out['mean']) <= 1e-9


@pytest.mark.parametrize('dim,neval,alpha,beta,adapt', [
    (1, 500, 0.5, 0.75, True),     # one axis
    (3, 60, 0.5, 0.75, True),      # a handful of evaluations: few hypercubes, few increments
    (6, 3000, 0.5, 0.0, True),     # beta = 0: uniform allocation, no sigf
    (9, 4000, 0.5, 0.75, True),    # above 8 dimensions: the generic-dimension kernel
    (12, 3000, 0.0, 0.75, True),   # alpha = 0: the map stays as it is
    (4, 3000, 0.5, 0.75, False),   # adapt = False: neither sigf nor the map change
])
def test_fused_fp64_edge_shapes_match_oracle(dim, neval, alpha, beta, adapt):
    """Fused FP64 iterations (Philox draws, one vg_iterate call each) ==
    oracle on the same draws, for shapes and settings at the edges of the
    sizing and adapt logic; each iteration starts from the oracle's state."""
    f = vg.Gaussian(a=20.0, c=0.45, dim=dim)
    I = vg.Integrator(dim * [[0, 1]], neval=neval, precision='fp64', seed=5, alpha=alpha, beta=beta,
                      adapt=adapt)
    st = O.State(dim * [[0, 1]], neval, alpha=alpha, beta=beta)
    assert list(I.nstrat) == list(st.nstrat)
    assert list(I.map.ninc) == list(st.ninc)
    for itn in range(1, 4):
        set_state(I, st.grid, st.sigf, st.sum_sigf)
        r = I(f, nitn=1)
        out = st.iterate(f.kind, f.params(dim), seed=5, stream=0, itn=itn, adapt=adapt)
        assert I.last_neval == out['neval']
        assert list(I.neval_hcube_range) == list(out['range'])
        assert rel(r.itn_results[0].mean, out['mean']) <= RTOL
        assert rel(r.itn_results[0].var, out['var']) <= RTOL
        assert rel(I.sigf, st.sigf) <= RTOL
        g = I.map.grid
        for d in range(dim):
            K = st.ninc[d]
            assert np.max(np.abs(g[d, :K + 1] - st.grid[d, :K + 1])) <= RTOL


def test_dropin_matches_fused_fp64():
    """lbatch torch integrand path == fused built-in path (same draws)."""
    f = vg.Ridge(M=40, s=0.05)
    I1 = vg.Integrator(4 * [[0, 1]], neval=5000, precision='fp64', seed=7)
    I2 = vg.Integrator(4 * [[0, 1]], neval=5000, precision='fp64', seed=7)

    @vg.lbatchintegrand
    def g(x):
        return f(x)

    r1 = I1(f, nitn=3)
    r2 = I2(g, nitn=3)
    for a, b in zip(r1.itn_results, r2.itn_results):
        assert rel(a.mean, b.mean) <= 1e-10
        assert rel(a.var, b.var) <= 1e-8


def test_fp32_gauss_config1_statistics():
    f = vg.Gaussian(a=100.0, c=0.5, dim=4)
    I = vg.Integrator(4 * [[0, 1]], seed=2024)
    I(f, nitn=10, neval=1e4, alpha=0.5, beta=0.75)
    r = I(f, nitn=10, neval=1e4)
    exact = f.exact(4)
    assert abs(r.mean - exact) < 3 * r.sdev, (r, exact)
    assert r.sdev / exact < 5e-3


def test_fp32_ridge_config2_statistics():
    f = vg.Ridge(M=1000, s=0.01)
    I = vg.Integrator(4 * [[0, 1]], seed=77)
    I(f, nitn=10, neval=1e6)
    r = I(f, nitn=10, neval=1e6)
    exact = f.exact(4)
    assert abs(r.mean - exact) < 3 * r.sdev, (r, exact)
    assert r.dof == 9


def test_nan_integrand_raises():
    @vg.lbatchintegrand
    def bad(x):
        out = torch.ones(x.shape[0], dtype=x.dtype, device=x.device)
        out[0] = float('nan')
        return out

    I = vg.Integrator(2 * [[0, 1]], seed=1)
    with pytest.raises(ValueError):
        I(bad, nitn=1, neval=1000)


def test_integrand_exception_propagates():
    @vg.lbatchintegrand
    def bad(x):
        return 1 / 0.

    I = vg.Integrator(2 * [[0, 1]], seed=1)
    with pytest.raises(ZeroDivisionError):
        I(bad, nitn=1, neval=100)


def test_constant_integrand_epsilon_guard():
    # test_vegas.py:1272-1296: sdev ratios exactly 1 and 2 from the EPSILON guard
    I = vg.Integrator([(0, 1)], neval=100, alpha=0, seed=3, precision='fp64')
    res = I(vg.Constant(7.0), nitn=4)
    np.testing.assert_almost_equal(res.itn_results[0].sdev / res.itn_results[1].sdev, 1.0, 7)
    np.testing.assert_almost_equal(res.itn_results[0].sdev / res.sdev, 2.0, 7)
    np.testing.assert_almost_equal(res.mean, 7.0, 7)
    res = I(vg.Constant(0.0), nitn=4)
    assert res.mean == 0.0


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_reduce_kept_matches_reduce(precision):
    """vg_sample_keep + vg_reduce_kept (the reduction streams the kept
    Jacobians and training bins) == vg_sample + vg_reduce (the reduction
    regenerates every sample) on the same allocation and integrand values:
    mean, variance, sum_sigf and sigf bit for bit (same arithmetic, static
    tile partials in a fixed order); the training histogram bit for bit in
    FP64 and at 1e-6 relative in FP32 (FP32 atomic adds in arrival order)."""
    L = N.load()
    f = vg.Gaussian(a=30.0, c=0.45, dim=4)
    A = vg.Integrator(4 * [[0, 1]], neval=200000, precision=precision, seed=21)
    A(f, nitn=2)                               # a non-uniform map and sigf
    B = vg.Integrator(4 * [[0, 1]], neval=200000, precision=precision, seed=21)
    set_state(B, A.map.grid, A.sigf, A.sum_sigf)
    stream = N.stream_ptr(A.device)
    res = []
    for I, kept in ((A, False), (B, True)):
        it, ncap = I._struct()
        I._allocate(it)
        n = int(I._read_stats().neval)
        keep = I._keep_buffer(it, ncap) if kept else None
        x, _, _, _ = I._points(it, ncap, 9, None, want_w=False, keep=keep)
        fx = torch.zeros(ncap, dtype=x.dtype, device=x.device)
        fx[:n] = f(x[:n])
        fdt = N.VG_F64 if precision == 'fp64' else N.VG_F32
        if kept:
            N.check(L.vg_reduce_kept(ctypes.byref(it), 9, None, N.ptr(fx), fdt, N.ptr(keep), keep.numel(),
                                     stream))
        else:
            N.check(L.vg_reduce(ctypes.byref(it), 9, None, N.ptr(fx), fdt, stream))
        st = I._read_stats()
        res.append((st, I.sigf.copy(), I.map.sum_f.cpu().numpy().copy(), I.map.n_f.cpu().numpy().copy(), n))
    (sa, ga, ha, ca, na), (sb, gb, hb, cb, nb) = res
    assert na == nb
    assert sa.mean == sb.mean and sa.var == sb.var and sa.sum_sigf == sb.sum_sigf
    assert np.array_equal(ga, gb)
    assert np.array_equal(ca, cb) and 0 < ca.sum() <= na * 4
    tol = 1e-12 if precision == 'fp64' else 1e-6
    assert np.max(np.abs(ha - hb)) <= tol * np.max(np.abs(ha))


def test_stepwise_builtin_path_matches_pipelined(tmp_path):
    """A built-in integrand with a host decision per iteration (rtol stop,
    analyzer, save) runs the same kernels as the pipelined call: identical
    iteration results on the same draws; rtol stops the loop; the analyzer
    sees every iteration; save writes the running result.  FP64, compared
    at the FP64 parity tolerance: the training histogram's FP64 atomics add
    in arrival order, so the adapted maps of two runs differ at the 1e-16
    level."""
    import pickle
    f = vg.Gaussian(a=60.0, c=0.45, dim=3)
    A = vg.Integrator(3 * [[0, 1]], neval=20000, seed=17, precision='fp64')
    B = vg.Integrator(3 * [[0, 1]], neval=20000, seed=17, precision='fp64')
    ra = A(f, nitn=6)
    seen = []

    class Watch(object):
        def begin(self, itn, integrator):
            seen.append(('begin', itn))

        def end(self, itn_result, result):
            seen.append(('end', itn_result.mean))

    out = str(tmp_path / 'r.pkl')
    rb = B(f, nitn=6, rtol=1e-15, analyzer=Watch(), save=out)
    assert len(ra.itn_results) == len(rb.itn_results) == 6
    assert rel([x.mean for x in rb.itn_results], [x.mean for x in ra.itn_results]) <= RTOL
    assert rel([x.sdev for x in rb.itn_results], [x.sdev for x in ra.itn_results]) <= RTOL
    ga, gb = np.nan_to_num(A.map.grid), np.nan_to_num(B.map.grid)
    assert np.max(np.abs(ga - gb)) <= RTOL and rel(B.sigf, A.sigf) <= 1e-10
    assert len(seen) == 12 and seen[0] == ('begin', 0)
    with open(out, 'rb') as fh:
        assert abs(pickle.load(fh).mean - rb.mean) <= 1e-15 * abs(rb.mean)
    C = vg.Integrator(3 * [[0, 1]], neval=20000, seed=17, precision='fp64')
    rc = C(f, nitn=6, rtol=0.5)
    assert rc.nitn == 1


def test_speculative_rtol_path_leaves_the_state_of_the_stop():
    """An rtol stop without other host hooks runs one iteration ahead of the
    host and undoes it at the stop: the same iterations, results and final
    state (map, sigf, sum_sigf, iteration counter) as the iteration-by-
    iteration loop (here: the same call with an analyzer), and the next call
    continues identically (FP64, parity tolerance)."""
    f = vg.Gaussian(a=60.0, c=0.45, dim=3)

    class Quiet(object):
        def begin(self, itn, integrator):
            pass

        def end(self, itn_result, result):
            pass

    A = vg.Integrator(3 * [[0, 1]], neval=20000, seed=29, precision='fp64')
    B = vg.Integrator(3 * [[0, 1]], neval=20000, seed=29, precision='fp64')
    ra = A(f, nitn=40, rtol=2e-3)
    rb = B(f, nitn=40, rtol=2e-3, analyzer=Quiet())
    assert 1 < ra.nitn < 40 and ra.nitn == rb.nitn
    assert rel([x.mean for x in ra.itn_results], [x.mean for x in rb.itn_results]) <= RTOL
    assert A._itn == B._itn == ra.nitn
    assert rel(A.sum_sigf, B.sum_sigf) <= RTOL and rel(A.sigf, B.sigf) <= 1e-10
    ga, gb = np.nan_to_num(A.map.grid), np.nan_to_num(B.map.grid)
    assert np.max(np.abs(ga - gb)) <= RTOL
    B.set(analyzer=None)
    ra2, rb2 = A(f, nitn=2), B(f, nitn=2)
    assert rel([x.mean for x in ra2.itn_results], [x.mean for x in rb2.itn_results]) <= RTOL
