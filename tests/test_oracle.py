"""Pin the oracle (CPU restatement) before trusting it as the GPU checker.

1. Known-answer tests transcribed from the reference's own suite
   (tests/test_vegas.py of vegas 6.4.1).
2. Replays of traces recorded from the compiled reference
   (tests/golden/make_golden.py): the oracle must reproduce the reference's
   FP64 results bit for bit (its operation order is the reference's).
3. Philox4x32-10 known-answer vectors (Random123 distribution).
"""
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


# --------------------------------------------------------------------------
# known answers (reference tests/test_vegas.py)
# --------------------------------------------------------------------------
def test_philox_kat():
    assert [hex(v) for v in O.philox([0, 0, 0, 0], [0, 0])] == \
        ['0x6627e8d5', '0xe169c58d', '0xbc57ac4c', '0x9b00dbd8']
    assert [hex(v) for v in O.philox([0xffffffff] * 4, [0xffffffff] * 2)] == \
        ['0x408f276d', '0x41c83b0e', '0xa20bc7c6', '0x6d5451fd']
    assert [hex(v) for v in O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                     [0xa4093822, 0x299f31d0])] == \
        ['0xd16cfe09', '0x94fdcceb', '0x5001e420', '0x24126ea1']


def test_uniform_ranges():
    u = np.array([O.uniform_f64(5, 0, 1, i, d) for i in range(2000) for d in range(5)])
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.02
    v = np.array([O.uniform_f32(5, 0, 1, i, d) for i in range(2000) for d in range(5)])
    assert v.min() >= 0.0 and v.max() < 1.0 and abs(v.mean() - 0.5) < 0.02


def test_map_known_answer():
    # test_vegas.py:76-95
    grid = np.array([[0., 1., 3.], [-2., 0., 6.]])
    inc = np.diff(grid, axis=1)
    y = np.array([[0, 0], [0.25, 0.25], [0.5, 0.5], [0.75, 0.75], [1.0, 1.0]])
    x, jac = O.map_points(grid, inc, [2, 2], y)
    np.testing.assert_allclose(x, [[0, -2], [0.5, -1], [1, 0], [2, 3], [3, 6]])
    np.testing.assert_allclose(jac, [8, 8, 48, 48, 48])


def test_init_regrid_known_answer():
    # test_vegas.py:39-63: AdaptiveMap(grid, ninc) regrids with adapt(ninc=)
    g, inc, _ = O.adapt([[0, 0.4, 1], [-2, 0., 4]], np.diff([[0, 0.4, 1], [-2, 0., 4]], axis=1),
                        [2, 2], None, None, 0.0, 4)
    np.testing.assert_allclose(g, [[0, 0.2, 0.4, 0.7, 1.], [-2., -1., 0., 2., 4.]])
    np.testing.assert_allclose(inc, [[0.2, 0.2, 0.3, 0.3], [1, 1, 2, 2]])
    g, inc = O.make_uniform([0, -2], [1, 4], [2, 2])
    np.testing.assert_allclose(g, [[0, 0.5, 1.], [-2., 1., 4.]])


def _adapt_loop(F, lims, ninc, alpha, nitn, ys):
    grid, inc = O.make_uniform([l[0] for l in lims], [l[1] for l in lims], ninc)
    ninc = np.array(ninc, np.int64)
    for _ in range(nitn):
        x, jac = O.map_points(grid, inc, ninc, ys)
        # f * jac (map Jacobian), as the reference test builds it
        f = F(x) * jac
        sum_f, n_f = O.add_training_data(ninc, inc.shape[1], ys, f)
        grid, inc, _ = O.adapt(grid, inc, ninc, sum_f, n_f, alpha)
    return grid


def test_adapt_fixed_points():
    # test_vegas.py:142-207 (2-pt Gauss-Legendre abscissas, analytic fixed points)
    g = 1. / 3. ** 0.5
    yg = [(1 - g) / 4., (1 + g) / 4, (3 - g) / 4, (3 + g) / 4.]
    ys = np.array([[yi] for yi in yg])
    grid = _adapt_loop(lambda x: x[:, 0] ** 2, [[0, 2]], [2], 2., 60, ys)
    np.testing.assert_allclose(grid, [[0, 2. / 2. ** (1. / 3.), 2.]])
    ys2 = np.array([[yi, yj] for yi in yg for yj in yg])
    F = lambda x: x[:, 0] * x[:, 1] ** 2  # noqa: E731
    want = [[0, 2. * 2. ** (-0.5), 2.], [0, 4. * 2 ** (-1. / 3.), 4.]]
    np.testing.assert_allclose(_adapt_loop(F, [[0, 2], [0, 4]], [2, 2], 2., 60, ys2), want)
    np.testing.assert_allclose(_adapt_loop(F, [[0, 2], [0, 4]], [2, 2], -2., 20, ys2), want)


def test_adapt_no_change():
    # test_vegas.py:145-160: already adapted / alpha = 0
    grid, inc = O.make_uniform([0, -1], [2, 1], [2, 2])
    y = np.array([[0.25, 0.25], [0.75, 0.75]])
    x, jac = O.map_points(grid, inc, [2, 2], y)
    sf, nf = O.add_training_data([2, 2], 2, y, jac)
    g, _, _ = O.adapt(grid, inc, [2, 2], sf, nf, 1.5)
    np.testing.assert_allclose(g, [[0., 1., 2.], [-1, 0, 1]])
    grid = np.array([[0, 1.5, 2], [-1, 0, 1]])
    inc = np.diff(grid, axis=1)
    g, _, _ = O.adapt(grid, inc, [2, 2], sf, nf, 0.0)
    np.testing.assert_allclose(g, grid)


@pytest.mark.parametrize('kw,nstrat,ninc,neval,mnh', [
    (dict(dim=2, neval=234), [5, 5], [20, 20], 234, None),
    (dict(dim=2, nstrat=[1, 1], neval=1000), [1, 1], [100, 100], 1000, 1000),
    (dict(dim=2, nstrat=[10, 11], neval=880), [10, 11], [80, 88], 880, 2),
    (dict(dim=2, nstrat=[7, 9], neval=2000), [7, 9], [196, 198], 2000, 7),
    (dict(dim=2, neval=3100), [20, 19], None, 3100, 2),
    (dict(dim=2, neval=3500), [21, 20], None, 3500, 2),
    (dict(dim=2, neval=1300), [13, 12], [130, 120], 1300, 2),
    (dict(dim=4, neval=1e4), [6, 6, 6, 5], [996, 996, 996, 1000], 10000, None),
    (dict(dim=4, neval=1e6), [19, 19, 19, 18], [988, 988, 988, 990], 1000000, None),
])
def test_sizing_known_answer(kw, nstrat, ninc, neval, mnh):
    # test_vegas.py:561-595, 733-772, 973-982 and the configs' sizes
    s = O.sizing(**kw)
    assert list(s['nstrat']) == nstrat
    if ninc is not None:
        assert list(s['ninc']) == ninc
    assert s['neval'] == neval
    if mnh is not None:
        assert s['min_neval_hcube'] == mnh


def test_sizing_errors():
    with pytest.raises(ValueError):
        O.sizing(2, nstrat=[7, 9], neval=20)
    with pytest.raises(MemoryError):
        O.sizing(3, neval=1000, max_mem=10)


def test_ravg_known_answer():
    # test_vegas.py:216-236
    mean, sdev, chi2, dof, Q = O.weighted_average([1., 2., 3.], [1., 4., 9.])
    np.testing.assert_allclose(mean, 1.346938775510204)
    np.testing.assert_allclose(sdev, 0.8571428571428571)
    np.testing.assert_allclose(chi2, 0.5306122448979592)
    assert dof == 2
    np.testing.assert_allclose(Q, 0.7669711269557102)


# --------------------------------------------------------------------------
# replays of reference traces (bit-exact)
# --------------------------------------------------------------------------
def replay(tr, beta=0.75, alpha=0.5, adapt=True):
    nstrat = tr['nstrat']
    ninc = tr['ninc']
    H = int(np.prod(nstrat))
    neval = int(tr['neval'])
    nf = float(tr['neval_frac'])
    mnh = int(tr['min_neval_hcube'])
    mxh = int(tr['max_neval_hcube'])
    grid = tr['grid_init']
    sigf = tr['sigf_init'] if len(tr['sigf_init']) else np.ones(H)
    sum_sigf = float(tr['sum_sigf_init'])
    for k in range(int(tr['nitn'])):
        inc = np.diff(np.nan_to_num(grid), axis=1)
        adaptive_alloc = beta > 0 and H > 1
        neval_sigf = nf * neval / sum_sigf if (beta > 0 and sum_sigf > 0) else 0.0
        nh, rng, tot = O.alloc(sigf, neval_sigf, adaptive_alloc, mnh, mxh, int(neval / H))
        assert tot == int(tr['last_neval%d' % k])
        assert list(rng) == list(tr['range%d' % k])
        u = tr['u%d' % k].astype(np.float64) * 2.0 ** -24
        y, x, w, hc = O.points(nstrat, np.nan_to_num(grid), inc, ninc, nh, u=u)
        f = tr['f%d' % k]
        adaptive = adaptive_alloc and adapt
        mean, var, sigf_new, ss, fdv2 = O.reduce(nh, w, f, beta=beta, adaptive=adaptive, sigf=sigf)
        assert mean[0] == tr['mean%d' % k]
        assert var[0, 0] ** 0.5 == tr['sdev%d' % k]
        if adaptive:
            assert np.array_equal(sigf_new, tr['sigf%d' % k])
            if ss > 0:
                assert ss == tr['sum_sigf%d' % k]
                sum_sigf = ss
            sigf = sigf_new
        if adapt and alpha > 0:
            sum_f, n_f = O.add_training_data(ninc, inc.shape[1], y, fdv2)
            grid_new, _, _ = O.adapt(np.nan_to_num(grid), inc, ninc, sum_f, n_f, alpha)
            want = tr['grid%d' % k]
            ok = ~np.isnan(want)
            assert np.array_equal(grid_new[ok], want[ok])
            grid = want
        else:
            assert np.array_equal(np.nan_to_num(grid), np.nan_to_num(tr['grid%d' % k]))


def test_replay_gauss4():
    replay(load('ref_gauss4_injected.npz'))


def test_replay_ridge():
    replay(load('ref_ridge_injected.npz'))


def test_replay_constant_epsilon_guard():
    tr = load('ref_const_injected.npz')
    replay(tr, alpha=0.0)
    # the EPSILON guard makes each iteration's sdev identical (test_vegas.py:1272-1296)
    assert tr['sdev0'] == tr['sdev1'] == tr['sdev2'] and tr['sdev0'] > 0


def test_replay_beta0():
    replay(load('ref_beta0_injected.npz'), beta=0.0)


def test_map_edges_golden():
    c = load('ref_map_adapt.npz')
    g = np.nan_to_num(c['map_grid'])
    x, jac = O.map_points(g, np.diff(g, axis=1), c['map_ninc'], c['map_y'])
    assert np.array_equal(x, c['map_x'])
    assert np.array_equal(jac, c['map_jac'])


def test_adapt_golden():
    c = load('ref_map_adapt.npz')
    for k in range(int(c['n_adapt'])):
        p = 'adapt%d_' % k
        ninc = c[p + 'ninc_in']
        g = np.nan_to_num(c[p + 'grid_in'])
        inc = np.diff(g, axis=1)
        for d in range(len(ninc)):  # inc beyond ninc[d] is never read
            inc[d, ninc[d]:] = 0.0
        if bool(c[p + 'train']):
            sf, nf = O.add_training_data(ninc, inc.shape[1], c[p + 'y'], c[p + 'f'])
            assert np.array_equal(sf, c[p + 'sum_f'])
            assert np.array_equal(nf, c[p + 'n_f'])
        else:
            sf = nf = None
        gn, _, _ = O.adapt(g, inc, ninc, sf, nf, float(c[p + 'alpha']), c[p + 'new_ninc'])
        want = c[p + 'grid_out']
        ok = ~np.isnan(want)
        assert np.array_equal(gn[ok], want[ok]), k


def test_alloc_golden():
    c = load('ref_map_adapt.npz')
    for k in range(int(c['n_alloc'])):
        neval, nf, mnh, mxh, H = c['alloc%d_params' % k]
        ss = float(c['alloc%d_sum_sigf' % k])
        nh, rng, tot = O.alloc(c['alloc%d_sigf' % k], nf * neval / ss, True, int(mnh), int(mxh),
                               int(neval / H))
        assert np.array_equal(nh, c['alloc%d_neval_h' % k])
        assert list(rng) == list(c['alloc%d_range' % k])


# --------------------------------------------------------------------------
# live comparison with the compiled reference (development container only)
# --------------------------------------------------------------------------
def _ref():
    try:
        import build_ref
        if not build_ref.built():
            return None
        return build_ref.import_reference()
    except Exception:
        return None


def test_live_reference_sizing_sweep():
    v = _ref()
    if v is None:
        pytest.skip('compiled reference not available here')
    for dim in (1, 2, 3, 4, 5, 8, 9, 16):
        for neval in (50, 234, 1000, 3100, 1e4, 2 ** 20, 1e6, 1e7):
            try:
                I = v.Integrator(dim * [[0, 1]], neval=neval)
            except MemoryError:
                continue
            s = O.sizing(dim, neval=neval)
            assert list(I.nstrat) == list(s['nstrat'])
            assert list(I.map.ninc) == list(s['ninc'])
            assert I.min_neval_hcube == s['min_neval_hcube']


def replay_ate(tr, alpha=0.5):
    """adapt_to_errors=True trace: increments = strata, uniform allocation,
    the map trained on each hypercube's |variance| at the hypercube's last
    sample (pyx:1372, 1662, 2181-2193)."""
    nstrat, ninc = tr['nstrat'], tr['ninc']
    assert np.array_equal(nstrat, ninc)
    H = int(np.prod(nstrat))
    neval = int(tr['neval'])
    mnh, mxh = int(tr['min_neval_hcube']), int(tr['max_neval_hcube'])
    grid = tr['grid_init']
    for k in range(int(tr['nitn'])):
        inc = np.diff(np.nan_to_num(grid), axis=1)
        nh, rng, tot = O.alloc(np.ones(H), 0.0, False, mnh, mxh, int(neval / H))
        assert tot == int(tr['last_neval%d' % k])
        assert list(rng) == list(tr['range%d' % k])
        u = tr['u%d' % k].astype(np.float64) * 2.0 ** -24
        y, x, w, hc = O.points(nstrat, np.nan_to_num(grid), inc, ninc, nh, u=u)
        mean, var, _, _, _, hv = O.reduce(nh, w, tr['f%d' % k], adaptive=False, hc_var=True)
        assert mean[0] == tr['mean%d' % k]
        assert var[0, 0] ** 0.5 == tr['sdev%d' % k]
        last = np.cumsum(nh) - 1
        sum_f, n_f = O.add_training_data(ninc, inc.shape[1], y[last], hv)
        grid_new, _, _ = O.adapt(np.nan_to_num(grid), inc, ninc, sum_f, n_f, alpha)
        want = tr['grid%d' % k]
        ok = ~np.isnan(want)
        assert np.array_equal(grid_new[ok], want[ok])
        grid = want


def test_replay_adapt_to_errors():
    tr = load('ref_ate_injected.npz')
    sz = O.sizing(2, neval=2000, adapt_to_errors=True)
    assert list(sz['nstrat']) == list(tr['nstrat']) and list(sz['ninc']) == list(tr['ninc'])
    replay_ate(tr)


def test_invmap_golden():
    c = load('ref_invmap.npz')
    g = np.nan_to_num(c['inv_grid'])
    y, jac = O.invmap(g, np.diff(g, axis=1), c['inv_ninc'], c['inv_x'])
    assert np.array_equal(y, c['inv_y'])
    assert np.array_equal(jac, c['inv_jac'])


def test_adapt_to_samples_golden():
    c = load('ref_invmap.npz')
    g = np.nan_to_num(c['ats_grid_in'])
    grid, inc, ninc = O.adapt_to_samples(g, np.diff(g, axis=1), c['ats_ninc_in'], c['ats_x'],
                                         c['ats_f'], nitn=4, alpha=0.8)
    assert list(ninc) == list(c['ats_ninc_out'])
    want = c['ats_grid_out']
    ok = ~np.isnan(want)
    assert np.array_equal(grid[ok], want[ok])
