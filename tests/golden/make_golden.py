"""Generate golden vectors from the compiled reference vegas (vegas 6.4.1).

Run in the development container, where the reference sources exist:

    python oracle/build_ref.py          # compiles src/vegas/_vegas.pyx out of tree
    python tests/golden/make_golden.py  # writes tests/golden/*.npz

The fixtures let the oracle (and, through it, the CUDA path) be pinned on a
machine without the reference.  Every integrator trace is recorded in
"injected-sample" mode: ``ran_array_generator`` hands the reference uniforms
u = k / 2**24 (k drawn from a seeded numpy generator, stored as uint32), and
the integrand wrapper records the exact f values the reference consumed.

Per iteration a trace stores the state the reference ended with (grid, sigf,
sum_sigf) plus the iteration's mean, var, last_neval and neval_hcube_range;
the state before iteration k is the state after iteration k-1 (the initial
state is the freshly constructed integrator's).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
import build_ref  # noqa: E402

U_SCALE = 2.0 ** -24


class Recorder(object):
    """ran_array_generator that records its draws as uint32 k (u = k/2^24)."""

    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)
        self.draws = []

    def __call__(self, size):
        k = self.rng.integers(0, 2 ** 24, size=size, dtype=np.uint32)
        self.draws.append(k)
        return k.astype(np.float64) * U_SCALE

    def take(self):
        out = np.concatenate(self.draws, axis=0) if self.draws else np.zeros((0, 0), np.uint32)
        self.draws = []
        return out


def valid_grid(m):
    ninc = np.asarray(m.ninc)
    K = int(ninc.max())
    g = np.full((len(ninc), K + 1), np.nan)
    for d in range(len(ninc)):
        g[d, :ninc[d] + 1] = np.asarray(m.grid)[d, :ninc[d] + 1]
    return g


def trace(v, limits, fcn_np, nitn, neval, seed, **kargs):
    """Run the reference integrator nitn times (nitn=1 each) recording everything."""
    rec = Recorder(seed)
    integ = v.Integrator(limits, neval=neval, ran_array_generator=rec, **kargs)
    fvals = []

    @v.lbatchintegrand
    def f(x):
        fx = fcn_np(np.asarray(x))
        if np.asarray(x).shape[0] > 1:     # skip the one-point probe call (pyx:3080)
            fvals.append(np.array(fx, dtype=np.float64))
        return fx

    out = dict(
        nstrat=np.asarray(integ.nstrat, np.int64),
        ninc=np.asarray(integ.map.ninc, np.int64),
        grid_init=valid_grid(integ.map),
        sigf_init=np.array(integ.sigf, float),
        sum_sigf_init=np.array(integ.sum_sigf),
        min_neval_hcube=np.array(integ.min_neval_hcube),
        max_neval_hcube=np.array(integ.max_neval_hcube),
        neval=np.array(integ.neval),
        neval_frac=np.array(integ.neval_frac),
        nitn=np.array(nitn),
    )
    for k in range(nitn):
        fvals.clear()
        r = integ(f, nitn=1)
        u = rec.take()
        fx = np.concatenate(fvals)
        assert fx.shape[0] == u.shape[0], (fx.shape, u.shape)
        res = r.itn_results[-1]
        out['u%d' % k] = u.astype(np.uint32)
        out['f%d' % k] = fx
        out['mean%d' % k] = np.array(res.mean)
        # sdev exactly as the reference formed it: var ** 0.5 (pyx:3144)
        out['sdev%d' % k] = np.array(list(res.internaldata[1].values())[0])
        out['sigf%d' % k] = np.array(integ.sigf, float)
        out['sum_sigf%d' % k] = np.array(integ.sum_sigf)
        out['grid%d' % k] = valid_grid(integ.map)
        out['last_neval%d' % k] = np.array(integ.last_neval)
        out['range%d' % k] = np.array(integ.neval_hcube_range, np.int64)
    return out


def gauss4(x):
    return (100 / np.pi) ** 2 * np.exp(-100 * np.sum((x - 0.5) ** 2, axis=1))


def ridge(x, M=1000, s=0.01):
    dim = x.shape[1]
    c = (np.arange(M) + 0.5) / M
    acc = np.zeros(x.shape[0])
    for j in range(M):
        r2 = np.zeros(x.shape[0])
        for d in range(dim):
            r2 += (x[:, d] - c[j]) * (x[:, d] - c[j])
        acc += np.exp(-r2 / (2 * s * s))
    return (2 * np.pi * s * s) ** (-0.5 * dim) * acc / M


def const7(x):
    return 7 * np.ones(x.shape[0], float)


def peak2(x):
    return np.exp(-50 * (x[:, 0] - 0.3) ** 2) * (1 + x[:, 1] ** 2)


def ate_trace(v):
    """adapt_to_errors=True: map increments = strata, uniform allocation, the
    map trained on each hypercube's variance at its last sample."""
    return trace(v, 2 * [[0, 1]], peak2, nitn=3, neval=2000, seed=5, alpha=0.5,
                 adapt_to_errors=True)


def adapt_cases(v):
    """Direct AdaptiveMap cases: map edges, training skips, adapt variants."""
    rng = np.random.default_rng(7)
    cases = {}
    # map incl. y == 0 and y == 1 (iy == ninc branch, pyx:354-359)
    m = v.AdaptiveMap([[0, 0.3, 1.0], [-2, -1.5, 0, 6]], ninc=[5, 7])
    y = np.concatenate([rng.random((64, 2)), [[0., 0.], [1., 1.], [0.2, 1.0], [1.0, 0.5]]])
    x = np.empty_like(y)
    jac = np.empty(len(y))
    m.map(y, x, jac)
    cases['map_grid'] = valid_grid(m)
    cases['map_ninc'] = np.asarray(m.ninc, np.int64)
    cases['map_y'] = y
    cases['map_x'] = x
    cases['map_jac'] = jac
    # training with y in {0, 1} skipped (pyx:460) then adapt variants
    idx = 0
    for ninc, alpha, new_ninc, train in [
            ([6, 6], 0.5, None, True), ([10, 7], 1.5, None, True), ([8, 8], -2.0, None, True),
            ([9, 12], 0.0, [5, 20], True), ([20, 20], 0.7, [4, 9], True),
            ([5, 9], 0.5, None, False), ([1, 4], 0.5, None, True), ([2, 3], 2.0, [3, 3], True)]:
        m = v.AdaptiveMap([[0, 1], [-1, 2]], ninc=ninc)
        g0 = valid_grid(m)
        y = rng.random((200, 2))
        y[:5, 0] = 0.0
        y[5:10, 1] = 1.0
        f = np.exp(-10 * (y[:, 0] - 0.3) ** 2) * (1 + y[:, 1] ** 3)
        f[::17] = 0.0
        if train:
            m.add_training_data(y, f)
            sum_f = np.array(m.sum_f)
            n_f = np.array(m.n_f)
        else:
            sum_f = n_f = np.zeros((2, max(ninc)))
        m.adapt(alpha=alpha, ninc=new_ninc)
        p = 'adapt%d_' % idx
        cases[p + 'grid_in'] = g0
        cases[p + 'ninc_in'] = np.array(ninc, np.int64)
        cases[p + 'y'] = y
        cases[p + 'f'] = f
        cases[p + 'train'] = np.array(train)
        cases[p + 'sum_f'] = sum_f
        cases[p + 'n_f'] = n_f
        cases[p + 'alpha'] = np.array(alpha)
        cases[p + 'new_ninc'] = np.array(new_ninc if new_ninc is not None else ninc, np.int64)
        cases[p + 'grid_out'] = valid_grid(m)
        idx += 1
    cases['n_adapt'] = np.array(idx)
    return cases


def invmap_cases(v):
    """AdaptiveMap.invmap on an adapted map (points inside, on nodes, outside
    the grid) and adapt_to_samples.  Equal ninc on every axis: with unequal
    ninc the reference's rows are zero-padded and numpy.searchsorted sees an
    unsorted row."""
    rng = np.random.default_rng(13)
    out = {}
    m = v.AdaptiveMap([[0, 1], [-2, 3]], ninc=[9, 9])
    y0 = rng.random((400, 2))
    m.add_training_data(y0, np.exp(-20 * (y0[:, 0] - 0.4) ** 2) + y0[:, 1] ** 2)
    m.adapt(alpha=1.0)
    g = np.asarray(m.grid)
    x = np.concatenate([rng.uniform([-0.1, -2.5], [1.1, 3.5], (200, 2)),
                        np.stack([g[0, :9], g[1, 1:10]], axis=1),
                        [[0.0, -2.0], [1.0, 3.0], [-1e-9, 3.0 + 1e-9]]])
    y = np.empty_like(x)
    jac = np.empty(len(x))
    m.invmap(x, y, jac)
    out['inv_grid'] = valid_grid(m)
    out['inv_ninc'] = np.asarray(m.ninc, np.int64)
    out['inv_x'] = x
    out['inv_y'] = y
    out['inv_jac'] = jac
    # adapt_to_samples: a 3-d map adapted to samples of a peaked function
    m2 = v.AdaptiveMap([[0, 1], [0, 2], [-1, 1]], ninc=[50, 50, 50])
    xs = np.column_stack([rng.random(3000), 2 * rng.random(3000), 2 * rng.random(3000) - 1])
    fs = np.exp(-30 * (xs[:, 0] - 0.3) ** 2 - 10 * (xs[:, 1] - 1.2) ** 2) * (1 + xs[:, 2] ** 2)
    out['ats_grid_in'] = valid_grid(m2)
    out['ats_ninc_in'] = np.asarray(m2.ninc, np.int64)
    m2.adapt_to_samples(xs, fs, nitn=4, alpha=0.8)
    out['ats_x'] = xs
    out['ats_f'] = fs
    out['ats_grid_out'] = valid_grid(m2)
    out['ats_ninc_out'] = np.asarray(m2.ninc, np.int64)
    return out


def alloc_cases(v):
    """Allocation from a given sigf, incl. the max_neval_hcube clamp."""
    rng = np.random.default_rng(11)
    out = {}
    for k, (dim, neval, mx) in enumerate([(3, 2000, 50000), (2, 5000, 40), (4, 30000, 200)]):
        integ = v.Integrator(dim * [[0, 1]], neval=neval, max_neval_hcube=mx,
                             ran_array_generator=np.random.default_rng(k).random)
        H = integ.nhcube
        sigf = rng.random(H) ** 4
        sigf[rng.random(H) < 0.1] = 0.0
        sigf[0] = 50.0
        integ.set(sigf=sigf)
        hc = np.concatenate([np.asarray(b[-1]) for b in integ.random_batch(yield_hcube=True)])
        out['alloc%d_sigf' % k] = np.asarray(integ.sigf, float)
        out['alloc%d_sum_sigf' % k] = np.array(integ.sum_sigf)
        out['alloc%d_neval_h' % k] = np.bincount(hc, minlength=H).astype(np.int64)
        out['alloc%d_range' % k] = np.asarray(integ.neval_hcube_range, np.int64)
        out['alloc%d_params' % k] = np.array([integ.neval, integ.neval_frac, integ.min_neval_hcube,
                                              integ.max_neval_hcube, H], float)
    out['n_alloc'] = np.array(3)
    return out


def restrat_f(x):
    """Integrand whose structure sits in directions 0 and 1 (weak in 2)."""
    return np.exp(-40.0 * (x[:, 0] - 0.3) ** 2 - 25.0 * (x[:, 1] - 0.6) ** 2) * (1.0 + 0.2 * x[:, 2])


RESTRAT_CASES = [
    dict(seed=11, train=dict(nitn=4), args=dict(nitn=2, ndy=5)),
    dict(seed=12, train=dict(nitn=3), args=dict(nitn=1, ndy=4, below_avg_nstrat=1, gamma=0.5)),
]


def restratify_cases(V):
    """vegas.restratify (src/vegas/__init__.py:1313-1592) on a trained dim-6
    integrator, in injected-sample mode.  The reference's internal I/dI
    integrand returns a gvar BufferDict; the stand-in flattens it to an
    array-valued integrand (same numbers, key order I then dI[mu, i]), and
    the wrapper below hands restratify the dictionary view it indexes."""

    class Restrat(V.restratifyIntegrator):
        def __call__(self, fcn, **kargs):
            r = V.Integrator.__call__(self, fcn, **kargs)
            phase = self.__dict__.get('_phase', 0)
            self._phase = phase + 1
            if phase == 0:
                flat = np.asarray(r, dtype=object)
                d = _ResultDict(I=flat[0], dI=flat[1:].reshape(self.dim, self.ndy))
                d.Q = r.Q
                d.summary = r.summary
                return d
            self._training = r
            return r

    out = {}
    for c, case in enumerate(RESTRAT_CASES):
        rec = Recorder(case['seed'])
        integ = V.Integrator(6 * [[0, 1]], neval=4000, alpha=0.5, ran_array_generator=rec)
        f = V.lbatchintegrand(restrat_f)
        r0 = integ(f, **case['train'])
        R = Restrat(integ, f, **case['args'])
        pre = 'c%d_' % c
        out[pre + 'nstrat_before'] = np.asarray(R.old_nstrat, np.int64)
        out[pre + 'train_mean'] = np.array(r0.mean)
        out[pre + 'I'] = np.array([R.I.mean, R.I.sdev])
        out[pre + 'dI_mean'] = np.array([[g.mean for g in row] for row in R.dI])
        out[pre + 'dI_sdev'] = np.array([[g.sdev for g in row] for row in R.dI])
        out[pre + 'weight_mean'] = np.array([g.mean for g in R.weight])
        out[pre + 'weight_sdev'] = np.array([g.sdev for g in R.weight])
        out[pre + 'Q'] = np.array(R.Q)
        out[pre + 'nstrat_after'] = np.asarray(R.nstrat, np.int64)
        out[pre + 'neval_after'] = np.array(R.neval)
        tr = R._training
        out[pre + 'itn_mean'] = np.array([g.mean for g in tr.itn_results])
        out[pre + 'itn_sdev'] = np.array([g.sdev for g in tr.itn_results])
        out[pre + 'grid_after'] = valid_grid(R.map)
        out[pre + 'sum_sigf_after'] = np.array(R.sum_sigf)
    out['ncases'] = np.array(len(RESTRAT_CASES))
    return out


def arr_f(x):
    """Three-component integrand (correlated components)."""
    x = np.asarray(x)
    g = np.exp(-20.0 * np.sum((x - 0.45) ** 2, axis=1))
    return np.stack([g, x[:, 0] * g, x[:, 1] * x[:, 2] * g], axis=1)


def array_cases(v):
    """Array-valued integrand, correlated and not (RAvgArray, pyx:2579-2879;
    per-hypercube covariance sums, pyx:2149-2172), injected-sample mode."""
    from gvar import evalcov
    out = {}
    for c, corr in enumerate((True, False)):
        rec = Recorder(40 + c)
        integ = v.Integrator(3 * [[0, 1]], neval=3000, ran_array_generator=rec, correlate_integrals=corr)
        r = integ(v.lbatchintegrand(arr_f), nitn=3)
        pre = 'c%d_' % c
        out[pre + 'itn_mean'] = np.array([[g.mean for g in res] for res in r.itn_results])
        out[pre + 'itn_cov'] = np.array([evalcov(list(res)) for res in r.itn_results])
        out[pre + 'mean'] = np.array([g.mean for g in r])
        out[pre + 'cov'] = evalcov(list(r))
        out[pre + 'chi2'] = np.array(r.chi2)
        out[pre + 'Q'] = np.array(r.Q)
    return out


def jac_f(x, jac):
    """Integrand that uses dx/dy per direction (uses_jac, pyx:265-295, 2127)."""
    x = np.asarray(x)
    jac = np.asarray(jac)
    return np.exp(-x[:, 0]) * jac[:, 0] / (1.0 + jac[:, 1])


def uses_jac_cases(v):
    """uses_jac=True on a map adapted to peak2 (injected uniforms): the
    integrand receives jac[n, dim] = dx/dy per direction."""
    rec = Recorder(60)
    integ = v.Integrator(2 * [[0, 1]], neval=2000, ran_array_generator=rec)
    integ(v.lbatchintegrand(peak2), nitn=3)
    r = integ(v.lbatchintegrand(jac_f), nitn=2, uses_jac=True)
    return dict(itn_mean=np.array([g.mean for g in r.itn_results]),
                itn_sdev=np.array([g.sdev for g in r.itn_results]),
                mean=np.array(r.mean), sdev=np.array(r.sdev))


class _ResultDict(dict):
    pass


def main(only=None):
    build_ref.build()
    v = build_ref.import_reference()
    if only == ['restratify']:
        V = build_ref.import_reference_package()
        np.savez_compressed(os.path.join(HERE, 'ref_restratify.npz'), **restratify_cases(V))
        return
    if only == ['array']:
        np.savez_compressed(os.path.join(HERE, 'ref_array.npz'), **array_cases(v))
        return
    if only == ['uses_jac']:
        np.savez_compressed(os.path.join(HERE, 'ref_uses_jac.npz'), **uses_jac_cases(v))
        return
    np.savez_compressed(os.path.join(HERE, 'ref_gauss4_injected.npz'),
                        **trace(v, 4 * [[0, 1]], gauss4, nitn=3, neval=10000, seed=1,
                                alpha=0.5, beta=0.75))
    np.savez_compressed(os.path.join(HERE, 'ref_ridge_injected.npz'),
                        **trace(v, 4 * [[0, 1]], ridge, nitn=3, neval=8000, seed=2,
                                alpha=0.5, beta=0.75))
    np.savez_compressed(os.path.join(HERE, 'ref_const_injected.npz'),
                        **trace(v, [[0, 1]], const7, nitn=3, neval=100, seed=3, alpha=0.0))
    np.savez_compressed(os.path.join(HERE, 'ref_beta0_injected.npz'),
                        **trace(v, [[0, np.pi], [-np.pi / 2, np.pi / 2]],
                                lambda x: (np.sin(x[:, 0]) ** 2 + np.cos(x[:, 1]) ** 2) / np.pi ** 2,
                                nitn=2, neval=3000, seed=4, beta=0.0))
    np.savez_compressed(os.path.join(HERE, 'ref_map_adapt.npz'), **adapt_cases(v), **alloc_cases(v))
    np.savez_compressed(os.path.join(HERE, 'ref_ate_injected.npz'), **ate_trace(v))
    np.savez_compressed(os.path.join(HERE, 'ref_invmap.npz'), **invmap_cases(v))
    for f in sorted(os.listdir(HERE)):
        if f.endswith('.npz'):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == '__main__':
    # no argument: every fixture; "restratify", "array" or "uses_jac": that fixture only
    main(sys.argv[1:] or None)
