"""Python face of the vegas+ oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the checker for the CUDA path: a CPU restatement of the
reference algorithm (src/vegas/_vegas.pyx, vegas 6.4.1).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU baseline and its
``--impl reference`` arm) may import this module.  The product package
``vegas_gb300`` never does.

* ``sizing`` restates the host-side integer logic of ``Integrator.set``
  (_vegas.pyx:1256-1446) in Python.
* Everything numeric is in ``vegas_oracle.c`` (same directory), compiled by
  ``build()`` into ``oracle/_build/libvegas_oracle.so`` and bound here with
  ctypes.

Parity status: pinned.  ``tests/test_oracle.py`` checks this restatement
against the reference's own known-answer tests (tests/test_vegas.py) and
against golden vectors produced by the compiled reference
(``tests/golden/make_golden.py``).
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'libvegas_oracle.so')
SRC = os.path.join(HERE, 'vegas_oracle.c')

TINY = 1e-257
EPSILON = np.finfo(float).eps * 1e4

F_GAUSS, F_RIDGE, F_LORENTZ, F_MIXTURE, F_LATTICE, F_CONST = range(6)


def build(force=False):
    """Compile the C restatement with gcc (portable flags, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + '.%d.tmp' % os.getpid()
    subprocess.run(['gcc', '-O2', '-ffp-contract=off', '-fPIC', '-shared', '-Wall',
                    '-o', tmp, SRC, '-lm', '-lpthread'], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        i64, i32, u32, u64, dbl = (ctypes.c_int64, ctypes.c_int, ctypes.c_uint32,
                                   ctypes.c_uint64, ctypes.c_double)
        L.vo_philox4x32_10.argtypes = [P, P, P]
        L.vo_uniform_f64.argtypes = [u64, u32, u32, u64, i32]
        L.vo_uniform_f64.restype = dbl
        L.vo_uniform_f32.argtypes = [u64, u32, u32, u64, i32]
        L.vo_uniform_f32.restype = ctypes.c_float
        L.vo_strata_pow.argtypes = [dbl, i32]
        L.vo_strata_pow.restype = dbl
        L.vo_make_uniform.argtypes = [i32, P, P, P, P, i64, P, i64]
        L.vo_map.argtypes = [i32, P, P, i64, P, i64, i64, P, P, P]
        L.vo_add_training_data.argtypes = [i32, P, i64, i64, P, P, P, P]
        L.vo_invmap.argtypes = [i32, P, P, i64, P, i64, i64, P, P, P]
        L.vo_adapt.argtypes = [i32, P, P, i64, P, i64, P, P, dbl, P, P, i64, P, i64]
        L.vo_alloc.argtypes = [i64, P, dbl, i32, i64, i64, i64, P, P]
        L.vo_alloc.restype = i64
        L.vo_points.argtypes = [i32, P, P, P, i64, P, i64, i64, P, P, u64, u32, u32, P, P, P, P]
        L.vo_reduce.argtypes = [i64, P, i32, P, P, i32, dbl, P, P, P, P, P, P]
        L.vo_eval.argtypes = [i32, P, i32, i64, P, P]
        L.vo_iterate.argtypes = [i32, i32, P, P, P, P, i64, P, i64, i64, P, P, i64, dbl, i64,
                                 i64, dbl, dbl, i32, i32, u64, u32, u32, i32, P]
        L.vo_iterate.restype = i32
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ---------------------------------------------------------------------------
# host sizing -- Integrator.set, _vegas.pyx:1256-1446
# ---------------------------------------------------------------------------
def sizing(dim, neval=1000, neval_frac=0.75, beta=0.75, maxinc_axis=1000, max_mem=1e9,
           min_neval_batch=100000, max_neval_hcube=50000, nstrat=None,
           uniform_nstrat=False, adapt_to_errors=False, minimize_mem=False):
    """Return dict(nstrat, ninc, neval, nhcube, min_neval_hcube) as Integrator.set.

    Follows _vegas.pyx:1335-1407 for a freshly constructed integrator given
    either ``neval`` or ``nstrat`` (as the constructor does, pyx:1172-1176).
    """
    nf = 0 if (beta == 0 or adapt_to_errors) else neval_frac
    neval = int(neval)
    if nstrat is not None:                                    # pyx:1335-1342
        nstrat = np.array(nstrat, dtype=np.intp)
        nhcube = int(np.prod(nstrat))
        if neval is None:
            neval = int(2. * nhcube / (1. - nf))
        elif neval < 2. * nhcube / (1. - nf):
            raise ValueError('neval too small')
    else:                                                     # pyx:1343-1366
        # a complex power in the reference (see vo_strata_pow)
        ns = int(lib().vo_strata_pow((1 - nf) * neval / 2., dim))
        if ns < 1:
            ns = 1
        d = int((math.log((1 - nf) * neval / 2.) - dim * math.log(ns)) / math.log(1 + 1. / ns))
        if ((ns + 1) ** d * ns ** (dim - d)) > max_mem and not minimize_mem:
            raise MemoryError('work arrays larger than max_mem')
        if uniform_nstrat:
            d = 0
        nstrat = np.empty(dim, np.intp)
        nstrat[:d] = ns + 1
        nstrat[d:] = ns
    if adapt_to_errors:                                       # pyx:1369-1386
        ninc = np.array(nstrat, dtype=np.intp)
    else:
        ni = min(int(neval / 10.), maxinc_axis)
        ninc = np.empty(dim, np.intp)
        for d in range(dim):
            if ni >= nstrat[d]:
                ninc[d] = int(ni / nstrat[d]) * nstrat[d]
            elif nstrat[d] <= maxinc_axis:
                ninc[d] = nstrat[d]
            else:
                nstrat[d] = int(nstrat[d] / ni) * ni
                ninc[d] = ni
    nhcube = int(np.prod(nstrat))                              # pyx:1397-1407
    if nhcube == 1:
        min_neval_hcube = int(neval)
    else:
        min_neval_hcube = int((1 - nf) * neval / nhcube)
    if min_neval_hcube < 2:
        min_neval_hcube = 2
    workspace = min_neval_batch + max_neval_hcube             # pyx:1437-1441
    if workspace > neval:
        workspace = neval + 1
    if (3 * dim + 3) * workspace + (0 if minimize_mem else nhcube) > max_mem:
        raise MemoryError('work arrays larger than max_mem')
    return dict(nstrat=np.asarray(nstrat), ninc=ninc, neval=neval, nhcube=nhcube,
                min_neval_hcube=min_neval_hcube)


# ---------------------------------------------------------------------------
# numeric kernels (C)
# ---------------------------------------------------------------------------
def philox(ctr, key):
    c = _c(ctr, np.uint32)
    k = _c(key, np.uint32)
    o = np.empty(4, np.uint32)
    lib().vo_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def uniform_f64(seed, stream, itn, i, d):
    return lib().vo_uniform_f64(seed, stream, itn, i, d)


def uniform_f32(seed, stream, itn, i, d):
    return lib().vo_uniform_f32(seed, stream, itn, i, d)


def make_uniform(xl, xu, ninc):
    xl = _c(xl, float)
    xu = _c(xu, float)
    ninc = _c(ninc, np.int64)
    dim = len(ninc)
    K = int(ninc.max())
    grid = np.zeros((dim, K + 1))
    inc = np.zeros((dim, K))
    lib().vo_make_uniform(dim, _p(xl), _p(xu), _p(ninc), _p(grid), K + 1, _p(inc), K)
    return grid, inc


def map_points(grid, inc, ninc, y):
    ninc = _c(ninc, np.int64)
    grid = _c(grid, float)
    inc = _c(inc, float)
    y = _c(y, float)
    n, dim = y.shape
    x = np.empty_like(y)
    jac = np.empty(n)
    lib().vo_map(dim, _p(ninc), _p(grid), grid.shape[1], _p(inc), inc.shape[1], n, _p(y), _p(x),
                 _p(jac))
    return x, jac


def invmap(grid, inc, ninc, x):
    """AdaptiveMap.invmap (pyx:362-413): returns y, jac."""
    ninc = _c(ninc, np.int64)
    grid = _c(grid, float)
    inc = _c(inc, float)
    x = _c(x, float)
    n, dim = x.shape
    y = np.empty_like(x)
    jac = np.empty(n)
    lib().vo_invmap(dim, _p(ninc), _p(grid), grid.shape[1], _p(inc), inc.shape[1], n, _p(x), _p(y),
                    _p(jac))
    return y, jac


def adapt_to_samples(grid, inc, ninc, x, fx, nitn=5, alpha=1.0, maxinc_axis=1000):
    """AdaptiveMap.adapt_to_samples (pyx:728-790) composed from the oracle's
    invmap, add_training_data and adapt: returns grid, inc, ninc."""
    ninc = _c(ninc, np.int64)
    fx = _c(fx, float)
    old_ninc = max(int(max(ninc)), maxinc_axis)
    tmp_ninc = int(min(old_ninc, x.shape[0] / 10.))
    if tmp_ninc < 2:
        raise ValueError('not enough samples')
    grid, inc, ninc = adapt(grid, inc, ninc, None, None, 0.0, tmp_ninc)
    for _ in range(nitn):
        y, jac = invmap(grid, inc, ninc, x)
        sum_f, n_f = add_training_data(ninc, inc.shape[1], y, (jac * fx) ** 2)
        grid, inc, ninc = adapt(grid, inc, ninc, sum_f, n_f, alpha, tmp_ninc)
    if tmp_ninc != old_ninc:
        grid, inc, ninc = adapt(grid, inc, ninc, None, None, 0.0, old_ninc)
    return grid, inc, ninc


def add_training_data(ninc, ldi, y, f, sum_f=None, n_f=None):
    ninc = _c(ninc, np.int64)
    y = _c(y, float)
    f = _c(f, float)
    n, dim = y.shape
    if sum_f is None:
        sum_f = np.zeros((dim, ldi))
        n_f = np.zeros((dim, ldi)) + TINY
    lib().vo_add_training_data(dim, _p(ninc), ldi, n, _p(y), _p(f), _p(sum_f), _p(n_f))
    return sum_f, n_f


def adapt(grid, inc, ninc, sum_f, n_f, alpha, new_ninc=None):
    ninc = _c(ninc, np.int64)
    grid = _c(grid, float)
    inc = _c(inc, float)
    dim = len(ninc)
    new_ninc = ninc.copy() if new_ninc is None else _c(
        np.full(dim, new_ninc) if np.ndim(new_ninc) == 0 else new_ninc, np.int64)
    K = int(new_ninc.max())
    ng = np.zeros((dim, K + 1))
    ni = np.zeros((dim, K))
    if sum_f is not None:
        sum_f = _c(sum_f, float)
        n_f = _c(n_f, float)
    lib().vo_adapt(dim, _p(ninc), _p(grid), grid.shape[1], _p(inc), inc.shape[1], _p(sum_f),
                   _p(n_f), float(alpha), _p(new_ninc), _p(ng), K + 1, _p(ni), K)
    return ng, ni, new_ninc


def alloc(sigf, neval_sigf, adaptive, min_neval_hcube, max_neval_hcube, avg_neval_hcube):
    sigf = _c(sigf, float)
    H = len(sigf)
    nh = np.empty(H, np.int64)
    rng = np.empty(2, np.int64)
    tot = lib().vo_alloc(H, _p(sigf), float(neval_sigf), int(adaptive), int(min_neval_hcube),
                         int(max_neval_hcube), int(avg_neval_hcube), _p(nh), _p(rng))
    return nh, rng, int(tot)


def points(nstrat, grid, inc, ninc, neval_h, u=None, seed=0, stream=0, itn=0):
    nstrat = _c(nstrat, np.int64)
    ninc = _c(ninc, np.int64)
    grid = _c(grid, float)
    inc = _c(inc, float)
    neval_h = _c(neval_h, np.int64)
    dim = len(nstrat)
    n = int(neval_h.sum())
    if u is not None:
        u = _c(u, float)
        assert u.shape == (n, dim)
    y = np.empty((n, dim))
    x = np.empty((n, dim))
    w = np.empty(n)
    hc = np.empty(n, np.int64)
    lib().vo_points(dim, _p(nstrat), _p(ninc), _p(grid), grid.shape[1], _p(inc), inc.shape[1],
                    len(neval_h), _p(neval_h), _p(u), seed, stream, itn, _p(y), _p(x), _p(w),
                    _p(hc))
    return y, x, w, hc


def reduce(neval_h, wgt, fx, beta=0.75, adaptive=True, sigf=None, hc_var=False):
    """Returns mean, var, sigf, sum_sigf, fdv2 (and, with hc_var, the
    per-hypercube |variance| that adapt_to_errors trains the map on)."""
    neval_h = _c(neval_h, np.int64)
    wgt = _c(wgt, float)
    fx = _c(fx, float)
    if fx.ndim == 1:
        fx = fx.reshape(-1, 1)
    s = fx.shape[1]
    H = len(neval_h)
    mean = np.zeros(s)
    var = np.zeros((s, s))
    sigf = np.ones(H) if sigf is None else _c(sigf, float).copy()
    ss = np.zeros(1)
    fdv2 = np.empty(len(wgt))
    hv = np.empty(H) if hc_var else None
    lib().vo_reduce(H, _p(neval_h), s, _p(wgt), _p(fx), int(adaptive), float(beta), _p(mean),
                    _p(var), _p(sigf), _p(ss), _p(fdv2), _p(hv))
    for a in range(s):
        for b in range(a):
            var[b, a] = var[a, b]
    if hc_var:
        return mean, var, sigf, float(ss[0]), fdv2, hv
    return mean, var, sigf, float(ss[0]), fdv2


def evaluate(kind, params, x):
    x = _c(x, float)
    p = _c(params, float)
    n, dim = x.shape
    f = np.empty(n)
    lib().vo_eval(kind, _p(p), dim, n, _p(x), _p(f))
    return f


class State(object):
    """Integrator state for the multi-threaded oracle driver ``iterate``."""

    def __init__(self, limits, neval, nitn_hint=None, alpha=0.5, beta=0.75, neval_frac=0.75,
                 maxinc_axis=1000, max_neval_hcube=50000, nstrat=None, adapt_to_errors=False):
        limits = np.asarray(limits, float)
        dim = len(limits)
        sz = sizing(dim, neval=neval, neval_frac=neval_frac, beta=beta, maxinc_axis=maxinc_axis,
                    max_neval_hcube=max_neval_hcube, nstrat=nstrat, adapt_to_errors=adapt_to_errors)
        self.adapt_to_errors = bool(adapt_to_errors)
        self.dim = dim
        self.nstrat = sz['nstrat'].astype(np.int64)
        # AdaptiveMap(limits) then set() regrids with adapt(ninc=...), pyx:1386
        g1 = np.array([[lo, hi] for lo, hi in limits])
        i1 = (g1[:, 1] - g1[:, 0]).reshape(dim, 1)
        grid, inc, ninc = adapt(g1, i1, np.ones(dim, np.int64), None, None, 0.0,
                                sz['ninc'].astype(np.int64))
        self.grid, self.inc, self.ninc = grid, inc, ninc
        self.H = sz['nhcube']
        self.neval = sz['neval']
        self.min_neval_hcube = sz['min_neval_hcube']
        self.max_neval_hcube = max_neval_hcube
        self.neval_frac = neval_frac
        self.alpha = alpha
        self.beta = beta
        self.sigf = np.ones(self.H)
        self.sum_sigf = float(self.H)

    def iterate(self, kind, params, seed=1, stream=0, itn=0, nthreads=1, adapt=True):
        out = np.zeros(5)
        ss = np.array([self.sum_sigf])
        p = _c(params, float)
        rc = lib().vo_iterate(self.dim, kind, _p(p), _p(self.nstrat), _p(self.ninc), _p(self.grid),
                              self.grid.shape[1], _p(self.inc), self.inc.shape[1], self.H,
                              _p(self.sigf), _p(ss), self.neval, self.neval_frac,
                              self.min_neval_hcube, self.max_neval_hcube, self.alpha, self.beta,
                              int(adapt), int(self.adapt_to_errors), seed, stream, itn, nthreads,
                              _p(out))
        assert rc == 0
        self.sum_sigf = float(ss[0])
        return dict(mean=out[0], var=out[1], neval=int(out[2]), range=(int(out[3]), int(out[4])))


def gammaQ(a, x):
    import scipy.special
    return float(scipy.special.gammaincc(a, x))


def weighted_average(means, variances):
    """RAvg.add weighted average (pyx:2392-2410): returns mean, sdev, chi2, dof, Q."""
    w = [1 / (v if v > TINY else TINY) for v in variances]
    var = 1. / np.sum(w)
    mean = np.sum([wi * m for wi, m in zip(w, means)]) * var
    chi2 = 0.0
    if len(means) > 1:
        for m, wi in zip(means, w):
            chi2 += (mean - m) ** 2 * wi
    dof = len(means) - 1
    Q = gammaQ(dof / 2., chi2 / 2.) if dof > 0 else float('nan')
    return mean, math.sqrt(var), chi2, dof, Q
