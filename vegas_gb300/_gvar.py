"""Gaussian random variables for integration results.

The reference returns results built on the third-party ``gvar`` package
(``RAvg`` derives from ``gvar.GVar``, _vegas.pyx:2276).  ``gvar`` is not a
dependency here: this module provides the small part of that interface the
results need -- a mean, a linear combination of independent unit "primary"
noises (so correlated arrays and ``evalcov`` work), linear error propagation
through + - * / and powers, comparisons of means, and the compact
``mean(err)`` string format.
"""
import itertools
import math

import numpy as np
import scipy.special

_counter = itertools.count()


class GVar(object):
    """mean + sum_k der[k] * e_k with independent unit primaries e_k."""

    __slots__ = ('_mean', '_der')

    def __init__(self, mean, der):
        self._mean = float(mean)
        self._der = dict(der)

    @property
    def internaldata(self):
        return (self._mean, self._der)

    @property
    def mean(self):
        return self._mean

    @property
    def var(self):
        return float(sum(c * c for c in self._der.values()))

    @property
    def sdev(self):
        return math.sqrt(self.var)

    def _lin(self, other, a, b, mean):
        der = {k: a * v for k, v in self._der.items()}
        if isinstance(other, GVar):
            for k, v in other._der.items():
                der[k] = der.get(k, 0.0) + b * v
        return GVar(mean, der)

    def __add__(self, o):
        return self._lin(o, 1.0, 1.0, self._mean + (o._mean if isinstance(o, GVar) else o))

    __radd__ = __add__

    def __sub__(self, o):
        return self._lin(o, 1.0, -1.0, self._mean - (o._mean if isinstance(o, GVar) else o))

    def __rsub__(self, o):
        return (-self) + o

    def __neg__(self):
        return GVar(-self._mean, {k: -v for k, v in self._der.items()})

    def __pos__(self):
        return self

    def __mul__(self, o):
        if isinstance(o, GVar):
            return self._lin(o, o._mean, self._mean, self._mean * o._mean)
        o = float(o)
        return GVar(self._mean * o, {k: v * o for k, v in self._der.items()})

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, GVar):
            return self._lin(o, 1.0 / o._mean, -self._mean / o._mean ** 2, self._mean / o._mean)
        o = float(o)
        return GVar(self._mean / o, {k: v / o for k, v in self._der.items()})

    def __rtruediv__(self, o):
        o = float(o)
        m = o / self._mean
        return GVar(m, {k: -m / self._mean * v for k, v in self._der.items()})

    def __pow__(self, p):
        p = float(p)
        m = self._mean ** p
        dm = p * self._mean ** (p - 1.0) if p != 0.0 else 0.0
        return GVar(m, {k: dm * v for k, v in self._der.items()})

    # comparisons act on the means, as gvar's do
    def __lt__(self, o):
        return self._mean < float(o)

    def __gt__(self, o):
        return self._mean > float(o)

    def __le__(self, o):
        return self._mean <= float(o)

    def __ge__(self, o):
        return self._mean >= float(o)

    def __float__(self):
        return self._mean

    def __format__(self, spec):
        return format(str(self), spec)

    def __str__(self):
        return fmt(self._mean, self.sdev)

    def __repr__(self):
        return str(self)


def fmt(mean, sdev):
    """``mean(err)`` with two significant digits in the error (gvar style)."""
    if not math.isfinite(mean):
        return '%g(%g)' % (mean, sdev)
    if not (sdev > 0) or not math.isfinite(sdev):
        return '%.8g(0)' % mean
    ndec = 1 - int(math.floor(math.log10(sdev)))
    err = int(round(sdev * 10 ** ndec)) if ndec >= 0 else int(round(sdev))
    if err >= 100 and ndec > 0:
        ndec -= 1
        err = int(round(sdev * 10 ** ndec))
    if ndec <= 0:
        return '%d(%d)' % (int(round(mean)), int(round(sdev)))
    if sdev >= 1.0:
        return '%.*f(%.*f)' % (ndec, mean, ndec, sdev)
    return '%.*f(%d)' % (ndec, mean, err)


def gvar(mean, unc):
    """gvar(mean, sdev) -> GVar; gvar(mean_array, cov_matrix) -> correlated array."""
    mean_a = np.asarray(mean, float)
    unc_a = np.asarray(unc, float)
    if mean_a.shape == ():
        return GVar(float(mean_a), {next(_counter): float(unc_a)})
    if unc_a.shape == mean_a.shape:
        out = np.empty(mean_a.shape, object)
        for idx in np.ndindex(mean_a.shape):
            out[idx] = GVar(mean_a[idx], {next(_counter): float(unc_a[idx])})
        return out
    m = mean_a.reshape(-1)
    cov = unc_a.reshape(m.size, m.size)
    val, vec = np.linalg.eigh(0.5 * (cov + cov.T))
    val = np.clip(val, 0.0, None)
    keys = [next(_counter) for _ in range(m.size)]
    out = np.empty(m.size, object)
    for i in range(m.size):
        out[i] = GVar(m[i], {keys[j]: vec[i, j] * math.sqrt(val[j])
                             for j in range(m.size) if val[j] > 0})
    return out.reshape(mean_a.shape)


def _flat(g):
    if isinstance(g, GVar):
        return [g]
    return list(np.asarray(g, dtype=object).flat)


def mean(g):
    if isinstance(g, GVar):
        return g.mean
    a = np.asarray(g)
    if a.dtype == object:
        return np.array([x.mean if isinstance(x, GVar) else float(x) for x in a.flat]).reshape(a.shape)
    return a


def sdev(g):
    if isinstance(g, GVar):
        return g.sdev
    a = np.asarray(g)
    if a.dtype == object:
        return np.array([x.sdev if isinstance(x, GVar) else 0.0 for x in a.flat]).reshape(a.shape)
    return np.zeros(a.shape)


def evalcov(g):
    gl = _flat(g)
    n = len(gl)
    cov = np.zeros((n, n))
    for i in range(n):
        for j in range(i + 1):
            di, dj = gl[i]._der, gl[j]._der
            s = sum(v * dj[k] for k, v in di.items() if k in dj)
            cov[i, j] = cov[j, i] = s
    return cov


def corr(a, b):
    c = evalcov([a, b])
    return c[0, 1] / math.sqrt(c[0, 0] * c[1, 1])


def gammaQ(a, x):
    """Regularised upper incomplete gamma function Q(a, x)."""
    return float(scipy.special.gammaincc(a, x))


def svd_inverse_sqrt(mat, svdcut):
    """Rows w_i with sum_i w_i w_i^T = pinv(mat), dropping eigenmodes below
    |svdcut| * max eigenvalue (negative svdcut semantics of gvar.SVD)."""
    mat = np.asarray(mat, float)
    val, vec = np.linalg.eigh(0.5 * (mat + mat.T))
    keep = val >= abs(svdcut) * np.max(np.fabs(val)) if val.size else np.zeros(0, bool)
    val = val[keep]
    vec = vec[:, keep].T
    return vec / np.sqrt(val)[:, None]
