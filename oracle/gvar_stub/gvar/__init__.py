"""Minimal stand-in for the third-party ``gvar`` package (pinned by the
reference at ``gvar>=13.1.5``, pyproject.toml:28), written for this repository.

TEST INFRASTRUCTURE ONLY.  It exists so that the reference vegas Cython module
(src/vegas/_vegas.pyx), compiled out of tree by ``oracle/build_ref.py``, can be
imported in the development container to generate golden vectors.  Nothing in
the product package imports it.

It restates only what the reference's hot path touches:

* ``GVar`` / ``gvar()``: Gaussian variables carried as (mean, {primary: coeff})
  so that correlated arrays (``gvar(mean_vec, cov)``) and ``evalcov`` work.
  ``RAvg`` subclasses ``GVar`` and re-initialises through ``internaldata``
  (_vegas.pyx:2305, 2403).
* ``RNG`` = numpy Generator, ``ranseed`` (used for ``xsample``,
  _vegas.pyx:1253; hot-path draws are injected through
  ``ran_array_generator``, _vegas.pyx:1678-1679).
* ``gammaQ`` = regularised upper incomplete gamma (scipy ``gammaincc``),
  ``SVD`` (eigen-decomposition with a negative ``svdcut`` that drops small
  modes), ``mean``/``sdev``/``evalcov``, ``dumps``/``loads`` = pickle.
* ``BufferDict`` supports only what ``vegas.restratify``'s internal
  integrand uses (src/vegas/__init__.py:1390-1419): an empty dictionary
  filled with rbatch arrays (batch index last) and flattened by
  ``_r2lbatch()`` to one lbatch array ``[nbatch, size]`` in key order, which
  the reference then integrates as an array-valued integrand.  Any other use
  raises.
"""
import itertools
import math
import pickle

import numpy
import scipy.special

_counter = itertools.count()


class GVarRef(object):
    pass


class GVar(object):
    """Gaussian random variable: mean plus linear combination of primaries."""

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

    def __call__(self):
        return self._mean + self.sdev * RNG.normal()

    # arithmetic (linear propagation)
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

    def __mul__(self, o):
        if isinstance(o, GVar):
            return self._lin(o, o._mean, self._mean, self._mean * o._mean)
        return GVar(self._mean * o, {k: v * o for k, v in self._der.items()})

    __rmul__ = __mul__

    def __truediv__(self, o):
        if isinstance(o, GVar):
            return self._lin(o, 1.0 / o._mean, -self._mean / o._mean ** 2, self._mean / o._mean)
        return GVar(self._mean / o, {k: v / o for k, v in self._der.items()})

    def __pow__(self, p):
        p = float(p)
        m = self._mean ** p
        dm = p * self._mean ** (p - 1.0) if p != 0.0 else 0.0
        return GVar(m, {k: dm * v for k, v in self._der.items()})

    # comparisons act on the means, as in gvar
    def __lt__(self, o):
        return self._mean < (o._mean if isinstance(o, GVar) else o)

    def __gt__(self, o):
        return self._mean > (o._mean if isinstance(o, GVar) else o)

    def __le__(self, o):
        return self._mean <= (o._mean if isinstance(o, GVar) else o)

    def __ge__(self, o):
        return self._mean >= (o._mean if isinstance(o, GVar) else o)

    def __str__(self):
        return fmt(self._mean, self.sdev)

    __repr__ = __str__


def fmt(mean, sdev):
    """Compact 'mean(err)' notation with two significant digits of error."""
    if not (sdev > 0) or not math.isfinite(sdev):
        return '%g(0)' % mean
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


def _new_primary(sdev):
    return {next(_counter): float(sdev)}


def gvar(*args):
    if len(args) == 1 and isinstance(args[0], GVar):
        return args[0]
    mean, unc = args
    mean_a = numpy.asarray(mean, float)
    unc_a = numpy.asarray(unc, float)
    if mean_a.shape == ():
        return GVar(float(mean_a), _new_primary(float(unc_a)))
    if unc_a.shape == mean_a.shape:
        out = numpy.empty(mean_a.shape, object)
        for idx in numpy.ndindex(mean_a.shape):
            out[idx] = GVar(mean_a[idx], _new_primary(unc_a[idx]))
        return out
    # correlated: cov matrix over flattened mean
    m = mean_a.reshape(-1)
    cov = unc_a.reshape(m.size, m.size)
    val, vec = numpy.linalg.eigh(0.5 * (cov + cov.T))
    val = numpy.clip(val, 0.0, None)
    keys = [next(_counter) for _ in range(m.size)]
    out = numpy.empty(m.size, object)
    for i in range(m.size):
        der = {}
        for j in range(m.size):
            c = vec[i, j] * math.sqrt(val[j])
            if c != 0.0:
                der[keys[j]] = c
        out[i] = GVar(m[i], der)
    return out.reshape(mean_a.shape)


def gvar_factory(cov=None):
    return gvar


def _flat(g):
    if isinstance(g, GVar):
        return [g]
    return list(numpy.asarray(g, dtype=object).flat)


def mean(g):
    if isinstance(g, GVar):
        return g.mean
    a = numpy.asarray(g)
    if a.dtype == object:
        return numpy.array([x.mean if isinstance(x, GVar) else x for x in a.flat], float).reshape(a.shape)
    return a


def sdev(g):
    if isinstance(g, GVar):
        return g.sdev
    a = numpy.asarray(g)
    if a.dtype == object:
        return numpy.array([x.sdev if isinstance(x, GVar) else 0.0 for x in a.flat], float).reshape(a.shape)
    return numpy.zeros(a.shape, float)


def var(g):
    return sdev(g) ** 2


def evalcov(g):
    gl = _flat(g)
    n = len(gl)
    cov = numpy.zeros((n, n), float)
    for i in range(n):
        for j in range(i + 1):
            di, dj = gl[i]._der, gl[j]._der
            s = sum(v * dj[k] for k, v in di.items() if k in dj)
            cov[i, j] = cov[j, i] = s
    return cov


def corr(a, b):
    c = evalcov([a, b])
    return c[0, 1] / math.sqrt(c[0, 0] * c[1, 1])


class SVD(object):
    """Eigen-decomposition of a symmetric matrix; svdcut<0 drops small modes."""

    def __init__(self, mat, svdcut=None, rescale=False):
        mat = numpy.asarray(mat, float)
        if rescale:
            d = numpy.sqrt(numpy.fabs(numpy.diag(mat)))
            d[d == 0] = 1.0
            self.D = 1.0 / d
            mat = (mat * self.D[:, None]) * self.D[None, :]
        else:
            self.D = None
        val, vec = numpy.linalg.eigh(mat)
        keep = numpy.ones(val.shape, bool)
        if svdcut is not None and svdcut < 0:
            keep = val >= abs(svdcut) * numpy.max(numpy.fabs(val))
        elif svdcut is not None and svdcut > 0:
            val = numpy.maximum(val, svdcut * numpy.max(numpy.fabs(val)))
        self.val = val[keep]
        self.vec = vec[:, keep].T

    def decomp(self, n=1):
        w = self.vec * (self.val ** (n / 2.0))[:, None]
        if self.D is not None:
            w = w * (self.D ** (-n))[None, :]
        return w


def gammaQ(a, x):
    return float(scipy.special.gammaincc(a, x))


RNG = numpy.random.default_rng(0)


def ranseed(seed=None, size=None):
    global RNG
    if seed is None:
        seed = int(numpy.random.SeedSequence().entropy % (2 ** 31))
    RNG = numpy.random.default_rng(seed)
    return seed


def randint(lo, hi, size=None):
    return RNG.integers(lo, hi, size=size)


def dumps(obj, protocol=None):
    return pickle.dumps(obj, protocol=protocol)


def loads(s):
    return pickle.loads(s)


def remove_gvars(x, gvlist):
    return x


def distribute_gvars(x, gvlist):
    return x


def tabulate(x, **kargs):
    return str(x)


class BufferDict(dict):
    """Empty dictionary of rbatch arrays, flattened by ``_r2lbatch``."""
    shape = None

    def __init__(self, *args, **kargs):
        if args or kargs:
            raise NotImplementedError('BufferDict is not provided by the oracle gvar stand-in')
        super(BufferDict, self).__init__()

    def _r2lbatch(self):
        cols = []
        for k in self:
            v = numpy.asarray(self[k], float)
            cols.append(v.reshape(-1, v.shape[-1]).T)
        return (numpy.ascontiguousarray(numpy.concatenate(cols, axis=1)),)


def asbufferdict(x):
    raise NotImplementedError('BufferDict is not provided by the oracle gvar stand-in')
