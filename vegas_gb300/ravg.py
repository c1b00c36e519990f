"""Running averages of per-iteration estimates (RAvg, RAvgArray).

Same semantics as the reference's result classes (src/vegas/_vegas.pyx,
RAvg pyx:2276-2451, RAvgArray pyx:2579-2879): inverse-variance weighted
averages across iterations when ``weighted`` (the default while adapting),
plain averages otherwise, chi**2, degrees of freedom and Q.  The per-iteration
mean and variance come from the GPU (FP64); combining at most a few dozen
numbers stays on the host, as in the reference.
"""
import math
import pickle

import numpy as np

from . import _gvar as gv
from ._gvar import GVar

TINY = 1e-257                       # _vegas.pyx:34
EPSILON = np.finfo(float).eps * 1e4  # _vegas.pyx:36


class RAvg(GVar):
    """Running average of scalar Monte Carlo estimates (pyx:2276)."""

    __slots__ = ('weighted', '_wlist', '_mlist', '_msum', '_varsum', '_n', 'itn_results',
                 'sum_neval', 'rescale', '_wbuf', '_mbuf')

    def __init__(self, weighted=True, itn_results=None, sum_neval=0, _rescale=True):
        super(RAvg, self).__init__(0.0, {})
        self.rescale = None
        self.weighted = bool(weighted)
        self._wlist = []
        self._mlist = []
        self._wbuf = np.empty(16)   # the weights and means as arrays (same values as the lists)
        self._mbuf = np.empty(16)
        self._msum = 0.0
        self._varsum = 0.0
        self._n = 0
        self.itn_results = []
        if itn_results is not None:
            if isinstance(itn_results, bytes):
                itn_results = pickle.loads(itn_results)
            for r in itn_results:
                self.add(r)
        self.sum_neval = sum_neval

    def __reduce__(self):
        return (RAvg, (self.weighted, pickle.dumps(self.itn_results), self.sum_neval))

    def extend(self, ravg):
        """Merge the results of ``ravg`` after those already in ``self``."""
        for r in ravg.itn_results:
            self.add(r)
        self.sum_neval += ravg.sum_neval

    def add(self, g):
        """Add estimate ``g`` (a GVar) to the running average (pyx:2392-2410)."""
        self.add_many((g,))

    def add_many(self, gs):
        """Add several estimates in order.  The weighted average after the
        last one depends only on the full lists (the reference recomputes it
        from them at every ``add``), so it is formed once, with the same
        numpy sums -- over arrays holding the lists' values, which numpy sums
        exactly as it sums the lists, at array rather than Python-loop cost
        per iteration; the unweighted running sums are accumulated in order."""
        for g in gs:
            self.itn_results.append(g)
            self._mlist.append(g.mean)
            if self.weighted:
                k = len(self._wlist)
                w = 1 / (g.var if g.var > TINY else TINY)
                self._wlist.append(w)
                if k == self._wbuf.shape[0]:
                    self._wbuf = np.concatenate([self._wbuf, np.empty(k)])
                    self._mbuf = np.concatenate([self._mbuf, np.empty(k)])
                self._wbuf[k] = w
                self._mbuf[k] = g.mean
            else:
                self._msum += g.mean
                self._varsum += g.var
                self._n += 1
        if not self._mlist:
            return
        if self.weighted:
            k = len(self._wlist)
            var = 1. / np.sum(self._wbuf[:k])
            sdev = np.sqrt(var)
            mean = np.sum(self._wbuf[:k] * self._mbuf[:k]) * var
        else:
            mean = self._msum / self._n
            sdev = np.sqrt(self._varsum / self._n ** 2)
        g2 = gv.gvar(mean, sdev)
        self._mean, self._der = g2._mean, g2._der

    @property
    def chi2(self):
        if len(self.itn_results) <= 1:
            return 0.0
        if self.weighted:
            wavg = self.mean
            ans = 0.0
            for m, w in zip(self._mlist, self._wlist):
                ans += (wavg - m) ** 2 * w
            return ans
        wavg = self.mean
        return np.sum([(m - wavg) ** 2 for m in self._mlist]) / (self._varsum / self._n)

    @property
    def dof(self):
        return len(self.itn_results) - 1

    @property
    def nitn(self):
        return len(self.itn_results)

    @property
    def Q(self):
        return gv.gammaQ(self.dof / 2., self.chi2 / 2.) if self.dof > 0 and self.chi2 >= 0 \
            else float('nan')

    @property
    def avg_neval(self):
        return self.sum_neval / self.nitn if self.nitn > 0 else 0

    def converged(self, rtol, atol):
        return self.sdev < atol + rtol * abs(self.mean)

    def summary(self, extended=False, weighted=None):
        """Iteration-by-iteration table (pyx:2412-2451)."""
        if weighted is None:
            weighted = self.weighted
        acc = RAvg(weighted=weighted)
        lines = []
        for i, res in enumerate(self.itn_results):
            acc.add(res)
            lines.append(('%3d' % (i + 1), '%-15s' % res, '%-15s' % acc,
                          '%8.2f' % (acc.chi2 / acc.dof if i != 0 else 0.0),
                          '%8.2f' % (acc.Q if i != 0 else 1.0)))
        return _table(lines, weighted)


def _table(lines, weighted):
    nchar = [0] * 5
    for data in lines:
        for i, d in enumerate(data):
            nchar[i] = max(nchar[i], len(d))
    fmt = '%%%ds   %%-%ds %%-%ds %%%ds %%%ds\n' % tuple(nchar)
    ans = fmt % ('itn', 'integral', 'wgt average' if weighted else 'average', 'chi2/dof', 'Q')
    ans += len(ans[:-1]) * '-' + '\n'
    for data in lines:
        ans += fmt % data
    return ans


class RAvgArray(np.ndarray):
    """Running average of array-valued estimates (pyx:2579).

    Weighted averages use the inverse covariance of each iteration, with
    eigenmodes below EPSILON*len*1e4 of the largest dropped (pyx:2715-2722).
    """

    def __new__(cls, shape=None, weighted=True, itn_results=None, sum_neval=0, rescale=True):
        if shape is None:
            if not itn_results:
                raise ValueError('must specify shape or itn_results')
            shape = np.shape(itn_results[0])
        obj = np.ndarray.__new__(cls, shape=shape, dtype=object)
        obj.flat = [gv.gvar(0., 0.) for _ in range(obj.size)]
        obj.weighted = bool(weighted)
        obj.rescale = (True if rescale is True else rescale) if weighted else None
        obj._wlist = []
        obj._mlist = []
        obj._msum = 0.
        obj._covsum = 0.
        obj._n = 0
        obj._invw = None
        obj.itn_results = []
        obj.sum_neval = sum_neval
        if itn_results is not None:
            for r in itn_results:
                obj.add(r)
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        for k, v in (('weighted', True), ('rescale', True), ('_wlist', []), ('_mlist', []),
                     ('_msum', 0.), ('_covsum', 0.), ('_n', 0), ('_invw', None),
                     ('itn_results', []), ('sum_neval', 0)):
            setattr(self, k, getattr(obj, k, v))

    def __reduce__(self):
        return (_rebuild_ravgarray, (self.shape, self.weighted, pickle.dumps(
            [(gv.mean(r), gv.evalcov(r)) for r in self.itn_results]), self.sum_neval,
            self.rescale))

    @staticmethod
    def _w(matrix):
        return gv.svd_inverse_sqrt(matrix, -EPSILON * len(matrix) * 1e4)

    def add(self, g):
        g = np.asarray(g)
        self.itn_results.append(g)
        g = g.reshape(-1)
        if self.weighted:
            if not hasattr(self, '_rescale_v'):
                if self.rescale is not None:
                    rs = np.fabs(gv.mean(g) if self.rescale is True
                                 else np.asarray(self.rescale).reshape(-1))
                    gsd = gv.sdev(g)
                    idx = gsd > rs
                    rs[idx] = gsd[idx]
                    rs[rs <= 0] = 1.
                    self._rescale_v = rs
                else:
                    self._rescale_v = 1.
            gm = gv.mean(g) / self._rescale_v
            gc = gv.evalcov(g) / np.outer(np.ones(g.size) * self._rescale_v,
                                          np.ones(g.size) * self._rescale_v)
            for i in range(len(gc)):
                if gc[i, i] <= 0:
                    gc[i, i] = TINY
            self._mlist.append(gm)
            self._wlist.append(self._w(gc))
            invcov = np.sum([w.T.dot(w) for w in self._wlist], axis=0)
            invw = self._w(invcov)
            cov = invw.T.dot(invw)
            mean = 0.0
            for m, w in zip(self._mlist, self._wlist):
                for wj in w:
                    wj_m = wj.dot(m)
                    for iw in invw:
                        mean = mean + iw * iw.dot(wj) * wj_m
            rs = self._rescale_v * np.ones(g.size)
            res = gv.gvar(mean * rs, cov * np.outer(rs, rs))
        else:
            gm = gv.mean(g)
            gc = gv.evalcov(g)
            self._mlist.append(gm)
            self._msum = self._msum + gm
            self._covsum = self._covsum + gc
            self._invw = None
            self._n += 1
            res = gv.gvar(self._msum / self._n, self._covsum / self._n ** 2)
        self.flat[:] = np.asarray(res, dtype=object).reshape(-1)

    @property
    def chi2(self):
        if len(self.itn_results) <= 1:
            return 0.0
        if self.weighted:
            ans = 0.0
            wavg = gv.mean(self).reshape(-1) / self._rescale_v
            for w, m in zip(self._wlist, self._mlist):
                for wi in w:
                    ans += wi.dot(m - wavg) ** 2
            return ans
        if self._invw is None:
            self._invw = self._w(self._covsum / self._n)
        wavg = gv.mean(self).reshape(-1)
        ans = 0.0
        for m in self._mlist:
            for iw in self._invw:
                ans += iw.dot(wavg - m) ** 2
        return ans

    @property
    def dof(self):
        if len(self.itn_results) <= 1:
            return 0
        if not self.weighted:
            if self._invw is None:
                self._invw = self._w(self._covsum / self._n)
            return (len(self.itn_results) - 1) * len(self._invw)
        return int(np.sum([len(w) for w in self._wlist])) - self.size

    @property
    def nitn(self):
        return len(self.itn_results)

    @property
    def Q(self):
        if self.dof <= 0 or self.chi2 < 0:
            return float('nan')
        return gv.gammaQ(self.dof / 2., self.chi2 / 2.)

    @property
    def avg_neval(self):
        return self.sum_neval / self.nitn if self.nitn > 0 else 0

    def converged(self, rtol, atol):
        return bool(np.all(gv.sdev(self) < atol + rtol * np.abs(gv.mean(self))))

    def summary(self, extended=False, weighted=None, rescale=None):
        if weighted is None:
            weighted = self.weighted
        if rescale is None:
            rescale = self.rescale
        acc = RAvgArray(self.shape, weighted=weighted, rescale=rescale)
        lines = []
        for i, res in enumerate(self.itn_results):
            acc.add(res)
            lines.append(('%3d' % (i + 1), '%-15s' % np.asarray(res).flat[0],
                          '%-15s' % acc.flat[0],
                          '%8.2f' % (acc.chi2 / acc.dof if i != 0 else 0.0),
                          '%8.2f' % (acc.Q if i != 0 else 1.0)))
        return _table(lines, weighted)


def _rebuild_ravgarray(shape, weighted, itn, sum_neval, rescale):
    res = [gv.gvar(m, c) for m, c in pickle.loads(itn)]
    out = RAvgArray(shape, weighted=weighted, sum_neval=sum_neval, rescale=rescale)
    for r in res:
        out.add(np.asarray(r).reshape(shape))
    return out


class RAvgDict(dict):
    """Running average of dictionary-valued estimates (pyx:2453-2545).

    Keys map to GVars or arrays of GVars; the values share one flat
    RAvgArray (``rarray``), so correlations between keys are kept.
    ``layout`` is a list of (key, shape) in the integrand's key order.
    """

    def __init__(self, layout, weighted=True, sum_neval=0, rescale=True):
        super(RAvgDict, self).__init__()
        self.layout = [(k, tuple(s)) for k, s in layout]
        self.size = int(sum(int(np.prod(s)) if s else 1 for _, s in self.layout))
        self.rarray = RAvgArray((self.size,), weighted=weighted, rescale=rescale)
        self.weighted = weighted
        self.itn_results = []
        self.sum_neval = sum_neval
        self._fill()

    def _slices(self):
        o = 0
        for k, s in self.layout:
            n = int(np.prod(s)) if s else 1
            yield k, s, slice(o, o + n)
            o += n

    def _fill(self):
        flat = np.asarray(self.rarray, dtype=object).reshape(-1)
        for k, s, sl in self._slices():
            dict.__setitem__(self, k, flat[sl][0] if s == () else flat[sl].reshape(s))

    def unflatten(self, flat):
        """Dictionary of the flat vector's pieces in this layout."""
        flat = np.asarray(flat, dtype=object).reshape(-1)
        out = {}
        for k, s, sl in self._slices():
            out[k] = flat[sl][0] if s == () else flat[sl].reshape(s)
        return out

    def add(self, g):
        """Add one iteration's estimates: a dict in this layout, or the flat vector."""
        if isinstance(g, dict):
            flat = np.concatenate([np.asarray(g[k], dtype=object).reshape(-1) for k, _ in self.layout])
        else:
            flat = np.asarray(g, dtype=object).reshape(-1)
        self.itn_results.append(self.unflatten(flat))
        self.rarray.add(flat)
        self._fill()

    def extend(self, ravg):
        for r in ravg.itn_results:
            self.add(r)
        self.sum_neval += ravg.sum_neval

    @property
    def buf(self):
        return np.asarray(self.rarray, dtype=object).reshape(-1)

    @property
    def chi2(self):
        return self.rarray.chi2

    @property
    def dof(self):
        return self.rarray.dof

    @property
    def Q(self):
        return self.rarray.Q

    @property
    def nitn(self):
        return len(self.itn_results)

    @property
    def avg_neval(self):
        return self.sum_neval / self.nitn if self.nitn > 0 else 0

    def converged(self, rtol, atol):
        b = self.buf
        return bool(np.all(gv.sdev(b) < atol + rtol * np.abs(gv.mean(b))))

    def summary(self, extended=False, weighted=None, rescale=None):
        return self.rarray.summary(extended=False, weighted=weighted, rescale=rescale)
