"""Expectation values with respect to a probability density: PDFIntegrator.

Follows the reference's ``vegas.PDFIntegrator`` (src/vegas/__init__.py:373-1189)
as a consumer of the batch-integrand path of ``Integrator``: the parameters
``p`` of a multi-dimensional distribution are re-expressed through the
principal axes of a Gaussian ``param`` (mean ``m``, covariance ``C``),

    p = m + V diag(sqrt(lambda)) chiv,      chiv = scale * tan(theta),

with ``C = V diag(lambda) V^T`` (eigenvalues below ``svdcut * max`` raised to
that floor, __init__.py:482-485), and vegas integrates over ``theta`` in
``[-atan(limit/scale), atan(limit/scale)]^d`` on a map pre-adapted to the
Gaussian (``_make_map``, __init__.py:576-592).  The integrand is a dictionary
with ``pdf(p) dp/dtheta`` and ``f(p) pdf(p) dp/dtheta`` (``_f_lbatch``,
__init__.py:594-630); the expectation value is the ratio of the two
integrals, with its error from their covariance.  Everything runs on the
GPU: the integrand is a torch batch function of the CUDA tensor ``theta``.

Differences from the reference, stated: ``param`` is given as a GVar array
(``vegas_gb300.gvar(mean, cov)``), a dictionary of them, or a (mean, cov)
pair -- there is no ``gvar.PDF`` / ``BufferDict`` machinery (the third-party
``gvar`` package is not a dependency); ``stats`` returns means and standard
deviations (no ``moments`` / ``histograms``); the random numbers of
``_make_map`` come from numpy's generator seeded by the integrator's seed.
"""
import math

import numpy as np
import torch

from . import _gvar as gv
from .adaptive_map import AdaptiveMap
from .integrands import lbatchintegrand
from .integrator import Integrator


class _GaussParam(object):
    """Mean, principal axes and scales of the Gaussian ``param`` (the part
    of ``gvar.PDF`` the integrator uses), with the flat <-> structured
    layout of the parameters."""

    def __init__(self, param, svdcut):
        self.layout = None            # None: flat array of shape `shape`; else [(key, shape), ...]
        if isinstance(param, tuple) and len(param) == 2:
            mean = np.asarray(param[0], float)
            cov = np.asarray(param[1], float).reshape(mean.size, mean.size)
            self.shape = mean.shape
        elif isinstance(param, dict):
            self.layout = []
            flat = []
            for k, v in param.items():
                a = np.asarray(v, dtype=object)
                self.layout.append((k, a.shape))
                flat.extend(a.reshape(-1))
            mean = np.array([x.mean for x in flat])
            cov = gv.evalcov(flat)
            self.shape = mean.shape
        else:
            a = np.asarray(param, dtype=object)
            flat = list(a.reshape(-1))
            mean = np.array([x.mean for x in flat])
            cov = gv.evalcov(flat)
            self.shape = a.shape
        self.mean = mean.reshape(-1)
        self.size = self.mean.size
        cov = 0.5 * (cov + cov.T)
        val, vec = np.linalg.eigh(cov)
        if svdcut:
            floor = abs(svdcut) * np.max(val)
            val = np.where(val < floor, floor, val)
        if np.any(val <= 0):
            raise ValueError('param covariance is not positive definite (raise svdcut)')
        self.axes = vec * np.sqrt(val)[None, :]      # p = mean + axes @ chiv
        self.dp_dchiv = float(np.prod(np.sqrt(val)))
        self._t = {}

    def tensors(self, device, dtype):
        key = (str(device), dtype)
        if key not in self._t:
            self._t[key] = (torch.as_tensor(self.mean, dtype=dtype, device=device),
                            torch.as_tensor(self.axes, dtype=dtype, device=device))
        return self._t[key]

    def pflat(self, chiv):
        """Parameters [n, size] for chiv [n, size]."""
        m, A = self.tensors(chiv.device, chiv.dtype)
        return m[None, :] + chiv @ A.t()

    def structured(self, p):
        """p [n, size] in the layout of ``param``: a tensor [n, *shape] or a
        dictionary of [n, *shape_k] tensors (batch index first)."""
        n = p.shape[0]
        if self.layout is None:
            return p.reshape((n,) + tuple(self.shape))
        out, o = {}, 0
        for k, sh in self.layout:
            sz = int(np.prod(sh)) if sh else 1
            out[k] = p[:, o:o + sz].reshape((n,) + tuple(sh))
            o += sz
        return out


def _batch_values(fcn, p):
    """f(p) for a batch (batch index first); rbatch functions get the batch
    index last and return it last."""
    if getattr(fcn, 'fcntype', 'lbatch') == 'rbatch':
        if isinstance(p, dict):
            q = {k: v.movedim(0, -1) for k, v in p.items()}
        else:
            q = p.movedim(0, -1)
        out = fcn(q)
        if hasattr(out, 'keys'):
            return {k: torch.as_tensor(v).movedim(-1, 0) for k, v in out.items()}
        return torch.as_tensor(out).movedim(-1, 0)
    return fcn(p)


class PDFEV(object):
    """Expectation value <f(p)> = int f pdf / int pdf (scalar f): a GVar-like
    ratio with the integrals' correlation; ``pdfnorm`` is int pdf."""

    def __init__(self, results):
        self.results = results
        num, den = results['f(p)*pdf'], results['pdf']
        self.pdfnorm = den
        self.value = _ratio(num, den)

    def __getattr__(self, k):
        return getattr(self.__dict__['value'], k)

    def __str__(self):
        return str(self.value)

    __repr__ = __str__


class PDFEVArray(np.ndarray):
    """Expectation values of an array-valued f(p) (GVar array)."""

    def __new__(cls, results):
        num, den = results['f(p)*pdf'], results['pdf']
        num = np.asarray(num, dtype=object)
        val = np.empty(num.shape, object)
        for idx in np.ndindex(num.shape):
            val[idx] = _ratio(num[idx], den)
        obj = val.view(cls)
        obj.pdfnorm = den
        obj.results = results
        return obj

    def __array_finalize__(self, obj):
        if obj is None:
            return
        self.pdfnorm = getattr(obj, 'pdfnorm', None)
        self.results = getattr(obj, 'results', None)


def _ratio(num, den):
    """num / den with linear error propagation through both (correlated)."""
    return _as_gvar(num) / _as_gvar(den)


def _as_gvar(x):
    if isinstance(x, gv.GVar):
        return x
    if hasattr(x, '_der'):
        return gv.GVar(float(x.mean), x._der)
    return gv.GVar(float(x), {})


class PDFIntegrator(Integrator):
    """vegas integrator for expectation values with respect to a PDF
    (reference ``vegas.PDFIntegrator``, src/vegas/__init__.py:373-1189).

    Args:
        param: the Gaussian that defines the integration variables -- a GVar
            array (``vegas_gb300.gvar(mean, cov)``), a dictionary of GVars /
            GVar arrays, or a ``(mean, cov)`` pair.  Its PDF is the one used
            when ``pdf`` is None.
        pdf: None, or a batch function ``pdf(p)`` of the parameters in
            ``param``'s layout (batch index first for lbatch functions, last
            for rbatchintegrand); need not be normalised.
        adapt_to_pdf: vegas adapts to the PDF (True) or to f(p) pdf(p).
        limit: each variable ranges over ``limit`` standard deviations of
            ``param`` on either side of its mean.
        scale: the variables emphasise ``scale`` standard deviations.
        svdcut: eigenvalues of ``param``'s covariance below ``svdcut`` times
            the largest are raised to that floor.
        **kargs: settings of the underlying Integrator (``uses_jac`` is
            ignored, as in the reference).
    """

    def __init__(self, param, pdf=None, adapt_to_pdf=True, limit=100., scale=1., svdcut=1e-15, **kargs):
        if param is None:
            raise ValueError('param must be specified')
        kargs = dict(kargs)
        kargs.pop('uses_jac', None)
        self.param_pdf = _GaussParam(param, svdcut)
        self.limit = abs(float(limit))
        self.scale = abs(float(scale))
        self.pdf = pdf
        self.adapt_to_pdf = bool(adapt_to_pdf)
        seed = kargs.get('seed', Integrator.defaults.get('seed'))
        nodes = self._make_map(self.limit / self.scale, seed, kargs.get('device'))
        super(PDFIntegrator, self).__init__(AdaptiveMap(self.param_pdf.size * [nodes],
                                                        device=kargs.get('device')), **kargs)

    def _make_map(self, limit, seed, device):
        """One axis of the map, pre-adapted to the Gaussian in theta (the
        reference's _make_map, __init__.py:576-592: 2000 random points, 10
        adapt steps with alpha 1.5 on 100 increments); returns its nodes."""
        rng = np.random.default_rng(None if seed is None else (int(seed) * 7919 + 17) & ((1 << 63) - 1))
        ny = 2000
        lim = math.atan(limit)
        m = AdaptiveMap([[-lim, lim]], ninc=100, device=device)
        y = torch.as_tensor(rng.random((ny, 1)), dtype=torch.float64, device=m.device)
        theta = torch.empty_like(y)
        jac = torch.empty(ny, dtype=torch.float64, device=m.device)
        for _ in range(10):
            m.map(y, theta, jac)
            t = torch.tan(theta[:, 0])
            x = self.scale * t
            fx = (t ** 2 + 1) * torch.exp(-(x ** 2) / 2.)
            m.add_training_data(y, (jac * fx) ** 2)
            m.adapt(alpha=1.5)
        return np.array(m.grid[0][:int(m.ninc[0]) + 1])

    def _integrand(self, f):
        pp, scale, pdf, adapt_to_pdf = self.param_pdf, self.scale, self.pdf, self.adapt_to_pdf
        norm = 1.0 / math.sqrt(2 * math.pi)

        @lbatchintegrand
        def fcn(theta):
            t = torch.tan(theta)
            chiv = scale * t
            dp_dtheta = torch.prod(scale * (t * t + 1.), dim=1) * pp.dp_dchiv
            p = pp.structured(pp.pflat(chiv))
            if pdf is None:
                dens = torch.prod(torch.exp(-(chiv * chiv) / 2.) * norm, dim=1) / pp.dp_dchiv
            else:
                dens = torch.as_tensor(_batch_values(pdf, p), device=theta.device).reshape(theta.shape[0])
            w = dp_dtheta * dens
            if f is None:
                return {'pdf': w}
            fp = _batch_values(f, p)
            ans = {}
            if adapt_to_pdf:
                ans['pdf'] = w
            if hasattr(fp, 'keys'):
                for k in fp:
                    v = torch.as_tensor(fp[k], device=theta.device)
                    ans[('f(p)*pdf', k)] = v * w.reshape((-1,) + (v.dim() - 1) * (1,))
            else:
                v = torch.as_tensor(fp, device=theta.device, dtype=w.dtype)
                ans['f(p)*pdf'] = v * w.reshape((-1,) + (v.dim() - 1) * (1,))
            if not adapt_to_pdf:
                ans['pdf'] = w
            return ans

        return fcn

    def __call__(self, f=None, save=None, saveall=None, **kargs):
        """Expectation value of f(p) (a PDFEV / PDFEVArray / dict of them);
        with f None, the integral of the PDF (an RAvgDict with ``pdfnorm``)."""
        kargs = dict(kargs)
        kargs.pop('uses_jac', None)
        for k in ('pdf', 'adapt_to_pdf'):
            if k in kargs:
                setattr(self, k, kargs.pop(k))
        results = super(PDFIntegrator, self).__call__(self._integrand(f), save=save, saveall=saveall,
                                                      **kargs)
        if results['pdf'].mean == 0:
            raise RuntimeError('Integral of PDF vanishes; increase neval?')
        if f is None:
            results.pdfnorm = results['pdf']
            return results
        keys = [k for k in results.keys() if k != 'pdf']
        if keys == ['f(p)*pdf']:
            if np.ndim(results['f(p)*pdf']) == 0:
                return PDFEV(results)
            return PDFEVArray(results)
        out = {}
        den = results['pdf']
        for k in keys:
            name = k[1]
            v = np.asarray(results[k], dtype=object)
            if v.shape == ():
                out[name] = _ratio(v.item() if hasattr(v, 'item') else v, den)
            else:
                r = np.empty(v.shape, object)
                for idx in np.ndindex(v.shape):
                    r[idx] = _ratio(v[idx], den)
                out[name] = r
        return out

    def stats(self, f, **kargs):
        """Mean and standard deviation of f(p) under the PDF (from the
        integrals of f pdf, f^2 pdf and pdf; __init__.py:729-946 without
        moments and histograms): a GVar-like ``mean(sdev)`` per component,
        the vegas error of each in ``vegas_mean`` / ``vegas_sdev``."""

        def f2(p):
            v = _batch_values(f, p)
            if hasattr(v, 'keys'):
                out = {}
                for k in v:
                    t = torch.as_tensor(v[k])
                    out[('m', k)] = t
                    out[('m2', k)] = t * t
                return out
            t = torch.as_tensor(v)
            return {'m': t, 'm2': t * t}

        r = self(lbatchintegrand(f2), **kargs)
        res = _Stats()
        names = sorted({k[1] for k in r if isinstance(k, tuple)}, key=str) if any(
            isinstance(k, tuple) for k in r) else [None]
        for name in names:
            m = r['m'] if name is None else r[('m', name)]
            m2 = r['m2'] if name is None else r[('m2', name)]
            mean = np.asarray(gv.mean(m), float)
            var = np.asarray(gv.mean(m2), float) - mean ** 2
            sd = np.sqrt(np.clip(var, 0.0, None))
            val = gv.gvar(mean, sd)
            res.vegas_mean[name] = m
            res.vegas_sdev[name] = sd
            res[name] = val
        return res[None] if names == [None] else res

    def sample(self, nbatch, mode='rbatch'):
        """Weighted sample (wgts, p) of the PDF: sum_i wgts[i] g(p_i)
        estimates <g(p)> (__init__.py:1049-1188); p in param's layout with
        the batch index last ('rbatch') or first ('lbatch')."""
        wgt, theta = super(PDFIntegrator, self).sample(nbatch=nbatch, mode='lbatch')
        pp = self.param_pdf
        t = torch.tan(theta)
        chiv = self.scale * t
        dp_dtheta = torch.prod(self.scale * (t * t + 1.), dim=1) * pp.dp_dchiv
        p = pp.structured(pp.pflat(chiv))
        if self.pdf is None:
            dens = torch.prod(torch.exp(-(chiv * chiv) / 2.) / math.sqrt(2 * math.pi), dim=1) / pp.dp_dchiv
        else:
            dens = torch.as_tensor(_batch_values(self.pdf, p), device=theta.device).reshape(theta.shape[0])
        w = wgt.to(dens.dtype) * dp_dtheta * dens
        w = w / w.sum()
        if mode == 'rbatch':
            p = {k: v.movedim(0, -1) for k, v in p.items()} if isinstance(p, dict) else p.movedim(0, -1)
        return w, p


class _Stats(dict):
    """Results of PDFIntegrator.stats: component -> mean(sdev), with the
    vegas results behind them."""

    def __init__(self):
        super(_Stats, self).__init__()
        self.vegas_mean = {}
        self.vegas_sdev = {}
