"""Integrand adapters and built-in integrands.

* ``lbatchintegrand`` / ``LBatchIntegrand`` (and the legacy aliases
  ``batchintegrand`` / ``BatchIntegrand``) mark batch integrands exactly as in
  the reference (src/vegas/_vegas.pyx:3386-3438): the function receives
  ``x[i, d]`` -- here a CUDA ``torch`` tensor ``[n, dim]`` -- and returns
  ``f[i]`` (a tensor, or anything ``torch.as_tensor`` accepts).
* Built-in integrands (``Gaussian``, ``Ridge``, ``LorentzianProduct``,
  ``GaussianMixture``, ``LatticeAction``, ``Constant``) are the synthetic
  workloads of the benchmarks.  The Integrator evaluates them inside its
  fused CUDA kernel; calling one directly evaluates it with torch ops (handy
  as an ordinary lbatch integrand, e.g. to exercise the drop-in path).
"""
import math

import numpy as np
import torch

from . import _native as N


class LBatchIntegrand(object):
    """Wrapper for lbatch integrands (pyx:3386-3406)."""

    def __init__(self, fcn=None):
        self.fcn = self if fcn is None else fcn

    @property
    def fcntype(self):
        return 'lbatch'

    def __call__(self, *args, **kargs):
        return self.fcn(*args, **kargs)

    def __getattr__(self, attr):
        if attr == 'fcn':
            raise AttributeError(attr)
        return getattr(self.fcn, attr)


def lbatchintegrand(f):
    """Decorator marking a batch integrand ``f(x[n, dim]) -> f[n]`` (pyx:3408-3438)."""
    try:
        f.fcntype = 'lbatch'
        return f
    except Exception:
        return LBatchIntegrand(f)


class RBatchIntegrand(object):
    """Batch index on the right: ``f(x[dim, n]) -> f[n]`` (pyx:3440-3455)."""

    def __init__(self, fcn=None):
        self.fcn = self if fcn is None else fcn

    @property
    def fcntype(self):
        return 'rbatch'

    def __call__(self, *args, **kargs):
        return self.fcn(*args, **kargs)

    def __getattr__(self, attr):
        if attr == 'fcn':
            raise AttributeError(attr)
        return getattr(self.fcn, attr)


def rbatchintegrand(f):
    try:
        f.fcntype = 'rbatch'
        return f
    except Exception:
        return RBatchIntegrand(f)


batchintegrand = lbatchintegrand
BatchIntegrand = LBatchIntegrand


class BuiltinIntegrand(object):
    """An integrand the fused kernel evaluates itself (no Python call)."""
    fcntype = 'lbatch'
    kind = None

    def params(self, dim):
        raise NotImplementedError

    def exact(self, dim):
        """Closed-form integral over the unit hypercube when known, else None."""
        return None


class Gaussian(BuiltinIntegrand):
    """``norm * exp(-a * sum_d (x_d - c)^2)`` (config 1 with a=100, c=0.5)."""
    kind = N.VG_F_GAUSS

    def __init__(self, a=100.0, c=0.5, norm=None, dim=4):
        self.a, self.c = float(a), float(c)
        self.norm = float((a / math.pi) ** (dim / 2.0)) if norm is None else float(norm)

    def params(self, dim):
        return [self.a, self.c, self.norm]

    def __call__(self, x):
        return self.norm * torch.exp(-self.a * ((x - self.c) ** 2).sum(dim=1))

    def exact(self, dim):
        s = 1.0 / math.sqrt(2 * self.a)
        one = 0.5 * (math.erf((1 - self.c) / (s * math.sqrt(2))) + math.erf(self.c / (s * math.sqrt(2))))
        return self.norm * (math.sqrt(math.pi / self.a)) ** dim * one ** dim


class Ridge(BuiltinIntegrand):
    """Mean of M normalised Gaussians of width s centred at c_j (1,...,1),
    c_j = (j + 1/2)/M (the vegas tutorial's ridge; config 2)."""
    kind = N.VG_F_RIDGE

    def __init__(self, M=1000, s=0.01):
        self.M, self.s = int(M), float(s)

    def params(self, dim):
        return [float(self.M), self.s]

    def __call__(self, x):
        dim = x.shape[1]
        c = (torch.arange(self.M, dtype=x.dtype, device=x.device) + 0.5) / self.M
        out = torch.zeros(x.shape[0], dtype=x.dtype, device=x.device)
        for j0 in range(0, self.M, 128):
            cj = c[j0:j0 + 128]
            r2 = ((x[:, None, :] - cj[None, :, None]) ** 2).sum(dim=2)
            out += torch.exp(-r2 / (2 * self.s ** 2)).sum(dim=1)
        return out * (2 * math.pi * self.s ** 2) ** (-0.5 * dim) / self.M

    def exact(self, dim):
        c = (np.arange(self.M) + 0.5) / self.M
        from scipy.special import ndtr
        one = ndtr((1 - c) / self.s) - ndtr(-c / self.s)
        return float(np.mean(one ** dim))


class LorentzianProduct(BuiltinIntegrand):
    """``prod_d (w_d/pi) / ((x_d - c_d)^2 + w_d^2)`` (config 3)."""
    kind = N.VG_F_LORENTZ

    def __init__(self, c, w):
        self.c = np.asarray(c, float)
        self.w = np.asarray(w, float)

    def params(self, dim):
        return list(self.c) + list(self.w)

    def __call__(self, x):
        c = torch.as_tensor(self.c, dtype=x.dtype, device=x.device)
        w = torch.as_tensor(self.w, dtype=x.dtype, device=x.device)
        return torch.prod((w / math.pi) / ((x - c) ** 2 + w ** 2), dim=1)

    def exact(self, dim):
        return float(np.prod((np.arctan((1 - self.c) / self.w) + np.arctan(self.c / self.w)) / np.pi))


class GaussianMixture(BuiltinIntegrand):
    """Equal-weight mixture of K normalised Gaussians N(x; c_k, sigma) (config 4)."""
    kind = N.VG_F_MIXTURE

    def __init__(self, centers, sigma=0.03):
        self.centers = np.asarray(centers, float)
        self.sigma = float(sigma)

    def params(self, dim):
        return [float(len(self.centers)), self.sigma] + list(self.centers.reshape(-1))

    def __call__(self, x):
        c = torch.as_tensor(self.centers, dtype=x.dtype, device=x.device)
        r2 = ((x[:, None, :] - c[None, :, :]) ** 2).sum(dim=2)
        dim = x.shape[1]
        norm = (2 * math.pi * self.sigma ** 2) ** (-0.5 * dim)
        return norm * torch.exp(-r2 / (2 * self.sigma ** 2)).mean(dim=1)

    def exact(self, dim):
        from scipy.special import ndtr
        c = self.centers
        one = ndtr((1 - c) / self.sigma) - ndtr(-c / self.sigma)
        return float(np.mean(np.prod(one, axis=1)))


class LatticeAction(BuiltinIntegrand):
    """``exp(-S)``, S = sum_i (x_{i+1}-x_i)^2/(2a) + a (x_i^2/2 + lam x_i^4),
    periodic (config 5: anharmonic oscillator path integral)."""
    kind = N.VG_F_LATTICE

    def __init__(self, a=0.5, lam=0.1):
        self.a, self.lam = float(a), float(lam)

    def params(self, dim):
        return [self.a, self.lam]

    def __call__(self, x):
        xn = torch.roll(x, -1, dims=1)
        S = ((xn - x) ** 2 / (2 * self.a) + self.a * (x ** 2 / 2 + self.lam * x ** 4)).sum(dim=1)
        return torch.exp(-S)

    def exact(self, dim, lo=-5.0, hi=5.0, nodes=400):
        """Integral over [lo, hi]^dim in FP64 by the transfer matrix: the
        periodic chain integrates to Tr(T^dim) with T(x, y) =
        exp(-(x-y)^2/(2a) - a (V(x) + V(y))/2), V = x^2/2 + lam x^4, here
        discretised by Gauss-Legendre quadrature (nodes points) and summed
        over the eigenvalues of the symmetric quadrature matrix."""
        t, wq = np.polynomial.legendre.leggauss(int(nodes))
        x = 0.5 * (hi - lo) * t + 0.5 * (hi + lo)
        wq = 0.5 * (hi - lo) * wq
        V = x ** 2 / 2 + self.lam * x ** 4
        T = np.exp(-(x[:, None] - x[None, :]) ** 2 / (2 * self.a) - self.a * (V[:, None] + V[None, :]) / 2)
        sw = np.sqrt(wq)
        ev = np.linalg.eigvalsh(sw[:, None] * T * sw[None, :])
        return float(np.sum(ev ** int(dim)))


class Constant(BuiltinIntegrand):
    kind = N.VG_F_CONST

    def __init__(self, value=1.0):
        self.value = float(value)

    def params(self, dim):
        return [self.value]

    def __call__(self, x):
        return torch.full((x.shape[0],), self.value, dtype=x.dtype, device=x.device)
