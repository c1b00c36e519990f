"""y-space restratification: ``restratify(integ, f)``.

Mirrors ``vegas.restratify`` / ``restratifyIntegrator``
(src/vegas/__init__.py:1313-1592).  vegas+ spreads its y-space strata evenly
over the directions; ``restratify`` measures, with the integrator's current
map, how much the integral of ``f`` varies along each direction of y and
moves the strata to the directions where it varies most:

1. integrate ``I`` = the integral of f together with ``dI[d][i]`` = the part
   of it from ``i/ndy <= y[d] <= (i+1)/ndy`` (both ends inclusive, as the
   reference bins), ``nitn`` iterations with the map frozen (``alpha=0``)
   and uncorrelated components;
2. weight[d] = ndy * sum_i (dI[d][i] - I/ndy)**2;
3. new nstrat[d] proportional to the weight (damped by ``gamma``), keeping
   the number of hypercubes about the same: directions are fixed in order of
   increasing target, each truncated to an integer >= 1 (or set to
   ``below_avg_nstrat`` when its weight is below the average), and the
   truncation error is spread over the directions still open;
4. ``nitn`` adaptive iterations of ``f`` with the new strata (results
   discarded), so the returned integrator is trained.

On the GPU: x arrives as a CUDA tensor; y comes from the map's inverse
(``vg_invmap``), the sums per direction and bin are the components of a
dictionary-valued integrand reduced by the array-reduction kernel.  When
``uses_jac`` is set the integrand receives dx/dy per direction (the
integrator's ``jac1d``), the meaning ``uses_jac`` has everywhere else; the
reference passes the product Jacobian from ``invmap`` at this one call.
PDFIntegrator is not part of this package, so ``f`` is required.
"""
import numpy as np
import torch

from . import _gvar as gv
from .integrands import BuiltinIntegrand
from .integrator import Integrator


class _IdIIntegrand(object):
    """Dictionary-valued lbatch integrand {'I': f(x), 'dI': f(x) per y bin}
    (src/vegas/__init__.py:1390-1419)."""

    fcntype = 'lbatch'

    def __init__(self, integ):
        self.integ = integ

    def __call__(self, x, jac=None):
        integ = self.integ
        n, dim = x.shape
        y = torch.empty_like(x)
        j = torch.empty(n, dtype=x.dtype, device=x.device)
        integ.map.invmap(x, y, j)
        fcn = integ.f
        if isinstance(fcn, BuiltinIntegrand):
            fx = torch.as_tensor(fcn(x), device=x.device)
        else:
            fx = integ._eval_batch(fcn, integ._classify(fcn), x, jac)
        fI = fx.reshape(n, -1)[:, 0].to(x.dtype)
        yst = torch.as_tensor(integ.yst, dtype=x.dtype, device=x.device)
        yb = y[:, :, None]
        inside = (yst[:-1] <= yb) & (yb <= yst[1:])            # [n, dim, ndy]
        dI = fI[:, None, None] * inside.to(x.dtype)
        return {'I': fI, 'dI': dI}


class restratifyIntegrator(Integrator):
    """Copy of ``integ`` with strata redistributed for ``f``
    (src/vegas/__init__.py:1314-1434).  Attributes ``I``, ``dI`` (GVar
    array [dim, ndy]), ``weight`` (GVar array [dim]), ``Q``, ``old_nstrat``."""

    def __init__(self, integ, f, nitn=1, ndy=5, below_avg_nstrat=None, verbose=False, gamma=1.,
                 **vargs):
        if f is None:
            raise ValueError('restratify needs the integrand f')
        super(restratifyIntegrator, self).__init__(integ)
        self.set(vargs)
        self.f = f
        self.ndy = int(ndy)
        self.yst = np.linspace(0, 1, self.ndy + 1)
        self.old_nstrat = np.array(self.nstrat)

        # I and dI with the map frozen
        save = self.set(correlate_integrals=False, nitn=nitn, alpha=0, adapt=True)
        result = self(_IdIIntegrand(self))
        self.set(save)
        self.I = result['I']
        self.dI = result['dI']
        self.Q = result.Q
        if verbose:
            print('\n==================== restratify')
            print('BEFORE:')
            print(result.summary()[:-1])
            print('nstrat =', np.array2string(self.old_nstrat, max_line_width=60, prefix=9 * ' '))
            print('nhcube =', np.prod(self.old_nstrat), '\n')

        # weights: variance of dI/dy[d] as a step function
        dim = len(self.old_nstrat)
        self.weight = np.zeros(dim, object)
        dIavg = self.I / self.ndy
        for mu in range(dim):
            self.weight[mu] = np.sum((self.dI[mu] - dIavg) ** 2) * self.ndy
        if verbose:
            print('WEIGHTS:')
            for mu in range(dim):
                print('  weight %-3d %s' % (mu, self.weight[mu]))
        self.set(nstrat=_new_nstrat(self.weight, self.old_nstrat, gamma, below_avg_nstrat,
                                    self.nstrat),
                 neval=self.neval)

        # train the new strata
        save = self.set(nitn=nitn, adapt=True)
        training = self(f)
        self.set(save)
        if verbose:
            print('\nAFTER:')
            print(training.summary()[:-1])
            print('nstrat =', np.array2string(np.asarray(self.nstrat), max_line_width=60,
                                              prefix=9 * ' '))
            print('nhcube =', np.prod(self.nstrat))
            print(20 * '=')


def _new_nstrat(weight, old_nstrat, gamma, below_avg_nstrat, like):
    """Strata per direction from the weights (src/vegas/__init__.py:1347-1363).

    Operations on the weights follow the order the reference applies them to
    its GVar objects (sequential sums and products), so the float results
    -- and the integer truncations that depend on them -- are the same."""
    dim = len(old_nstrat)
    w = [float(g) for g in weight]
    w_sum = w[0]
    w_prod = w[0]
    for v in w[1:]:
        w_sum = w_sum + v
        w_prod = w_prod * v
    w_avg = w_sum / dim
    w_gm = w_prod ** (1 / dim)
    nstrat_gm = np.prod(old_nstrat) ** (1 / dim)
    ratio = np.array([(w[mu] / w_gm) * nstrat_gm / old_nstrat[mu] for mu in range(dim)])
    nstrat = old_nstrat * ratio ** gamma
    nleft = dim
    musort = np.array(np.argsort(nstrat))
    new_nstrat = np.array(like)
    for mu in musort:
        new_nstrat[mu] = nstrat[mu] if nstrat[mu] > 1 else 1
        if below_avg_nstrat and w[mu] < w_avg:
            new_nstrat[mu] = below_avg_nstrat
        nleft -= 1
        if nleft > 0:
            nstrat[musort[-nleft:]] *= (nstrat[mu] / new_nstrat[mu]) ** (1 / nleft)
            nstrat[mu] = new_nstrat[mu]
    return new_nstrat


def restratify(integ, f=None, nitn=1, ndy=5, below_avg_nstrat=None, verbose=False, gamma=1.,
               **vargs):
    """Integrator with y-space strata optimised for ``f``
    (src/vegas/__init__.py:1457-1592).  ``integ`` should already be adapted
    to ``f``; typical use::

        integ = vegas_gb300.Integrator(20 * [[0, 1]])
        integ(f, neval=400_000, nitn=10)                        # train
        integ = vegas_gb300.restratify(integ, f, nitn=3)        # new strata
        result = integ(f, nitn=10)
    """
    return restratifyIntegrator(integ, f=f, nitn=nitn, ndy=ndy, below_avg_nstrat=below_avg_nstrat,
                                verbose=verbose, gamma=gamma, **vargs)
