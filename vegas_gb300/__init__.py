"""vegas_gb300 -- vegas+ adaptive Monte Carlo integration on NVIDIA GB300.

Drop-in for the hot path of gplepage/vegas (``vegas.Integrator``,
``AdaptiveMap``, ``RAvg``/``RAvgArray``, ``lbatchintegrand``) with the
numerics in hand-written sm_103a CUDA behind a C ABI
(include/vegas_gb300.h, libvegas_gb300.so).
"""
from .adaptive_map import AdaptiveMap
from .integrands import (BatchIntegrand, Constant, Gaussian, GaussianMixture, LatticeAction,
                         LBatchIntegrand, LorentzianProduct, RBatchIntegrand, Ridge,
                         batchintegrand, lbatchintegrand, rbatchintegrand)
from .integrator import Integrator, reporter, strata
from .ravg import RAvg, RAvgArray, RAvgDict
from .restratify import restratify, restratifyIntegrator
from ._gvar import GVar, gvar
from . import checkpoint

__version__ = '0.1.0'

__all__ = ['AdaptiveMap', 'Integrator', 'RAvg', 'RAvgArray', 'RAvgDict', 'reporter', 'lbatchintegrand',
           'batchintegrand', 'rbatchintegrand', 'LBatchIntegrand', 'BatchIntegrand',
           'RBatchIntegrand', 'Gaussian', 'Ridge', 'LorentzianProduct', 'GaussianMixture',
           'LatticeAction', 'Constant', 'GVar', 'gvar', 'strata', 'restratify',
           'restratifyIntegrator']
