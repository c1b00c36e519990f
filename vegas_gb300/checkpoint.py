"""Checkpoints interchangeable with the reference vegas.

The reference pickles an ``AdaptiveMap`` as ``(AdaptiveMap, (grid,))`` with
``grid`` = ``extract_grid()`` (src/vegas/_vegas.pyx:150-167) and an
``Integrator`` as ``(Integrator, (map,), settings)`` where the settings are
its ``defaults`` (less the map) plus ``nstrat`` and ``sigf``
(_vegas.pyx:1194-1207), restored through ``set()`` (:1209-1211).  This
package pickles the same structures under its own class names, so a map or
integrator trained on the GPU and one trained by the reference on a CPU
carry the same state:

* ``dumps_reference(obj)`` writes a pickle of a ``vegas_gb300`` map or
  integrator that the reference's ``pickle.loads`` turns into
  ``vegas.AdaptiveMap`` / ``vegas.Integrator`` (the settings limited to the
  keys the reference knows);
* ``loads(data, device=None)`` / ``load(file, device=None)`` read a pickle
  written by either package into this package's classes, on ``device``.

``RAvg`` results are not converted: the reference stores their iterations
through ``gvar.dumps``, which needs the third-party ``gvar`` to read.
"""
import importlib
import io
import pickle
import sys
import types

import numpy as np

from .adaptive_map import AdaptiveMap
from .integrator import Integrator

REF_MODULE = 'vegas._vegas'
# the reference's Integrator.defaults, less 'map' (_vegas.pyx:1115-1140)
REF_SETTINGS = ('neval', 'maxinc_axis', 'min_neval_batch', 'max_neval_hcube', 'gpu_pad', 'neval_frac',
                'max_mem', 'nitn', 'alpha', 'beta', 'adapt', 'correlate_integrals', 'minimize_mem',
                'adapt_to_errors', 'uniform_nstrat', 'rtol', 'atol', 'analyzer', 'ran_array_generator',
                'sync_ran', 'mpi', 'uses_jac', 'nproc')


def _ref_classes():
    """The reference's AdaptiveMap and Integrator classes when the reference
    is importable, else placeholders registered under its module name while
    a pickle is written (pickle records classes by module and name only)."""
    try:
        mod = importlib.import_module(REF_MODULE)
        return mod.AdaptiveMap, mod.Integrator, None
    except ImportError:
        pass
    saved = {k: sys.modules.get(k) for k in ('vegas', REF_MODULE)}
    pkg = types.ModuleType('vegas')
    pkg.__path__ = []
    mod = types.ModuleType(REF_MODULE)
    for name in ('AdaptiveMap', 'Integrator'):
        cls = type(name, (object,), {'__module__': REF_MODULE})
        setattr(mod, name, cls)
    pkg._vegas = mod
    sys.modules['vegas'] = pkg
    sys.modules[REF_MODULE] = mod
    return mod.AdaptiveMap, mod.Integrator, saved


class _RefPickler(pickle.Pickler):
    def __init__(self, f, protocol, classes):
        super(_RefPickler, self).__init__(f, protocol)
        self.ref_map, self.ref_integ = classes

    def reducer_override(self, obj):
        if isinstance(obj, AdaptiveMap):
            grid = [[float(v) for v in row] for row in obj.extract_grid()]
            return (self.ref_map, (grid,))
        if isinstance(obj, Integrator):
            odict = {k: getattr(obj, k) for k in REF_SETTINGS}
            odict['nstrat'] = np.asarray(obj.nstrat)
            odict['sigf'] = np.asarray(obj.sigf, dtype=float)
            return (self.ref_integ, (obj.map,), odict)
        return NotImplemented


def dumps_reference(obj, protocol=pickle.HIGHEST_PROTOCOL):
    """Pickle ``obj`` (an AdaptiveMap or Integrator of this package, or a
    container of them) in the reference's class names."""
    ref_map, ref_integ, saved = _ref_classes()
    try:
        buf = io.BytesIO()
        _RefPickler(buf, protocol, (ref_map, ref_integ)).dump(obj)
        return buf.getvalue()
    finally:
        if saved is not None:
            for k, v in saved.items():
                if v is None:
                    sys.modules.pop(k, None)
                else:
                    sys.modules[k] = v


def dump_reference(obj, file, protocol=pickle.HIGHEST_PROTOCOL):
    data = dumps_reference(obj, protocol)
    if hasattr(file, 'write'):
        file.write(data)
    else:
        with open(file, 'wb') as f:
            f.write(data)


class _Unpickler(pickle.Unpickler):
    def __init__(self, f, device):
        super(_Unpickler, self).__init__(f)
        self.device = device

    def find_class(self, module, name):
        ours = module.startswith('vegas_gb300')
        if module == REF_MODULE or ours:
            dev = self.device
            if name == 'AdaptiveMap':
                return lambda grid, ninc=None: AdaptiveMap(grid, ninc=ninc, device=dev)
            if name == 'Integrator':
                return lambda map, **kargs: Integrator(map, device=dev, **kargs)
            if ours:
                return super(_Unpickler, self).find_class(module, name)
            raise pickle.UnpicklingError('reference class %s.%s has no counterpart here' % (module, name))
        return super(_Unpickler, self).find_class(module, name)


def loads(data, device=None):
    """Read a map or integrator pickled by the reference or by this package."""
    return _Unpickler(io.BytesIO(data), device).load()


def load(file, device=None):
    if hasattr(file, 'read'):
        return loads(file.read(), device)
    with open(file, 'rb') as f:
        return loads(f.read(), device)
