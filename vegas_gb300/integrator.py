"""vegas+ Integrator on the GPU.

Python face of the reference's ``vegas.Integrator`` (src/vegas/_vegas.pyx:
834-2230): the same constructor, ``defaults``, ``set`` semantics, ``__call__``
(fcn, save, saveall, **kargs), ``random_batch``/``random``/``sample``,
``settings`` and pickling.  Everything numeric runs in libvegas_gb300.so:

* built-in integrands (vegas_gb300.integrands) run fused: one allocation and
  one persistent kernel per iteration, no host round trip except reading the
  80-byte iteration record;
* lbatch integrands receive CUDA tensors ``x[n, dim]`` (FP32 by default, FP64
  with ``precision='fp64'``) and return ``f[n]``; the reduction then runs on
  the device.  The points of an iteration are all in HBM already, so a batch
  holds as many as ``max_mem`` allows (at least ``min_neval_batch``, the
  reference's lower bound on a batch): normally the whole iteration in one
  call.

Extra settings beyond the reference's: ``precision`` ('fp32' | 'fp64'),
``seed`` (Philox key), ``device``.
"""
import ctypes
import math
import os
import pickle
import sys
import time

import numpy as np
import torch

from . import _native as N
from . import _gvar as gv
from .adaptive_map import AdaptiveMap, _device
from .integrands import BuiltinIntegrand
from .ravg import RAvg, RAvgArray, RAvgDict

HUGE = 10 ** (sys.float_info.max_10_exp - 50)  # _vegas.pyx:35

# attribute types of the reference's typed Integrator fields (_vegas.pxd:35-62)
_INT = ('neval', 'min_neval_batch', 'maxinc_axis', 'max_neval_hcube', 'nitn', 'nproc')
_FLOAT = ('neval_frac', 'max_mem', 'alpha', 'rtol', 'atol', 'beta')
_BOOL = ('gpu_pad', 'adapt', 'correlate_integrals', 'minimize_mem', 'adapt_to_errors',
         'sync_ran', 'mpi', 'uniform_nstrat', 'uses_jac')


class Integrator(object):
    r"""Adaptive multidimensional Monte Carlo integration (vegas+), on a GPU.

    ``Integrator(map, **kargs)`` where ``map`` is a list of ``[xl, xu]``
    limits, an :class:`AdaptiveMap` or another Integrator (whose map, sigf
    and strata are copied, pyx:1149-1162).
    """

    defaults = dict(
        map=None,
        neval=1000,
        maxinc_axis=1000,
        min_neval_batch=100000,
        max_neval_hcube=50000,
        gpu_pad=False,
        neval_frac=0.75,
        max_mem=1e9,
        nitn=10,
        alpha=0.5,
        beta=0.75,
        adapt=True,
        correlate_integrals=True,
        minimize_mem=False,
        adapt_to_errors=False,
        uniform_nstrat=False,
        rtol=0,
        atol=0,
        analyzer=None,
        ran_array_generator=None,
        sync_ran=True,
        mpi=False,
        uses_jac=False,
        nproc=1,
        precision='fp32',
        seed=None,
    )

    def __init__(self, map, **kargs):
        self.neval_hcube_range = None
        self.last_neval = 0
        self._itn = 0
        self._work = None
        self._stats = None
        self._sigf = None
        self.sum_sigf = HUGE
        self.nhcube = 1
        self.min_neval_hcube = 2
        self.device = _device(kargs.pop('device', None))
        for k, v in Integrator.defaults.items():
            if k != 'map':
                setattr(self, k, v)
        if isinstance(map, Integrator):
            self._set_map(map)
            args = {k: getattr(map, k) for k in Integrator.defaults if k != 'map'}
            self._sigf = map._sigf.clone() if map._sigf is not None else None
            self.sum_sigf = float(self._sigf.sum()) if self._sigf is not None else HUGE
            self.nstrat = np.array(map.nstrat)
            if 'nstrat' not in kargs:
                kargs['nstrat'] = map.nstrat
                if 'neval' not in kargs:
                    kargs['neval'] = map.neval
        else:
            args = {k: v for k, v in Integrator.defaults.items() if k != 'map'}
            self._set_map(map)
            self.nstrat = np.zeros(self.map.dim, np.int64)
        args.update(kargs)
        if 'nstrat' in kargs and 'neval' not in kargs and 'neval' in args:
            del args['neval']
        if 'neval' in kargs and 'nstrat' not in kargs and 'nstrat' in args:
            del args['nstrat']
        if args.get('seed') is None:
            args['seed'] = int.from_bytes(os.urandom(8), 'little') >> 1
        self.set(args)

    # ---------------------------------------------------------------- state
    def _set_map(self, map):
        if isinstance(map, AdaptiveMap):
            self.map = AdaptiveMap(map, device=self.device)
        elif isinstance(map, Integrator):
            self.map = AdaptiveMap(map.map, device=self.device)
        else:
            if hasattr(map, 'keys'):
                raise NotImplementedError('dictionary integration regions are not supported yet')
            lim = np.array(map, dtype=float)
            if lim.ndim < 2 or lim.shape[-1] != 2:
                raise ValueError('integration limits must be [[xl, xu], ...]')
            self.map = AdaptiveMap(lim.reshape(-1, 2), device=self.device)
        self.xsample = np.array([0.5 * (a + b) for a, b in self.map.region()])

    @property
    def dim(self):
        return self.map.dim

    @property
    def sigf(self):
        return np.zeros(0) if self._sigf is None else self._sigf.cpu().numpy()

    def __reduce__(self):
        odict = {k: getattr(self, k) for k in Integrator.defaults if k != 'map'}
        odict['nstrat'] = np.asarray(self.nstrat)
        odict['sigf'] = self.sigf
        return (Integrator, (self.map,), odict)

    def __setstate__(self, odict):
        self.set(odict)

    def set(self, ka={}, **kargs):
        """Reset parameters; returns the old values (pyx:1256-1446)."""
        if kargs:
            kargs.update(ka)
        else:
            kargs = dict(ka)
        old_val = dict()
        nstrat = None
        for k in kargs:
            if k == 'map':
                old_val['map'] = self.map
                self._set_map(kargs['map'])
            elif k == 'nstrat':
                if kargs['nstrat'] is None:
                    continue
                old_val['nstrat'] = self.nstrat
                nstrat = np.array(kargs['nstrat'], dtype=np.int64)
            elif k == 'sigf':
                old_val['sigf'] = self.sigf
                s = np.fabs(np.asarray(kargs['sigf'], float))
                self._sigf = torch.from_numpy(s.copy()).to(self.device)
                self.sum_sigf = float(np.sum(s))
            elif k in Integrator.defaults:
                old_val[k] = getattr(self, k, None)
                v = kargs[k]
                if k in _INT and v is not None:
                    v = int(v)
                elif k in _FLOAT and v is not None:
                    v = float(v)
                elif k in _BOOL and v is not None:
                    v = bool(v)
                setattr(self, k, v)
            elif k not in ['nhcube_batch', 'max_nhcube']:
                raise AttributeError('no parameter named "%s"' % str(k))
        if self.precision not in ('fp32', 'fp64'):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        # sanity checks (pyx:1319-1330)
        if nstrat is not None:
            if len(nstrat) != self.map.dim:
                raise ValueError('nstrat[d] has wrong length: %d not %d' % (len(nstrat), self.map.dim))
            if np.any(nstrat < 1):
                raise ValueError('bad nstrat: ' + str(nstrat))
        if self.neval_frac < 0 or self.neval_frac >= 1:
            raise ValueError('neval_frac = {} but require 0 <= neval_frac < 1'.format(self.neval_frac))
        if 'neval' in old_val and self.neval < 2:
            raise ValueError('neval>2 required, not ' + str(self.neval))
        dim = self.map.dim
        # strata and increments (pyx:1333-1407), host logic in the C ABI
        if nstrat is not None:
            mode = 1
        elif 'neval' in old_val or 'neval_frac' in old_val:
            mode = 0
        else:
            mode = 2
        nstrat_in = nstrat if nstrat is not None else np.asarray(self.nstrat, np.int64)
        sz = strata(dim, mode, self.neval, 'neval' in old_val, nstrat_in, self.neval_frac,
                    self.beta, self.adapt_to_errors, self.uniform_nstrat, self.max_mem,
                    self.minimize_mem, self.maxinc_axis)
        if mode == 1 and 'neval' not in old_val:
            old_val['neval'] = self.neval
        self.neval = sz['neval']
        nstrat = sz['nstrat']
        ninc = sz['ninc']
        mnh = sz['min_neval_hcube']
        if not np.array_equal(self.map.ninc, ninc):
            self.map.adapt(ninc=ninc)
        if not np.array_equal(np.asarray(self.nstrat), nstrat):
            if 'sigf' not in old_val:
                old_val['sigf'] = self.sigf
                self._sigf = None
                self.sum_sigf = HUGE
            self.nstrat = nstrat
        self.nhcube = int(np.prod(self.nstrat))
        self.min_neval_hcube = int(mnh)
        if self.beta >= 0 and self.nhcube > 1 and (self._sigf is None or
                                                   self._sigf.numel() != self.nhcube):
            self._sigf = torch.ones(self.nhcube, dtype=torch.float64, device=self.device)
            self.sum_sigf = float(self.nhcube)
        if self._sigf is None:
            self._sigf = torch.ones(max(self.nhcube, 1), dtype=torch.float64, device=self.device)
        workspace = self.min_neval_batch + self.max_neval_hcube
        if workspace > self.neval:
            workspace = self.neval + 1
        if (3 * dim + 3) * workspace + (0 if self.minimize_mem else self.nhcube) > self.max_mem:
            raise MemoryError('work arrays larger than max_mem; reduce min_neval_batch or '
                              'max_neval_hcube (or increase max_mem)')
        geometry = (tuple(int(v) for v in np.asarray(self.nstrat).reshape(-1)), self.nhcube,
                    tuple(int(v) for v in np.asarray(self.map.ninc).reshape(-1)), self.neval,
                    self.neval_frac, self.min_neval_hcube, self.max_neval_hcube, self.precision)
        if geometry != getattr(self, '_geometry', None):
            # a new workspace (zeroed: the allocation keeps its ticket and
            # epoch words there) for the new strata / capacity
            self._work = None
            self._geometry = geometry
        return old_val

    # ----------------------------------------------------- device plumbing
    def _struct(self):
        it = N.VgIntegrator()
        it.dim = self.dim
        it.precision = N.VG_F64 if self.precision == 'fp64' else N.VG_F32
        it.nhcube = self.nhcube
        for d in range(self.dim):
            it.nstrat[d] = int(self.nstrat[d])
            it.ninc[d] = int(self.map._ninc[d])
        g, inc = self.map.grid_tensor, self.map.inc_tensor
        it.grid = g.data_ptr()
        it.inc = inc.data_ptr()
        it.ldg = g.shape[1]
        it.ldi = inc.shape[1]
        it.sigf = self._sigf.data_ptr()
        it.neval = self.neval
        it.neval_frac = self.neval_frac
        it.min_neval_hcube = self.min_neval_hcube
        it.max_neval_hcube = self.max_neval_hcube
        it.alpha = self.alpha
        it.beta = self.beta
        it.adapt = int(self.adapt)
        it.adapt_to_errors = int(self.adapt_to_errors)
        it.seed = int(self.seed) & ((1 << 64) - 1)
        it.stream_id = getattr(self, '_stream_id', 0)   # Philox stream (0; batched integrals use their index)
        it.tile = 0
        L = N.load()
        ncap = L.vg_neval_cap(ctypes.byref(it))
        need = L.vg_workspace_bytes(ctypes.byref(it), 0)
        if self._work is None or self._work.numel() < need:
            self._work = torch.zeros(need, dtype=torch.uint8, device=self.device)
        if self._stats is None:
            self._stats = torch.zeros(ctypes.sizeof(N.VgStats), dtype=torch.uint8, device=self.device)
        if self.map.sum_f is None or self.map.sum_f.shape != inc.shape:
            self.map.sum_f = torch.zeros(inc.shape, dtype=torch.float64, device=self.device)
            self.map.n_f = torch.zeros(inc.shape, dtype=torch.int64, device=self.device)
        it.sum_f = self.map.sum_f.data_ptr()
        it.n_f = self.map.n_f.data_ptr()
        it.stats = self._stats.data_ptr()
        it.work = self._work.data_ptr()
        it.work_bytes = self._work.numel()
        return it, int(ncap)

    def _put_sum_sigf(self):
        """The device record reset with the carried sum_sigf (the rest is
        written by the iteration), enqueued on the current stream without a
        host wait."""
        N.check(N.load().vg_stats_reset(N.ptr(self._stats), float(self.sum_sigf), N.stream_ptr(self.device)))

    def _read_stats(self):
        b = self._stats.cpu().numpy().tobytes()
        return N.VgStats.from_buffer_copy(b)

    def _allocate(self, it):
        self._put_sum_sigf()
        L = N.load()
        N.check(L.vg_allocate(ctypes.byref(it), N.stream_ptr(self.device)))

    # ------------------------------------------------------------- sampling
    def _points(self, it, ncap, itn, u, want_y=False, want_hc=False, want_w=True, keep=None, bufs=None):
        """x (and y, weights, hypercubes) of the current allocation; with
        ``keep`` (a device buffer of vg_keep_bytes) the sampler also keeps
        each sample's Jacobian and training bins for vg_reduce_kept.  With
        ``bufs`` (a dict) the output tensors are kept there and reused by
        the next call of the same size."""
        L = N.load()
        dt = torch.float64 if self.precision == 'fp64' else torch.float32

        def out(name, shape, dtype):
            if bufs is None:
                return torch.empty(shape, dtype=dtype, device=self.device)
            t = bufs.get(name)
            if t is None or tuple(t.shape) != tuple(shape) or t.dtype != dtype:
                t = bufs[name] = torch.empty(shape, dtype=dtype, device=self.device)
            return t

        x = out('x', (ncap, self.dim), dt)
        y = out('y', (ncap, self.dim), dt) if want_y else None
        w = out('w', (ncap,), torch.float64) if want_w else None
        hc = out('hc', (ncap,), torch.int64) if want_hc else None
        if keep is None:
            N.check(L.vg_sample(ctypes.byref(it), itn, N.ptr(u), N.ptr(x), N.ptr(y), N.ptr(w),
                                N.ptr(hc), ncap, N.stream_ptr(self.device)))
        else:
            N.check(L.vg_sample_keep(ctypes.byref(it), itn, N.ptr(u), N.ptr(x), N.ptr(y), N.ptr(w),
                                     N.ptr(hc), ncap, N.ptr(keep), keep.numel(), N.stream_ptr(self.device)))
        return x, y, w, hc

    def _keep_buffer(self, it, ncap):
        """Device buffer for the kept Jacobians and training bins of one
        iteration's samples (reused across iterations)."""
        L = N.load()
        need = int(L.vg_keep_bytes(ctypes.byref(it), ncap))
        if getattr(self, '_keep', None) is None or self._keep.numel() < need:
            self._keep = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._keep

    def _draw_u(self, n):
        """Injected uniforms [n, dim] (FP64, device) from ran_array_generator,
        requested in the reference's batch sizes (pyx:1692-1732)."""
        gen = self.ran_array_generator
        parts = []
        nh = self._neval_h_host()
        csum = np.cumsum(nh)
        start, base = 0, 0
        H = len(nh)
        while start < H:
            # first hypercube where the batch reaches min_neval_batch
            target = base + self.min_neval_batch
            end = int(np.searchsorted(csum, target, side='left'))
            end = min(end, H - 1)
            nb = int(csum[end] - base)
            parts.append(np.asarray(gen((nb, self.dim)), dtype=np.float64).reshape(nb, self.dim))
            base = int(csum[end])
            start = end + 1
        u = np.concatenate(parts, axis=0)
        assert u.shape[0] == n
        return torch.from_numpy(np.ascontiguousarray(u)).to(self.device)

    def _neval_h_host(self):
        # neval_h lives at the start of the workspace (int32 per hypercube)
        return self._work[:4 * self.nhcube].view(torch.int32).cpu().numpy().astype(np.int64)

    def random_batch(self, yield_hcube=False, yield_y=False):
        """Batches of integration points and weights of one iteration
        (pyx:1601-1634): yields (x, [y,] wgt, [hcube]) as CUDA tensors."""
        it, ncap = self._struct()
        self._allocate(it)
        st = self._read_stats()
        n = int(st.neval)
        self.last_neval = n
        self.neval_hcube_range = np.array([st.range_lo, st.range_hi])
        u = self._draw_u(n) if self.ran_array_generator is not None else None
        self._itn += 1
        x, y, w, hc = self._points(it, ncap, self._itn & 0xffffffff, u, yield_y, yield_hcube)
        nb = max(1, int(self.min_neval_batch))
        for lo in range(0, n, nb):
            hi = min(n, lo + nb)
            ans = (x[lo:hi],)
            if yield_y:
                ans += (y[lo:hi],)
            ans += (w[lo:hi],)
            if yield_hcube:
                ans += (hc[lo:hi],)
            yield ans

    random_vec = random_batch

    def random(self, yield_hcube=False, yield_y=False):
        """Point-by-point version of random_batch (pyx:1770-1814)."""
        for b in self.random_batch(yield_hcube=yield_hcube, yield_y=yield_y):
            for i in range(b[0].shape[0]):
                yield tuple(t[i] for t in b)

    def sample(self, nbatch=None, mode='rbatch'):
        """Random sample (wgt, x) with sum(wgt*f(x)) estimating the integral (pyx:1816-1863)."""
        neval = self.last_neval if self.last_neval > 0 else self.neval
        nbatch = neval if nbatch is None else int(nbatch)
        nit = nbatch // neval
        if nit * neval < nbatch:
            nit += 1
        xs, ws = [], []
        for _ in range(nit):
            for x, w in self.random_batch():
                xs.append(x)
                ws.append(w)
        x = torch.cat(xs, dim=0)
        w = torch.cat(ws) / nit
        if mode == 'rbatch':
            x = x.t()
        return w, x

    # ------------------------------------------------------------ integrate
    def _classify(self, fcn):
        if isinstance(fcn, BuiltinIntegrand):
            return 'builtin'
        ft = getattr(fcn, 'fcntype', 'scalar')
        if ft == 'lbatch':
            return 'lbatch'
        if ft == 'rbatch':
            return 'rbatch'
        return 'scalar'

    def _eval_batch_size(self):
        """Points per integrand call: at least min_neval_batch (the
        reference's lower bound on a batch, pyx:1692-1710), as many as
        max_mem (floats) allows for x, jac and f."""
        per_point = 2 * self.dim + 2
        return max(1, int(self.min_neval_batch), int(self.max_mem // per_point))

    def _eval_batch(self, fcn, kind, x, jac=None, layout=None):
        """fcn on a batch; with uses_jac, jac[n, dim] = dx/dy per direction is
        passed as ``jac=`` (transposed for rbatch, per point for scalar
        integrands), as in the reference (pyx:2127, 3309-3316)."""
        n = x.shape[0]
        if kind == 'lbatch':
            f = fcn(x) if jac is None else fcn(x, jac=jac)
            if layout is not None:
                return self._flatten_dict(f, kind, n, layout)
        elif kind == 'rbatch':
            f = fcn(x.t()) if jac is None else fcn(x.t(), jac=jac.t())
            if layout is not None:
                return self._flatten_dict(f, kind, n, layout)
        else:
            xc = x.cpu().numpy()
            if jac is None:
                f = [fcn(xi) for xi in xc]
            else:
                jc = jac.cpu().numpy()
                f = [fcn(xi, jac=ji) for xi, ji in zip(xc, jc)]
            if layout is not None:
                f = [np.concatenate([np.asarray(fi[k], dtype=float).reshape(-1) for k, _ in layout])
                     for fi in f]
            f = np.array([np.asarray(fi, dtype=float).reshape(-1) for fi in f], dtype=float)
            if f.ndim == 2 and f.shape[1] == 1:
                f = f[:, 0]
        if kind == 'rbatch' and not isinstance(f, torch.Tensor):
            f = torch.as_tensor(np.asarray(f, dtype=float), device=self.device)
        if kind == 'rbatch':
            f = f.to(self.device)
            if f.dim() > 1:   # rbatch returns [..., n]: batch index last
                f = f.reshape(-1, x.shape[0]).t()
        if not isinstance(f, torch.Tensor):
            f = torch.as_tensor(np.asarray(f, dtype=float), device=self.device)
        f = f.to(self.device)
        if f.dim() > 1:
            f = f.reshape(f.shape[0], -1)   # [n, s], s = size of one integrand value
        return f

    def _fshape(self, fcn, kind, x1, j1=None):
        """Shape of one integrand value, from an evaluation at one point (the
        reference takes it from a sample evaluation, pyx:3068-3082): a tuple
        for arrays, a list of (key, shape) for dictionary-valued integrands."""
        if kind == 'lbatch':
            out = fcn(x1) if j1 is None else fcn(x1, jac=j1)
            if hasattr(out, 'keys'):
                return [(k, tuple(torch.as_tensor(out[k]).shape)[1:]) for k in out]
            return tuple(torch.as_tensor(out).shape)[1:]
        if kind == 'rbatch':
            out = fcn(x1.t()) if j1 is None else fcn(x1.t(), jac=j1.t())
            if hasattr(out, 'keys'):
                return [(k, tuple(torch.as_tensor(out[k]).shape)[:-1]) for k in out]
            return tuple(torch.as_tensor(out).shape)[:-1]
        xc = x1[0].cpu().numpy()
        out = fcn(xc) if j1 is None else fcn(xc, jac=j1[0].cpu().numpy())
        if hasattr(out, 'keys'):
            return [(k, tuple(np.shape(out[k]))) for k in out]
        return tuple(np.shape(out))

    def _flatten_dict(self, out, kind, n, layout):
        """[n, s] tensor of a dictionary-valued batch in the layout's key order."""
        parts = []
        for k, _ in layout:
            v = torch.as_tensor(out[k], device=self.device)
            if kind == 'rbatch':
                v = v.reshape(-1, n).t()
            parts.append(v.reshape(n, -1).to(torch.float64))
        return torch.cat(parts, dim=1)

    def _reduce_array(self, it, f, fdt, w):
        """Mean and (co)variance of every component of an array integrand."""
        L = N.load()
        s = int(f.shape[1])
        corr = 1 if self.correlate_integrals else 0
        need = int(L.vg_reduce_array_work_bytes(s, corr))
        work = torch.empty(need, dtype=torch.uint8, device=self.device)
        mean = torch.empty(s, dtype=torch.float64, device=self.device)
        var = torch.empty((s, s), dtype=torch.float64, device=self.device)
        N.check(L.vg_reduce_array(ctypes.byref(it), N.ptr(f), fdt, s, corr, N.ptr(w), N.ptr(mean),
                                  N.ptr(var), N.ptr(work), need, N.stream_ptr(self.device)))
        return mean.cpu().numpy(), var.cpu().numpy()

    def __call__(self, fcn, save=None, saveall=None, **kargs):
        """Integrate ``fcn``; returns an :class:`RAvg` (pyx:1912-2230)."""
        if kargs:
            self.set(kargs)
        if isinstance(fcn, type):
            raise ValueError('integrand given is a class, not an object -- need to initialize?')
        kind = self._classify(fcn)
        result = RAvg(weighted=self.adapt)
        if kind == 'builtin' and self.ran_array_generator is None and not self.uses_jac:
            if self.analyzer is None and save is None and saveall is None:
                if self.rtol == 0 and self.atol == 0:
                    return self._call_pipelined(fcn, result)
                return self._call_speculative(fcn, result)
            return self._call_stepwise(fcn, result, save, saveall)
        L = N.load()
        stream = N.stream_ptr(self.device)
        dt = torch.float64 if self.precision == 'fp64' else torch.float32
        fshape = None
        for itn in range(self.nitn):
            arr = None
            if self.analyzer is not None:
                self.analyzer.begin(itn, self)
            it, ncap = self._struct()
            self._allocate(it)
            self._itn += 1
            itn_word = self._itn & 0xffffffff
            u = None
            if kind == 'builtin' and self.uses_jac:
                raise ValueError('uses_jac=True needs an integrand that accepts jac=')
            if kind == 'builtin' and self.ran_array_generator is None:
                p = fcn.params(self.dim)
                N.check(L.vg_fused_iteration(ctypes.byref(it), itn_word, None, int(fcn.kind),
                                             N.dbl_array(p), len(p), stream))
            else:
                st = self._read_stats()
                n = int(st.neval)
                if self.ran_array_generator is not None:
                    u = self._draw_u(n)
                if kind == 'builtin':
                    p = fcn.params(self.dim)
                    N.check(L.vg_fused_iteration(ctypes.byref(it), itn_word, N.ptr(u),
                                                 int(fcn.kind), N.dbl_array(p), len(p), stream))
                else:
                    # the sampler keeps each sample's Jacobian and training
                    # bins, so the reduction streams them instead of
                    # regenerating the samples; the weights are written only
                    # while an array-valued integrand may need them
                    keep = self._keep_buffer(it, ncap)
                    want_w = fshape is None or bool(fshape)
                    x, yv, w, _ = self._points(it, ncap, itn_word, u, want_y=self.uses_jac, want_w=want_w,
                                               keep=keep)
                    jac = self.map.jac1d(yv[:n]) if self.uses_jac else None
                    f = None
                    nb = self._eval_batch_size()
                    for lo in range(0, n, nb):
                        hi = min(n, lo + nb)
                        if fshape is None:
                            fshape = self._fshape(fcn, kind, x[:1],
                                                  None if jac is None else jac[:1])
                        layout = fshape if isinstance(fshape, list) else None
                        fb = self._eval_batch(fcn, kind, x[lo:hi],
                                              None if jac is None else jac[lo:hi], layout)
                        if fb.shape[0] != hi - lo:
                            raise ValueError('integrand returned %d values for %d points'
                                             % (fb.shape[0], hi - lo))
                        if f is None:
                            if layout is not None:
                                s_f = int(sum(int(np.prod(sh)) if sh else 1 for _, sh in layout))
                            else:
                                s_f = int(np.prod(fshape)) if fshape else 1
                            f = torch.empty((ncap, s_f) if fshape else ncap, dtype=dt,
                                            device=self.device)
                        f[lo:hi] = fb.reshape(hi - lo).to(dt) if f.dim() == 1 \
                            else fb.reshape(hi - lo, -1).to(dt)
                    if bool(torch.isnan(f[:n]).any()):
                        raise ValueError('integrand evaluates to nan')
                    fdt = N.VG_F64 if dt == torch.float64 else N.VG_F32
                    f0 = f if f.dim() == 1 else f[:, 0].contiguous()
                    N.check(L.vg_reduce_kept(ctypes.byref(it), itn_word, N.ptr(u), N.ptr(f0), fdt, N.ptr(keep),
                                             keep.numel(), stream))
                    if f.dim() > 1:
                        arr = self._reduce_array(it, f, fdt, w)
            # adapt the map on the device before reading the iteration record
            N.check(L.vg_end_iteration(ctypes.byref(it), stream))
            st = self._read_stats()
            self._take_record(st)
            if arr is not None:
                # array- or dictionary-valued integrand: RAvgArray of the
                # integrand's shape / RAvgDict of its keys
                # (VegasIntegrand.format_result, pyx:3127-3147)
                mean_a, var_a = arr
                if self.correlate_integrals:
                    g = gv.gvar(mean_a, var_a)
                else:
                    g = gv.gvar(mean_a, np.sqrt(np.clip(np.diag(var_a), 0.0, None)))
                if isinstance(fshape, list):
                    if not isinstance(result, RAvgDict):
                        result = RAvgDict(fshape, weighted=self.adapt)
                    result.add(np.asarray(g, dtype=object).reshape(-1))
                else:
                    if not isinstance(result, RAvgArray):
                        result = RAvgArray(fshape, weighted=self.adapt)
                    result.add(np.asarray(g, dtype=object).reshape(fshape))
            else:
                result.add(gv.gvar(st.mean, st.var ** 0.5))
            result.sum_neval += self.last_neval
            if self.analyzer is not None:
                self.analyzer.end(result.itn_results[-1], result)
            if save is not None:
                _save(save, result)
            if saveall is not None:
                _save(saveall, (result, self))
            if result.converged(self.rtol, self.atol):
                break
        return result

    def _take_record(self, st):
        """Checks of one iteration's device record; the integrator's copies
        of its neval, neval range and sum_sigf."""
        if st.status == N.VG_ERR_MEMORY:
            raise MemoryError('iteration exceeded its evaluation capacity')
        elif st.status == N.VG_ERR_TIMEOUT:
            raise N.VegasTimeout('a bounded device-side wait gave up (allocation look-back); '
                                 'the iteration scheduled no work')
        elif st.status != 0:
            raise N.VegasError('device status %d' % st.status)
        if st.nan_seen:
            raise ValueError('integrand evaluates to nan')
        self.last_neval = int(st.neval)
        self.neval_hcube_range = np.array([st.range_lo, st.range_hi])
        if self.beta > 0 and self.adapt and self.nhcube > 1:
            self.sum_sigf = float(st.sum_sigf)

    def _records_host(self, n):
        sz = ctypes.sizeof(N.VgStats)
        buf = getattr(self, '_rec_host', None)
        if buf is None or buf.shape[0] < n:
            buf = torch.empty((max(n, 16), sz), dtype=torch.uint8, pin_memory=True)
            self._rec_host = buf
        return buf

    def _call_pipelined(self, fcn, result):
        """__call__ for a built-in integrand when no iteration needs a host
        decision (no rtol/atol stop, analyzer or save): every iteration --
        allocation, fused evaluate+reduce, adapt, one ``vg_iterate`` call
        that overlaps the adapt with the iteration sums -- is enqueued without
        waiting, and each iteration's record is copied to pinned host memory
        on the same stream; the records are read once after the last
        iteration.  Same kernels and results as the iteration-by-iteration
        loop, without a host round trip per iteration."""
        L = N.load()
        stream = N.stream_ptr(self.device)
        it, ncap = self._struct()
        self._put_sum_sigf()
        p = fcn.params(self.dim)
        params = N.dbl_array(p)
        nitn = int(self.nitn)
        host = self._records_host(nitn)
        for k in range(nitn):
            self._itn += 1
            N.check(L.vg_iterate(ctypes.byref(it), self._itn & 0xffffffff, int(fcn.kind), params, len(p),
                                 stream))
            host[k].copy_(self._stats, non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        raw = host[:nitn].numpy().tobytes()
        sz = ctypes.sizeof(N.VgStats)
        gs = []
        for k in range(nitn):
            st = N.VgStats.from_buffer_copy(raw, k * sz)
            self._take_record(st)
            gs.append(gv.gvar(st.mean, st.var ** 0.5))
            result.sum_neval += self.last_neval
        result.add_many(gs)
        return result

    def _call_stepwise(self, fcn, result, save, saveall):
        """__call__ for a built-in integrand when iterations need a host
        decision (rtol/atol stop, analyzer, save): one ``vg_iterate`` call
        per iteration (the kernels of the pipelined path), its record copied
        to pinned host memory and waited for on an event; sum_sigf stays on
        the device between iterations.  The analyzer, save and stopping rule
        run after each iteration as in the reference (pyx:2086-2226)."""
        L = N.load()
        stream = N.stream_ptr(self.device)
        it, ncap = self._struct()
        self._put_sum_sigf()
        p = fcn.params(self.dim)
        params = N.dbl_array(p)
        host = self._records_host(1)
        sz = ctypes.sizeof(N.VgStats)
        done = torch.cuda.Event()
        for itn in range(int(self.nitn)):
            if self.analyzer is not None:
                self.analyzer.begin(itn, self)
            self._itn += 1
            N.check(L.vg_iterate(ctypes.byref(it), self._itn & 0xffffffff, int(fcn.kind), params, len(p),
                                 stream))
            host[0].copy_(self._stats, non_blocking=True)
            done.record(torch.cuda.current_stream(self.device))
            done.synchronize()
            st = N.VgStats.from_buffer_copy(host[0].numpy().tobytes()[:sz])
            self._take_record(st)
            result.add(gv.gvar(st.mean, st.var ** 0.5))
            result.sum_neval += self.last_neval
            if self.analyzer is not None:
                self.analyzer.end(result.itn_results[-1], result)
            if save is not None:
                _save(save, result)
            if saveall is not None:
                _save(saveall, (result, self))
            if result.converged(self.rtol, self.atol):
                break
        return result

    def _call_speculative(self, fcn, result):
        """__call__ for a built-in integrand with an rtol/atol stop and no
        other host hook: iteration k + 1 is enqueued before iteration k's
        record is read, so the GPU never waits for the host.  After each
        iteration the map and sigf are copied to one of two backup slots on
        the device; when the stopping rule (pyx:2226) or an error ends the
        loop at iteration k, the iteration already enqueued after it is
        undone from slot k -- the integrator is left exactly as the
        iteration-by-iteration loop leaves it, and the next call draws the
        same random numbers."""
        L = N.load()
        stream = N.stream_ptr(self.device)
        cur = torch.cuda.current_stream(self.device)
        it, ncap = self._struct()
        self._put_sum_sigf()
        p = fcn.params(self.dim)
        params = N.dbl_array(p)
        nitn = int(self.nitn)
        grid, inc, sigf = self.map.grid_tensor, self.map.inc_tensor, self._sigf
        bk = [(torch.empty_like(grid), torch.empty_like(inc), torch.empty_like(sigf)) for _ in range(2)]
        host = self._records_host(2)
        sz = ctypes.sizeof(N.VgStats)
        done = [torch.cuda.Event(), torch.cuda.Event()]
        itn0 = self._itn

        def enqueue(k):
            N.check(L.vg_iterate(ctypes.byref(it), (itn0 + k + 1) & 0xffffffff, int(fcn.kind), params, len(p),
                                 stream))
            host[k % 2].copy_(self._stats, non_blocking=True)
            done[k % 2].record(cur)
            g, i, s_ = bk[k % 2]
            g.copy_(grid, non_blocking=True)
            i.copy_(inc, non_blocking=True)
            s_.copy_(sigf, non_blocking=True)

        def undo(k):   # back to the state after iteration k
            g, i, s_ = bk[k % 2]
            grid.copy_(g, non_blocking=True)
            inc.copy_(i, non_blocking=True)
            sigf.copy_(s_, non_blocking=True)
            cur.synchronize()

        enqueue(0)
        for k in range(nitn):
            ahead = k + 1 < nitn
            if ahead:
                enqueue(k + 1)
            done[k % 2].synchronize()
            st = N.VgStats.from_buffer_copy(host[k % 2].numpy().tobytes()[:sz])
            self._itn = itn0 + k + 1
            try:
                self._take_record(st)
            except Exception:
                if ahead:
                    undo(k)
                raise
            result.add(gv.gvar(st.mean, st.var ** 0.5))
            result.sum_neval += self.last_neval
            if result.converged(self.rtol, self.atol):
                if ahead:
                    undo(k)
                break
        return result

    # --------------------------------------------------------------- report
    def settings(self, ngrid=0):
        """Text summary of the settings (pyx:1448-1590)."""
        nhcube = int(np.prod(self.nstrat))
        neval = nhcube * self.min_neval_hcube if self.beta <= 0 else self.neval
        ans = 'Integrator Settings:\n'
        if self.beta > 0 and not self.adapt_to_errors:
            ans += '    %.6g (approx) integrand evaluations in each of %d iterations\n' % (
                self.neval, self.nitn)
        else:
            ans += '    %.6g integrand evaluations in each of %d iterations\n' % (neval, self.nitn)
        ans += '    number of: strata/axis = %s\n' % np.array2string(
            np.asarray(self.nstrat), max_line_width=80, prefix=29 * ' ')
        ans += '               increments/axis = %s\n' % np.array2string(
            np.asarray(self.map.ninc), max_line_width=80, prefix=33 * ' ')
        ans += '               h-cubes = %.6g  processors = %d\n' % (nhcube, self.nproc)
        max_neval_hcube = max(self.max_neval_hcube, self.min_neval_hcube)
        ans += '               evaluations/batch >= %.2g\n' % (float(self.min_neval_batch),)
        ans += '               %d <= evaluations/h-cube <= %.2g\n' % (
            int(self.min_neval_hcube), float(max_neval_hcube))
        ans += '    minimize_mem = %s  adapt_to_errors = %s  adapt = %s\n' % (
            str(self.minimize_mem), str(self.adapt_to_errors), str(self.adapt))
        ans += '    accuracy: relative = %g  absolute = %g\n' % (self.rtol, self.atol)
        if not self.adapt:
            ans += '    damping: alpha = %g  beta= %g\n\n' % (0., 0.)
        else:
            ans += '    damping: alpha = %g  beta= %g\n\n' % (self.alpha, self.beta)
        limits = ['({:.5}, {:.5})'.format(*l) for l in self.map.region()]
        entries = [(str(a), lim) for a, lim in enumerate(limits)]
        w1 = max(len('axis'), max(len(e[0]) for e in entries))
        w2 = max(len('integration limits'), max(len(e[1]) for e in entries))
        lines = ['{:>{w1}}    {:>{w2}}'.format('axis', 'integration limits', w1=w1, w2=w2)]
        lines.append(len(lines[0]) * '-')
        for a, lim in entries:
            lines.append('{:>{w1}}    {:>{w2}}'.format(a, lim, w1=w1, w2=w2))
        ans += '    ' + '\n    '.join(lines) + '\n'
        if ngrid > 0:
            ans += '\n' + self.map.settings(ngrid=ngrid)
        return ans


def strata(dim, mode, neval, neval_given, nstrat, neval_frac=0.75, beta=0.75,
           adapt_to_errors=False, uniform_nstrat=False, max_mem=1e9, minimize_mem=False,
           maxinc_axis=1000):
    """Strata, increments and min_neval_hcube of Integrator.set (pyx:1333-1407).

    mode 0: from neval; 1: explicit nstrat; 2: keep nstrat.  Host logic in
    the C ABI (vg_set_strata), which reproduces the reference's complex-power
    rounding of the strata count."""
    neval = ctypes.c_int64(int(neval))
    ns_out = (ctypes.c_int64 * dim)()
    ninc_out = (ctypes.c_int64 * dim)()
    mnh = ctypes.c_int64(0)
    nstrat_in = N.i64_array(nstrat if nstrat is not None else np.zeros(dim, np.int64))
    L = N.load()
    N.check(L.vg_set_strata(dim, mode, ctypes.byref(neval), 1 if neval_given else 0, nstrat_in,
                            float(neval_frac), float(beta), int(adapt_to_errors),
                            int(uniform_nstrat), float(max_mem), int(minimize_mem),
                            int(maxinc_axis), ns_out, ninc_out, ctypes.byref(mnh)))
    return dict(neval=int(neval.value), nstrat=np.array(list(ns_out), np.int64),
                ninc=np.array(list(ninc_out), np.int64), min_neval_hcube=int(mnh.value))


def _save(dest, obj):
    if isinstance(dest, str):
        with open(dest, 'wb') as f:
            pickle.dump(obj, f)
    else:
        pickle.dump(obj, dest)


class reporter(object):
    """Analyzer printing a report after each iteration (pyx:2232-2269)."""

    def __init__(self, ngrid=0):
        self.ngrid = ngrid
        self.clock = time.perf_counter

    def begin(self, itn, integrator):
        self.integrator = integrator
        self.itn = itn
        self.t0 = self.clock()
        if itn == 0:
            print(integrator.settings())
        sys.stdout.flush()

    def end(self, itn_ans, ans):
        print("    itn %2d: %s\n all itn's: %s" % (self.itn + 1, itn_ans, ans))
        print('    neval = %s  neval/h-cube = %s\n    chi2/dof = %.2f  Q = %.2f  time = %.2f' % (
            format(self.integrator.last_neval, '.6g'), tuple(self.integrator.neval_hcube_range),
            ans.chi2 / ans.dof if ans.dof > 0 else 0, ans.Q if ans.dof > 0 else 1.,
            self.clock() - self.t0))
        print(self.integrator.map.settings(ngrid=self.ngrid))
        print('')
        sys.stdout.flush()
