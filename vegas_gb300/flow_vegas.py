"""vegas+ with a learned proposal: a coupling-layer normalising flow composed
with the adapted AdaptiveMap (no counterpart in the reference).

Plain phase: ordinary vegas+ (``Integrator``) adapts its map and strata.
Flow phase: the adapted map is frozen and the flow is inserted between the
stratified sampler and the map, acting on vegas's y-space:

    y (stratified, Philox) --flow--> y' in [0,1]^d --frozen AdaptiveMap--> x

The integrand seen on the stratified y-space is

    f_eff(y) = f(x) * J_map(y') * |dy'/dy| = f(x) * J_map(y') * exp(-logdet(y')),

and vegas+'s stratification (allocation by sigf, per-hypercube variances)
runs on f_eff with the identity map.  Every sample carries the flow's exact
log-determinant, so each iteration's estimate stays unbiased whatever the
flow's parameters.

Training.  With q the density of y' when y is uniform and g = f J_map, the
estimator's variance is V = int g^2/q dy' - I^2, and
    grad V = -E_p[(g^2 / (q p)) grad log q],
p the stratified sampling density of y' (p = q * s(y), s proportional to the
evaluations n_h of the sample's hypercube).  Per sample the weight is
f_eff^2 / n_h on the loss -sum_i w_i logdet(y'_i) (chi^2 / variance loss).
Because the map is frozen and sits after the flow, log q depends on the
flow's parameters only through logdet: the gradient is exact.  The first
``kl_itn`` flow iterations use the KL weights |f_eff| / n_h instead, which
are far less heavy-tailed while the flow is still far from the target.

Gate.  Plain vegas+ is both the fallback and the judge: its variance per
evaluation (iteration variance x evaluations) over the plain phase is the
bar.  After ``grace`` flow iterations, a flow iteration that does not beat
it counts as a loss; after ``patience`` losses in a row the flow is switched
off for good and iterations continue with plain vegas+, whose map and strata
were left untouched by the flow phase.
"""
import ctypes
import math
import time

import numpy as np
import torch

from . import _native as N
from . import _gvar as gv
from .adaptive_map import AdaptiveMap
from .flow import Flow
from .integrands import BuiltinIntegrand
from .integrator import Integrator
from .ravg import RAvg


class FlowIntegrator(object):
    """vegas+ over ``limits`` with a coupling-layer flow in its y-space.

    Args:
        limits: ``[[xl, xu], ...]`` integration box.
        nlayers, K: flow coupling layers and spline bins (hidden width 128).
        train_batch: samples per Adam step (drawn from the iteration's samples).
        train_steps: Adam steps per iteration.
        lr: Adam learning rate.
        plain_itn: iterations of plain vegas+ before the flow starts.
        kl_itn: first flow iterations trained with KL weights (then chi^2).
        train_itn: flow iterations that train the flow; later ones only
            sample with it (None: train on every flow iteration).
        grace: first flow iterations that are not judged.
        patience: judged flow iterations that may lose in a row.
        gate: 'eval' (variance per evaluation) or 'time' (variance x seconds
            per evaluation).
        **kargs: vegas settings of the underlying Integrator (neval, nitn,
            alpha, beta, seed, ...).
    """

    def __init__(self, limits, nlayers=6, K=32, train_batch=1 << 15, train_steps=4, lr=1e-3,
                 plain_itn=10, kl_itn=10, train_itn=None, grace=10, patience=3, gate='eval',
                 flow_seed=0, device=None, **kargs):
        kargs.setdefault('precision', 'fp32')
        if kargs['precision'] != 'fp32':
            raise ValueError('the flow path computes in FP32 (precision="fp32")')
        self.vegas = Integrator(limits, device=device, **kargs)
        self.device = self.vegas.device
        self.dim = self.vegas.dim
        self.flow = Flow(self.dim, nlayers=nlayers, K=K, seed=flow_seed, device=self.device, lr=lr)
        self.train_batch = int(train_batch)
        self.train_steps = int(train_steps)
        self.plain_itn = int(plain_itn)
        self.kl_itn = int(kl_itn)
        self.train_itn = None if train_itn is None else int(train_itn)
        self.grace = int(grace)
        self.patience = int(patience)
        if gate not in ('eval', 'time'):
            raise ValueError("gate must be 'eval' or 'time'")
        self.gate = gate
        self.flow_on = False
        self.flow_dead = False
        self.plain_scores = []
        self.losing = 0
        self.strat = None            # stratification integrator on [0,1]^d (flow phase)
        self._bufs = {}              # per-iteration device buffers, reused
        self.map = None              # frozen AdaptiveMap (flow phase)
        self._nit = 0
        self._flow_nit = 0
        self.history = []            # per iteration: dict(flow, mean, sdev, neval, score, seconds)
        self._tseed = (int(self.vegas.seed) * 0x9E3779B97F4A7C15 + 0x632BE5AB) & ((1 << 64) - 1)
        self._tstep = 0
        self._zs = self._ws = self._scr = None

    @property
    def plain_score(self):
        return min(self.plain_scores) if self.plain_scores else None

    # ---------------------------------------------------------- flow phase
    def _start_flow(self):
        v = self.vegas
        self.map = AdaptiveMap(v.map, device=self.device)
        keep = ('neval', 'beta', 'neval_frac', 'min_neval_batch', 'max_neval_hcube', 'maxinc_axis',
                'max_mem')
        args = {k: getattr(v, k) for k in keep}
        s = Integrator([[0.0, 1.0]] * self.dim, device=self.device, alpha=0.0, adapt=True,
                       precision='fp32', seed=(int(v.seed) * 2654435761 + 1) & ((1 << 63) - 1),
                       **args)
        if not np.array_equal(np.asarray(s.nstrat), np.asarray(v.nstrat)):
            s.set(nstrat=np.asarray(v.nstrat))
        if s._sigf.numel() == v._sigf.numel():
            s._sigf.copy_(v._sigf)       # the flow starts as the identity: the strata carry over
            s.sum_sigf = v.sum_sigf
        self.strat = s
        self.flow_on = True
        self.losing = 0

    def _feff(self, fcn, x, jac, ld, out):
        """out[:n] = f(x) * jac * exp(-ld) (FP32); x in the integration box."""
        n = x.shape[0]
        L = N.load()
        stream = N.stream_ptr(self.device)
        if isinstance(fcn, BuiltinIntegrand):
            p = fcn.params(self.dim)
            N.check(L.vg_eval_points(int(fcn.kind), N.dbl_array(p), len(p), self.dim, n, N.ptr(x),
                                     N.dbl_array([0.0] * self.dim), N.dbl_array([1.0] * self.dim),
                                     N.ptr(ld), N.ptr(jac), N.ptr(out), stream))
            return
        ft = getattr(fcn, 'fcntype', 'scalar')
        if ft == 'rbatch':
            f = fcn(x.t())
        elif ft == 'lbatch':
            f = fcn(x)
        else:
            raise ValueError('the flow path needs a batch integrand (lbatchintegrand / rbatchintegrand)')
        f = torch.as_tensor(f, device=self.device).reshape(n)
        if f.dtype != torch.float32:
            f = f.to(torch.float32)
        f = f.contiguous()
        N.check(L.vg_weight_points(n, N.ptr(f), N.ptr(jac), N.ptr(ld), N.ptr(out), stream))

    def _buf(self, name, *shape):
        """A float32 device tensor of the given shape, kept for reuse."""
        t = self._bufs.get(name)
        if t is None or tuple(t.shape) != shape:
            t = self._bufs[name] = torch.empty(shape, dtype=torch.float32, device=self.device)
        return t

    def _flow_iteration(self, fcn, train):
        s = self.strat
        L = N.load()
        stream = N.stream_ptr(self.device)
        it, ncap = s._struct()
        s._allocate(it)
        n = int(s._read_stats().neval)
        s._itn += 1
        itn_word = s._itn & 0xffffffff
        # the iteration's device buffers are kept and reused (no allocator traffic per iteration)
        yv, _, wgt, hc = s._points(it, ncap, itn_word, None, want_hc=train, bufs=self._bufs)
        yv = yv[:n]
        yp, ld = self.flow.sample(yv, z=self._buf('yp', ncap, self.dim)[:n], ld=self._buf('ld', ncap)[:n])
        x = self._buf('xm', ncap, self.dim)[:n]
        jac = self._buf('jac', ncap)[:n]
        self.map.map(yp, x, jac)
        f = self._buf('f', ncap)
        self._feff(fcn, x, jac, ld, f)
        N.check(L.vg_reduce(ctypes.byref(it), itn_word, None, N.ptr(f), N.VG_F32, stream))
        if train and self.train_steps > 0:
            m = min(self.train_batch, n)
            if self._zs is None or self._zs.shape[0] != m:
                self._zs = torch.empty((m, self.dim), dtype=torch.float32, device=self.device)
                self._ws = torch.empty(m, dtype=torch.float32, device=self.device)
                self._scr = torch.empty(m + 1, dtype=torch.float64, device=self.device)
            nh = s._work[:4 * s.nhcube].view(torch.int32)
            chi2 = 1 if self._flow_nit > self.kl_itn else 0
            for _ in range(self.train_steps):
                self._tstep += 1
                N.check(L.vg_flow_train_batch(n, m, self._tseed, self._tstep & 0xffffffff, self.dim,
                                              N.ptr(yp), N.ptr(f), N.ptr(wgt), N.ptr(hc), N.ptr(nh),
                                              chi2, N.ptr(self._zs), N.ptr(self._ws), N.ptr(self._scr),
                                              stream))
                self.flow.train_step_normalized(self._zs, self._ws)
        N.check(L.vg_end_iteration(ctypes.byref(it), stream))
        st = s._read_stats()
        if st.status != 0:
            raise N.VegasError('device status %d' % st.status)
        if st.nan_seen:
            raise ValueError('integrand evaluates to nan')
        s.last_neval = int(st.neval)
        if s.beta > 0 and s.nhcube > 1:
            s.sum_sigf = float(st.sum_sigf)
        return float(st.mean), float(st.var), int(st.neval)

    def _plain_iteration(self, fcn):
        old = self.vegas.nitn
        self.vegas.nitn = 1
        try:
            r = self.vegas(fcn)
        finally:
            self.vegas.nitn = old
        v = r.itn_results[-1]
        return float(v.mean), float(v.sdev) ** 2, int(self.vegas.last_neval)

    def __call__(self, fcn, nitn=None, train=True, **kargs):
        """Run ``nitn`` iterations; returns an RAvg of them (as Integrator.__call__)."""
        if kargs:
            self.vegas.set(kargs)
        nitn = self.vegas.nitn if nitn is None else int(nitn)
        result = RAvg(weighted=self.vegas.adapt)
        for _ in range(nitn):
            self._nit += 1
            if not self.flow_on and not self.flow_dead and self._nit > self.plain_itn:
                self._start_flow()
            use_flow = self.flow_on
            t0 = time.perf_counter()
            if use_flow:
                self._flow_nit += 1
                tr = train and (self.train_itn is None or self._flow_nit <= self.train_itn)
                mean, var, neval = self._flow_iteration(fcn, tr)
            else:
                mean, var, neval = self._plain_iteration(fcn)
            sec = time.perf_counter() - t0
            score = var * neval * (sec / neval if self.gate == 'time' else 1.0)
            self.history.append(dict(flow=use_flow, mean=mean, sdev=math.sqrt(max(var, 0.0)),
                                     neval=neval, score=score, seconds=sec))
            if not use_flow:
                # the last few plain iterations (adapted) set the bar
                self.plain_scores = (self.plain_scores + [score])[-3:]
            elif self._flow_nit > self.grace:
                if self.plain_score is not None and score >= self.plain_score:
                    self.losing += 1
                    if self.losing >= self.patience:
                        self.flow_on = False
                        self.flow_dead = True
                else:
                    self.losing = 0
            result.add(gv.gvar(mean, math.sqrt(max(var, 0.0))))
            result.sum_neval += neval
        return result
