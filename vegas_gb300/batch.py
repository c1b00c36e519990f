"""Many independent vegas+ integrals in one persistent GPU launch.

No counterpart in the reference (one ``Integrator`` call integrates one
integrand).  ``BatchIntegrator`` holds the state of every integral -- the
same per-integral state an ``Integrator`` has (AdaptiveMap grid, strata and
their sigf, training histogram, iteration record) -- in a few device arenas,
and runs ``nitn`` vegas+ iterations of all of them in one kernel
(``vg_batch_launch``: one persistent kernel per dimension bucket -- dim
<= 4, <= 8, <= 16 -- on forked streams), optionally replayed from a CUDA
graph.  The tile configuration of each bucket's kernel (samples per thread,
CTAs per SM) is picked by a small autotuner that times each configuration on
a sample of the bucket's integrals.
"""
import ctypes
import math
import time

import numpy as np
import torch

from . import _native as N
from .adaptive_map import _device
from .integrands import LatticeAction, LorentzianProduct
from .integrator import strata

_LDP = 32   # parameters per integral in the packed table (Lorentzian: 2*dim <= 32)
_KINDS = {LorentzianProduct: N.VG_F_LORENTZ, LatticeAction: N.VG_F_LATTICE}


def _align(n, a=256):
    return (n + a - 1) // a * a


class BatchIntegrator(object):
    """vegas+ on many integrals of one built-in integrand family.

    Args:
        integrands: list of ``LorentzianProduct`` (over the unit cube) or of
            ``LatticeAction`` (over ``limits``), dimension <= 16 each.
        nevals: evaluations per iteration of each integral.
        dims: dimension of each integral (needed for ``LatticeAction``).
        limits: (lo, hi) of every axis (default (0, 1)).
        group: CTAs per integral (None: as many as fit when every integral
            gets at least two, else 1 = one CTA per integral from a queue);
            more than one only when all integrals share a dimension bucket.
        nitn, nwarm: iterations per launch and warm-up iterations excluded
            from the weighted average (the reference's ``nitn`` of an adapt
            call followed by a final call).
        alpha, beta, seed: as ``Integrator``; integral j uses Philox stream j.
        variant: tile configuration per dimension bucket, a sequence of 3
            (or one int for all buckets); None: autotune.
        precision: 'fp32' (default: FP32 sampling, map and evaluation,
            float-float and FP64 sums) or 'fp64' (the parity configuration:
            everything in FP64, the arithmetic of ``Integrator(precision=
            'fp64')``; Lorentzian products of dim <= 8 only, no autotuning).
    """

    def __init__(self, integrands, nevals, nitn=16, nwarm=8, alpha=0.5, beta=0.75, seed=1,
                 variant=None, device=None, neval_frac=0.75, max_neval_hcube=50000, dims=None,
                 limits=(0.0, 1.0), group=None, precision='fp32'):
        self.device = _device(device)
        if precision not in ('fp32', 'fp64'):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.precision = precision
        self.integrands = list(integrands)
        self.njobs = len(self.integrands)
        if self.njobs < 1:
            raise ValueError('no integrands')
        kinds = {_KINDS.get(type(f)) for f in self.integrands}
        if None in kinds or len(kinds) != 1:
            raise NotImplementedError('batched launch: one family of LorentzianProduct or LatticeAction')
        self.kind = kinds.pop()
        self.limits = (float(limits[0]), float(limits[1]))
        self.group_req = group
        self.nitn, self.nwarm = int(nitn), int(nwarm)
        if not 0 <= self.nwarm < self.nitn:
            raise ValueError('need 0 <= nwarm < nitn')
        self.alpha, self.beta, self.seed = float(alpha), float(beta), int(seed)
        self.neval_frac, self.max_neval_hcube = float(neval_frac), int(max_neval_hcube)
        if dims is None:
            dims = [len(f.c) for f in self.integrands]
        self.dims = np.array(dims, np.int64)
        if self.dims.max() > 16:
            raise NotImplementedError('batched launch: dimension <= 16')
        self._layout(np.asarray(nevals, np.int64))
        self._itn = 0
        self.variant = None
        self._graph = None
        if precision == 'fp64':
            variant = (N.VG_BATCH_CFG_F64,) * 3
        elif variant is None:
            variant = self.autotune()
        self.set_variant(variant)

    # ------------------------------------------------------------- layout
    def _layout(self, nevals):
        L = N.load()
        nj = self.njobs
        self.its = (N.VgIntegrator * nj)()
        sizes = []
        self.nstrat, self.ninc, self.nhcube, self.neval = [], [], [], []
        for j in range(nj):
            d = int(self.dims[j])
            sz = strata(d, 0, int(nevals[j]), True, np.zeros(d, np.int64), self.neval_frac, self.beta)
            it = self.its[j]
            it.dim = d
            it.precision = N.VG_F64 if self.precision == 'fp64' else N.VG_F32
            H = int(np.prod(sz['nstrat']))
            it.nhcube = H
            K = int(sz['ninc'].max())
            for k in range(d):
                it.nstrat[k] = int(sz['nstrat'][k])
                it.ninc[k] = int(sz['ninc'][k])
            it.ldg, it.ldi = K + 1, K
            it.neval = sz['neval']
            it.neval_frac = self.neval_frac
            it.min_neval_hcube = sz['min_neval_hcube']
            it.max_neval_hcube = self.max_neval_hcube
            it.alpha, it.beta = self.alpha, self.beta
            it.adapt = 1
            it.adapt_to_errors = 0
            it.seed = self.seed & ((1 << 64) - 1)
            it.stream_id = j
            it.tile = 0
            work = int(L.vg_workspace_bytes(ctypes.byref(it), 0))
            sizes.append((d * (K + 1) * 8, d * K * 8, H * 8, d * K * 8, d * K * 8,
                          ctypes.sizeof(N.VgStats), work))
            self.nstrat.append(sz['nstrat'])
            self.ninc.append(sz['ninc'])
            self.nhcube.append(H)
            self.neval.append(sz['neval'])
        offs = []
        o = 0
        for s in sizes:
            row = []
            for b in s:
                row.append(o)
                o = _align(o + b)
            offs.append(row)
        self.arena = torch.zeros(o, dtype=torch.uint8, device=self.device)
        base = self.arena.data_ptr()
        host_init = []
        for j in range(nj):
            it = self.its[j]
            og, oi, osg, osf, onf, ost, ow = offs[j]
            it.grid, it.inc, it.sigf = base + og, base + oi, base + osg
            it.sum_f, it.n_f, it.stats = base + osf, base + onf, base + ost
            it.work, it.work_bytes = base + ow, sizes[j][6]
            host_init.append((j, og, oi, osg, ost))
        # initial state: uniform grids, sigf = 1, sum_sigf = nhcube
        arena = self.arena
        for j, og, oi, osg, ost in host_init:
            d, K = int(self.dims[j]), int(self.its[j].ldi)
            g = np.zeros((d, K + 1))
            inc = np.zeros((d, K))
            for k in range(d):
                nk = int(self.ninc[j][k])
                g[k, :nk + 1] = np.linspace(self.limits[0], self.limits[1], nk + 1)
                inc[k, :nk] = np.diff(g[k, :nk + 1])
            arena[og:og + g.nbytes].copy_(torch.from_numpy(g.view(np.uint8).reshape(-1)))
            arena[oi:oi + inc.nbytes].copy_(torch.from_numpy(inc.view(np.uint8).reshape(-1)))
            H = self.nhcube[j]
            arena[osg:osg + 8 * H].view(torch.float64).fill_(1.0)
            st = N.VgStats()
            st.sum_sigf = float(H)
            arena[ost:ost + ctypes.sizeof(st)].copy_(
                torch.frombuffer(bytearray(bytes(st)), dtype=torch.uint8))
        self._stats_off = [h[4] for h in host_init]
        # integrand parameters, outputs, job table, queue order
        self.params = np.zeros((nj, _LDP))
        self.nparams = np.zeros(nj, np.int32)
        for j, f in enumerate(self.integrands):
            p = f.params(int(self.dims[j]))
            self.params[j, :len(p)] = p
            self.nparams[j] = len(p)
        self.out = torch.zeros((nj, self.nitn, 3), dtype=torch.float64, device=self.device)
        self.res = torch.zeros((nj, 4), dtype=torch.float64, device=self.device)
        self.table = torch.empty(int(L.vg_batch_table_bytes(nj)), dtype=torch.uint8, device=self.device)
        # queue order: grouped by dimension bucket, largest first in each
        self.bucket = np.where(self.dims <= 4, 0, np.where(self.dims <= 8, 1, 2))
        cost = np.array([self.neval[j] * (1 + self.dims[j]) for j in range(nj)])
        order = np.lexsort((-cost, self.bucket)).astype(np.int32)
        self.seg = np.zeros(6, np.int32)
        for b in range(3):
            pos = np.nonzero(self.bucket[order] == b)[0]
            self.seg[2 * b] = int(pos[0]) if len(pos) else 0
            self.seg[2 * b + 1] = len(pos)
        self.order = torch.tensor(order, device=self.device)
        self.queue = torch.zeros(3, dtype=torch.int32, device=self.device)
        self.sync = torch.zeros(nj, dtype=torch.int32, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)

    # ----------------------------------------------------------- launching
    def set_variant(self, variant):
        if np.ndim(variant) == 0:
            variant = (int(variant),) * 3
        cfg = np.array([int(v) for v in variant], np.int32)
        if cfg.shape != (3,):
            raise ValueError('variant: one configuration per dimension bucket (3)')
        L = N.load()
        smem = np.zeros(3, np.uint64)
        grid = np.zeros(3, np.int32)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        N.check(L.vg_batch_prepare(ctypes.cast(self.its, ctypes.c_void_p), self.njobs, self.kind,
                                   vp(self.params), _LDP, vp(self.nparams), self.nitn,
                                   N.ptr(self.out), N.ptr(self.res), N.ptr(self.sync), vp(cfg),
                                   N.ptr(self.table), self.table.numel(), vp(smem), vp(grid),
                                   N.stream_ptr(self.device)))
        self._cfg, self._smem, self._grid = cfg, smem, grid
        self.variant = tuple(int(v) for v in cfg)
        present = [b for b in range(3) if self.seg[2 * b + 1] > 0]
        self.groups = np.ones(3, np.int32)
        if len(present) == 1:
            b = present[0]
            if self.group_req is None:
                g = int(grid[b]) // int(self.seg[2 * b + 1])
                self.groups[b] = g if g >= 2 else 1
            else:
                self.groups[b] = int(self.group_req)
        elif self.group_req is not None and int(self.group_req) > 1:
            raise ValueError('groups of CTAs per integral need integrals of one dimension bucket')
        self.group = int(self.groups.max())
        self.grid = int(grid.max())
        self._graph = None

    def launch(self):
        """nitn iterations of every integral (asynchronous): one persistent
        kernel per dimension bucket."""
        L = N.load()
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        N.check(L.vg_batch_launch(N.ptr(self.table), self.njobs, self.kind, self.nitn, self.nwarm,
                                  (self._itn + 1) & 0xffffffff, N.ptr(self.order), vp(self.seg),
                                  N.ptr(self.queue), N.ptr(self.sync), vp(self.groups), N.ptr(self.status),
                                  vp(self._smem), vp(self._grid), vp(self._cfg), N.stream_ptr(self.device)))
        self._itn += self.nitn

    def capture(self):
        """Capture one launch in a CUDA graph (replayed by ``run(graph=True)``).
        The iteration counter of a replayed graph is fixed at capture; every
        replay continues from the state the previous one left."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.launch()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self._graph = g
        return g

    def run(self, graph=False):
        """Run nitn iterations of every integral; returns results (see results())."""
        if graph:
            if self._graph is None:
                self.capture()
            self._graph.replay()
        else:
            self.launch()
        return self.results()

    def results(self):
        """Per integral: mean, sdev, chi2, dof of the weighted average over the
        iterations after the warm-up ones (numpy [njobs, 4])."""
        if int(self.status.item()) != 0:
            raise N.VegasTimeout('batched launch: a group barrier timed out (status %d)'
                                 % int(self.status.item()))
        return self.res.cpu().numpy()

    def iterations(self):
        """Every iteration's (mean, variance, evaluations) (numpy [njobs, nitn, 3])."""
        return self.out.cpu().numpy()

    def timeline(self):
        """One launch with every integral's start and end recorded on the
        device (globaltimer): returns (start_ns, end_ns, sm) arrays
        [njobs], times relative to the earliest start.  The job table is
        rebuilt with the instrumentation for this launch and without it
        afterwards."""
        L = N.load()
        stamps = torch.zeros(3 * self.njobs, dtype=torch.int64, device=self.device)
        N.check(L.vg_batch_set_stamps(N.ptr(stamps)))
        try:
            self.set_variant(self.variant)
        finally:
            N.check(L.vg_batch_set_stamps(None))
        self.launch()
        torch.cuda.synchronize(self.device)
        self.set_variant(self.variant)
        s = stamps.view(self.njobs, 3).cpu().numpy()
        t0 = s[:, 0].min()
        return s[:, 0] - t0, s[:, 1] - t0, s[:, 2]

    def integrator_struct(self, j):
        """The C-ABI record of integral j (device pointers into the arena:
        grid, inc, sigf, training histogram, stats, workspace)."""
        return self.its[j]

    def state(self, j):
        """Views into the arena of integral j's device state: ``grid``
        [dim, ldg] and ``inc`` [dim, ldi] (FP64), ``sigf`` [nhcube], the
        ``stats`` record (bytes, ``N.VgStats``) and ``neval_h`` [nhcube]
        (int32, the last iteration's allocation, at the start of its
        workspace).  Writing into them changes the integral's state."""
        it = self.its[j]
        base = self.arena.data_ptr()
        d, H = int(it.dim), int(it.nhcube)

        def view(ptr, nbytes):
            o = int(ptr) - base
            return self.arena[o:o + nbytes]

        return {
            'grid': view(it.grid, 8 * d * it.ldg).view(torch.float64).view(d, int(it.ldg)),
            'inc': view(it.inc, 8 * d * it.ldi).view(torch.float64).view(d, int(it.ldi)),
            'sigf': view(it.sigf, 8 * H).view(torch.float64),
            'stats': view(it.stats, ctypes.sizeof(N.VgStats)),
            'neval_h': view(it.work, 4 * H).view(torch.int32),
        }

    def read_stats(self, j):
        """Integral j's iteration record (``N.VgStats``: sum_sigf, neval, range...)."""
        b = self.state(j)['stats'].cpu().numpy().tobytes()
        return N.VgStats.from_buffer_copy(b)

    def put_sum_sigf(self, j, value):
        """Set integral j's carried sum_sigf (the allocation's normaliser)."""
        st = self.read_stats(j)
        st.sum_sigf = float(value)
        self.state(j)['stats'].copy_(torch.frombuffer(bytearray(bytes(st)), dtype=torch.uint8))

    def evaluations(self):
        """Evaluations of the last launch summed over integrals and iterations
        (the allocations' actual counts, read back from the device)."""
        return int(round(float(self.out[:, :, 2].sum().item())))

    def nominal_evaluations(self):
        """The requested neval of every integral times nitn (the allocation
        gives each iteration about this many; rounding down per hypercube
        usually gives fewer)."""
        return int(sum(self.neval)) * self.nitn

    # ------------------------------------------------------------ autotune
    def autotune(self, sample=256, reps=2):
        """Time every tile configuration of each dimension bucket's kernel on
        a sample of that bucket's integrals (fresh copies, one launch each
        after a warm-up launch) and return the fastest per bucket."""
        L = N.load()
        nv = int(L.vg_batch_variants())
        rng = np.random.default_rng(12345)
        best = [0, 0, 0]
        self.tuning = {}
        for b in range(3):
            members = np.nonzero(self.bucket == b)[0]
            if len(members) == 0:
                continue
            idx = np.sort(rng.choice(members, size=min(sample, len(members)), replace=False))
            best_t = float('inf')
            for v in range(nv):
                try:
                    probe = BatchIntegrator([self.integrands[i] for i in idx], [self.neval[i] for i in idx],
                                            nitn=2, nwarm=1, alpha=self.alpha, beta=self.beta,
                                            seed=self.seed, variant=v, device=self.device,
                                            neval_frac=self.neval_frac,
                                            max_neval_hcube=self.max_neval_hcube,
                                            dims=[int(self.dims[i]) for i in idx], limits=self.limits,
                                            group=self.group_req)
                except (ValueError, MemoryError, NotImplementedError, N.VegasError):
                    continue   # configuration unavailable for this family / size
                probe.launch()
                torch.cuda.synchronize(self.device)
                t0 = time.perf_counter()
                for _ in range(reps):
                    probe.launch()
                torch.cuda.synchronize(self.device)
                t = (time.perf_counter() - t0) / reps
                self.tuning['%d/%d' % (b, v)] = t
                if t < best_t:
                    best[b], best_t = v, t
                del probe
        return tuple(best)
