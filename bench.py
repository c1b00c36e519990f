"""Benchmark: vegas+ on the ridge integrand (dim 4, M=1000 Gaussians of width
0.01 on the diagonal), neval = 1e6 evaluations per iteration, FP32 sampling /
map / evaluation with FP64 sums -- the vegas+ ridge workload.

A step is one full vegas+ iteration: allocation of evaluations to the
123462 hypercubes, Philox sampling + map + fused integrand evaluation +
per-hypercube two-pass reduction + training histogram, and the grid adapt.

Arms
  (default)          this library on the GPU(s); one JSON line on rank 0.
  --impl reference   the reference algorithm on the host cores: the CPU
                     restatement in oracle/ (the reference's Cython cannot be
                     built on the GPU host), all host threads, same workload.

JSON keys follow the benchmark contract: value = evaluations/s with inputs
resident in HBM (device loop, CUDA events on the launching stream); e2e = the
same through the public API (Integrator.__call__ per step, host buffers for
the integrand parameters and the result); roofline of the dominant kernel;
cpu_baseline; clocks sampled during the timed region.  Further lines: the
time to 1e-4 relative error (plain and flow-augmented vegas+), the batched
launch of 4096 integrals, the 64-coupling lattice scan, the FP64 dim-4 case
and the drop-in path (a torch integrand through the public API, with the HBM
roofline of the sampling and reduction kernels).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'time to 1e-4 rel. error & evals/s: flow-vegas+ vs plain vegas+, 1 GB300'
WORKLOAD = 'vegas+ ridge: dim=4, M=1000 Gaussians s=0.01 on the diagonal, neval=1e6/itn, ' \
           'ninc=1000 (actual [988,988,988,990]), nstrat [19,19,19,18], alpha=0.5, beta=0.75'
NEVAL = 1000000
DIM = 4
RIDGE_M, RIDGE_S = 1000, 0.01


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3000)
    ap.add_argument('--warmup', type=int, default=10)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-tta', action='store_true')
    ap.add_argument('--device-loop-only', action='store_true',
                    help='run only the device-resident iteration loop (for profilers)')
    ap.add_argument('--case', default='ridge',
                    choices=['ridge', 'flow', 'flow_train', 'batch', 'dropin', 'lattice'],
                    help='with --device-loop-only: which kernel family to run (for profilers): '
                         'ridge = the fused vegas+ iteration, flow = the flow sampling pass '
                         '(dim 8, 2^18 rows), flow_train = flow training steps (dim 8, 2^15 rows: '
                         'forward, per layer backward + weight gradients, Adam), '
                         'batch = the batched launch on 256 Lorentzian integrals, '
                         'dropin = the drop-in path (torch integrand, sampling and reduction kernels), '
                         'lattice = the lambda-scan launch on 16 couplings x 2e6 evaluations')
    ap.add_argument('--no-batch', action='store_true', help='skip the batched many-integral line')
    ap.add_argument('--no-reference-runs', action='store_true',
                    help='skip the normal-mode comparisons with oracle runs of the same workloads')
    return ap.parse_args()


# ------------------------------------------------------------------ clocks
class ClockSampler(object):
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            p = [q.strip() for q in ln.split(',')]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(smax) if smax else None, 'reasons': sorted(reasons),
                'samples': len(sm)}


# --------------------------------------------------------------- GPU arm
def profile_case(args, dev):
    """Short device loops of one kernel family, for ncu captures."""
    import torch
    if args.case == 'flow':
        from vegas_gb300.flow import Flow
        fl = Flow(8, seed=1, device=dev)
        g = torch.Generator(device=dev).manual_seed(0)
        fl.theta.add_(0.05 * torch.randn(fl.theta.shape, device=dev, generator=g))  # non-uniform splines
        fl.refresh()
        u = torch.rand(1 << 18, 8, device=dev, generator=g)
        for _ in range(args.warmup + args.steps):
            fl.sample(u)
    elif args.case == 'flow_train':
        from vegas_gb300.flow import Flow
        fl = Flow(8, seed=3, device=dev)
        g = torch.Generator(device=dev).manual_seed(0)
        z = torch.rand(1 << 15, 8, device=dev, generator=g)
        w = 2 * torch.rand(1 << 15, device=dev, generator=g)
        for _ in range(args.warmup + args.steps):
            fl.train_step_normalized(z, w)
    elif args.case == 'dropin':
        # the drop-in path's sampling and reduction kernels, 1e7 evaluations
        dropin_line(dev, neval=10 ** 7, nitn=1, reps=max(1, args.steps))
    elif args.case == 'batch':
        from vegas_gb300.batch import BatchIntegrator
        fs, nevals, _ = batch_workload(256)
        B = BatchIntegrator(fs, nevals, nitn=2, nwarm=1, seed=99, device=dev, variant=(1, 1, 0))
        for _ in range(args.warmup + args.steps):
            B.launch()
    elif args.case == 'lattice':
        import numpy as np
        import vegas_gb300 as vg
        from vegas_gb300.batch import BatchIntegrator
        lams = np.exp(np.linspace(np.log(0.01), np.log(1.0), 16))
        fs = [vg.LatticeAction(0.5, float(l)) for l in lams]
        B = BatchIntegrator(fs, [2 * 10 ** 6] * 16, nitn=2, nwarm=1, seed=7, dims=[16] * 16,
                            limits=(-5.0, 5.0), device=dev, variant=(0, 0, 2))
        for _ in range(args.warmup + args.steps):
            B.launch()
    torch.cuda.synchronize()


def batch_workload(njobs=4096, seed=2024):
    """The batched workload: Lorentzian products, dim ~ U{3..9}, centres
    U[0.2,0.8]^d, widths log-U[0.01,0.1], neval log-U[1e4,1e6] (seeded)."""
    import numpy as np
    import vegas_gb300 as vg
    rng = np.random.default_rng(seed)
    dims = rng.integers(3, 10, njobs)
    fs = []
    for d in dims:
        c = rng.uniform(0.2, 0.8, int(d))
        w = np.exp(rng.uniform(np.log(0.01), np.log(0.1), int(d)))
        fs.append(vg.LorentzianProduct(c, w))
    nevals = np.exp(rng.uniform(np.log(1e4), np.log(1e6), njobs)).astype(np.int64)
    return fs, nevals, dims


def dropin_line(dev, neval=10 ** 7, nitn=5, reps=5):
    """The drop-in path: a torch lbatch integrand (the dim-4 Gaussian
    (100/pi)^2 exp(-100 sum (x-1/2)^2) written in torch ops) through
    Integrator.__call__ -- sampling + map kernel (vg_sample_keep), the
    integrand's own torch kernels, reduction + training histogram kernel
    (vg_reduce_kept), adapt.  Evaluations/s through the API, and the HBM
    roofline of the sampling and reduction kernels: algorithmic bytes per
    evaluation (x (4 dim), the Jacobian (4) and the training bins (2 dim)
    written by the sampler; f, the Jacobian and the bins read by the
    reduction) over their CUDA-event times, against the measured copy
    bandwidth."""
    import math
    import numpy as np
    import torch
    import vegas_gb300 as vg
    from vegas_gb300 import _native as N
    dim = 4

    @vg.lbatchintegrand
    def gauss(x):
        return (100.0 / math.pi) ** 2 * torch.exp(-100.0 * ((x - 0.5) ** 2).sum(dim=1))

    integ = vg.Integrator(dim * [[0, 1]], neval=neval, seed=31, device=dev)
    integ(gauss, nitn=3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = integ(gauss, nitn=nitn)
    torch.cuda.synchronize()
    api_s = time.perf_counter() - t0
    # kernel timings on the launching stream
    L = N.load()
    stream = N.stream_ptr(dev)
    it, ncap = integ._struct()
    integ._allocate(it)
    n = int(integ._read_stats().neval)
    x = torch.empty((ncap, dim), dtype=torch.float32, device=dev)
    keep = integ._keep_buffer(it, ncap)
    cur = torch.cuda.current_stream(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]

    def sample():   # x, and each sample's Jacobian and training bins kept for the reduction
        N.check(L.vg_sample_keep(ctypes.byref(it), 7, None, N.ptr(x), None, None, None, ncap, N.ptr(keep),
                                 keep.numel(), stream))

    sample()
    f = gauss(x[:n])
    fb = torch.zeros(ncap, dtype=torch.float32, device=dev)
    fb[:n] = f

    def reduce():   # reads f, the kept Jacobians and bins
        N.check(L.vg_reduce_kept(ctypes.byref(it), 7, None, N.ptr(fb), N.VG_F32, N.ptr(keep), keep.numel(),
                                 stream))

    reduce()
    torch.cuda.synchronize()
    ev[0].record(cur)
    for _ in range(reps):
        sample()
    ev[1].record(cur)
    for _ in range(reps):
        f = gauss(x[:n])
    ev[2].record(cur)
    for _ in range(reps):
        reduce()
    ev[3].record(cur)
    torch.cuda.synchronize()
    t_s = ev[0].elapsed_time(ev[1]) / 1e3 / reps
    t_f = ev[1].elapsed_time(ev[2]) / 1e3 / reps
    t_r = ev[2].elapsed_time(ev[3]) / 1e3 / reps
    peaks = {}
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'MEASURED_PEAKS.json')) as fh:
            peaks = json.load(fh)
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get('hbm_gbs', 6800.0))
    # algorithmic bytes per evaluation: the sampler writes x (4 dim), the
    # Jacobian (4) and the training bins (2 dim); the reduction reads f (4),
    # the Jacobian and the bins
    b_s, b_r = 6 * dim + 4, 4 + 4 + 2 * dim
    ex1 = math.erf(math.sqrt(100.0) * 0.5)   # (100/pi)^2 exp(-100 sum (x-1/2)^2) over [0,1]^4
    exact = ex1 ** 4
    return {
        'fp32_vs_fp64_oracle': {'oracle': 'exact value erf(5)^4 in FP64', 'exact': exact,
                                'rel_dev': r.mean / exact - 1.0, 'pull': (r.mean - exact) / r.sdev},
        'workload': 'drop-in path: torch lbatch integrand (dim-4 Gaussian, torch ops) through '
                    'Integrator.__call__, neval %.0e/itn, FP32 sampling, FP64 sums' % neval,
        'value': r.sum_neval / api_s, 'unit': 'evals/s', 'neval_per_iteration': n,
        'result': str(r),
        'seconds_per_iteration': {'api': api_s / nitn, 'sample_kernel': t_s, 'integrand_torch': t_f,
                                  'reduce_kernel': t_r},
        'roofline': {
            'bound': 'hbm', 'unit': 'GB/s', 'peak': hbm,
            'peak_source': 'MEASURED_PEAKS.json hbm_gbs' if 'hbm_gbs' in peaks else 'fallback',
            'traffic_source': 'dram__bytes_read.sum + dram__bytes_write.sum per launch (ncu, '
                              'bench.py --device-loop-only --case dropin, about 9.3e6 evaluations)',
            'sample_kernel': {'bytes_per_eval': b_s, 'achieved': b_s * n / t_s / 1e9,
                              'frac': b_s * n / t_s / 1e9 / hbm, 'traffic': 227.2e6,
                              'writes': 'x (FP32, 4 dim B), Jacobian (4 B), training bins (2 dim B)'},
            'reduce_kernel': {'bytes_per_eval': b_r, 'achieved': b_r * n / t_r / 1e9,
                              'frac': b_r * n / t_r / 1e9 / hbm, 'traffic': 179.3e6,
                              'reads': 'f (4 B), Jacobian (4 B), training bins (2 dim B); forms the '
                                       'two-pass hypercube sums and the training histogram'}},
    }


def batched_line(dev, reps=2):
    """4096 integrals x (8 + 8) iterations in one persistent launch per
    replay of a CUDA graph; evals/s over the whole job and the pulls against
    the closed form."""
    import numpy as np
    import torch
    from vegas_gb300.batch import BatchIntegrator
    fs, nevals, dims = batch_workload()
    t0 = time.perf_counter()
    B = BatchIntegrator(fs, nevals, nitn=16, nwarm=8, seed=99, device=dev)
    t_setup = time.perf_counter() - t0
    B.capture()
    B._graph.replay()                     # warm-up replay (adapts the maps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        B._graph.replay()
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3 / reps
    res = B.results()
    exact = np.array([f.exact(int(d)) for f, d in zip(fs, dims)])
    pulls = (res[:, 0] - exact) / res[:, 1]
    # where the launch's time goes: every integral's start and end (device
    # globaltimer) in one more, instrumented launch
    t_s, t_e, _ = B.timeline()
    span = float(t_e.max()) / 1e9
    dur = (t_e - t_s) / 1e9
    bucket = np.where(dims <= 4, 0, np.where(dims <= 8, 1, 2))
    timeline = {'launch_span_s': span, 'longest_integral_s': float(dur.max()),
                'longest_integral_dim': int(dims[int(np.argmax(dur))]),
                'longest_integral_neval': int(nevals[int(np.argmax(dur))]),
                'last_start_s': float(t_s.max()) / 1e9,
                'per_bucket_end_s': {str(b): float(t_e[bucket == b].max()) / 1e9 for b in range(3)
                                     if np.any(bucket == b)},
                'note': 'one instrumented launch; the tail is span - last_start_s (no integral left to start)'}
    return {
        'timeline': timeline,
        'workload': '4096 Lorentzian-product integrals, dim U{3..9}, centres U[0.2,0.8]^d, widths '
                    'log-U[0.01,0.1], neval log-U[1e4,1e6] per integral, nitn 8+8, one persistent '
                    'kernel per 16 iterations replayed from a CUDA graph, FP32 eval + FP64 sums',
        'evals_per_launch': B.evaluations(), 'seconds_per_launch': secs,
        'value': B.evaluations() / secs, 'unit': 'evals/s', 'variant': B.variant,
        'autotune_seconds': {str(k): v for k, v in getattr(B, 'tuning', {}).items()},
        'setup_seconds': t_setup, 'integrals': len(fs),
        'pull_rms': float(np.sqrt(np.mean(pulls ** 2))), 'pull_max_abs': float(np.max(np.abs(pulls))),
        'rel_err_median': float(np.median(res[:, 1] / np.abs(res[:, 0]))),
        'fp32_vs_fp64_oracle': {
            'oracle': 'closed-form Lorentzian integrals in FP64 (LorentzianProduct.exact)',
            'max_rel_dev': float(np.max(np.abs(res[:, 0] / exact - 1))),
            'median_rel_dev': float(np.median(np.abs(res[:, 0] / exact - 1))),
            'pull_rms': float(np.sqrt(np.mean(pulls ** 2)))},
        # Lorentz factor per axis: subtract, FMA, reciprocal, multiply
        'nominal_evals_per_launch': B.nominal_evaluations(),
        'roofline': issue_roofline(dims, B.iterations()[:, :, 2].sum(axis=1), secs, lambda d: 4 * d, 2070.0),
    }


def issue_roofline(dims, nevals, seconds, integrand_ops, clock_mhz):
    """Issue-rate model of a batched launch: thread instructions per
    evaluation from op counts -- Philox4x32-10 (10 rounds of 2 wide
    multiplies, 2 three-input XORs and 2 key adds, plus 4 conversions: 80
    per 4 uniforms), the map (12 per axis: stratum coordinate, scale, floor,
    table load, FMA, Jacobian, training bin), the integrand (integrand_ops(d))
    and the per-sample reduction (30 + d: weight, histogram atomics,
    float-float two-pass sums) -- against 128 thread instructions per cycle
    and SM."""
    import numpy as np
    d = np.asarray(dims, np.int64)
    ops = 80 * ((d + 3) // 4) + 12 * d + integrand_ops(d) + 30 + d
    work = float(np.sum(ops * np.asarray(nevals, np.float64)))
    peak = 152 * 128 * clock_mhz * 1e6
    return {'bound': 'issue (model)', 'achieved': work / seconds / 1e12, 'peak': peak / 1e12,
            'unit': 'T thread-instr/s', 'frac': work / seconds / peak,
            'ops_per_evaluation_mean': float(np.sum(ops * np.asarray(nevals, np.float64)) /
                                             np.sum(np.asarray(nevals, np.float64))),
            'peak_source': '152 SMs x 4 schedulers x 32 lanes x %.0f MHz' % clock_mhz}


def lattice_line(dev, reps=2):
    """64 couplings lambda log-spaced in [0.01, 1] of the dim-16 periodic
    lattice action on [-5, 5]^16 (a = 0.5), 1e7 evaluations per lambda and
    iteration, nitn 8+8, in one launch (cooperative groups of CTAs per
    lambda); errors against the FP64 transfer-matrix value."""
    import numpy as np
    import torch
    import vegas_gb300 as vg
    from vegas_gb300.batch import BatchIntegrator
    lams = np.exp(np.linspace(np.log(0.01), np.log(1.0), 64))
    fs = [vg.LatticeAction(0.5, float(l)) for l in lams]
    t0 = time.perf_counter()
    B = BatchIntegrator(fs, [10 ** 7] * 64, nitn=16, nwarm=8, seed=7, dims=[16] * 64,
                        limits=(-5.0, 5.0), device=dev)
    t_setup = time.perf_counter() - t0
    B.run()                               # warm-up launch (adapts the maps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        B.launch()
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3 / reps
    res = B.results()
    exact = np.array([f.exact(16) for f in fs])
    pulls = (res[:, 0] - exact) / res[:, 1]
    return {
        'workload': 'dim-16 periodic lattice action exp(-sum[(x_{i+1}-x_i)^2/(2a) + a(x_i^2/2 + '
                    'lambda x_i^4)]), a=0.5, x in [-5,5]^16, 64 lambda log-spaced in [0.01,1], '
                    '1e7 evals/itn per lambda, nitn 8+8, one cooperative launch, FP32 eval, FP64 RAvg',
        'evals_per_launch': B.evaluations(), 'seconds_per_launch': secs,
        'value': B.evaluations() / secs, 'unit': 'evals/s', 'variant': B.variant,
        'ctas_per_lambda': B.group, 'setup_seconds': t_setup,
        'pull_rms': float(np.sqrt(np.mean(pulls ** 2))), 'pull_max_abs': float(np.max(np.abs(pulls))),
        'rel_err_median': float(np.median(res[:, 1] / np.abs(res[:, 0]))),
        'oracle': 'transfer matrix, 400-node Gauss-Legendre, FP64 (LatticeAction.exact)',
        # action per axis: difference, square, x^2, x^4 and the FMAs (6), plus one exp
        'nominal_evals_per_launch': B.nominal_evaluations(),
        'roofline': issue_roofline([16] * 64, B.iterations()[:, :, 2].sum(axis=1), secs, lambda d: 6 * d + 2,
                                   2070.0),
        'fp32_vs_fp64_oracle_max_rel_dev': float(np.max(np.abs(res[:, 0] / exact - 1))),
    }


def _jsonable(o):
    """JSON encoder fallback for numpy scalars and arrays."""
    import numpy as np
    if isinstance(o, np.generic):
        return o.item()
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(type(o).__name__)


def lattice_flow_line(dev, nlam=8, neval=1 << 20, train_itn=100, train_steps=2):
    """The flow on the lattice couplings: for a subset of the 64 lambda of
    the scan, flow-augmented vegas+ (FlowIntegrator: 6 coupling layers,
    32-bin splines, 2x128 conditioners, as on the mixture) against plain
    vegas+ at the same evaluations per iteration; variance per evaluation,
    seconds per iteration, pulls against the FP64 transfer-matrix value and
    the gate's decision (plain vegas+ judges by variance per evaluation)."""
    import numpy as np
    import torch
    import vegas_gb300 as vg
    from vegas_gb300.flow_vegas import FlowIntegrator
    # every 9th coupling of the 64-coupling scan (log-spaced in [0.01, 1]) and the last
    scan = np.exp(np.linspace(np.log(0.01), np.log(1.0), 64))
    lams = [float(v) for v in scan[np.linspace(0, 63, nlam).round().astype(int)]]
    out = {'workload': 'dim-16 periodic lattice action, a=0.5, x in [-5,5]^16, lambda in %s, %d evaluations '
                       'per iteration; plain vegas+ 50 + 20 iterations; flow-augmented vegas+ 30 plain + %d '
                       'flow (trained, %d Adam steps each) + 20 measured'
                       % ([round(v, 4) for v in lams], neval, train_itn, train_steps), 'per_lambda': {}}
    lim = 16 * [[-5.0, 5.0]]
    for lam in lams:
        f = vg.LatticeAction(0.5, float(lam))
        ex = f.exact(16)
        I = vg.Integrator(lim, neval=neval, seed=3, device=dev)
        I(f, nitn=50)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = I(f, nitn=20)
        torch.cuda.synchronize()
        tp = (time.perf_counter() - t0) / 20
        fi = FlowIntegrator(lim, neval=neval, seed=3, device=dev, plain_itn=30, kl_itn=10, train_itn=train_itn,
                            grace=10, patience=3, train_steps=train_steps, train_batch=1 << 15, lr=1e-3)
        fi(f, nitn=30 + train_itn)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rf = fi(f, nitn=20)
        torch.cuda.synchronize()
        tf = (time.perf_counter() - t0) / 20
        vp = r.sdev ** 2 * r.sum_neval / ex ** 2
        vf = rf.sdev ** 2 * rf.sum_neval / ex ** 2
        out['per_lambda'][str(lam)] = {
            'exact': ex, 'plain': str(r), 'plain_pull': (r.mean - ex) / r.sdev if r.sdev > 0 else None,
            'plain_rel_var_per_eval': vp, 'plain_seconds_per_iteration': tp,
            'flow': str(rf), 'flow_pull': (rf.mean - ex) / rf.sdev if rf.sdev > 0 else None,
            'flow_rel_var_per_eval': vf, 'flow_seconds_per_iteration': tf,
            'flow_active_at_end': bool(fi.flow_on),
            'variance_per_eval_ratio_flow_over_plain': vf / vp if vp > 0 else None,
            'variance_x_time_ratio_flow_over_plain': (vf * tf) / (vp * tp) if vp > 0 and tp > 0 else None}
    rv = [v['variance_per_eval_ratio_flow_over_plain'] for v in out['per_lambda'].values()]
    rt = [v['variance_x_time_ratio_flow_over_plain'] for v in out['per_lambda'].values()]
    out['summary'] = {
        'couplings': len(rv),
        'geo_mean_variance_per_eval_ratio': float(np.exp(np.mean(np.log(rv)))),
        'geo_mean_variance_x_time_ratio': float(np.exp(np.mean(np.log(rt)))),
        'flow_wins_variance_x_time': int(sum(1 for x in rt if x < 1.0)),
        'max_abs_flow_pull': float(max(abs(v['flow_pull']) for v in out['per_lambda'].values())),
        'note': 'ratios below 1: the flow is better; per coupling the better of the two is what a gate on '
                'variance x time would keep'}
    return out


def max_over_ranks(value, world, device=None):
    """Largest value over the ranks of the job (the timing rule of the
    benchmark: a step lasts as long as its slowest replica)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(base, rank):
    """Seed of a replica: replicas are independent vegas+ runs (own Philox
    key, stream = rank); nothing is exchanged on the data path."""
    return (int(base) + 7919 * int(rank)) & ((1 << 63) - 1)


def ridge_fp64_line(dev, nitn=20, warm=5):
    """The ridge workload with sampling, map and evaluation in FP64 (all
    1000 Gaussian terms per evaluation, as the reference computes them):
    evaluations/s of the device loop (vg_iterate, CUDA events), the
    same-precision companion of the FP64 CPU baseline."""
    import torch
    import vegas_gb300 as vg
    from vegas_gb300 import _native as N
    L = N.load()
    f = vg.Ridge(M=RIDGE_M, s=RIDGE_S)
    I = vg.Integrator(DIM * [[0, 1]], neval=NEVAL, precision='fp64', seed=64, device=dev)
    it, ncap = I._struct()
    I._put_sum_sigf()
    params = N.dbl_array(f.params(DIM))
    stream = N.stream_ptr(dev)
    for k in range(warm):
        N.check(L.vg_iterate(ctypes.byref(it), k + 1, f.kind, params, 2, stream))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(nitn):
        N.check(L.vg_iterate(ctypes.byref(it), warm + k + 1, f.kind, params, 2, stream))
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3 / nitn
    n = int(I._read_stats().neval)
    return {'workload': 'vegas+ ridge as the headline line, sampling / map / evaluation in FP64 (1000 '
                        'terms per evaluation)', 'value': n / secs, 'unit': 'evals/s',
            'seconds_per_iteration': secs, 'iterations': nitn, 'neval_per_iteration': n}


def config1_line(dev, nitn=20):
    """The CPU-sized workload: dim 4, f = (100/pi)^2 exp(-100 sum (x-1/2)^2),
    neval 1e4/itn, FP64 throughout.  Latency per iteration through the public
    API (one call of nitn iterations, enqueued back to back, records read at
    the end) and for iterations captured in a CUDA graph (allocation, fused
    evaluation + reduction, adapt; the iteration record copied on the
    device)."""
    import ctypes
    import torch
    import vegas_gb300 as vg
    from vegas_gb300 import _native as N
    L = N.load()
    f = vg.Gaussian(a=100.0, c=0.5, dim=4)
    integ = vg.Integrator(4 * [[0, 1]], neval=10000, precision='fp64', seed=31, device=dev)
    integ(f, nitn=3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = integ(f, nitn=nitn)
    torch.cuda.synchronize()
    t_api = (time.perf_counter() - t0) / nitn
    # CUDA graph of nitn iterations; sum_sigf carries over in the device record
    g_int = vg.Integrator(4 * [[0, 1]], neval=10000, precision='fp64', seed=32, device=dev)
    it, ncap = g_int._struct()
    g_int._put_sum_sigf()
    params = N.dbl_array(f.params(4))
    recs = torch.empty((nitn, ctypes.sizeof(N.VgStats)), dtype=torch.uint8, device=dev)
    s = torch.cuda.Stream(device=dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            sp = N.stream_ptr(dev)
            for k in range(nitn):
                N.check(L.vg_iterate(ctypes.byref(it), k + 1, f.kind, params, 3, sp))
                recs[k].copy_(g_int._stats)
    torch.cuda.current_stream(dev).wait_stream(s)
    graph.replay()                         # warm-up replay
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    graph.replay()
    e1.record()
    torch.cuda.synchronize()
    t_graph = e0.elapsed_time(e1) / 1e3 / nitn
    return {'workload': 'dim 4, (100/pi)^2 exp(-100 sum (x-1/2)^2), neval 1e4/itn, ninc 1000, '
                        'alpha 0.5, beta 0.75, FP64 throughout',
            'seconds_per_iteration_api': t_api, 'seconds_per_iteration_graph': t_graph,
            'result': str(r), 'exact': f.exact(4)}


def gpu_arm(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    import vegas_gb300 as vg
    from vegas_gb300 import _native as N

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        dist.init_process_group('nccl')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    L = N.load()
    if args.device_loop_only and args.case != 'ridge':
        profile_case(args, dev)
        return

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    f = vg.Ridge(M=RIDGE_M, s=RIDGE_S)
    exact = f.exact(DIM)
    # -------- device loop (inputs resident; value, roofline)
    integ = vg.Integrator(DIM * [[0, 1]], neval=NEVAL, seed=replica_seed(1234, rank), device=dev)
    it, ncap = integ._struct()
    it.stream_id = rank
    stream = N.stream_ptr(dev)
    params = N.dbl_array(f.params(DIM))
    integ._put_sum_sigf()
    l2_flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(itn, ev=None):
        if ev is None:   # one call: allocation, fused kernel + finalize, adapt (overlapped)
            N.check(L.vg_iterate(ctypes.byref(it), itn, f.kind, params, 2, stream))
            return
        # the same kernels with events around the fused kernel + finalize
        N.check(L.vg_allocate(ctypes.byref(it), stream))
        ev[0].record()
        N.check(L.vg_fused_iteration(ctypes.byref(it), itn, None, f.kind, params, 2, stream))
        ev[1].record()
        N.check(L.vg_end_iteration(ctypes.byref(it), stream))

    itn = 1
    for _ in range(args.warmup):
        step(itn)
        itn += 1
    barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
            torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    neval_tot = 0
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    for k in range(args.steps):
        l2_flush.fill_(float(k))          # evict L2 between timed iterations
        e0, e1, e2, e3 = evs[k]
        e0.record()
        step(itn)
        e3.record()
        itn += 1
    barrier()
    clk = clocks.stop()
    if args.device_loop_only:
        return
    # the fused kernel + finalize alone (roofline), in the same conditions,
    # over as many further iterations (not part of the timed steps)
    for k in range(args.steps):
        l2_flush.fill_(float(k))
        step(itn, evs[k][1:3])
        itn += 1
    torch.cuda.synchronize()
    step_ms = [evs[k][0].elapsed_time(evs[k][3]) for k in range(args.steps)]
    kern_ms = [evs[k][1].elapsed_time(evs[k][2]) for k in range(args.steps)]
    st = integ._read_stats()
    neval_step = int(st.neval)
    t_total = max_over_ranks(sum(step_ms) / 1e3, world, dev)
    value = world * neval_step * args.steps / t_total
    # -------- roofline of the fused kernel: SFU-bound (one ex2 per Gaussian term)
    kern_s = statistics.median(kern_ms) / 1e3
    ex2_per_launch = neval_step * RIDGE_M
    # Gaussian terms the kernel evaluates: those that can be nonzero in FP32
    # (the others are exactly zero and skipped); counted in one extra,
    # untimed iteration
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    N.check(L.vg_set_term_counter(N.ptr(cnt)))
    params_c = N.dbl_array(f.params(DIM))   # rebuilt so the counter is attached
    N.check(L.vg_allocate(ctypes.byref(it), stream))
    N.check(L.vg_fused_iteration(ctypes.byref(it), itn, None, f.kind, params_c, 2, stream))
    N.check(L.vg_set_term_counter(None))
    torch.cuda.synchronize()
    executed = int(cnt.item())
    achieved = executed / kern_s / 1e9
    peak = measure_ex2_peak(L, dev)
    model = ridge_issue_model(executed / neval_step)
    clk_max = float(clk.get('sm_max_mhz') or 2070.0)
    issue_peak = 152 * 128 * clk_max * 1e6
    model_rate = model['total'] * neval_step / kern_s
    # -------- e2e through the public API: one call of K iterations (each
    # iteration's record read back to pinned host memory), and K calls of one
    # iteration each
    integ2 = vg.Integrator(DIM * [[0, 1]], neval=NEVAL, seed=replica_seed(99, rank), device=dev)
    integ2(f, nitn=args.warmup)
    barrier()
    t0 = time.perf_counter()
    r = integ2(f, nitn=args.steps)
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e = world * r.sum_neval / t_e2e
    barrier()
    t0 = time.perf_counter()
    ne2 = 0
    for _ in range(args.steps):
        integ2(f, nitn=1)
        ne2 += integ2.last_neval
    barrier()
    t_call = max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e_call = world * ne2 / t_call
    # -------- time to 1e-4 relative error (plain vegas+, public API, fresh map)
    tta = None
    if not args.no_tta:
        integ3 = vg.Integrator(DIM * [[0, 1]], neval=NEVAL, seed=replica_seed(4242, rank), device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r3 = integ3(f, nitn=5000, rtol=1e-4)
        torch.cuda.synchronize()
        pull3 = (r3.mean - exact) / r3.sdev
        tta = {'ridge_plain': {
            'seconds': time.perf_counter() - t0, 'iterations': r3.nitn,
            'result': str(r3), 'rel_err': r3.sdev / abs(r3.mean),
            'exact': exact, 'pull': pull3,
            'reached': bool(r3.sdev / abs(r3.mean) <= 1e-4 and abs(pull3) <= 3.0),
            'chi2_dof': (r3.chi2 / r3.dof if r3.dof > 0 else 0.0)}}
        if rank == 0:
            tta['mixture_flow_vs_plain'] = tta_flow_vs_plain(dev)
    batched = lattice = small = dropin = ridge64 = refruns = None
    if rank == 0:
        small = config1_line(dev)
        dropin = dropin_line(dev)
        ridge64 = ridge_fp64_line(dev)
        if not args.no_reference_runs:
            refruns = reference_runs(dev)
    lattice_flow = None
    if not args.no_batch and rank == 0:
        batched = batched_line(dev)
        lattice = lattice_line(dev)
        lattice_flow = lattice_flow_line(dev)
    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return
    out = {
        'metric': METRIC, 'value': value, 'unit': 'evals/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': 1e3 * t_total / args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 (sample/map/eval), f64 (sums)',
        'data': 'synthetic (analytic integrand, Philox4x32-10 sampling)',
        'config': {'workload': WORKLOAD, 'neval_per_step': neval_step, 'l2_flush': True,
                   'parallelism': 'replicas' if world > 1 else 'single'},
        'e2e': {'value': e2e, 'unit': 'evals/s', 'h2d_bytes_per_step': 8 * len(f.params(DIM)),
                'd2h_bytes_per_step': ctypes.sizeof(N.VgStats),
                'call': 'Integrator(f, nitn=%d): every iteration enqueued, its record copied to '
                        'pinned host memory; inputs = the integrand parameters of each launch'
                        % args.steps,
                'per_call': {'value': e2e_call, 'unit': 'evals/s',
                             'call': '%d calls Integrator(f, nitn=1), host round trip each'
                                     % args.steps}},
        # per timed step: allocation, fused tile kernel, finalize, adapt
        'gpu_launches': 4 * args.steps,
        'roofline': {'bound': 'issue (model)', 'achieved': model_rate / 1e12, 'peak': issue_peak / 1e12,
                     'unit': 'T thread-instr/s', 'frac': model_rate / issue_peak,
                     'traffic': 1.70e6,
                     'traffic_source': 'dram__bytes_read.sum + dram__bytes_write.sum of one fused '
                                       'tile_kernel launch (ncu, bench.py --device-loop-only)',
                     'kernel': 'ridge iteration: fused tile_kernel (evaluate + reduce) + finalize '
                               '(CUDA events on the launching stream, median over the timed steps)',
                     'algorithmic': 'thread instructions per evaluation from op counts (ridge_issue_model) '
                                    'x %d evaluations per launch' % neval_step,
                     'model_per_eval': model,
                     'peak_source': '152 SMs x 4 schedulers x 32 lanes x %.0f MHz (maximum SM clock)'
                                    % clk_max,
                     'sfu': {'executed_ex2_per_launch': executed,
                             'achieved': achieved, 'peak': peak, 'unit': 'Gex2/s',
                             'frac_executed': achieved / peak,
                             'reference_terms_equivalent': ex2_per_launch / kern_s / 1e9,
                             'note': 'the reference evaluates all M=1000 terms (%d ex2 per launch); the '
                                     'kernel evaluates only those that can be nonzero in FP32 (identical '
                                     'f), so the reference-terms rate is not a utilisation' % ex2_per_launch,
                             'peak_source': 'MUFU ex2 probe kernel on this GPU (vg_probe_mufu_ex2)'}},
        'clocks': clk,
        'time_to_1e-4': tta,
        'batched': batched,
        'lattice_scan': lattice,
        'lattice_flow': lattice_flow,
        'small_fp64': small,
        'dropin': dropin,
        'ridge_fp64': ridge64,
        'reference_runs': refruns,
    }
    if not args.no_cpu_baseline and world == 1:
        out['cpu_baseline'] = cpu_baseline(iters=2)
    print(json.dumps(out, default=_jsonable))


MIX_DIM, MIX_NEVAL = 8, 1 << 20
MIX_WORKLOAD = ('flow-augmented vegas+: dim=8, equal-weight mixture of 4 normalised Gaussians '
                '(sigma=0.03) at seeded centres U[0.15,0.85]^8 (numpy default_rng(4)), 2^20 '
                'evaluations/itn; flow: 6 coupling layers, 32-bin piecewise-quadratic splines, '
                'conditioner MLP 2x128 BF16 on tcgen05 tensor cores')


def mixture_integrand():
    import numpy as np
    import vegas_gb300 as vg
    rng = np.random.default_rng(4)
    return vg.GaussianMixture(rng.uniform(0.15, 0.85, (4, MIX_DIM)), sigma=0.03)


def _tta_run(step, warm_itn, cap_s, target=1e-4, exact=None):
    """Wall-clock time until the running result (iterations after the first
    warm_itn) reaches target relative error.  step() runs one iteration and
    returns (mean, var, neval).  Past cap_s the time is extrapolated with the
    1/n error law from the accumulated precision.  With the exact value
    given, the target counts as reached only when the result also lies
    within 3 standard deviations of it (a biased result reaches nothing):
    "reached" says so, and "pull" is (mean - exact) / sdev."""
    import torch
    from vegas_gb300 import RAvg, gvar
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(warm_itn):
        step()
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    r = RAvg()
    neval = 0
    means = []
    while True:
        m, v, ne = step()
        r.add(gvar(m, max(v, 0.0) ** 0.5))
        means.append(m)
        neval += ne
        rel = r.sdev / abs(r.mean) if r.mean != 0 else float('inf')
        t = time.perf_counter() - t0
        if rel <= target or t > cap_s:
            break
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    t_acc = t - t_warm
    est = t if rel <= target else t_warm + t_acc * (rel / target) ** 2
    out = {'seconds': est, 'measured_seconds': t, 'extrapolated': rel > target,
           'warmup_seconds': t_warm, 'warmup_iterations': warm_itn, 'iterations': r.nitn,
           'evaluations': neval, 'result': str(r), 'mean': r.mean, 'sdev': r.sdev, 'rel_err': rel,
           'var_per_eval': (r.sdev ** 2) * neval,
           'chi2_dof': (r.chi2 / r.dof if r.dof > 0 else 0.0)}
    if exact is not None:
        out['exact'] = exact
        out['pull'] = (r.mean - exact) / r.sdev if r.sdev > 0 else None
        out['reached'] = bool(rel <= target and out['pull'] is not None and abs(out['pull']) <= 3.0)
    if len(means) > 2:
        # the plain (unweighted) mean of the iterations: unbiased where the
        # inverse-variance weighting is not, with the error from the spread
        # of the iterations; its time to the target by the 1/n law
        import numpy as np
        mu = float(np.mean(means))
        su = float(np.std(means, ddof=1) / len(means) ** 0.5)
        relu = su / abs(mu) if mu != 0 else float('inf')
        u = {'mean': mu, 'sdev': su, 'rel_err': relu,
             'seconds': t if relu <= target else t_warm + t_acc * (relu / target) ** 2,
             'extrapolated': bool(relu > target)}
        if exact is not None and su > 0:
            u['pull'] = (mu - exact) / su
        out['unweighted_average'] = u
    return out


def tta_flow_vs_plain(dev, cap_s=30.0):
    """Time to 1e-4 relative error on the flow workload: plain vegas+ (fused
    kernel path) against flow-augmented vegas+ (FlowIntegrator)."""
    import vegas_gb300 as vg
    from vegas_gb300.flow_vegas import FlowIntegrator
    f = mixture_integrand()
    exact = f.exact(MIX_DIM)
    lim = MIX_DIM * [[0.0, 1.0]]
    plain = vg.Integrator(lim, neval=MIX_NEVAL, seed=777, device=dev)

    def pstep():
        old = plain.nitn
        plain.nitn = 1
        rr = plain(f)
        plain.nitn = old
        v = rr.itn_results[-1]
        return v.mean, v.sdev ** 2, plain.last_neval

    out = {'workload': MIX_WORKLOAD, 'exact': exact}
    out['plain'] = _tta_run(pstep, 10, cap_s, exact=exact)
    # training schedule: 10 plain iterations, then 100 flow iterations with
    # 2 Adam steps of 2^15 samples each (30 on the KL loss, 70 on the
    # variance loss), then the frozen flow.  The training is not bitwise
    # reproducible and its outcome spreads from run to run; over 10 seeds
    # this schedule reached 1e-4 in 0.47-0.57 s in 9 runs (one run's flow
    # under-sampled a mode: 0.43 s, pull beyond 3 sigma), where 40 x 4 steps
    # with 10 KL iterations spread over 0.50-1.30 s
    fi = FlowIntegrator(lim, neval=MIX_NEVAL, seed=777, device=dev, plain_itn=10, kl_itn=30,
                        train_itn=100, grace=10, patience=3, train_steps=2, train_batch=1 << 15,
                        lr=1e-3)

    def fstep():
        fi(f, nitn=1)
        h = fi.history[-1]
        return h['mean'], h['sdev'] ** 2, h['neval']

    out['flow'] = _tta_run(fstep, 110, cap_s, exact=exact)
    out['flow']['training'] = ('10 plain + 100 training iterations (2 Adam steps of 2^15 samples each; '
                               '30 on the KL loss, 70 on the variance loss) in the warm-up; the iterations '
                               'after it use the frozen flow')
    out['flow']['flow_active_at_end'] = bool(fi.flow_on)
    # time-to-accuracy counts only a run that reached 1e-4 within 3 sigma
    # of the exact value; plain vegas+ on this multimodal integrand
    # converges to a biased value (see reference_runs.config4_mixture)
    # the times to a correct 1e-4: a run that stopped at 1e-4 more than 3
    # sigma from the exact value counts with the time its plain (unweighted)
    # average of the iterations needs to reach 1e-4 (unbiased, extrapolated)
    def correct_time(r):
        if r['reached']:
            return r['seconds'], 'weighted average (RAvg)'
        u = r.get('unweighted_average')
        if u is not None and u.get('pull') is not None and abs(u['pull']) <= 3.0:
            return u['seconds'], 'plain mean of the iterations' + (' (extrapolated)' if u['extrapolated'] else '')
        return None, 'not reached'
    tp, how_p = correct_time(out['plain'])
    tf, how_f = correct_time(out['flow'])
    out['seconds_to_correct_1e-4'] = {'plain': tp, 'plain_how': how_p, 'flow': tf, 'flow_how': how_f}
    out['speedup'] = tp / tf if (tp and tf) else None
    out['speedup_note'] = ('flow over plain vegas+, times to a 1e-4 result within 3 sigma of the exact value; '
                           'plain reached=%s with its weighted average, flow reached=%s'
                           % (out['plain']['reached'], out['flow']['reached']))
    return out


# ------------------------------------------------- normal-mode comparisons
def _combined(a_mean, a_sdev, b_mean, b_sdev):
    d = (a_sdev ** 2 + b_sdev ** 2) ** 0.5
    return (a_mean - b_mean) / d if d > 0 else None


def _oracle_run(st, kind, params, nwarm, nitn, seed, nthreads):
    """The oracle (the reference algorithm in FP64 on the host) for nwarm
    adapting iterations then nitn more: per-iteration (mean, var), the
    weighted average (RAvg.add, pyx:2392-2410) and the wall time."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    t0 = time.perf_counter()
    ms, vs = [], []
    neval = 0
    for k in range(nwarm + nitn):
        out = st.iterate(kind, params, seed=seed, stream=0, itn=k + 1, nthreads=nthreads)
        if k >= nwarm:
            ms.append(out['mean'])
            vs.append(out['var'])
            neval += out['neval']
    dt = time.perf_counter() - t0
    mean, sdev, chi2, dof, Q = O.weighted_average(ms, vs)
    ms = np.asarray(ms)
    return {'mean': mean, 'sdev': sdev, 'chi2_dof': chi2 / dof if dof else 0.0, 'Q': Q,
            'unweighted_mean': float(ms.mean()),
            'unweighted_sdev': float(ms.std(ddof=1) / len(ms) ** 0.5) if len(ms) > 1 else 0.0,
            'seconds': dt, 'evaluations': neval, 'iterations': nitn, 'warmup_iterations': nwarm,
            'threads': nthreads}


def _gpu_run(I, f, nwarm, nitn):
    """The same on the GPU through the public API: per-iteration results
    after nwarm adapting iterations, weighted and unweighted averages."""
    import numpy as np
    import torch
    if nwarm:
        I(f, nitn=nwarm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = I(f, nitn=nitn)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    ms = np.array([x.mean for x in r.itn_results])
    return {'mean': r.mean, 'sdev': r.sdev, 'chi2_dof': r.chi2 / r.dof if r.dof else 0.0, 'Q': r.Q,
            'unweighted_mean': float(ms.mean()),
            'unweighted_sdev': float(ms.std(ddof=1) / len(ms) ** 0.5) if len(ms) > 1 else 0.0,
            'seconds': dt, 'evaluations': int(r.sum_neval), 'iterations': nitn, 'warmup_iterations': nwarm,
            'precision': I.precision}


def _pulls(runs, exact):
    """Each run's pull against the exact value (weighted and unweighted
    averages) and the combined-sigma pull of every GPU run against the
    oracle run."""
    for k, r in runs.items():
        if not isinstance(r, dict) or 'mean' not in r:
            continue
        r['pull_vs_exact'] = (r['mean'] - exact) / r['sdev'] if r['sdev'] > 0 else None
        r['rel_dev_vs_exact'] = r['mean'] / exact - 1.0
        if r.get('unweighted_sdev'):
            r['unweighted_pull_vs_exact'] = (r['unweighted_mean'] - exact) / r['unweighted_sdev']
    o = runs['oracle']
    for k, r in runs.items():
        if k != 'oracle' and isinstance(r, dict) and 'mean' in r:
            r['combined_pull_vs_oracle'] = _combined(r['mean'], r['sdev'], o['mean'], o['sdev'])
    runs['exact'] = exact
    return runs


def reference_runs(dev):
    """Normal-mode results on the GPU against oracle runs of the same
    workload (independent draws: the oracle is the reference algorithm in
    FP64 on the host cores), combined-sigma pulls, and each against the
    exact value.  Config 1: dim-4 Gaussian, 1e4/itn, 10+10, FP64.  Config 2:
    the ridge, 1e6/itn, 10+10, FP32 on the GPU (and FP64).  Config 4: plain
    vegas+ on the 8-d Gaussian mixture, 2^20/itn, 10 + 150 iterations in
    FP32 and FP64 on the GPU and in the oracle -- the weighted average
    (RAvg) and the plain mean of the iterations, to attribute the bias of
    plain vegas+ on this multimodal integrand."""
    import vegas_gb300 as vg
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    cores = os.cpu_count() or 1
    out = {}
    # config 1
    f = vg.Gaussian(a=100.0, c=0.5, dim=4)
    runs = {'gpu_fp64': _gpu_run(vg.Integrator(4 * [[0, 1]], neval=10000, precision='fp64', seed=101,
                                               device=dev), f, 10, 10),
            'gpu_fp32': _gpu_run(vg.Integrator(4 * [[0, 1]], neval=10000, seed=102, device=dev), f, 10, 10),
            'oracle': _oracle_run(O.State(4 * [[0, 1]], 10000), O.F_GAUSS, f.params(4), 10, 10, 103, 1)}
    out['config1_gauss4'] = _pulls(runs, f.exact(4))
    # config 2
    f = vg.Ridge(M=RIDGE_M, s=RIDGE_S)
    runs = {'gpu_fp32': _gpu_run(vg.Integrator(DIM * [[0, 1]], neval=NEVAL, seed=201, device=dev), f, 10, 10),
            'gpu_fp64': _gpu_run(vg.Integrator(DIM * [[0, 1]], neval=NEVAL, precision='fp64', seed=202,
                                               device=dev), f, 10, 10),
            'oracle': _oracle_run(O.State(DIM * [[0, 1]], NEVAL), O.F_RIDGE, [RIDGE_M, RIDGE_S], 10, 10, 203,
                                  cores)}
    out['config2_ridge'] = _pulls(runs, f.exact(DIM))
    # config 4, plain vegas+
    f = mixture_integrand()
    lim = MIX_DIM * [[0.0, 1.0]]
    n4 = 150
    runs = {'gpu_fp32': _gpu_run(vg.Integrator(lim, neval=MIX_NEVAL, seed=401, device=dev), f, 10, n4),
            'gpu_fp64': _gpu_run(vg.Integrator(lim, neval=MIX_NEVAL, precision='fp64', seed=402, device=dev),
                                 f, 10, n4),
            'oracle': _oracle_run(O.State(lim, MIX_NEVAL), O.F_MIXTURE, f.params(MIX_DIM), 10, n4, 403, cores)}
    out['config4_mixture_plain'] = _pulls(runs, f.exact(MIX_DIM))
    out['note'] = ('gpu_* and oracle are independent runs (own Philox streams); combined_pull_vs_oracle = '
                   '(I_gpu - I_oracle) / sqrt(sdev_gpu^2 + sdev_oracle^2); the oracle is the reference '
                   'algorithm restated in C, FP64, on %d host threads' % cores)
    return out


def ridge_issue_model(terms_per_eval, dim=DIM):
    """Issue-rate model of the fused FP32 ridge iteration: thread
    instructions per evaluation from the algorithm's op counts.

      Philox4x32-10 for the sample's uniforms: 80 per 4 uniforms (10 rounds
        of 2 wide multiplies, 2 three-input XORs, 2 key adds; 4 conversions)
      map, per axis: stratum coordinate, bin index, table load, node + inc
        x fraction, Jacobian factor, training bin -- 12
      ridge: mean and spread of x (3 dim + 1), exponent offset and centre
        (2), window of the Gaussian terms that can be nonzero in FP32 (15),
        final scale (3); per evaluated term: subtract, FMA, ex2, add and a
        quarter of a vector shared load -- 4.25
      per-sample reduction: weight and fdv2 (4), training histogram (3 per
        axis), float-float two-pass hypercube sums (30)

    The terms are the ones the kernel evaluates (those that can be nonzero
    in FP32; the others are exactly zero), counted per iteration.  Peak: 152
    SMs x 4 schedulers x 32 lanes per cycle at the maximum SM clock."""
    philox = 80 * ((dim + 3) // 4)
    mapping = 12 * dim
    integrand = (3 * dim + 1) + 2 + 15 + 3 + 4.25 * terms_per_eval
    reduction = 4 + 3 * dim + 30
    return {'philox': philox, 'map': mapping, 'integrand': integrand, 'reduction': reduction,
            'total': philox + mapping + integrand + reduction, 'terms_per_eval': terms_per_eval}


def measure_ex2_peak(L, dev):
    """MUFU ex2 throughput of this GPU (G ex2/s), measured by a probe kernel."""
    import torch
    from vegas_gb300 import _native as N
    nthreads = 152 * 2048 * 4
    iters = 4096
    out = torch.empty(nthreads, dtype=torch.float32, device=dev)
    s = N.stream_ptr(dev)
    for _ in range(2):
        N.check(L.vg_probe_mufu_ex2(N.ptr(out), nthreads, iters, s))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    N.check(L.vg_probe_mufu_ex2(N.ptr(out), nthreads, iters, s))
    e1.record()
    torch.cuda.synchronize()
    return nthreads * iters * 8 / (e0.elapsed_time(e1) / 1e3) / 1e9


# ------------------------------------------------------------ CPU baseline
def _cpu_tta(st, kind, params, nwarm, seed, nthreads, cap_s, target=1e-4, exact=None):
    """The oracle's time to `target` relative error on one workload: nwarm
    adapting iterations, then iterations until the weighted average reaches
    the target or cap_s passes (then extrapolated with the 1/n law)."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    t0 = time.perf_counter()
    k = 0
    for _ in range(nwarm):
        k += 1
        st.iterate(kind, params, seed=seed, itn=k, nthreads=nthreads)
    t_warm = time.perf_counter() - t0
    ms, vs = [], []
    ne = 0
    rel = float('inf')
    while True:
        k += 1
        out = st.iterate(kind, params, seed=seed, itn=k, nthreads=nthreads)
        ms.append(out['mean'])
        vs.append(out['var'])
        ne += out['neval']
        mean, sdev, chi2, dof, Q = O.weighted_average(ms, vs)
        rel = sdev / abs(mean) if mean != 0 else float('inf')
        t = time.perf_counter() - t0
        if rel <= target or t > cap_s:
            break
    t_acc = t - t_warm
    r = {'seconds': t if rel <= target else t_warm + t_acc * (rel / target) ** 2,
         'measured_seconds': t, 'extrapolated': rel > target, 'iterations': len(ms),
         'warmup_iterations': nwarm, 'evaluations': ne, 'rel_err': rel, 'mean': mean, 'sdev': sdev,
         'evals_per_s': ne / t_acc if t_acc > 0 else None, 'threads': nthreads}
    if exact is not None:
        r['pull'] = (mean - exact) / sdev if sdev > 0 else None
    return r


def cpu_baseline(iters=2, kind='port'):
    """The reference algorithm on the host cores (the C restatement in
    oracle/, FP64): the ridge workload at all cores (the reported value)
    and at one core; the oracle's time to 1e-4 relative error on the dim-4
    Gaussian (1e4/itn, one core) and the ridge (all cores); and per-
    evaluation rates on bounded subsets of the batched Lorentzian workload
    (32 of its 4096 integrals, 2 iterations each), the 8-d mixture (2
    iterations of 2^20) and the lattice scan (1 of its 64 couplings, 2
    iterations of 1e7), from which the full workloads' CPU times are
    extrapolated."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    import vegas_gb300 as vg
    cores = os.cpu_count() or 1
    st = O.State(DIM * [[0, 1]], NEVAL)
    t0 = time.perf_counter()
    ne = 0
    for k in range(iters):
        out = st.iterate(O.F_RIDGE, [RIDGE_M, RIDGE_S], seed=5, itn=k + 1, nthreads=cores)
        ne += out['neval']
    dt = time.perf_counter() - t0
    # one core, one iteration of the same workload
    st1 = O.State(DIM * [[0, 1]], NEVAL)
    t1 = time.perf_counter()
    ne1 = st1.iterate(O.F_RIDGE, [RIDGE_M, RIDGE_S], seed=6, itn=1, nthreads=1)['neval']
    t1 = time.perf_counter() - t1
    # the CPU-sized workload (dim 4 Gaussian, neval 1e4, FP64): seconds per
    # iteration of the reference algorithm on one core
    f1 = vg.Gaussian(a=100.0, c=0.5, dim=4)
    stg = O.State(4 * [[0, 1]], 10000)
    tg = time.perf_counter()
    for k in range(20):
        stg.iterate(O.F_GAUSS, f1.params(4), seed=5, itn=k + 1, nthreads=1)
    tg = (time.perf_counter() - tg) / 20
    tta = {'config1_gauss4_1core': _cpu_tta(O.State(4 * [[0, 1]], 10000), O.F_GAUSS, f1.params(4), 10, 7, 1,
                                            10.0, exact=f1.exact(4)),
           'config2_ridge_all_cores': _cpu_tta(O.State(DIM * [[0, 1]], NEVAL), O.F_RIDGE, [RIDGE_M, RIDGE_S], 5,
                                               8, cores, 15.0, exact=vg.Ridge(M=RIDGE_M, s=RIDGE_S).exact(DIM))}
    # bounded subsets of the larger workloads
    subsets = {}
    fs, nevals, dims = batch_workload()
    rng = np.random.default_rng(1)
    idx = rng.choice(len(fs), 32, replace=False)
    t3, n3 = time.perf_counter(), 0
    for i in idx:
        s3 = O.State(int(dims[i]) * [[0, 1]], int(nevals[i]))
        for k in range(2):
            n3 += s3.iterate(O.F_LORENTZ, fs[i].params(int(dims[i])), seed=9, itn=k + 1, nthreads=cores)['neval']
    t3 = time.perf_counter() - t3
    # the full launch's evaluations: nominal neval x 16 iterations, scaled by
    # the subset's actual / nominal ratio (the allocation rounds down)
    total3 = float(np.sum(nevals)) * 16 * n3 / (2.0 * float(np.sum(nevals[idx])))
    subsets['config3_batched_lorentz'] = {
        'sample': '32 of the 4096 integrals, 2 iterations each', 'evaluations': n3, 'seconds': t3,
        'evals_per_s': n3 / t3, 'extrapolated_seconds_full_launch': total3 / (n3 / t3),
        'full_launch_evaluations': total3}
    fm = mixture_integrand()
    s4 = O.State(MIX_DIM * [[0.0, 1.0]], MIX_NEVAL)
    t4, n4 = time.perf_counter(), 0
    for k in range(2):
        n4 += s4.iterate(O.F_MIXTURE, fm.params(MIX_DIM), seed=9, itn=k + 1, nthreads=cores)['neval']
    t4 = time.perf_counter() - t4
    subsets['config4_mixture_plain'] = {'sample': '2 iterations of 2^20', 'evaluations': n4, 'seconds': t4,
                                        'evals_per_s': n4 / t4}
    s5 = O.State(16 * [[-5.0, 5.0]], 10 ** 7)
    t5, n5 = time.perf_counter(), 0
    for k in range(2):
        n5 += s5.iterate(O.F_LATTICE, [0.5, 0.1], seed=9, itn=k + 1, nthreads=cores)['neval']
    t5 = time.perf_counter() - t5
    total5 = 64.0 * 16 * n5 / 2.0   # per-lambda actual evaluations of this sample
    subsets['config5_lattice_scan'] = {
        'sample': '1 of the 64 couplings (lambda 0.1), 2 iterations of 1e7', 'evaluations': n5, 'seconds': t5,
        'evals_per_s': n5 / t5, 'extrapolated_seconds_full_launch': total5 / (n5 / t5),
        'full_launch_evaluations': total5}
    return {'value': ne / dt, 'unit': 'evals/s', 'cores': cores, 'kind': kind,
            'sample': '%d full iterations of the ridge workload (neval=1e6 each), FP64, %d threads'
                      % (iters, cores),
            'one_core': {'value': ne1 / t1, 'unit': 'evals/s', 'sample': '1 iteration of 1e6, 1 thread'},
            'small_fp64_seconds_per_iteration_1core': tg,
            'time_to_1e-4': tta, 'subsets': subsets,
            'host': {'nproc': cores, 'machine': os.uname().machine}}


def reference_arm(args):
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    cores = os.cpu_count() or 1
    st = O.State(DIM * [[0, 1]], NEVAL)
    itn = 1
    for _ in range(args.warmup):
        st.iterate(O.F_RIDGE, [RIDGE_M, RIDGE_S], seed=5, itn=itn, nthreads=cores)
        itn += 1
    t0 = time.perf_counter()
    ne = 0
    for _ in range(args.steps):
        out = st.iterate(O.F_RIDGE, [RIDGE_M, RIDGE_S], seed=5, itn=itn, nthreads=cores)
        ne += out['neval']
        itn += 1
    dt = time.perf_counter() - t0
    v = ne / dt
    print(json.dumps({
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'evals/s', 'n_gpus': 0,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * dt / args.steps,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic', 'config': {'workload': WORKLOAD, 'neval_per_step': NEVAL},
        'cpu_baseline': {'value': v, 'unit': 'evals/s', 'cores': cores, 'kind': 'port',
                         'sample': 'each step one full iteration (neval=1e6), %d threads' % cores},
        'e2e': {'value': v, 'unit': 'evals/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }))


def main():
    args = parse()
    if args.impl == 'reference':
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == '__main__':
    main()
