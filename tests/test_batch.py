"""Batched launch (many integrals in one persistent kernel).

GPU tests: per-iteration parity with the single-integral fused path on the
same Philox streams (the kernels share the tile body: first iteration 1e-6
relative -- FP32 rounding of the two compilations, FP64 summation order;
later iterations 1e-4, the maps being adapted from FP32 histograms summed in
nondeterministic atomic order), agreement with the closed
form of Lorentzian products (|pull| < 5 per integral, mean pull^2 < 3), and a
CUDA-graph replay.  CPU test: the job-table size and variant count."""
import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300 import _native as N


def _lorentz(rng, dim):
    c = rng.uniform(0.2, 0.8, dim)
    w = np.exp(rng.uniform(np.log(0.01), np.log(0.1), dim))
    return vg.LorentzianProduct(c, w)


def test_batch_abi_sizes():
    L = N.load()
    assert L.vg_batch_variants() >= 2
    assert L.vg_batch_table_bytes(10) > L.vg_batch_table_bytes(1) > 0


@pytest.mark.gpu
@pytest.mark.parametrize('variant', [0, 1, 2])
def test_batch_matches_single_integral_path(variant):
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(3)
    dims, nevals = [3, 5, 9, 4], [10000, 30000, 20000, 50000]
    fs = [_lorentz(rng, d) for d in dims]
    B = BatchIntegrator(fs, nevals, nitn=4, nwarm=1, seed=77, variant=variant)
    B.run()
    torch.cuda.synchronize()
    out = B.iterations()
    for j, (f, d, ne) in enumerate(zip(fs, dims, nevals)):
        I = vg.Integrator(d * [[0, 1]], neval=ne, seed=77)
        I._stream_id = j
        for k in range(4):
            r = I(f, nitn=1)
            m, s = r.itn_results[-1].mean, r.itn_results[-1].sdev
            # first iteration: same samples; the FP32 arithmetic of the two
            # compiled kernels may round differently (contraction into FMAs
            # differs between instantiations), sums differ in FP64 order.
            # Later iterations start from maps adapted on FP32 shared-memory
            # histograms whose atomic-add order differs from run to run.
            tol = 1e-6 if k == 0 else 1e-4
            if k == 0:   # same allocation (uniform sigf): same evaluation count
                assert int(out[j, k, 2]) == I.last_neval
            assert abs(out[j, k, 0] - m) <= tol * abs(m), (j, k, out[j, k, 0], m)
            assert abs(out[j, k, 1] - s * s) <= tol * 10 * s * s, (j, k)


@pytest.mark.gpu
def test_batch_accuracy_and_graph_replay():
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(11)
    nj = 64
    dims = rng.integers(3, 10, nj)
    nevals = np.exp(rng.uniform(np.log(1e4), np.log(1e5), nj)).astype(np.int64)
    fs = [_lorentz(rng, int(d)) for d in dims]
    B = BatchIntegrator(fs, nevals, nitn=16, nwarm=8, seed=5)
    res = B.run(graph=True)
    torch.cuda.synchronize()
    exact = np.array([f.exact(int(d)) for f, d in zip(fs, dims)])
    pulls = (res[:, 0] - exact) / res[:, 1]
    assert np.all(np.isfinite(pulls))
    assert np.max(np.abs(pulls)) < 5, pulls
    assert np.mean(pulls ** 2) < 3, np.mean(pulls ** 2)
    res2 = B.run(graph=True)   # replay continues from the adapted state
    torch.cuda.synchronize()
    pulls2 = (res2[:, 0] - exact) / res2[:, 1]
    assert np.max(np.abs(pulls2)) < 5
    assert np.median(res2[:, 1]) <= np.median(res[:, 1]) * 1.5


@pytest.mark.gpu
def test_batch_group_mode_matches_queue_mode():
    """Cooperative groups of CTAs per integral give the queue mode's first
    iteration (same samples) and the closed-form answers (groups need the
    integrals of one dimension bucket)."""
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(21)
    dims, nevals = [5, 6, 8], [200000, 300000, 100000]
    fs = [_lorentz(rng, d) for d in dims]
    A = BatchIntegrator(fs, nevals, nitn=6, nwarm=2, seed=8, variant=0, group=1)
    B = BatchIntegrator(fs, nevals, nitn=6, nwarm=2, seed=8, variant=0, group=2)
    ra, rb = A.run(), B.run()
    oa, ob = A.iterations(), B.iterations()
    assert np.allclose(oa[:, 0, 0], ob[:, 0, 0], rtol=1e-6, atol=0)
    exact = np.array([f.exact(d) for f, d in zip(fs, dims)])
    for r in (ra, rb):
        assert np.max(np.abs((r[:, 0] - exact) / r[:, 1])) < 5
    with pytest.raises(ValueError):
        BatchIntegrator([_lorentz(rng, 3), _lorentz(rng, 6)], [10000, 10000], nitn=2, nwarm=1,
                        variant=0, group=2)


@pytest.mark.gpu
def test_batch_lattice_scan_against_transfer_matrix():
    """A small lambda scan of the periodic lattice action (dim 4 on
    [-5, 5]^4) in group mode, against the FP64 transfer-matrix value."""
    from vegas_gb300.batch import BatchIntegrator
    lams = np.exp(np.linspace(np.log(0.01), np.log(1.0), 8))
    fs = [vg.LatticeAction(0.5, float(l)) for l in lams]
    B = BatchIntegrator(fs, [200000] * len(fs), nitn=12, nwarm=6, seed=3, dims=[4] * len(fs),
                        limits=(-5.0, 5.0))
    res = B.run()
    exact = np.array([f.exact(4) for f in fs])
    pulls = (res[:, 0] - exact) / res[:, 1]
    assert np.max(np.abs(pulls)) < 5, pulls
