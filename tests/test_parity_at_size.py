"""Parity at the benchmark sizes, and the batched launch against the oracle.

1. The vegas+ ridge workload at its full size (dim 4, M = 1000 Gaussians of
   width 0.01, neval = 1e6: 123462 hypercubes, ninc [988, 988, 988, 990]) in
   FP64 with Philox draws, against the oracle on the same draws.  At this
   size the single-pass allocation's look-back spans about 120 blocks and
   thousands of hypercubes are cut by tile boundaries and merged across
   tiles -- paths the small parity cases never reach.  Each iteration starts
   the GPU from the oracle's state; neval_h is compared bit-exactly with the
   oracle's allocation from the same sigf (pyx:1692-1710), the iteration's
   mean and variance, sum_sigf, sigf and the adapted grid at 1e-12 relative
   (pyx:2136-2217, 467-594).  sigf is compared at 1e-12 relative to
   max(|sigf|, 1e-100): below that the hypercube's variance is a sum of
   squares in the FP64 subnormal range, where relative precision is lost in
   any summation order.

2. The batched launch in its FP64 parity configuration (the same
   allocation, tile body, cut-hypercube merge and adapt as the single
   integral FP64 path, run by one CTA per integral inside the persistent
   kernel): integrals of dims 3 to 8 in both dimension buckets, each
   iteration against the oracle on the same Philox stream (integral j =
   stream j) -- neval_h bit-exact from the same sigf, mean / variance /
   sigf / sum_sigf / grid at 1e-12.
"""
import os

import numpy as np
import pytest
import torch

import oracle as O
import vegas_gb300 as vg

pytestmark = pytest.mark.gpu
RTOL = 1e-12
NTHREADS = os.cpu_count() or 1


def rel(a, b, floor=1e-300):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def set_state(I, grid, sigf, sum_sigf):
    g = torch.from_numpy(np.nan_to_num(grid)).to(I.device)
    I.map._grid.copy_(g)
    I.map._inc.copy_(torch.diff(g, dim=1))
    I._sigf.copy_(torch.from_numpy(np.asarray(sigf, float)).to(I.device))
    I.sum_sigf = float(sum_sigf)


def oracle_alloc(st, sigf, sum_sigf):
    """The oracle's allocation (neval_h per hypercube) from a given sigf."""
    adaptive = st.beta > 0 and st.H > 1
    nsf = st.neval_frac * st.neval / sum_sigf if (st.beta > 0 and sum_sigf > 0) else 0.0
    nh, rng, tot = O.alloc(sigf, nsf, adaptive, st.min_neval_hcube, st.max_neval_hcube,
                           int(float(st.neval) / float(st.H)))
    return nh, rng, tot


def test_ridge_full_size_fp64_matches_oracle():
    f = vg.Ridge(M=1000, s=0.01)
    seed = 2024
    I = vg.Integrator(4 * [[0, 1]], neval=1000000, precision='fp64', seed=seed)
    st = O.State(4 * [[0, 1]], 1000000)
    assert list(st.nstrat) == [19, 19, 19, 18] and st.H == 123462
    assert list(I.nstrat) == list(st.nstrat)
    assert list(I.map.ninc) == list(st.ninc) == [988, 988, 988, 990]
    for itn in range(1, 3):
        set_state(I, st.grid, st.sigf, st.sum_sigf)
        nh_want, rng_want, tot_want = oracle_alloc(st, st.sigf.copy(), st.sum_sigf)
        r = I(f, nitn=1)
        out = st.iterate(f.kind, f.params(4), seed=seed, stream=0, itn=itn, nthreads=NTHREADS)
        assert I.last_neval == out['neval'] == tot_want
        assert list(I.neval_hcube_range) == list(out['range']) == list(rng_want)
        nh = I._neval_h_host()
        assert np.array_equal(nh, nh_want), int(np.sum(nh != nh_want))
        assert rel(r.itn_results[0].mean, out['mean']) <= RTOL
        assert rel(r.itn_results[0].var, out['var']) <= RTOL
        assert rel(I.sum_sigf, st.sum_sigf) <= RTOL
        assert rel(I.sigf, st.sigf, floor=1e-100) <= RTOL
        g = I.map.grid
        for d in range(4):
            K = st.ninc[d]
            assert np.max(np.abs(g[d, :K + 1] - st.grid[d, :K + 1])) <= RTOL


def _lorentz(rng, dim):
    c = rng.uniform(0.2, 0.8, dim)
    w = np.exp(rng.uniform(np.log(0.01), np.log(0.1), dim))
    return vg.LorentzianProduct(c, w)


def test_batch_fp64_matches_oracle():
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(17)
    dims = [3, 4, 5, 8, 6]
    nevals = [3000, 40000, 12000, 60000, 250000]
    fs = [_lorentz(rng, d) for d in dims]
    seed = 4321
    B = BatchIntegrator(fs, nevals, nitn=1, nwarm=0, seed=seed, precision='fp64')
    sts = [O.State(d * [[0, 1]], ne) for d, ne in zip(dims, nevals)]
    for j, s in enumerate(sts):
        assert list(B.nstrat[j]) == list(s.nstrat)
        assert list(B.ninc[j]) == list(s.ninc)
    for itn in range(1, 4):
        want = []
        for j, s in enumerate(sts):       # every integral starts from the oracle's state
            v = B.state(j)
            K = int(v['grid'].shape[1]) - 1
            v['grid'].copy_(torch.from_numpy(np.nan_to_num(s.grid[:, :K + 1])))
            v['inc'].copy_(torch.from_numpy(np.nan_to_num(s.inc[:, :K])))
            v['sigf'].copy_(torch.from_numpy(s.sigf))
            B.put_sum_sigf(j, s.sum_sigf)
            want.append(oracle_alloc(s, s.sigf.copy(), s.sum_sigf))
        B.launch()
        torch.cuda.synchronize()
        assert int(B.status.item()) == 0
        out = B.iterations()
        for j, (f, d, s) in enumerate(zip(fs, dims, sts)):
            o = s.iterate(f.kind, f.params(d), seed=seed, stream=j, itn=itn, nthreads=NTHREADS)
            nh_want, rng_want, tot_want = want[j]
            rec = B.read_stats(j)
            v = B.state(j)
            assert rec.status == 0
            assert rec.neval == o['neval'] == tot_want == int(out[j, 0, 2]), (j, itn)
            assert (rec.range_lo, rec.range_hi) == tuple(o['range']) == tuple(rng_want)
            nh = v['neval_h'].cpu().numpy().astype(np.int64)
            assert np.array_equal(nh, nh_want), (j, itn, int(np.sum(nh != nh_want)))
            assert rel(out[j, 0, 0], o['mean']) <= RTOL, (j, itn, out[j, 0, 0], o['mean'])
            assert rel(out[j, 0, 1], o['var']) <= RTOL, (j, itn)
            assert rel(rec.sum_sigf, s.sum_sigf) <= RTOL
            assert rel(v['sigf'].cpu().numpy(), s.sigf, floor=1e-100) <= RTOL
            g = v['grid'].cpu().numpy()
            for k in range(d):
                K = s.ninc[k]
                assert np.max(np.abs(g[k, :K + 1] - s.grid[k, :K + 1])) <= RTOL, (j, itn, k)


def test_batch_fp64_group_mode_matches_oracle():
    """The batched launch's cooperative group mode (G CTAs share each
    integral's tiles; two bounded group barriers per iteration; the
    finalize merges G partial sums) in the FP64 configuration against the
    oracle: integrals of one dimension bucket, neval_h bit-exact, mean /
    variance / sigf / grid at 1e-12."""
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(23)
    dims = [5, 6, 7, 8]
    nevals = [30000, 80000, 50000, 120000]
    fs = [_lorentz(rng, d) for d in dims]
    seed = 99
    B = BatchIntegrator(fs, nevals, nitn=1, nwarm=0, seed=seed, precision='fp64', group=3)
    assert B.group == 3
    sts = [O.State(d * [[0, 1]], ne) for d, ne in zip(dims, nevals)]
    for itn in range(1, 3):
        want = []
        for j, s in enumerate(sts):
            v = B.state(j)
            K = int(v['grid'].shape[1]) - 1
            v['grid'].copy_(torch.from_numpy(np.nan_to_num(s.grid[:, :K + 1])))
            v['inc'].copy_(torch.from_numpy(np.nan_to_num(s.inc[:, :K])))
            v['sigf'].copy_(torch.from_numpy(s.sigf))
            B.put_sum_sigf(j, s.sum_sigf)
            want.append(oracle_alloc(s, s.sigf.copy(), s.sum_sigf))
        B.launch()
        torch.cuda.synchronize()
        assert int(B.status.item()) == 0
        out = B.iterations()
        for j, (f, d, s) in enumerate(zip(fs, dims, sts)):
            o = s.iterate(f.kind, f.params(d), seed=seed, stream=j, itn=itn, nthreads=NTHREADS)
            nh_want, rng_want, tot_want = want[j]
            rec = B.read_stats(j)
            v = B.state(j)
            assert rec.neval == o['neval'] == tot_want, (j, itn)
            assert np.array_equal(v['neval_h'].cpu().numpy().astype(np.int64), nh_want)
            assert rel(out[j, 0, 0], o['mean']) <= RTOL, (j, itn, out[j, 0, 0], o['mean'])
            assert rel(out[j, 0, 1], o['var']) <= RTOL, (j, itn)
            assert rel(v['sigf'].cpu().numpy(), s.sigf, floor=1e-100) <= RTOL
            g = v['grid'].cpu().numpy()
            for k in range(d):
                K = s.ninc[k]
                assert np.max(np.abs(g[k, :K + 1] - s.grid[k, :K + 1])) <= RTOL, (j, itn, k)
