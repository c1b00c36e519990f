"""restratify: strata moved between directions of y (src/vegas/__init__.py:1313-1592).

Golden fixture: tests/golden/ref_restratify.npz, made by running the
reference's own ``restratify`` (make_golden.py restratify) in injected-sample
mode on a trained dim-6 integrator.

CPU: the weights and the new strata from the reference's I / dI (exact
integers; weights <= 1e-12 relative).  GPU (FP64, the same injected
uniforms): the whole ``restratify`` call -- I, dI, weights, Q at 1e-9
relative (the integrand is evaluated by torch instead of numpy), the new
strata bit-exact, the training iterations and the final grid at 1e-9.
FP32 with Philox draws: strata concentrate in the directions that matter
and the integral stays within 5 sigma of the exact value.
"""
import math
import os

import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300 import _gvar as gv
from vegas_gb300.restratify import _new_nstrat

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
U_SCALE = 2.0 ** -24
# the generator's cases (make_golden.RESTRAT_CASES)
CASES = [
    dict(seed=11, train=dict(nitn=4), args=dict(nitn=2, ndy=5)),
    dict(seed=12, train=dict(nitn=3), args=dict(nitn=1, ndy=4, below_avg_nstrat=1, gamma=0.5)),
]


def gold():
    return dict(np.load(os.path.join(GOLD, 'ref_restratify.npz')))


def rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


class Draws(object):
    """The fixture's injected uniforms: u = k / 2^24, k from default_rng(seed)."""

    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)

    def __call__(self, size):
        return self.rng.integers(0, 2 ** 24, size=size, dtype=np.uint32).astype(np.float64) * U_SCALE


@vg.lbatchintegrand
def restrat_f(x):
    return torch.exp(-40.0 * (x[:, 0] - 0.3) ** 2 - 25.0 * (x[:, 1] - 0.6) ** 2) * (1.0 + 0.2 * x[:, 2])


def weights_from(I, dI, ndy):
    """GVar weights exactly as restratify forms them, from independent GVars."""
    gI = gv.gvar(I[0], I[1])
    dIavg = gI / ndy
    out = []
    for mu in range(dI[0].shape[0]):
        row = gv.gvar(dI[0][mu], dI[1][mu])
        out.append(np.sum((row - dIavg) ** 2) * ndy)
    return out


@pytest.mark.parametrize('c', [0, 1])
def test_weights_and_strata_from_reference_integrals(c):
    g = gold()
    p = 'c%d_' % c
    a = CASES[c]['args']
    w = weights_from(g[p + 'I'], (g[p + 'dI_mean'], g[p + 'dI_sdev']), a['ndy'])
    assert rel([x.mean for x in w], g[p + 'weight_mean']) <= 1e-12
    assert rel([x.sdev for x in w], g[p + 'weight_sdev']) <= 1e-12
    ns = _new_nstrat(w, g[p + 'nstrat_before'], a.get('gamma', 1.0), a.get('below_avg_nstrat'),
                     g[p + 'nstrat_before'])
    assert np.array_equal(ns, g[p + 'nstrat_after'])


def test_new_strata_edge_cases():
    old = np.array([3, 3, 3, 3], np.int64)
    # equal weights: strata unchanged
    assert list(_new_nstrat([1.0] * 4, old, 1.0, None, old)) == [3, 3, 3, 3]
    # one direction dominant: all strata move there, others floor at 1
    ns = _new_nstrat([1.0, 1e-6, 1e-6, 1e-6], old, 1.0, None, old)
    assert ns[1:].tolist() == [1, 1, 1] and ns[0] >= 27
    # gamma = 0: no change
    assert list(_new_nstrat([5.0, 1.0, 0.1, 2.0], old, 0.0, None, old)) == [3, 3, 3, 3]


@pytest.mark.gpu
@pytest.mark.parametrize('c', [0, 1])
def test_restratify_matches_reference_fp64(c):
    g = gold()
    p = 'c%d_' % c
    case = CASES[c]
    draws = Draws(case['seed'])
    integ = vg.Integrator(6 * [[0, 1]], neval=4000, alpha=0.5, precision='fp64',
                          ran_array_generator=draws)
    assert list(integ.nstrat) == list(g[p + 'nstrat_before'])
    r0 = integ(restrat_f, **case['train'])
    assert rel(r0.mean, g[p + 'train_mean']) <= 1e-9
    R = vg.restratify(integ, restrat_f, **case['args'])
    assert rel([R.I.mean, R.I.sdev], g[p + 'I']) <= 1e-9
    assert rel([[x.mean for x in row] for row in R.dI], g[p + 'dI_mean']) <= 1e-9
    assert rel([[x.sdev for x in row] for row in R.dI], g[p + 'dI_sdev']) <= 1e-9
    assert rel([x.mean for x in R.weight], g[p + 'weight_mean']) <= 1e-9
    assert rel([x.sdev for x in R.weight], g[p + 'weight_sdev']) <= 1e-9
    if np.isnan(g[p + 'Q']):
        assert np.isnan(R.Q)
    else:
        assert abs(R.Q - float(g[p + 'Q'])) <= 1e-9
    assert np.array_equal(np.asarray(R.nstrat), g[p + 'nstrat_after'])
    assert R.neval == int(g[p + 'neval_after'])
    want = g[p + 'grid_after']
    ok = ~np.isnan(want)
    assert np.max(np.abs(R.map.grid[ok] - want[ok])) <= 1e-9
    assert rel(R.sum_sigf, g[p + 'sum_sigf_after']) <= 1e-9
    # the integrator keeps integrating with the new strata
    r1 = R(restrat_f, nitn=1)
    assert math.isfinite(r1.mean) and r1.sdev > 0


@pytest.mark.gpu
def test_restratify_fp32_concentrates_strata():
    dim = 8
    exact = (math.sqrt(math.pi / 40.0) * (math.erf(math.sqrt(40.0) * 0.7) + math.erf(math.sqrt(40.0) * 0.3)) / 2
             * math.sqrt(math.pi / 25.0) * (math.erf(5.0 * 0.4) + math.erf(5.0 * 0.6)) / 2 * 1.1)
    integ = vg.Integrator(dim * [[0, 1]], neval=200000, seed=7)
    integ(restrat_f, nitn=6)
    before = integ(restrat_f, nitn=4)
    R = vg.restratify(integ, restrat_f, nitn=2)
    ns = np.asarray(R.nstrat)
    assert ns[0] > 4 and ns[1] > 4
    assert np.all(ns[3:] == 1)
    after = R(restrat_f, nitn=4)
    assert abs(after.mean - exact) < 5 * after.sdev
    assert abs(before.mean - exact) < 5 * before.sdev
    assert after.sdev < before.sdev
