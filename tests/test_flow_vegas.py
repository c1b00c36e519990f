"""Flow-augmented vegas+ (FlowIntegrator) on the GPU.

* gain: on the non-separable 8-d mixture of 4 Gaussians, the trained
  flow's variance per evaluation is >= 5x below that of the same vegas+
  map and stratification without the flow (the method without the
  network), and below that of plain vegas+ given the same number of
  iterations (whose map keeps adapting).  The FP32 training histogram is
  summed with atomics, so plain vegas+'s maps -- and its variance on this
  multimodal integrand, which ranges over an order of magnitude -- differ
  from run to run; the frozen-map comparison shares the flow's base and is
  the stable measure of what the network adds;
* unbiasedness: the flow iterations' weighted average agrees with the exact
  integral within 5 sigma (every sample carries the flow's exact logdet);
* gate: on an integrand plain vegas+ integrates exactly (a constant), the
  flow cannot win and is switched off, after which plain vegas+ continues.
"""
import numpy as np
import pytest
import torch

import vegas_gb300 as vg

pytestmark = pytest.mark.gpu


def _mixture(dim=8, seed=4):
    rng = np.random.default_rng(seed)
    return vg.GaussianMixture(rng.uniform(0.15, 0.85, (4, dim)), sigma=0.03)


def test_flow_beats_plain_vegas_on_mixture():
    from vegas_gb300.flow_vegas import FlowIntegrator
    f = _mixture()
    exact = f.exact(8)
    neval = 1 << 18
    plain = vg.Integrator(8 * [[0, 1]], neval=neval, seed=11)
    plain(f, nitn=50)
    rp = plain(f, nitn=10)
    v_plain = np.median([r.sdev ** 2 for r in rp.itn_results]) * plain.last_neval
    # the training schedule of the benchmark (30 of the 100 training
    # iterations on the KL loss, 2 Adam steps each): the shorter 40 x 6-step
    # schedule left the flow short of the 5x gain in about one run in four
    F = FlowIntegrator(8 * [[0, 1]], neval=neval, seed=11, plain_itn=10, kl_itn=30, train_itn=100,
                       grace=1000, train_steps=2, train_batch=1 << 15)
    F(f, nitn=110)                     # 10 plain + 100 training flow iterations
    rf = F(f, nitn=20)                 # frozen flow
    assert F.flow_on
    # medians over 20 iterations each (a median of 10 variance estimates
    # moves by about 15 % with the rounding of the training run)
    v_flow = np.median([h['sdev'] ** 2 * h['neval'] for h in F.history[-20:]])
    # the same map and strata without the flow: plain vegas+ continued from
    # the integrator the flow was inserted into, map frozen (alpha = 0)
    base = vg.Integrator(F.vegas, alpha=0.0, seed=12)
    base(f, nitn=10)
    rb = base(f, nitn=20)
    v_base = np.median([r.sdev ** 2 for r in rb.itn_results]) * base.last_neval
    assert v_flow * 5 <= v_base, (v_flow, v_base, v_plain)
    assert v_flow <= v_plain, (v_flow, v_plain)
    assert abs(rf.mean - exact) < 5 * rf.sdev, (rf.mean, rf.sdev, exact)


def test_flow_switched_off_when_plain_vegas_wins():
    from vegas_gb300.flow_vegas import FlowIntegrator
    F = FlowIntegrator(4 * [[0, 1]], neval=20000, seed=3, plain_itn=4, kl_itn=2, grace=2, patience=2,
                       train_steps=1, train_batch=4096)
    r = F(vg.Constant(2.0), nitn=14)
    assert F.flow_dead and not F.flow_on
    assert abs(r.mean - 2.0) < 1e-6
    assert not F.history[-1]['flow']


@pytest.mark.gpu
def test_flow_on_lattice_is_unbiased():
    """The flow in vegas's y-space on the dim-16 lattice action (one coupling
    of the lambda scan): every flow iteration carries the flow's exact
    log-determinant, so the average of the flow iterations agrees with the
    FP64 transfer-matrix value (within 5 sigma), trained or not."""
    from vegas_gb300.flow_vegas import FlowIntegrator
    f = vg.LatticeAction(0.5, 0.05)
    ex = f.exact(16)
    fi = FlowIntegrator(16 * [[-5.0, 5.0]], neval=1 << 18, seed=21, plain_itn=20, kl_itn=5, train_itn=15,
                        grace=100, patience=3, train_steps=2, train_batch=1 << 13)
    fi(f, nitn=50)
    flows = [h for h in fi.history if h['flow']]
    assert len(flows) == 30
    w = np.array([1.0 / h['sdev'] ** 2 for h in flows[-15:]])
    m = np.array([h['mean'] for h in flows[-15:]])
    mean = float(np.sum(w * m) / np.sum(w))
    sdev = float(np.sum(w) ** -0.5)
    assert abs(mean - ex) < 5 * sdev, (mean, sdev, ex)
