"""Bounded device-side waits give up with a status the host reads, and the
context stays usable (no fault, no hang).

vg_set_wait_budget(0) gives every wait a budget of zero polls, so a wait
that finds its flag unset gives up at once -- deterministically, with no
spinning: the allocation's look-back (a block reads its predecessors'
published totals) and the batched launch's group barriers (a CTA waits for
the other CTAs of its integral).  The iteration then reports VG_ERR_TIMEOUT
(vegas_gb300._native.VegasTimeout) and schedules no work; with the default
budget restored, the next iterations are correct.  No counterpart in the
reference (no device waits); it raises exceptions for its own failures
(pyx:2133-2134, 1355-1356)."""
import numpy as np
import pytest

import vegas_gb300 as vg
from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_allocation_lookback_wait_gives_up_then_recovers():
    L = N.load()
    f = vg.Gaussian(a=40.0, c=0.5, dim=4)
    I = vg.Integrator(4 * [[0, 1]], neval=200000, seed=12)
    assert I.nhcube > 4 * 1024          # several allocation blocks: some must look back
    N.check(L.vg_set_wait_budget(0))
    try:
        with pytest.raises(N.VegasTimeout):
            I(f, nitn=1)
    finally:
        N.check(L.vg_set_wait_budget(-1))
    I2 = vg.Integrator(4 * [[0, 1]], neval=200000, seed=12)
    r = I2(f, nitn=4)
    assert abs(r.mean - f.exact(4)) < 5 * r.sdev, r


def test_batch_group_barrier_gives_up_then_recovers():
    from vegas_gb300.batch import BatchIntegrator
    rng = np.random.default_rng(5)
    fs = [vg.LorentzianProduct(rng.uniform(0.3, 0.7, 4), np.full(4, 0.05)) for _ in range(4)]
    L = N.load()
    N.check(L.vg_set_wait_budget(0))
    try:
        B = BatchIntegrator(fs, [20000] * 4, nitn=2, nwarm=1, seed=3, variant=0, group=2)
    finally:
        N.check(L.vg_set_wait_budget(-1))
    assert B.group == 2
    with pytest.raises(N.VegasTimeout):
        B.run()
    B.status.zero_()
    B.set_variant(B.variant)            # job table rebuilt with the default budget
    res = B.run()
    for k, fk in enumerate(fs):
        assert abs(res[k, 0] - fk.exact(4)) < 6 * res[k, 1], (k, res[k])
