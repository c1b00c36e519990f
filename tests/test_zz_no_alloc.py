"""vg_iteration_noalloc: a full vegas+ iteration whose scratch is a static
device array, for callers that cannot allocate device memory (plug-ins whose
host owns every device byte, services under a device-memory budget, callers
that must not allocate on their iteration path).

Checked through the C ABI against the ordinary path (vg_allocate +
vg_fused_iteration + vg_end_iteration with a caller workspace) on two calls
in a row, both paths starting each call from the same state, in both
precision modes.  FP64: the tolerance of the other FP64 parity tests (1e-12
relative).  FP32 (which also uses the FP32 grid table and the split
evaluation buffer of the scratch): the iteration sums are deterministic
(static per-tile partials summed in a fixed order), 1e-12 as well; the
adapted grid comes from an FP32 training histogram summed with atomics in
arrival order, so it is compared at 1e-5 relative, the FP32 first-iteration
tolerance of the batched tests widened by the adapt's cumulative sums.
This file is collected last so that a failure here does not hide any other
test."""
import ctypes

import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300 import _native as N

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def _state(I):
    return (I.map.grid_tensor.clone(), I.map.inc_tensor.clone(), I._sigf.clone(), I.sum_sigf)


def _load(I, st):
    g, inc, sigf, ss = st
    I.map.grid_tensor.copy_(g)
    I.map.inc_tensor.copy_(inc)
    I._sigf.copy_(sigf)
    I.sum_sigf = ss


def _rel(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize('precision', ['fp32', 'fp64'])
def test_noalloc_matches_workspace_path(precision):
    L = N.load()
    f = vg.Ridge(M=200, s=0.02)
    params = N.dbl_array(f.params(4))
    ref = vg.Integrator(4 * [[0, 1]], neval=20000, precision=precision, seed=31)
    new = vg.Integrator(4 * [[0, 1]], neval=20000, precision=precision, seed=31)
    grid_tol = RTOL if precision == 'fp64' else 1e-5
    stream = N.stream_ptr(ref.device)
    for call in range(2):
        _load(new, _state(ref))
        it_r, _ = ref._struct()
        ref._put_sum_sigf()
        N.check(L.vg_allocate(ctypes.byref(it_r), stream))
        N.check(L.vg_fused_iteration(ctypes.byref(it_r), call + 1, None, f.kind, params, 2, stream))
        N.check(L.vg_end_iteration(ctypes.byref(it_r), stream))
        st_r = ref._read_stats()
        it_n, _ = new._struct()
        it_n.work = None          # the no-alloc entry point must not need a workspace
        it_n.work_bytes = 0
        new._put_sum_sigf()
        N.check(L.vg_iteration_noalloc(ctypes.byref(it_n), call + 1, None, f.kind, params, 2,
                                       stream))
        st_n = new._read_stats()
        assert st_n.status == 0 and st_n.neval == st_r.neval
        assert _rel(st_n.mean, st_r.mean) <= RTOL
        assert _rel(st_n.var, st_r.var) <= RTOL
        assert _rel(st_n.sum_sigf, st_r.sum_sigf) <= RTOL
        assert _rel(new.sigf, ref.sigf) <= RTOL
        g_n, g_r = new.map.grid, ref.map.grid
        assert np.max(np.abs(g_n - g_r)) <= grid_tol * np.max(np.abs(g_r))
        ref.sum_sigf = float(st_r.sum_sigf)


def test_noalloc_rejects_oversized_iteration():
    L = N.load()
    big = vg.Integrator(4 * [[0, 1]], neval=int(2e7), seed=5)
    it, _ = big._struct()
    it.work = None
    it.work_bytes = 0
    assert L.vg_workspace_bytes(ctypes.byref(it), 0) > N.VG_NOALLOC_SCRATCH_BYTES
    with pytest.raises(MemoryError):
        N.check(L.vg_iteration_noalloc(ctypes.byref(it), 1, None, N.VG_F_GAUSS,
                                       N.dbl_array([100.0, 0.5, 1.0]), 3,
                                       N.stream_ptr(big.device)))
