"""Checkpoints shared with the reference (src/vegas/_vegas.pyx:150-167, 1194-1211).

CPU (development container, where the compiled reference exists; skipped
elsewhere): a map and an integrator trained by the reference load into this
package with bit-identical grid, strata and sigf, and this package's
pickles in the reference's class names load back into the reference the
same way.  GPU: a trained integrator written in the reference's format and
read back equals the one restored from this package's own pickle, and keeps
integrating.
"""
import pickle

import numpy as np
import pytest

import vegas_gb300 as vg
from vegas_gb300 import checkpoint


def _ref():
    try:
        import build_ref
        if not build_ref.built():
            return None
        return build_ref.import_reference()
    except Exception:
        return None


def _peak(x):
    x = np.asarray(x)
    return np.exp(-30.0 * np.sum((x - 0.4) ** 2, axis=1))


def _valid(m):
    g = np.asarray(m.grid)
    return [list(g[d, :int(m.ninc[d]) + 1]) for d in range(len(m.ninc))]


def _trained_reference(v):
    f = v.lbatchintegrand(_peak)
    # neval 1000: the default neval a pickled integrator is first rebuilt
    # with, so restoring it regrids nothing (and runs no device kernel)
    I = v.Integrator(3 * [[0, 1]], neval=1000, ran_array_generator=np.random.default_rng(3).random)
    I(f, nitn=4)
    I.set(ran_array_generator=None)
    return I


def test_reference_checkpoint_loads_here():
    v = _ref()
    if v is None:
        pytest.skip('compiled reference not available here')
    R = _trained_reference(v)
    m = checkpoint.loads(pickle.dumps(R.map), device='cpu')
    assert isinstance(m, vg.AdaptiveMap)
    assert _valid(m) == _valid(R.map)
    I = checkpoint.loads(pickle.dumps(R), device='cpu')
    assert isinstance(I, vg.Integrator)
    assert list(I.nstrat) == list(R.nstrat)
    assert list(I.map.ninc) == list(R.map.ninc)
    assert _valid(I.map) == _valid(R.map)
    assert np.array_equal(I.sigf, np.asarray(R.sigf))
    for k in ('neval', 'nitn', 'alpha', 'beta', 'neval_frac', 'max_neval_hcube', 'adapt'):
        assert getattr(I, k) == getattr(R, k), k


def test_checkpoint_written_here_loads_in_reference():
    v = _ref()
    if v is None:
        pytest.skip('compiled reference not available here')
    R = _trained_reference(v)
    mine = checkpoint.loads(pickle.dumps(R), device='cpu')
    back = pickle.loads(checkpoint.dumps_reference(mine))
    assert type(back) is v.Integrator
    assert list(back.nstrat) == list(R.nstrat)
    assert _valid(back.map) == _valid(R.map)
    assert np.array_equal(np.asarray(back.sigf), np.asarray(R.sigf))
    m = pickle.loads(checkpoint.dumps_reference(mine.map))
    assert type(m) is v.AdaptiveMap
    assert _valid(m) == _valid(R.map)


def test_reference_format_without_reference_module(monkeypatch):
    """Written with placeholder classes when the reference is not importable;
    the module table is left as it was."""
    import importlib
    import sys

    real = importlib.import_module

    def no_reference(name, *a, **k):
        if name.startswith('vegas'):
            raise ImportError(name)
        return real(name, *a, **k)

    monkeypatch.setattr(checkpoint.importlib, 'import_module', no_reference)
    before = {k: sys.modules.get(k) for k in ('vegas', 'vegas._vegas')}
    m = vg.AdaptiveMap([[0.0, 0.25, 1.0], [1.0, 2.0, 4.0, 8.0]], device='cpu')
    data = checkpoint.dumps_reference(m)
    assert b'vegas._vegas' in data and b'AdaptiveMap' in data
    assert {k: sys.modules.get(k) for k in before} == before
    m2 = checkpoint.loads(data, device='cpu')
    assert _valid(m2) == _valid(m)


@pytest.mark.gpu
def test_reference_format_round_trip_gpu():
    I = vg.Integrator(4 * [[0, 1]], neval=20000, seed=3)
    I(vg.Gaussian(), nitn=5)
    J = checkpoint.loads(checkpoint.dumps_reference(I))
    K = pickle.loads(pickle.dumps(I))
    assert list(J.nstrat) == list(K.nstrat) == list(I.nstrat)
    assert np.array_equal(J.map.grid, K.map.grid)
    assert np.array_equal(J.sigf, K.sigf)
    r = J(vg.Gaussian(), nitn=3)
    assert abs(r.mean - vg.Gaussian().exact(4)) < 5 * r.sdev
