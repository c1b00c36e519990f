"""AdaptiveMap.invmap and adapt_to_samples on the GPU (pyx:362-413, 728-790)
against golden vectors recorded from the compiled reference
(tests/golden/make_golden.py): invmap bit-exact in FP64 (same operation
order, correctly rounded divisions), adapt_to_samples' final grid within
1e-12 of the largest node (the device histogram and scans sum in a
different order)."""
import os

import numpy as np
import pytest
import torch

import vegas_gb300 as vg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def make_map(grid, ninc):
    g = np.nan_to_num(grid)
    return vg.AdaptiveMap([list(g[d, :ninc[d] + 1]) for d in range(len(ninc))])


def test_invmap_golden_fp64():
    c = load('ref_invmap.npz')
    m = make_map(c['inv_grid'], c['inv_ninc'])
    x = c['inv_x']
    y = np.empty_like(x)
    jac = np.empty(len(x))
    m.invmap(x, y, jac)
    assert np.array_equal(y, c['inv_y'])
    assert np.array_equal(jac, c['inv_jac'])
    # device tensors in place, and map(invmap(x)) = x inside the grid
    xt = torch.from_numpy(x).cuda()
    yt = torch.empty_like(xt)
    jt = torch.empty(len(x), dtype=torch.float64, device='cuda')
    m.invmap(xt, yt, jt)
    assert np.array_equal(yt.cpu().numpy(), c['inv_y'])
    x2 = torch.empty_like(yt)
    j2 = torch.empty_like(jt)
    m.map(yt, x2, j2)
    inside = ((yt > 0) & (yt < 1)).all(dim=1).cpu().numpy()
    assert np.max(np.abs(x2.cpu().numpy()[inside] - x[inside])) <= 1e-14


def test_invmap_fp32():
    # FP32 storage, FP64 arithmetic: the result is the FP64 invmap of the
    # float-rounded x, rounded to float (jac is piecewise constant, so a
    # point next to a node may change increment when x is rounded)
    c = load('ref_invmap.npz')
    m = make_map(c['inv_grid'], c['inv_ninc'])
    xt = torch.from_numpy(c['inv_x']).float().cuda()
    yt = torch.empty_like(xt)
    jt = torch.empty(len(xt), dtype=torch.float32, device='cuda')
    m.invmap(xt, yt, jt)
    x64 = xt.double()
    y64 = torch.empty_like(x64)
    j64 = torch.empty(len(xt), dtype=torch.float64, device='cuda')
    m.invmap(x64, y64, j64)
    assert torch.equal(yt, y64.float())
    assert torch.equal(jt, j64.float())
    assert np.max(np.abs(yt.cpu().numpy() - c['inv_y'])) <= 1e-6


def test_adapt_to_samples_golden():
    c = load('ref_invmap.npz')
    m = make_map(c['ats_grid_in'], c['ats_ninc_in'])
    m.adapt_to_samples(c['ats_x'], c['ats_f'], nitn=4, alpha=0.8)
    assert list(m.ninc) == list(c['ats_ninc_out'])
    want = c['ats_grid_out']
    ok = ~np.isnan(want)
    got = m.grid
    assert np.max(np.abs(got[ok] - want[ok])) <= 1e-12 * np.max(np.abs(want[ok]))
    # a callable f is called with x as given
    m2 = make_map(c['ats_grid_in'], c['ats_ninc_in'])
    vals = c['ats_f']
    m2.adapt_to_samples(c['ats_x'], lambda x: vals, nitn=4, alpha=0.8)
    assert np.array_equal(m2.grid[ok], got[ok]) or \
        np.max(np.abs(m2.grid[ok] - want[ok])) <= 1e-12 * np.max(np.abs(want[ok]))
    with pytest.raises(ValueError):
        make_map(c['ats_grid_in'], c['ats_ninc_in']).adapt_to_samples(c['ats_x'][:10], c['ats_f'][:10])
