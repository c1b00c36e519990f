"""PDFIntegrator (reference src/vegas/__init__.py:373-1189) as a consumer of
the batch-integrand path: expectation values under a correlated Gaussian and
under a user PDF, the PDF's normalisation, stats(), sample(), dictionary
parameters.  Checked against closed forms within 5 combined standard
deviations (the reference's own tests pin PDFIntegrator statistically,
tests/test_vegas.py), plus the exact identities of the variable change."""
import math

import numpy as np
import pytest
import torch

import vegas_gb300 as vg
from vegas_gb300.pdf_integrator import PDFIntegrator

MEAN = np.array([1.0, -2.0, 0.5])
COV = np.array([[1.0, 0.6, 0.1], [0.6, 2.0, -0.3], [0.1, -0.3, 0.5]])


def test_param_axes_cpu():
    """p = mean + axes chiv reproduces the covariance: axes axes^T = C, and
    dp/dchiv = sqrt(det C)."""
    from vegas_gb300.pdf_integrator import _GaussParam
    gp = _GaussParam((MEAN, COV), svdcut=1e-15)
    assert np.allclose(gp.axes @ gp.axes.T, COV, atol=1e-12)
    assert abs(gp.dp_dchiv - math.sqrt(np.linalg.det(COV))) < 1e-12
    g = vg.gvar(MEAN, COV)
    gp2 = _GaussParam(g, svdcut=1e-15)
    assert np.allclose(gp2.axes @ gp2.axes.T, COV, atol=1e-12)
    gd = _GaussParam({'a': g[:2], 'b': g[2]}, svdcut=1e-15)
    assert gd.layout == [('a', (2,)), ('b', ())]
    p = torch.zeros(5, 3, dtype=torch.float64)
    s = gd.structured(p)
    assert s['a'].shape == (5, 2) and s['b'].shape == (5,)


@pytest.mark.gpu
def test_expectations_under_gaussian():
    g = vg.gvar(MEAN, COV)
    I = PDFIntegrator(g, neval=20000, nitn=8, seed=5, precision='fp64')
    I(neval=20000, nitn=5)                    # adapt to the PDF

    @vg.lbatchintegrand
    def f(p):
        return torch.stack([p[:, 0], p[:, 1], p[:, 0] * p[:, 1]], dim=1)

    r = I(f, nitn=8)
    want = [MEAN[0], MEAN[1], COV[0, 1] + MEAN[0] * MEAN[1]]
    for k in range(3):
        assert abs(r[k].mean - want[k]) < 5 * r[k].sdev + 1e-9, (k, r[k], want[k])
    # the Gaussian PDF is normalised in chiv space
    assert abs(r.pdfnorm.mean - 1.0) < 5 * r.pdfnorm.sdev + 1e-9
    n = I(nitn=4)
    assert abs(n.pdfnorm.mean - 1.0) < 5 * n.pdfnorm.sdev + 1e-9


@pytest.mark.gpu
def test_user_pdf_and_stats():
    g = vg.gvar(MEAN[:2], COV[:2, :2])
    c = np.array([0.7, -1.5])
    s2 = 0.8

    @vg.lbatchintegrand
    def pdf(p):       # unnormalised Gaussian centred at c, variance s2 per axis
        return torch.exp(-((p - torch.as_tensor(c, dtype=p.dtype, device=p.device)) ** 2).sum(dim=1) / (2 * s2))

    I = PDFIntegrator(g, pdf=pdf, neval=20000, seed=8, precision='fp64')
    I(nitn=5)

    @vg.lbatchintegrand
    def f(p):
        return p[:, 0]

    r = I(f, nitn=8)
    assert abs(r.mean - c[0]) < 5 * r.sdev, r
    st = I.stats(f, nitn=8)
    assert abs(st.mean - c[0]) < 0.02
    assert abs(st.sdev - math.sqrt(s2)) < 0.02


@pytest.mark.gpu
def test_dict_param_and_sample():
    g = vg.gvar(MEAN, COV)
    I = PDFIntegrator({'a': g[:2], 'b': g[2]}, neval=20000, seed=11, precision='fp64')
    I(nitn=5)

    @vg.rbatchintegrand
    def f(p):     # rbatch: batch index last
        return {'ab': p['a'][0] * p['b'], 'b': p['b']}

    r = I(f, nitn=8)
    assert abs(r['b'].mean - MEAN[2]) < 5 * r['b'].sdev
    want = COV[0, 2] + MEAN[0] * MEAN[2]
    assert abs(r['ab'].mean - want) < 5 * r['ab'].sdev
    w, p = I.sample(nbatch=50000, mode='lbatch')
    assert abs(float(w.sum()) - 1.0) < 1e-9
    assert abs(float((w * p['b']).sum()) - MEAN[2]) < 0.05
