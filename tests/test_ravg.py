"""Host-side result classes against the reference's known answers
(tests/test_vegas.py:216-236, 313-335 of vegas 6.4.1)."""
import pickle

import numpy as np

from vegas_gb300 import RAvg, RAvgArray, gvar
from vegas_gb300 import _gvar as gv


def test_ravg_known_answer():
    a = RAvg()
    a.add(gvar(1, 1))
    a.add(gvar(2, 2))
    a.add(gvar(3, 3))
    np.testing.assert_allclose(a.mean, 1.346938775510204)
    np.testing.assert_allclose(a.sdev, 0.8571428571428571)
    assert a.dof == 2
    np.testing.assert_allclose(a.chi2, 0.5306122448979592)
    np.testing.assert_allclose(a.Q, 0.7669711269557102)
    assert str(a) == '1.35(86)'
    s = ["itn   integral        wgt average     chi2/dof        Q",
         "-------------------------------------------------------",
         "  1   1.0(1.0)        1.0(1.0)            0.00     1.00",
         "  2   2.0(2.0)        1.20(89)            0.20     0.65",
         "  3   3.0(3.0)        1.35(86)            0.27     0.77", ""]
    assert a.summary() == '\n'.join(s)


def test_ravg_unweighted():
    a = RAvg(weighted=False)
    for v in (1., 2., 3.):
        a.add(gvar(v, 0.1))
    np.testing.assert_allclose(a.mean, 2.0)
    np.testing.assert_allclose(a.sdev, 0.1 / 3 ** 0.5)
    assert a.dof == 2


def test_ravgarray_known_answer():
    a = RAvgArray((1, 2))
    a.add([[gvar(1, 1), gvar(10, 10)]])
    a.add([[gvar(2, 2), gvar(20, 20)]])
    a.add([[gvar(3, 3), gvar(30, 30)]])
    assert a.shape == (1, 2)
    np.testing.assert_allclose(a[0, 0].mean, 1.346938775510204)
    np.testing.assert_allclose(a[0, 0].sdev, 0.8571428571428571)
    assert a.dof == 4
    np.testing.assert_allclose(a.chi2, 2 * 0.5306122448979592)
    np.testing.assert_allclose(a.Q, 0.900374555485)
    assert str(a[0, 0]) == '1.35(86)' and str(a[0, 1]) == '13.5(8.6)'


def test_ravg_pickle_roundtrip():
    a = RAvg()
    for v, s in ((1., 1.), (2., 2.)):
        a.add(gvar(v, s))
    b = pickle.loads(pickle.dumps(a))
    assert b.mean == a.mean and b.sdev == a.sdev and b.nitn == 2


def test_correlated_gvar_algebra():
    x = gv.gvar([1.0, 2.0], [[1.0, 0.5], [0.5, 2.0]])
    c = gv.evalcov(x)
    np.testing.assert_allclose(c, [[1.0, 0.5], [0.5, 2.0]])
    d = x[0] - x[0]
    assert d.sdev == 0.0


def test_ravgdict_weighted_average():
    from vegas_gb300 import RAvgDict
    r = RAvgDict([('a', ()), ('b', (2,))])
    r.add({'a': gvar(1.0, 0.1), 'b': [gvar(2.0, 0.2), gvar(3.0, 0.3)]})
    r.add({'a': gvar(1.2, 0.1), 'b': [gvar(2.2, 0.2), gvar(3.3, 0.3)]})
    assert abs(r['a'].mean - 1.1) < 1e-12
    assert abs(r['a'].sdev - 0.1 / 2 ** 0.5) < 1e-12
    assert r['b'].shape == (2,) and abs(r['b'][1].mean - 3.15) < 1e-12
    assert r.nitn == 2 and r.dof == 3
    assert abs(r.chi2 - (0.2 ** 2 / 0.02 + 0.2 ** 2 / 0.08 + 0.3 ** 2 / 0.18)) < 1e-9
    assert r.converged(0.1, 0) and not r.converged(1e-6, 0)
