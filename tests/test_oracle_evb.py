"""CPU: the dE-EVB oracle (src/gradient.f90:361-386, 1228-1304) -- two
QMDFFs (the synthetic C20H42 and its 1,2-H-shift partner), every coupling
basis against central differences (Caracal's NUM_GRAD method), and the
lower-root properties of the 2x2 EVB matrix."""
import numpy as np
import pytest

from caracal_gb300 import qmdff as Q
from oracle import oracle as orc

BASES = {
    "const": dict(a=0.01),
    "1g": dict(a=0.01, b=50.0),
    "2g": dict(a=0.01, b=50.0, c=0.005, d=20.0, m=0.01),
    "3g": dict(a=0.01, b=50.0, c=0.005, d=20.0, m=0.01, e=0.002, f=10.0, n=-0.02),
    "sp": dict(a=0.01, b=50.0, c=0.02, d=30.0),
    "sd": dict(a=0.01, b=50.0, c=0.2, d=30.0),
    "sd2": dict(a=0.01, b=50.0, c=0.2, d=30.0, e=0.1, f=5.0),
    "sp2d": dict(a=0.01, b=50.0, c=0.02, d=30.0, e=0.01, f=5.0, g=0.3, h=40.0),
}


@pytest.fixture(scope="module")
def pair():
    ff = Q.alkane()
    return ff, Q.alkane_evb_partner(ff), Q.ElementTables.caracal()


@pytest.mark.parametrize("basis", list(BASES))
def test_evb_gradient_central_differences(pair, basis):
    ff, ff2, tab = pair
    orc.set_evb(ff, ff2, tab, basis, BASES[basis])
    x = ff.xyz + np.random.default_rng(1).normal(0, 0.05, ff.xyz.shape)
    V, g = orc.egrad("evb", x)
    h = 1e-5
    for a, d in [(0, 0), (5, 2), (21, 1), (40, 0), (61, 2), (1, 1)]:
        xp, xm = x.copy(), x.copy()
        xp[a, d] += h
        xm[a, d] -= h
        fd = (orc.egrad("evb", xp)[0][0] - orc.egrad("evb", xm)[0][0]) / (2 * h)
        assert abs(fd - g[0][a, d]) <= 1e-8 * np.max(np.abs(g[0]))


def test_evb_lower_root(pair):
    ff, ff2, tab = pair
    x = ff.xyz + np.random.default_rng(2).normal(0, 0.05, ff.xyz.shape)
    orc.set_qmdff(ff, tab)
    e1 = orc.egrad("qmdff", x)[0][0]
    orc.set_qmdff(ff2, tab)
    e2 = orc.egrad("qmdff", x)[0][0]
    orc.set_evb(ff, ff2, tab, "const", dict(a=0.0))
    assert abs(orc.egrad("evb", x)[0][0] - min(e1, e2)) < 1e-14
    orc.set_evb(ff, ff2, tab, "1g", dict(a=0.02, b=10.0))
    e = orc.egrad("evb", x)[0][0]
    assert e < min(e1, e2)
    V12 = 0.02 * np.exp(-10.0 * (e1 - e2) ** 2)
    assert abs(e - 0.5 * (e1 + e2 - np.sqrt((e1 - e2) ** 2 + 4 * V12 ** 2))) < 1e-14


FIT = {"1g": [0.01, 50.0], "2g": [0.01, 50.0, 0.005, 20.0, 0.01],
       "3g": [0.01, 50.0, 0.005, 20.0, 0.002, 10.0, 0.01, -0.02], "sp": [0.01, 50.0, 0.02, 30.0],
       "sd": [0.01, 50.0, 0.2, 30.0], "sd2": [0.01, 50.0, 0.2, 30.0, 0.1, 5.0],
       "sp2d": [0.01, 50.0, 0.02, 30.0, 0.01, 5.0, 0.3, 40.0],
       "sp2d3": [0.01, 50.0, 0.02, 30.0, 0.01, 5.0, 0.3, 40.0, 0.1, 8.0, 0.05, 12.0]}


def fit_data(m=200, seed=3):
    rng = np.random.default_rng(seed)
    e1 = rng.normal(0.0, 0.03, m)
    e2 = rng.normal(0.01, 0.03, m)
    eref = np.minimum(e1, e2) - np.abs(rng.normal(0.0, 0.004, m))
    return e1, e2, eref


@pytest.mark.parametrize("basis", list(FIT))
def test_fit_residual_and_jacobian(basis):
    e1, e2, eref = fit_data()
    x = np.array(FIT[basis])
    fvec, fjac = orc.evb_fit(basis, x, e1, e2, eref)
    # the residual is the squared deviation from the EVB lower root with |dE|
    dE = np.abs(e1 - e2)
    if basis == "1g":
        v = x[0] * np.exp(-x[1] * dE ** 2)
        np.testing.assert_allclose(fvec, (eref - 0.5 * (e1 + e2 - np.sqrt(dE ** 2 + 4 * v * v))) ** 2, rtol=1e-12)
    # fdjac2's forward differences agree with central differences of the residual
    for j in range(len(x)):
        h = 1e-6 * max(abs(x[j]), 1e-3)
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        cd = (orc.evb_fit(basis, xp, e1, e2, eref, jacobian=False) -
              orc.evb_fit(basis, xm, e1, e2, eref, jacobian=False)) / (2 * h)
        # forward differences carry O(h) truncation and rounding noise of
        # about eps * |E|^2 / h with fdjac2's step h = sqrt(eps) |x_j|
        hj = np.sqrt(np.finfo(float).eps) * abs(x[j])
        noise = 1e-15 * np.max(np.abs(eref)) ** 2 / hj
        assert np.max(np.abs(fjac[j] - cd)) <= 1e-5 * np.max(np.abs(cd)) + noise
