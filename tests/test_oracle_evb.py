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
    return ff, Q.alkane_evb_partner(ff), Q.ElementTables.d3_like()


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
