"""CPU: the oracle's restatement of Caracal's ANA_BRH2 surface (the BrH2
DIM-3C surface of POTLIB, src/egrad_brh2.f) against its pins: the zero of
energy and the valley energies its header documents (Br far from H2 at
RHH: 0; H far from HBr at RHX: DHH - DHX, the EASYBC - EASYAC of
PT5CM_brh2), central differences, exchange of the two H atoms and rigid
motions.  Parity unpinned beyond these: Caracal ships no BrH2 outputs."""
import numpy as np
import pytest

from oracle import oracle as orc

RHH, RHX, DHH, DHX = 1.4016, 2.673, 0.17447, 0.1439


def eg(q):
    V, g = orc.egrad("brh2", np.asarray(q, dtype=np.float64)[None])
    return V[0], g[0]


def geom(seed):
    rng = np.random.default_rng(seed)
    # H approaching the H end of H-Br, bent, atoms H, Br, H
    return np.array([[0.0, 0.0, -3.2], [0.0, 0.0, 2.7], [0.0, 0.3, 0.1]]) + rng.normal(0, 0.1, (3, 3))


def test_documented_asymptotes():
    V, _ = eg([[0.0, 0.0, 0.0], [30.0, 0.0, 0.0], [0.0, 0.0, RHH]])
    assert abs(V) < 1e-12                                        # Br + H2 at RHH: the zero
    V, _ = eg([[40.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, RHX]])
    assert abs(V - (DHH - DHX)) < 1e-12                          # H + HBr at RHX
    # both diatomics sit at their minima: stretching either raises V
    for q0, i, d in (([[0, 0, 0], [30.0, 0, 0], [0, 0, RHH]], 2, 2), ([[40.0, 0, 0], [0, 0, 0], [0, 0, RHX]], 2, 2)):
        q = np.array(q0, dtype=np.float64)
        e0 = eg(q)[0]
        for h in (-0.05, 0.05):
            qq = q.copy()
            qq[i, d] += h
            assert eg(qq)[0] > e0


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_central_differences(seed):
    q = geom(seed)
    _, g = eg(q)
    gn = np.zeros_like(q)
    h = 1e-6
    for i in range(3):
        for d in range(3):
            a, b = q.copy(), q.copy()
            a[i, d] += h
            b[i, d] -= h
            gn[i, d] = (eg(a)[0] - eg(b)[0]) / (2 * h)
    assert np.abs(g - gn).max() < 1e-8 * max(1.0, np.abs(g).max())


def test_symmetries():
    q = geom(5)
    V, g = eg(q)
    Vs, gs = eg(q[[2, 1, 0]])                   # the two H exchanged
    assert abs(Vs - V) < 1e-13 and np.abs(gs[[2, 1, 0]] - g).max() < 1e-12
    c, s = np.cos(0.9), np.sin(0.9)
    rot = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    Vr, gr = eg(q @ rot.T + np.array([1.0, -2.0, 0.5]))
    assert abs(Vr - V) < 1e-13 and np.abs(gr - g @ rot.T).max() < 1e-12
