"""CPU: the oracle's restatement of Caracal's ANA_OH3 surface
(src/egrad_oh3.f, Schatz-Elgersma OH + H2) against central finite
differences (Caracal's NUM_GRAD check) and the surface's limits.  No
reference outputs exist for this surface (parity unpinned)."""
import numpy as np
import pytest

from oracle import oracle as orc


def geometries():
    rng = np.random.default_rng(7)
    reac = np.array([[0, 0, 0], [1.83, 0, 0], [-0.5, 4.0, 0.2], [-0.4, 5.4, 0.3]], float)
    ts = np.array([[0, 0, 0], [1.83, 0, 0], [-0.6, 2.5, 0.1], [-0.8, 4.0, 0.2]], float)
    prod = np.array([[0, 0, 0], [1.81, 0, 0], [-0.45, 1.75, 0.0], [-1.0, 6.5, 0.5]], float)
    out = [reac, ts, prod]
    out += [g + rng.normal(0, 0.1, g.shape) for g in (reac, ts, prod) for _ in range(3)]
    return out


@pytest.mark.parametrize("k", range(12))
def test_gradient_matches_finite_differences(k):
    q = geometries()[k]
    _, g = orc.egrad("oh3", q[None])
    h = 1e-5
    gn = np.zeros_like(q)
    for i in range(4):
        for x in range(3):
            a, b = q.copy(), q.copy()
            a[i, x] += h
            b[i, x] -= h
            gn[i, x] = (orc.egrad("oh3", a[None])[0][0] - orc.egrad("oh3", b[None])[0][0]) / (2 * h)
    assert np.max(np.abs(g[0] - gn)) <= 1e-7 * max(1e-3, np.max(np.abs(gn)))


def test_limits():
    # OH + H2 far apart: the OH and H2 diatomics at their minima give ~0;
    # H2O + H lies below it (the reaction is exothermic on this surface)
    oh = np.array([[0, 0, 0], [1.8331, 0, 0]])
    far = np.vstack([oh, [[0, 40, 0], [0, 41.4, 0]]])
    e_reac = orc.egrad("oh3", far[None])[0][0]
    water = np.array([[0, 0, 0], [1.8081, 0, 0], [-0.4565, 1.7495, 0.0], [0, 0, 40.0]])
    e_prod = orc.egrad("oh3", water[None])[0][0]
    assert abs(e_reac) < 0.01
    assert e_prod < e_reac
