"""CPU: the oracle's restatement of Caracal's flexible SPC water box
(src/egrad_water.f90) against a pure-Python restatement on small boxes and
against central finite differences; the periodic set-up
(src/set_periodic.f90:78-104).  No reference outputs exist for this
surface (parity unpinned): these checks pin the restatement to the
reference's formulas, quirks included."""
import math

import numpy as np
import pytest

from caracal_gb300 import water as W
from oracle import oracle as orc

BOHR = 0.52917721092
HARTREE = 627.5094743


def py_water(x, nwater, box=None, cut=0.0, zahn=False, za=0.0, zp=0.0):
    """Straight loops over the reference's statements (energy only)."""
    f32 = lambda v: float(np.float32(v))  # noqa: E731  REAL(4) literals
    r0, r0hh = 1.0 / BOHR, 1.633 / BOHR
    de, a = 101.9188 / HARTREE, 2.567 * BOHR
    kt = 328.645606 / HARTREE * BOHR * BOHR
    krt = -211.4672 / HARTREE * BOHR * BOHR
    krr = f32(111.70765) / HARTREE * BOHR * BOHR
    sig, eps = 3.166 / BOHR, f32(0.1554) / HARTREE
    q = [-0.82, 0.41, 0.41] * nwater

    def img(d):
        if box is None:
            return d
        d = list(d)
        for k in range(3):
            while abs(d[k]) > 0.5 * box[k]:
                d[k] -= math.copysign(box[k], d[k])
        return d

    def norm(d):
        return math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])

    e = 0.0
    for w in range(nwater):
        o, h1, h2 = x[3 * w], x[3 * w + 1], x[3 * w + 2]
        d1 = norm(img(o - h1)) - r0
        d2 = norm(img(o - h2)) - r0
        dh = norm(img(h1 - h2)) - r0hh
        e += de * (1 - math.exp(a * d1)) ** 2 + de * (1 - math.exp(a * d2)) ** 2
        e += 0.5 * kt * dh ** 2 + krt * dh * (d1 + d2) + krr * d1 * d2
    n = 3 * nwater
    for i in range(n):
        for j in range(i + 1, n):
            if i // 3 == j // 3:
                continue
            r = norm(img(x[i] - x[j]))
            if not (r < cut or box is None):
                continue
            if zahn:
                e += q[i] * q[j] * (math.erfc(za * r) / r - zp * (r - cut))
            else:
                e += q[i] * q[j] / r
            if i % 3 == 0:  # name(i) == "O" (tested twice in the reference)
                s6 = (sig / r) ** 6
                e += 4 * eps * (s6 * s6 - s6)
    return e


@pytest.mark.parametrize("periodic,zahn", [(False, False), (True, False), (True, True)])
def test_oracle_matches_python_restatement(periodic, zahn):
    nw = 8
    x, length = W.water_box(nw, seed=3)
    rng = np.random.default_rng(1)
    x = x + rng.normal(0, 0.05, x.shape)
    if periodic:
        box, cut, za, zp = W.periodic_setup([length] * 3, 4.0, zahn)
        x = x + rng.normal(0, 0.5 * box[0], (1, 3))  # shift: images must matter
        orc.set_water(nw, box, cut, zahn, za, zp)
        ref = py_water(x, nw, box, cut, zahn, za, zp)
    else:
        orc.set_water(nw)
        ref = py_water(x, nw)
    V, g = orc.egrad("water", x[None])
    assert abs(V[0] - ref) <= 1e-12 * max(1.0, abs(ref))


@pytest.mark.parametrize("periodic", [False, True])
def test_oracle_gradient_matches_finite_differences(periodic):
    nw = 4
    x, length = W.water_box(nw, seed=5)
    x = x + np.random.default_rng(2).normal(0, 0.05, x.shape)
    if periodic:
        box, cut, za, zp = W.periodic_setup([length] * 3, 3.0, False)
        orc.set_water(nw, box, cut)
    else:
        orc.set_water(nw)
    _, g = orc.egrad("water", x[None])
    h = 1e-5
    gn = np.zeros_like(x)
    for i in range(x.shape[0]):
        for k in range(3):
            xp, xm = x.copy(), x.copy()
            xp[i, k] += h
            xm[i, k] -= h
            gn[i, k] = (orc.egrad("water", xp[None])[0][0] - orc.egrad("water", xm[None])[0][0]) / (2 * h)
    assert np.max(np.abs(g[0] - gn)) <= 1e-6 * np.max(np.abs(gn))


def test_lj_only_where_the_first_atom_is_oxygen():
    # two molecules far apart except for H(0) near O(1) and O(0)-H(1):
    # the pair (O0, H1) carries LJ, (H0, O1) none (src/egrad_water.f90:285)
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 1.0, 0],
                  [6.0, 0, 0], [5.0, 0, 0], [6.0, 1.0, 0]]) / BOHR
    orc.set_water(2)
    V, _ = orc.egrad("water", x[None])
    assert abs(V[0] - py_water(x, 2)) <= 1e-13
    sig, eps = 3.166 / BOHR, float(np.float32(0.1554)) / HARTREE
    lj = lambda r: 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)  # noqa: E731
    pairs_o_first = [(0, 3), (0, 4), (0, 5)]
    e_lj = sum(lj(np.linalg.norm(x[i] - x[j])) for i, j in pairs_o_first)
    # removing those three LJ terms leaves Coulomb + intramolecular only
    q = [-0.82, 0.41, 0.41] * 2
    e_coul = sum(q[i] * q[j] / np.linalg.norm(x[i] - x[j]) for i in range(3) for j in range(3, 6))
    orc.set_water(1)
    e1 = orc.egrad("water", x[None, :3])[0][0]
    e2 = orc.egrad("water", x[None, 3:])[0][0]
    assert abs(V[0] - (e1 + e2 + e_coul + e_lj)) <= 1e-13


def test_periodic_setup_follows_set_periodic():
    box, cut, za, zp = W.periodic_setup([20.0, 20.0, 20.0], 1.0)  # below 5 bohr
    assert cut == pytest.approx(10.0 / BOHR - 0.1)
    box, cut, za, zp = W.periodic_setup([30.0, 30.0, 30.0], 8.0)
    assert cut == pytest.approx(8.0 / BOHR)
    box, cut, za, zp = W.periodic_setup([12.0, 30.0, 30.0], 9.0)  # beyond half the box
    assert cut == pytest.approx(6.0 / BOHR - 0.1)
    box, cut, za, zp = W.periodic_setup([30.0] * 3, 4.0, zahn=True)
    assert cut == pytest.approx(10.0 / BOHR) and za == pytest.approx(0.2 * BOHR)
    acut = za * cut
    assert zp == pytest.approx(math.erfc(acut) / cut ** 2 + 2 * za / math.sqrt(math.pi) * math.exp(-acut ** 2) / cut)
