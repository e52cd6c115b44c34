"""CPU: umbrella sampling restatement (calc_xi mode 1, umbrella mode 0) and
the free-energy estimators (umbrella integration, WHAM).

Pins: the reference's explicit Hessian of xi against central differences of
its gradient; the bias gradient against central differences of
V = k/2 (xi - xi0)^2 - (1/beta) log fs at the centroid; umbrella integration
and WHAM on distributions whose free-energy profile is known in closed form.
"""
import numpy as np
import pytest

from caracal_gb300.pmf import umbrella_integration, wham
from caracal_gb300.units import K_BOLTZMANN_AU, beta_from_kelvin, dt_fs_to_au, mass_au
from caracal_gb300.workloads import ch4h_dividing_surface, ch4h_recross_definition
from oracle import oracle as orc

MASS = np.array([mass_au(s) for s in ("H", "C", "H", "H", "H", "H")])


def xidef():
    q0 = ch4h_dividing_surface()
    rd = ch4h_recross_definition(q0)
    return q0, rd, orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                                  (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                                  (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                                  rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])


def test_xi_hessian_matches_finite_differences():
    q0, _, xd = xidef()
    x = q0 + np.random.default_rng(1).normal(0, 0.05, q0.shape)
    xi, d, H = orc.calc_xi_umbrella(xd, x, MASS)
    h = 1e-5
    fd = np.zeros_like(H)
    for j in range(18):
        xp, xm = x.ravel().copy(), x.ravel().copy()
        xp[j] += h
        xm[j] -= h
        fd[:, j] = ((orc.calc_xi_umbrella(xd, xp.reshape(6, 3), MASS)[1] -
                     orc.calc_xi_umbrella(xd, xm.reshape(6, 3), MASS)[1]) / (2 * h)).ravel()
    assert np.max(np.abs(fd - H)) <= 1e-8 * np.max(np.abs(H))
    assert np.max(np.abs(H - H.T)) <= 1e-15 * np.max(np.abs(H))
    gx = np.zeros_like(d)
    for j in range(18):
        xp, xm = x.ravel().copy(), x.ravel().copy()
        xp[j] += h
        xm[j] -= h
        gx.ravel()[j] = (orc.calc_xi_umbrella(xd, xp.reshape(6, 3), MASS)[0] -
                         orc.calc_xi_umbrella(xd, xm.reshape(6, 3), MASS)[0]) / (2 * h)
    assert np.max(np.abs(gx - d)) <= 1e-8 * np.max(np.abs(d))


def test_bias_is_gradient_of_umbrella_potential():
    q0, _, xd = xidef()
    beta = beta_from_kelvin(500.0)
    cfg = orc.Config("ch4h", MASS, 4, dt_fs_to_au(0.1), beta)
    rng = np.random.default_rng(2)
    q = q0[None] + rng.normal(0, 0.03, (4, 6, 3))
    xi0, k = 0.97, 0.4
    xi, f = orc.umbrella_bias(cfg, xd, xi0, k, q, np.zeros_like(q))

    def V(c):
        x, d, _ = orc.calc_xi_umbrella(xd, c, MASS)
        fs = np.sqrt(np.sum(d * d / MASS[:, None]) / (2 * np.pi * beta))
        return 0.5 * k * (x - xi0) ** 2 - np.log(fs) / beta
    c = q.mean(axis=0)
    g = np.zeros(18)
    h = 1e-6
    for j in range(18):
        cp, cm = c.ravel().copy(), c.ravel().copy()
        cp[j] += h
        cm[j] -= h
        g[j] = (V(cp.reshape(6, 3)) - V(cm.reshape(6, 3))) / (2 * h)
    for b in range(4):   # every bead receives the centroid gradient (src/umbrella.f90:134-136)
        assert np.max(np.abs(f[b].ravel() - g)) <= 1e-7 * np.max(np.abs(g))
    assert xi == pytest.approx(orc.calc_xi_umbrella(xd, c, MASS)[0], rel=1e-15)


@pytest.mark.parametrize("slope", [0.0, 0.01])
def test_umbrella_integration_recovers_linear_profile(slope):
    beta = beta_from_kelvin(300.0)
    xw = np.linspace(-0.1, 1.1, 25)
    k = np.full_like(xw, 0.5)
    # harmonic windows on A = slope * xi: Gaussian with mean xi_i - slope/k and variance 1/(beta k)
    av = xw - slope / k
    va = 1.0 / (beta * k)
    lo, hi, nb = -0.05, 1.05, 111
    coord, pmf = umbrella_integration(xw, k, av, va, beta, lo, hi, nb, 1000)
    # Caracal stores the running integral up to the bin's upper edge at the
    # bin's midpoint and shifts by the minimum over all nbins entries, whose
    # last (never assigned) entry is 0
    dx = (hi - lo) / (nb - 1)
    ref = slope * (coord + 0.5 * dx - lo)
    ref = ref - min(ref.min(), 0.0)
    assert np.max(np.abs(pmf - ref)) <= 1e-10


def test_wham_recovers_flat_profile():
    kelvin = 300.0
    beta = 1.0 / (K_BOLTZMANN_AU * kelvin)
    xw = np.linspace(0.0, 1.0, 21)
    k = np.full_like(xw, 0.2)
    lo, hi, nb = -0.1, 1.1, 120
    dx = (hi - lo) / nb
    xj = lo + dx * np.arange(1, nb + 1)
    # expected counts under Caracal's restraint k (xi - xi_i)^2 on a flat profile
    hist = 1e6 * np.exp(-beta * k[:, None] * (xj[None, :] - xw[:, None]) ** 2)
    _, pmf = wham(hist, xw, k, kelvin, lo, hi, tol=1e-20)
    inner = pmf[10:-10]
    assert np.max(inner) - np.min(inner) <= 1e-8
    # the reference's own tolerance (1e-5 on sum (1 - f_new/f_old)^2) leaves
    # the profile flat to a small fraction of kT (in its printed units)
    _, pmf = wham(hist, xw, k, kelvin, lo, hi)
    kt = 627.509 * 0.52917721092 / beta
    assert np.max(pmf[10:-10]) - np.min(pmf[10:-10]) <= 0.05 * kt
