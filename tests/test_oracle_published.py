"""CPU: the oracle's analytic surfaces against published properties and the
one numeric output Caracal documents for them.

* ANA_CH4OH: Caracal's manual plots the IRC of examples/explore/ts_irc_ch4oh
  (manual/figures/irc_ch4oh.png, read into figure_irc_ch4oh.txt by
  tests/golden/reference/digitize_figures.py).  The saddle point is found
  here from the example's ts_start.xyz by Newton steps on the oracle's
  analytic gradient, and the path is traced with opt_irc's own Euler scheme
  (src/opt_irc.f90:107-330: a first step along the lowest mass-weighted
  Hessian mode, then unit steps of 0.005 along -g sqrt(m), a point every
  steplen = 0.05, stopping when the energy changes by < 1e-6 Hartree or
  the distance to the saddle stops growing).  The energies in the product
  valley and on the reactant side must lie on the plotted line.
* ANA_CH4H (J. C. Corchado, J. L. Bravo, J. Espinosa-Garcia, J. Chem. Phys.
  130, 184314 (2009)): reaction energy of CH4 + H -> CH3 + H2, 2.88 kcal/mol,
  and classical barrier 15.0 kcal/mol.
* ANA_OH3 (G. C. Schatz, H. Elgersma, Chem. Phys. Lett. 73, 21 (1980)):
  classical barrier 6.1 kcal/mol and reaction energy -15.2 kcal/mol of
  OH + H2 -> H2O + H.
"""
import os

import numpy as np
import pytest

from caracal_gb300 import keyfile as K
from caracal_gb300.units import angstrom_to_bohr
from conftest import ROOT
from oracle import oracle as orc

REF = os.path.join(ROOT, "tests", "golden", "reference")
KCAL = 627.5094740631                  # kcal/mol per Hartree
ANG = angstrom_to_bohr(1.0)
AMU = {"H": 1.00794, "C": 12.0107, "O": 15.9994}


def eg(pes, x):
    v, g = orc.egrad(pes, x[None])
    return v[0], g[0]


def hessian(pes, x, h=1e-4):
    n = x.size
    hm = np.zeros((n, n))
    for i in range(n):
        xp, xm = x.ravel().copy(), x.ravel().copy()
        xp[i] += h
        xm[i] -= h
        hm[i] = (eg(pes, xp.reshape(x.shape))[1] - eg(pes, xm.reshape(x.shape))[1]).ravel() / (2 * h)
    return 0.5 * (hm + hm.T)


def stationary_point(pes, x, iters=40):
    """Newton steps on the analytic gradient with the finite-difference
    Hessian, translations and rotations (|eigenvalue| < 1e-5) projected
    out: converges to the stationary point next to x.  Returns x, E, the
    largest gradient component and the Hessian's eigenvalues."""
    for _ in range(iters):
        _, g = eg(pes, x)
        if np.abs(g).max() < 1e-10:
            break
        w, u = np.linalg.eigh(hessian(pes, x))
        keep = np.abs(w) > 1e-5
        gq = u.T @ g.ravel()
        dx = -(u[:, keep] @ (gq[keep] / w[keep]))
        step = np.linalg.norm(dx)
        x = x + (dx * min(1.0, 0.2 / step)).reshape(x.shape)
    e, g = eg(pes, x)
    return x, e, np.abs(g).max(), np.linalg.eigvalsh(hessian(pes, x))


def irc_branch(pes, xts, ets, mode, mass, sign, euler=0.005, steplen=0.05, maxstep=200, ethr=1e-6):
    """One branch of opt_irc's Euler IRC: (s, E) every steplen."""
    nper, ntot = int(round(steplen / euler)), int(round(maxstep / euler * steplen))
    ds = euler if sign > 0 else -euler
    act, step, s = xts.copy(), sign * mode, ds
    ncorr = 0
    while True:                         # push off the saddle until E drops
        act = act - euler * step / np.linalg.norm(step)
        if ets - eg(pes, act)[0] > 0.0:
            break
        s += ds
        ncorr += 1
        assert ncorr <= 100
    out, e_last = [], 0.0
    for i in range(2 + ncorr, ntot + 1):
        d_before = np.linalg.norm(xts - act)
        e, g = eg(pes, act)
        st = g * np.sqrt(mass)[:, None]
        act = act - euler * st / np.linalg.norm(st)
        s += ds
        if i % nper == 0:
            out.append((s, e))
        if abs(e - e_last) < ethr or (np.linalg.norm(xts - act) <= d_before and i > 4):
            break
        e_last = e
    return out


def test_ch4oh_irc_lies_on_caracals_figure():
    sym, xyz = K.read_xyz(os.path.join(REF, "explore", "ts_irc_ch4oh", "ts_start.xyz"))
    mass = np.array([AMU[s] for s in sym])
    xts, ets, gmax, w = stationary_point("ch4oh", angstrom_to_bohr(np.array(xyz)))
    assert gmax < 1e-9 and np.count_nonzero(w < -1e-4) == 1          # a first-order saddle
    m3 = np.repeat(mass, 3)
    hw = hessian("ch4oh", xts) / np.sqrt(np.outer(m3, m3))
    mode = np.linalg.eigh(hw)[1][:, 0].reshape(xts.shape)
    path = sorted(irc_branch("ch4oh", xts, ets, mode, mass, +1) + [(0.0, ets)] +
                  irc_branch("ch4oh", xts, ets, mode, mass, -1))
    s, e = np.array(path).T
    fig = np.loadtxt(os.path.join(REF, "figure_irc_ch4oh.txt"))
    # which branch is which is the sign of an eigenvector: orient by the
    # product valley (the lower end)
    if e[0] > e[-1]:
        s = -s[::-1]
        e = e[::-1]
    # the saddle: the plotted maximum, -0.70489 Hartree (line centre,
    # +-1e-4 reading), against the Newton saddle
    assert abs(fig[:, 1].max() - ets) < 3e-4
    # the valleys, |s| >= 1.3 bohr amu^1/2 where the path is flat enough
    # that the reading error is the line width: within 1.5e-4 Hartree
    # (0.09 kcal/mol); the plot resolves 6e-5 Hartree per pixel
    flat = (np.abs(s) >= 1.3) & (s >= fig[0, 0]) & (s <= fig[-1, 0])
    assert flat.sum() >= 12
    ef = np.interp(s[flat], fig[:, 0], fig[:, 1])
    assert np.abs(ef - e[flat]).max() < 1.5e-4, np.c_[s[flat], e[flat], ef]
    # both ends: products CH3 + H2O near -0.7356, the CH4 + OH side near -0.7158
    assert abs(e[0] - (-0.7356)) < 3e-4 and abs(e[-1] - (-0.7158)) < 3e-4


def _tetra():
    s3 = 1.0 / np.sqrt(3.0)
    return np.array([[s3, s3, s3], [s3, -s3, -s3], [-s3, s3, -s3], [-s3, -s3, s3]])


def test_ch4h_published_energetics():
    v = _tetra()

    def geom(r_attacked, r_hh, r_other=1.09):
        q = np.zeros((6, 3))          # H (attacked), C, H, H, H, H (abstracting)
        q[0] = v[0] * r_attacked
        q[2], q[3], q[4] = v[1] * r_other, v[2] * r_other, v[3] * r_other
        q[5] = v[0] * (r_attacked + r_hh)
        return q * ANG

    xts, ets, gts, wts = stationary_point("ch4h", geom(1.40, 0.89))
    xr, er, gr, wr = stationary_point("ch4h", geom(1.09, 20.0))
    xp, ep, gp, wp = stationary_point("ch4h", geom(20.0, 0.74, 1.08))
    assert np.count_nonzero(wts < -1e-4) == 1 and np.count_nonzero(wr < -1e-4) == 0
    assert np.count_nonzero(wp < -1e-4) == 0 and max(gts, gr, gp) < 1e-6
    barrier, dE = (ets - er) * KCAL, (ep - er) * KCAL
    assert abs(dE - 2.88) < 0.02, dE
    assert abs(barrier - 15.0) < 0.1, barrier
    # the saddle is collinear C-H-H
    u, w2 = xts[0] - xts[1], xts[5] - xts[0]
    assert np.dot(u, w2) / np.linalg.norm(u) / np.linalg.norm(w2) > 1.0 - 1e-9


def test_oh3_published_energetics():
    def bent(r1, ang_deg):
        a = np.radians(ang_deg)
        return np.array([r1 * np.cos(a), r1 * np.sin(a), 0.0])

    # O, H (of OH), H, H
    ts0 = np.array([[0.0, 0.0, 0.0], bent(0.97, 97.0), [1.35, 0.0, 0.0], [2.17, 0.0, 0.0]]) * ANG
    re0 = np.array([[0.0, 0.0, 0.0], [0.97, 0.0, 0.0], [0.0, 20.0, 0.0], [0.0, 20.74, 0.0]]) * ANG
    pr0 = np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], bent(0.96, 104.5), [-20.0, 0.0, 0.0]]) * ANG
    xts, ets, gts, wts = stationary_point("oh3", ts0)
    xr, er, gr, wr = stationary_point("oh3", re0)
    xp, ep, gp, wp = stationary_point("oh3", pr0)
    assert np.count_nonzero(wts < -1e-4) == 1 and np.count_nonzero(wr < -1e-4) == 0
    assert np.count_nonzero(wp < -1e-4) == 0 and max(gts, gr, gp) < 1e-6
    barrier, dE = (ets - er) * KCAL, (ep - er) * KCAL
    assert abs(barrier - 6.1) < 0.05, barrier
    assert abs(dE - (-15.2)) < 0.05, dE


@pytest.mark.parametrize("name,xcol,lo,hi", [("pmf_h3", 1.0, 48.0, 49.0), ("kappa_h3", 50.0, 0.764, 0.770)])
def test_h_h2_figures_read_back(name, xcol, lo, hi):
    """The digitised H + H2 figures give the values the rate tests hold the
    engine to: PMF maximum ~48.5 kJ/mol at xi ~ 1, kappa(50 fs) ~ 0.767."""
    d = np.loadtxt(os.path.join(REF, f"figure_{name}.txt"))
    if name == "pmf_h3":
        i = np.argmax(d[:, 1])
        assert abs(d[i, 0] - xcol) < 0.01 and lo < d[i, 1] < hi
    else:
        assert lo < np.interp(xcol - 0.2, d[:, 0], d[:, 1]) < hi
