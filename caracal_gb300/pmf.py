"""Free-energy profiles from umbrella windows, as calc_rate computes them.

* Umbrella integration (Kaestner and Thiel; src/calc_rate.f90:1936-1998):
  for each bin centre xi of nbins points on [xi_min, xi_max], the mean force
  dA/dxi = sum_i N p_i(xi) [(xi - <xi>_i)/(beta var_i) - k_i (xi - xi_i)] /
  sum_i N p_i(xi) with Gaussian p_i of each window's mean and variance, then
  trapezoidal integration; the minimum is shifted to zero.
* WHAM (src/wham.f90): the self-consistent iteration of Caracal's routine with
  its conventions kept: restraint k (xi - xi_i)^2 without the factor 1/2, bin
  j at xi_min + j * bin_size, tolerance 1e-5 on sum (1 - f_new/f_old)^2, and
  the profile converted by 627.509 * bohr (kcal/mol scaled by the Bohr
  radius in Angstrom).  Caracal's own sampling loop leaves the histograms
  that feed its WHAM unfilled; here they come from the device
  (cr_engine_umbrella_stats).
All energies in Hartree unless stated.
"""
from __future__ import annotations

import numpy as np

from .units import BOHR_ANGSTROM, K_BOLTZMANN_AU


def umbrella_integration(xi_windows, kforce, average, variance, beta, xi_min, xi_max, nbins, nsamples):
    """(bin coordinates, PMF in Hartree) of umbrella integration.  The
    windows are xi_windows[i] with force constants kforce[i], sample means
    average[i] and variances variance[i]; nsamples is umbr_traj * umbr_step."""
    xw = np.asarray(xi_windows, dtype=float)
    k = np.asarray(kforce, dtype=float)
    av = np.asarray(average, dtype=float)
    va = np.asarray(variance, dtype=float)
    bin_size = (xi_max - xi_min) / (nbins - 1)
    x = xi_min + bin_size * np.arange(nbins)[:, None]          # (bins, windows)
    p = 1.0 / np.sqrt(2.0 * np.pi * va) * np.exp(-0.5 * (x - av) ** 2 / va)
    da = (1.0 / beta) * (x - av) / va - k * (x - xw)
    w = nsamples * p
    dA = np.sum(w * da, axis=1) / np.sum(w, axis=1)
    coord = np.zeros(nbins)
    pmf = np.zeros(nbins)
    acc = 0.0
    for i in range(nbins - 1):
        coord[i] = 0.5 * (xi_min + i * bin_size + xi_min + (i + 1) * bin_size)
        acc = acc + 0.5 * bin_size * (dA[i] + dA[i + 1])
        pmf[i] = acc
    pmf = pmf - pmf.min()  # over all nbins entries; the last one stays 0 (as Caracal's)
    return coord[:nbins - 1], pmf[:nbins - 1]


def wham(hist, xi_windows, kforce, kelvin, xi_min, xi_max, tol=1e-5, max_iter=100000):
    """(bin centres, PMF as Caracal prints it) from per-window histograms
    hist[window][bin] over [xi_min, xi_max)."""
    h = np.asarray(hist, dtype=float)
    nw, nbins = h.shape
    bin_size = (xi_max - xi_min) / nbins
    beta2 = 1.0 / K_BOLTZMANN_AU / kelvin
    ni = h.sum(axis=1)
    xj = xi_min + bin_size * np.arange(1, nbins + 1)
    pb = h / ni[:, None]
    W = np.exp(-beta2 * np.asarray(kforce)[:, None] * (xj[None, :] - np.asarray(xi_windows)[:, None]) ** 2)
    fi = np.ones(nw)
    for _ in range(max_iter):
        den = (ni[:, None] * W / fi[:, None]).sum(axis=0)
        num = (ni[:, None] * pb).sum(axis=0)
        pu = num / den
        pu[pu == 0.0] = 1e-15
        fnew = (W * pu[None, :]).sum(axis=1)
        eps = np.sum((1.0 - fnew / fi) ** 2)
        fi = fnew
        if not eps > tol:
            break
    pmin = np.max((1.0 / beta2) * np.log(pu))
    centres = xi_min + bin_size * (np.arange(1, nbins + 1) - 0.5)
    return centres, (-(1.0 / beta2) * np.log(pu) + pmin) * 627.509 * BOHR_ANGSTROM


def bimolecular_rate(kappa, pmf_max, pmf_min, r_inf, beta, mass_reac1, mass_reac2, npaths=1):
    """Caracal's BIMOLEC rate constant (src/calc_k_t.f90) in cm^3 mol^-1 s^-1:
    k = npaths kappa 4 pi R_inf^2 sqrt(1/(2 pi beta mu)) exp(-beta (W_max - W_min))
    in atomic units, converted with the reference's single-precision factor
    1e6 (a0^3 / t_au) N_A (its literals carry no D exponent)."""
    f32 = np.float32
    mu = mass_reac1 * mass_reac2 / (mass_reac1 + mass_reac2)
    k = npaths * kappa * 4.0 * np.pi * r_inf * r_inf * np.sqrt(1.0 / (2.0 * np.pi * beta * mu)) * \
        np.exp(-beta * (pmf_max - pmf_min))
    conv = f32(f32(5.2917721092e-11) ** 3) / f32(2.418884326505e-17)
    return float(k * float(f32(1e6)) * float(f32(conv)) * float(f32(6.02214179e23)))
