"""Caracal's flexible SPC water box (water_spc): periodic set-up and a
synthetic box builder.

The surface itself (src/egrad_water.f90:36-333, parameters
src/water_init.f90:74-103) runs on the device through
:class:`caracal_gb300.engine.WaterBox`.  :func:`periodic_setup` restates the
cutoff logic of src/set_periodic.f90:78-104 with the box lengths converted to
bohr as src/read_pes.f90:2728-2735 does; :func:`water_box` places molecules
at liquid density for synthetic runs.
"""
from __future__ import annotations

import math

import numpy as np

from .units import mass_au

BOHR = 0.52917721092                       # src/general.f90:256
SPI = 1.77245385090551599275151910313925   # sqrt(pi), src/qmdff.f90:47


def periodic_setup(box_angstrom, coul_cut_angstrom, zahn=False):
    """(box in bohr, coul_cut, zahn_a, zahn_par) as src/set_periodic.f90 sets
    them: a cutoff below 5 bohr becomes half the shortest box length minus
    0.1; the Zahn form fixes a = 0.2 bohr (sic) and the cutoff at 10 A; a
    cutoff beyond half the shortest box length is pulled back to it minus 0.1."""
    box = [float(x) / BOHR for x in box_angstrom]
    half = min(0.5 * b for b in box)
    cut = float(coul_cut_angstrom) / BOHR
    if cut < 5.0:
        cut = half - 0.1
    za = zp = 0.0
    if zahn:
        za = 0.2 * BOHR
        cut = 10.0 / BOHR
        acut = za * cut
        zp = math.erfc(acut) / cut ** 2 + 2 * za / SPI * math.exp(-acut ** 2) / cut
    if cut > half:
        cut = half - 0.1
    return box, cut, za, zp


def masses(nwater):
    """Atomic masses (a.u.) in the order O, H, H per molecule."""
    return np.array([mass_au("O"), mass_au("H"), mass_au("H")] * int(nwater))


def water_box(nwater, density_g_cm3=1.0, seed=0):
    """Coordinates (nwater * 3, 3) in bohr and the cubic box length in
    Angstrom: molecules at the model's equilibrium (r_OH = 1 A, r_HH = 1.633 A)
    on a simple cubic grid, randomly oriented."""
    n = int(nwater)
    vol_cm3 = n * 18.01528 / (6.02214076e23 * density_g_cm3)
    length = (vol_cm3 * 1e24) ** (1.0 / 3.0)  # Angstrom
    m = int(math.ceil(n ** (1.0 / 3.0)))
    step = length / m
    half_angle = math.asin(0.5 * 1.633 / 1.0)
    mol = np.array([[0.0, 0.0, 0.0],
                    [math.sin(half_angle), math.cos(half_angle), 0.0],
                    [-math.sin(half_angle), math.cos(half_angle), 0.0]])
    mol -= mol.mean(axis=0)
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        ix, iy, iz = k % m, (k // m) % m, k // (m * m)
        centre = (np.array([ix, iy, iz]) + 0.5) * step
        a = rng.normal(size=(3, 3))
        qm, r = np.linalg.qr(a)
        qm *= np.sign(np.diag(r))
        out.append(centre + mol @ qm.T)
    return np.concatenate(out) / BOHR, length
