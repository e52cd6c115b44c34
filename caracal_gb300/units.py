"""Unit conventions of Caracal's dynamic/calc_rate path (atomic units inside).

Constants and their origin in the reference:
  k_B = 0.316679D-5 Eh/K            src/dynamic.f90:79
  dt[a.u.] = dt[fs] / 2.41888428E-2  src/dynamic.f90:589 -- a REAL(4) literal, so the
                                     divisor is the float nearest 0.0241888428
  bohr = 0.52917721092 Angstrom      src/general.f90:256
  emass = 5.485799095d-4 amu         src/general.f90:252 (mass[a.u.] = amu / emass,
                                     src/atommass.f90:215-218)
"""
import numpy as np

K_BOLTZMANN_AU = 0.316679e-5
FS_PER_AU_REAL4 = float(np.float32(2.41888428e-2))
BOHR_ANGSTROM = 0.52917721092
EMASS_AMU = 5.485799095e-4

# element masses used on this path (src/atommass.f90:58-129)
AMU = {"H": 1.00782503207, "D": 2.0141017778, "C": 12.0, "O": 15.99491461956,
       "N": 14.0030740048, "F": 18.9984, "S": 32.06, "Cl": 34.96885268, "Ge": 72.61, "Br": 78.9183371}


def dt_fs_to_au(dt_fs: float) -> float:
    return float(dt_fs) / FS_PER_AU_REAL4


def beta_from_kelvin(kelvin: float) -> float:
    return 1.0 / (float(kelvin) * K_BOLTZMANN_AU)


def mass_au(symbol: str) -> float:
    return AMU[symbol.upper() if len(symbol) == 1 else symbol.capitalize()] / EMASS_AMU


def angstrom_to_bohr(x):
    return np.asarray(x, dtype=np.float64) / BOHR_ANGSTROM


def temperature_from_ekin(ekin: float, natoms: int, nbeads: int) -> float:
    """Caracal's printed temperature 2 Ekin / (3 k_B N P^2) (src/verlet.f90:1186-1188)."""
    return 2.0 * ekin / 3.0 / K_BOLTZMANN_AU / natoms / nbeads / nbeads


def nose_q_to_au(nose_q_steps: float, dt_fs: float) -> float:
    """NOSE_Q in time steps -> a.u. as Caracal computes it: nose_q*dt/2.41888428E-2
    with dt still in fs (src/dynamic.f90:578)."""
    return float(nose_q_steps) * float(dt_fs) / FS_PER_AU_REAL4
