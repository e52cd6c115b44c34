"""Caracal's keyword input for `dynamic` (the subset on this engine's path).

A key file is a list of lines; the first word of a line is the keyword
(case-insensitive), the rest its values, and a line `NAME {` opens a block
closed by `}`.  Read here, with Caracal's defaults and checks:

  general (src/dynamic.f90:243-320): XYZSTART file, RPMD_BEADS n, ENSEMBLE NVE|NVT|NPT,
    STEPS n, DELTAT dt_fs, TDUMP t_fs   (iwrite = nint(TDUMP / DELTAT))
  NVT { TEMP K, THERMOSTAT ANDERSEN|NOSE-HOOVER, ANDERSEN_STEP n, NOSE_DAMP n }
  NPT { TEMP K, PRES atm, THERMOSTAT ..., BAROSTAT BERENDSEN, ANDERSEN_STEP n,
    NOSE_DAMP n, BARO_DAMP n }  (src/dynamic.f90:478-580; periodic QMDFF only;
    BAROSTAT NOSE-HOOVER stops: its chain is not built here)
    (src/dynamic.f90:382-473; defaults TEMP 0, ANDERSEN_STEP 70, NOSE_DAMP 100)
  PES ANA_H3 | ANA_BRH2 | ANA_CH4H | ANA_CH4OH | ANA_OH3 | ANA_GEH4OH | QMDFF | DE_EVB
    (src/read_pes.f90:203, 413-631)
  QMDFF { FFNAMES file [file2], ESHIFT e1 [e2], COULOMB ZAHN, COUL_CUTOFF A,
    VDW_CUTOFF A }  (src/read_pes.f90:1745-1863; defaults 50 and 10)
  PERIODIC x y z (box edges, Angstrom; src/read_pes.f90:164-170) for QMDFF / DE_EVB
  DE_EVB { COUPLING basis }  with the parameters in evb_pars.dat
    (src/read_pes.f90:1928-1975, 2557-2600)
  E_CON (md_energies.dat), OUTPUT_SPARSE (no all-bead trajectory for P > 1)
  and, for this engine only, GPU_TRAJECTORIES n (independent trajectories
  stepped together; Caracal runs one) and SEED n.

Keywords outside this subset are reported by `unsupported`; NPT and the
other surfaces are not on this engine's path.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

ANALYTIC = {"ANA_H3": "h3", "ANA_CH4H": "ch4h", "ANA_CH4OH": "ch4oh", "ANA_OH3": "oh3", "ANA_GEH4OH": "geh4oh", "ANA_BRH2": "brh2"}
EVB_BASES = ("1g", "2g", "3g", "sp", "sd", "sd2", "sp2d")
KNOWN = {"XYZSTART", "RPMD_BEADS", "ENSEMBLE", "STEPS", "DELTAT", "TDUMP", "TDUMP_CUT", "PES", "NVT", "NVE", "NPT",
         "QMDFF", "DE_EVB", "GPU_TRAJECTORIES", "SEED", "E_CON", "OUTPUT_SPARSE", "READ_VEL", "PERIODIC", "}"}


class KeyError_(ValueError):
    """A key file Caracal would stop on (its `fatal`)."""


@dataclass
class DynamicInput:
    xyzstart: str = ""
    nbeads: int = 1
    ensemble: str = "NVE"
    nstep: int = 0
    dt_fs: float = 1.0
    tdump_fs: float = 1.0
    kelvin: float = 0.0
    thermostat: str = "none"
    andersen_step: int = 70
    nose_damp: float = 100.0
    pes: str = ""
    ffnames: list = field(default_factory=list)
    eshift: list = field(default_factory=list)
    coupling: str = "1g"
    ntraj: int = 1
    seed: int = 0
    energycon: bool = False      # E_CON: md_energies.dat (src/dynamic.f90:1130-1140)
    output_sparse: bool = False  # OUTPUT_SPARSE: no all-bead trajectory (src/dynamic.f90:1145-1155)
    read_vel: bool = False       # READ_VEL: start momenta from velocity_start.dat (src/dynamic.f90:1031-1059)
    box: list = field(default_factory=list)  # PERIODIC x y z (Angstrom); empty: not periodic
    zahn: bool = False           # QMDFF { COULOMB ZAHN }
    coul_cut: float = 50.0       # QMDFF { COUL_CUTOFF } (Angstrom where periodic)
    vdw_cut: float = 10.0        # QMDFF { VDW_CUTOFF } (Angstrom)
    pressure: float = 0.0        # NPT { PRES } (atm)
    barostat: str = ""           # NPT { BAROSTAT }: "berendsen"
    unsupported: list = field(default_factory=list)
    directory: str = "."

    @property
    def iwrite(self):
        """Steps between trajectory frames: Fortran nint(TDUMP / DELTAT)."""
        x = self.tdump_fs / self.dt_fs
        return int(x + 0.5) if x >= 0 else -int(-x + 0.5)


def _words(line):
    return line.split()


def _blocks(lines, name):
    """Lines inside every `name {` ... `}` block."""
    out = []
    for i, ln in enumerate(lines):
        head = ln.strip().upper().replace(" ", "")
        if head == name + "{":
            for ln2 in lines[i + 1:]:
                w = _words(ln2)
                if w and w[0] == "}":
                    break
                out.append(ln2)
            else:
                raise KeyError_(f"The {name} section has no second delimiter! (}})")
    return out


def parse(text, directory="."):
    """DynamicInput from the text of a key file."""
    lines = [ln.rstrip("\n") for ln in text.splitlines()]
    d = DynamicInput(directory=directory)
    inside = set()
    for name in ("NVT", "NVE", "QMDFF", "DE_EVB", "NPT"):
        for ln in _blocks(lines, name):
            inside.add(ln)
    for ln in lines:
        w = _words(ln)
        if not w or ln in inside:
            continue
        k = w[0].upper()
        if k == "XYZSTART":
            d.xyzstart = w[1]
        elif k == "RPMD_BEADS":
            d.nbeads = int(w[1])
        elif k == "ENSEMBLE":
            d.ensemble = w[1].upper()
        elif k == "STEPS":
            d.nstep = int(w[1])
        elif k == "DELTAT":
            d.dt_fs = float(w[1].replace("d", "e").replace("D", "E"))
        elif k == "TDUMP":
            d.tdump_fs = float(w[1].replace("d", "e").replace("D", "E"))
        elif k == "PES":
            d.pes = w[1].upper()
        elif k == "GPU_TRAJECTORIES":
            d.ntraj = int(w[1])
        elif k == "SEED":
            d.seed = int(w[1])
        elif k == "E_CON":
            d.energycon = True
        elif k == "OUTPUT_SPARSE":
            d.output_sparse = True
        elif k == "READ_VEL":
            d.read_vel = True
        elif k == "PERIODIC":
            try:
                d.box = [float(x) for x in w[1:4]]
            except ValueError:
                d.box = []
            if len(d.box) != 3:
                raise KeyError_("Correct format: PERIODIC [xlen,ylen,zlen (A)]")
        elif k.rstrip("{") not in KNOWN and not k.startswith("#") and not k.startswith("!"):
            d.unsupported.append(k)
    # checks of src/dynamic.f90:290-320
    if d.nbeads < 1:
        raise KeyError_("The number of RPMD beads must be positive!")
    if d.ensemble not in ("NVE", "NVT", "NPT"):
        raise KeyError_("No valid thermodynamic ensemble given! Choose either NVE, NVT or NPT.")
    if d.nstep < 1:
        raise KeyError_("The number of MD timesteps must be greater than zero!")
    if d.dt_fs < 1e-5:
        raise KeyError_("The MD timestep is too small to be useful!")
    if d.ensemble in ("NVT", "NPT"):
        thermo = "none"
        baro = "BERENDSEN"  # src/dynamic.f90:485 (the default)
        for ln in _blocks(lines, d.ensemble):
            w = _words(ln)
            k = w[0].upper()
            if k == "TEMP":
                d.kelvin = float(w[1])
            elif k == "THERMOSTAT":
                thermo = w[1].upper()
            elif k == "ANDERSEN_STEP":
                d.andersen_step = int(w[1])
            elif k == "NOSE_DAMP":
                d.nose_damp = float(w[1])
            elif k == "PRES" and d.ensemble == "NPT":
                d.pressure = float(w[1].replace("d", "e").replace("D", "E"))
            elif k == "BAROSTAT" and d.ensemble == "NPT":
                baro = w[1].upper() if len(w) > 1 else ""
        if d.kelvin < 0.0:
            raise KeyError_("Give a positive temperature!")
        if d.ensemble == "NPT":
            if baro == "NOSE-HOOVER":
                raise KeyError_("BAROSTAT NOSE-HOOVER (nhc_npt) is not on this engine's path; BERENDSEN is")
            if baro != "BERENDSEN":
                raise KeyError_("No valid barostat chosen! BERENDSEN and NOSE-HOOVER are available!")
            if d.pressure < 0.0:
                raise KeyError_("Give a positive pressure!")
            d.barostat = "berendsen"
        if thermo == "ANDERSEN":
            d.thermostat = "andersen"
        elif thermo == "NOSE-HOOVER":
            d.thermostat = "nhc"
        else:
            raise KeyError_("No availiable thermostat was chosen! Add the keyword THERMOSTAT!")
    if d.pes in ("QMDFF", "DE_EVB"):
        for ln in _blocks(lines, "QMDFF"):
            w = _words(ln)
            k = w[0].upper()
            if k == "FFNAMES":
                d.ffnames = w[1:3] if d.pes == "DE_EVB" else w[1:2]
            elif k == "ESHIFT":
                d.eshift = [float(x.replace("d", "e").replace("D", "E")) for x in w[1:3]]
            elif k == "COULOMB":
                # only ZAHN changes the Coulomb treatment; PPPME stops the run
                # (src/read_pes.f90:1832-1849), other names are just recorded
                if len(w) < 2:
                    raise KeyError_("Correct format: COULOMB [method]")
                if w[1].upper() == "PPPME":
                    raise KeyError_("The Particle Particle Particle Mesh Ewald (PPPME) method is not complete")
                d.zahn = w[1].upper() == "ZAHN"
            elif k == "COUL_CUTOFF":
                d.coul_cut = float(w[1])
            elif k == "VDW_CUTOFF":
                d.vdw_cut = float(w[1])
        if not d.ffnames:
            raise KeyError_("Please check the QMDFFNAMES keyword!")
    if d.pes == "DE_EVB":
        for ln in _blocks(lines, "DE_EVB"):
            w = _words(ln)
            if w[0].upper() == "COUPLING":
                d.coupling = w[1] if w[1] in EVB_BASES else "1g"
    if d.pes not in ANALYTIC and d.pes not in ("QMDFF", "DE_EVB"):
        raise KeyError_(f"PES {d.pes or '(none)'} is not on this engine's path")
    if d.box and d.pes in ANALYTIC:
        raise KeyError_("PERIODIC applies to QMDFF force fields on this engine")
    if d.ensemble == "NPT" and not d.box:
        raise KeyError_("The NPT ensemble can only be simulated in periodic systems!")
    if d.ensemble == "NPT" and d.pes != "QMDFF":
        raise KeyError_("NPT is built for one QMDFF force field on this engine")
    return d


def read(path):
    with open(path) as f:
        return parse(f.read(), directory=os.path.dirname(os.path.abspath(path)))


def read_xyz(path):
    """(symbols, coordinates in Angstrom) of the first frame of an xyz file."""
    with open(path) as f:
        n = int(f.readline().split()[0])
        f.readline()
        sym, xyz = [], []
        for _ in range(n):
            w = f.readline().split()
            sym.append(w[0])
            xyz.append([float(x) for x in w[1:4]])
    return sym, xyz


def read_velocities(path, natoms):
    """velocity_start.dat (src/dynamic.f90:1047-1059): two lines skipped, then
    per atom `idum idum vx vy vz`; returns (natoms, 3)."""
    with open(path) as f:
        lines = f.read().splitlines()
    v = np.zeros((natoms, 3))
    rows = [ln for ln in lines[2:] if ln.strip()]
    if len(rows) < natoms:
        raise KeyError_("velocity_start.dat has fewer lines than atoms")
    for i in range(natoms):
        w = rows[i].replace("d", "e").replace("D", "E").split()
        v[i] = [float(x) for x in w[2:5]]
    return v


def read_evb_pars(path, basis):
    """Coupling parameters from evb_pars.dat in the order of
    src/read_pes.f90:2565-2590 (a name line, then one value per line)."""
    order = {"1g": "ab", "2g": "abcdm", "3g": "abcdefmn", "sp": "abcd", "sd": "abcd", "sd2": "abcdef",
             "sp2d": "abcdefgh"}[basis]
    with open(path) as f:
        vals = [ln.split()[0] for ln in f.read().splitlines()[1:] if ln.split()]
    if len(vals) < len(order):
        raise KeyError_("The evb_pars.dat file contains too few lines or has a wrong formate!")
    return {k: float(v.replace("d", "e").replace("D", "E")) for k, v in zip(order, vals)}
