"""Synthetic workloads with the shapes of the engine's benchmark configurations.

Caracal ships no benchmark inputs, so each configuration is a seeded
synthetic input of the stated shape (geometry, bead count, trajectories,
temperature, time step).  Interpretations of under-specified geometry are
parameters here.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au

SEED = 20261203


@dataclass
class Workload:
    name: str
    pes: str
    symbols: list
    q0: np.ndarray          # (natoms, 3) bohr
    nbeads: int
    ntraj: int
    kelvin: float
    dt_fs: float
    nsteps: int
    thermostat: str
    sigma_bohr: float = 0.0
    andersen_step: int = 70
    pile_tau0_fs: float = 100.0
    transrot: bool = True
    seed: int = SEED
    extra: dict = field(default_factory=dict)

    @property
    def mass(self):
        return np.array([mass_au(s) for s in self.symbols])

    @property
    def dt_au(self):
        return dt_fs_to_au(self.dt_fs)

    @property
    def beta(self):
        return beta_from_kelvin(self.kelvin) if self.kelvin else float("inf")

    @property
    def pile_tau0_au(self):
        return dt_fs_to_au(self.pile_tau0_fs)

    @property
    def bead_steps(self):
        return self.nbeads * self.ntraj * self.nsteps


def h3_collinear(r_hh_ang=0.74, r_inc_ang=2.5):
    """Collinear H-H...H along z: H2 bond r_hh, incoming H r_inc from the nearer H."""
    z = np.array([0.0, r_hh_ang, r_hh_ang + r_inc_ang])
    q = np.zeros((3, 3))
    q[:, 2] = z
    return angstrom_to_bohr(q)


def h3_config(ntraj=64, nbeads=16, nsteps=1000, thermostat="pile", kelvin=300.0, dt_fs=0.1):
    """H + H2 on BKMP2: 3 atoms, 16 beads, 64 trajectories, 300 K, 0.1 fs, bead
    jitter sigma = 0.01 Angstrom, PILE tau0 = 100 fs (Andersen: ANDERSEN_STEP 70)."""
    return Workload(name=f"h3_bkmp2_P{nbeads}_T{ntraj}", pes="h3", symbols=["H", "H", "H"],
                    q0=h3_collinear(), nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs,
                    nsteps=nsteps, thermostat=thermostat, sigma_bohr=float(angstrom_to_bohr(0.01)))


def ch4h_dividing_surface(r_ch_ang=1.09, r_hh_ang=1.5):
    """CH4 (tetrahedral, r(CH) = r_ch) + H collinear with one C-H bond, r_hh
    beyond that bond's H (the H...H distance), in Caracal's atom order for
    ANA_CH4H: H (the attacked methane H), C, H, H, H, H_b (abstracting H)."""
    s3 = 1.0 / np.sqrt(3.0)
    v = np.array([[s3, s3, s3], [s3, -s3, -s3], [-s3, s3, -s3], [-s3, -s3, s3]])
    q = np.zeros((6, 3))
    q[0] = v[0] * r_ch_ang
    q[2], q[3], q[4] = v[1] * r_ch_ang, v[2] * r_ch_ang, v[3] * r_ch_ang
    q[5] = v[0] * (r_ch_ang + r_hh_ang)
    return angstrom_to_bohr(q)


def ch4h_config(ntraj=4096, nbeads=32, nsteps=2000, kelvin=500.0, dt_fs=0.1):
    """CH4 + H recrossing children: 6 atoms, 32 beads, 4096 NVE children from
    one dividing-surface geometry, momenta Maxwell at 500 K, 0.1 fs."""
    return Workload(name=f"ch4h_recross_P{nbeads}_T{ntraj}", pes="ch4h",
                    symbols=["H", "C", "H", "H", "H", "H"], q0=ch4h_dividing_surface(),
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps,
                    thermostat="none", sigma_bohr=0.0, transrot=False)


def ch4h_recross_definition(q0):
    """BIMOLEC mechanism of CH4 + H -> CH3 + H2 for Caracal's MECHA block
    (1-based atoms): reactant1 = CH4 (1-5), reactant2 = H_b (6), bond_form 1-6,
    bond_break 2-1; reference bond lengths from the dividing-surface geometry,
    DIST_INF 16 bohr, xi at the dividing surface 1.0."""
    q0 = np.asarray(q0)
    return dict(reac1=[1, 2, 3, 4, 5], reac2=[6], bond_form=(1, 6), bond_break=(2, 1),
                form_ref=float(np.linalg.norm(q0[0] - q0[5])),
                break_ref=float(np.linalg.norm(q0[1] - q0[0])), r_inf=16.0, xi_ideal=1.0)


def qmdff_config(ntraj=1024, nbeads=64, nsteps=500, kelvin=300.0, dt_fs=0.5, nc=20,
                 thermostat="andersen", andersen_step=70):
    """Synthetic QMDFF of C20H42 (62 atoms: the saturated 20-carbon chain), zig-zag
    r(CC) = 1.53 A, r(CH) = 1.09 A, tetrahedral angles: 64 beads, 1024 trajectories,
    NVT 300 K (Andersen, ANDERSEN_STEP 70), 0.5 fs, beads start on the reference
    geometry with 0.01 A jitter.  The force field itself is built by
    ``caracal_gb300.qmdff.alkane`` (extra["ff"])."""
    from . import qmdff as Q
    ff = Q.alkane(nc=nc)
    sym = ["C" if z == 6 else "H" for z in ff.at]
    return Workload(name=f"qmdff_c{nc}h{2 * nc + 2}_P{nbeads}_T{ntraj}", pes="qmdff", symbols=sym,
                    q0=ff.xyz.copy(), nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs,
                    nsteps=nsteps, thermostat=thermostat, andersen_step=andersen_step,
                    sigma_bohr=float(angstrom_to_bohr(0.01)), transrot=True, extra={"ff": ff})


def oh3_geometry():
    """OH + H2 approach in Caracal's ANA_OH3 atom order (O, H of OH, H, H):
    r(OH) = 0.97 A, H2 at 1.4 bohr, its near H 2.9 bohr from O (bohr)."""
    return np.array([[0.0, 0.0, 0.0], [1.83, 0.0, 0.0], [-0.6, 2.9, 0.1], [-0.8, 4.3, 0.2]])


def oh3_config(ntraj=4096, nbeads=32, nsteps=500, kelvin=300.0, dt_fs=0.1, thermostat="andersen",
               andersen_step=70):
    """OH + H2 on the Schatz-Elgersma surface (ANA_OH3): T trajectories of P beads
    near the reactant approach, NVT 300 K, 0.1 fs, 0.01 A bead jitter."""
    return Workload(name=f"oh3_P{nbeads}_T{ntraj}", pes="oh3", symbols=["O", "H", "H", "H"], q0=oh3_geometry(),
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps, thermostat=thermostat,
                    andersen_step=andersen_step, sigma_bohr=float(angstrom_to_bohr(0.01)), transrot=True)


def water_config(nwater=64, ntraj=64, nbeads=32, nsteps=500, kelvin=300.0, dt_fs=0.25, coul_cut_ang=6.0,
                 thermostat="andersen", andersen_step=70, zahn=False):
    """Periodic box of Caracal's flexible SPC water (water_spc): nwater
    molecules at 1 g/cm^3 on a cubic grid, randomly oriented (seed), cubic box,
    Coulomb cutoff coul_cut_ang (pulled below half the box as
    src/set_periodic.f90 does); NVT 300 K, 0.25 fs, beads start on the grid
    geometry with 0.01 A jitter."""
    from . import water as Wt
    x, length = Wt.water_box(nwater, seed=SEED)
    sym = ["O", "H", "H"] * nwater
    return Workload(name=f"water_spc_{nwater}_P{nbeads}_T{ntraj}", pes="water", symbols=sym, q0=x,
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps,
                    thermostat=thermostat, andersen_step=andersen_step,
                    sigma_bohr=float(angstrom_to_bohr(0.01)), transrot=True,
                    extra={"nwater": nwater, "box": [length] * 3, "coul_cut": coul_cut_ang, "zahn": zahn})


def ch4oh_geometry(r_ch_ang=1.09, r_ho_ang=1.3, r_oh_ang=0.97, angle_deg=100.0):
    """CH4 (tetrahedral, r(CH) = r_ch) + OH with O collinear with one C-H bond,
    r_ho beyond that bond's H, and the hydroxyl H at r_oh from O bent by angle_deg
    from the C-H axis, in Caracal's atom order for ANA_CH4OH: H (the attacked
    methane H), C, H, H, H, O, H(O)."""
    s3 = 1.0 / np.sqrt(3.0)
    v = np.array([[s3, s3, s3], [s3, -s3, -s3], [-s3, s3, -s3], [-s3, -s3, s3]])
    q = np.zeros((7, 3))
    q[0] = v[0] * r_ch_ang
    q[2], q[3], q[4] = v[1] * r_ch_ang, v[2] * r_ch_ang, v[3] * r_ch_ang
    q[5] = v[0] * (r_ch_ang + r_ho_ang)
    perp = np.cross(v[0], [0.0, 0.0, 1.0])
    perp /= np.linalg.norm(perp)
    a = np.radians(angle_deg)
    q[6] = q[5] + (-v[0] * np.cos(a) + perp * np.sin(a)) * r_oh_ang
    return angstrom_to_bohr(q)


def ch4h_md_config(ntraj=2048, nbeads=32, nsteps=1000, kelvin=500.0, dt_fs=0.1):
    """CH4 + H thermal trajectories (Andersen, ANDERSEN_STEP 70) from the
    dividing-surface geometry with 0.01 A bead jitter."""
    return Workload(name=f"ch4h_md_P{nbeads}_T{ntraj}", pes="ch4h",
                    symbols=["H", "C", "H", "H", "H", "H"], q0=ch4h_dividing_surface(),
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps,
                    thermostat="andersen", sigma_bohr=float(angstrom_to_bohr(0.01)))


def ch4oh_md_config(ntraj=512, nbeads=64, nsteps=1000, kelvin=300.0, dt_fs=0.1):
    """CH4 + OH thermal trajectories (Andersen, ANDERSEN_STEP 70), 7 atoms."""
    return Workload(name=f"ch4oh_md_P{nbeads}_T{ntraj}", pes="ch4oh",
                    symbols=["H", "C", "H", "H", "H", "O", "H"], q0=ch4oh_geometry(),
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps,
                    thermostat="andersen", sigma_bohr=float(angstrom_to_bohr(0.01)))


def geh4oh_geometry(r_geh_ang=1.525, r_ho_ang=1.5, r_oh_ang=0.97, angle_deg=100.0):
    """GeH4 + OH in Caracal's atom order for ANA_GEH4OH (H attacked, Ge, H, H,
    H, O, H(O)): the CH4 + OH arrangement with r(Ge-H) = 1.525 A."""
    return ch4oh_geometry(r_ch_ang=r_geh_ang, r_ho_ang=r_ho_ang, r_oh_ang=r_oh_ang, angle_deg=angle_deg)


def geh4oh_md_config(ntraj=512, nbeads=64, nsteps=1000, kelvin=300.0, dt_fs=0.1):
    """GeH4 + OH thermal trajectories (Andersen, ANDERSEN_STEP 70), 7 atoms."""
    return Workload(name=f"geh4oh_md_P{nbeads}_T{ntraj}", pes="geh4oh",
                    symbols=["H", "Ge", "H", "H", "H", "O", "H"], q0=geh4oh_geometry(),
                    nbeads=nbeads, ntraj=ntraj, kelvin=kelvin, dt_fs=dt_fs, nsteps=nsteps,
                    thermostat="andersen", sigma_bohr=float(angstrom_to_bohr(0.01)))


def mixed_classes(scale=1, nsteps=1000):
    """Four trajectory classes of uneven atom and bead counts stepped together:
    H3 (N=3) T=4096 P=8 (PILE), CH4H (N=6) T=2048 P=32, CH4OH (N=7) T=512
    P=64, QMDFF C20H42 (N=62) T=128 P=128 (Andersen); 147.5 M bead-steps in
    1000 steps.  Each class has its own noise seed; ``scale`` divides the
    trajectory counts (tests)."""
    t = lambda n: max(1, n // scale)  # noqa: E731
    out = [h3_config(ntraj=t(4096), nbeads=8, nsteps=nsteps, thermostat="pile"),
           ch4h_md_config(ntraj=t(2048), nbeads=32, nsteps=nsteps),
           ch4oh_md_config(ntraj=t(512), nbeads=64, nsteps=nsteps),
           qmdff_config(ntraj=t(128), nbeads=128, nsteps=nsteps)]
    for i, w in enumerate(out):
        w.seed = SEED + 1 + i
    return out
