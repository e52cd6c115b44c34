"""Caracal's `dynamic` program on the GPU engine: ``python -m caracal_gb300.dynamic dynamic.key``.

Reads the key file (``caracal_gb300.keyfile``), the XYZSTART geometry and the
force fields, starts every bead on the input structure with mdinit's momenta
(src/dynamic.f90:1307-1314, src/mdinit.f90:110-150; READ_VEL: velocity_start.dat),
advances the engine
TDUMP/DELTAT steps per launch and writes Caracal's output files at every dump
step (src/verlet.f90:780-800, 666-676, 1170-1205; src/dynamic.f90:1458-1486, 1676),
each frame from a page-locked snapshot while the GPU runs the next steps
(cr_engine_run_dump_async):

  trajectory.xyz       natoms*nbeads, a blank line (NpT: the box edges),
                       `name x y z` (Angstrom) for every bead (not with
                       OUTPUT_SPARSE and nbeads > 1)
  traj_centroid.xyz    the centroid frame (nbeads > 1)
  md_energies.dat      (E_CON) istep, Epot/P, Ekin/P, (Epot+Ekin)/P
  stdout               " Step: ... -- pot. energy: ... Hartree -- temperature: ... K";
                       NpT: step, Epot/P, T, volume (A^3), the pressure averaged
                       over the dump interval (atm), density (g/cm^3)

ENSEMBLE NPT (Berendsen barostat, periodic QMDFF) dumps synchronously: the
state, each trajectory's box and the pressure sum every TDUMP/DELTAT steps.

Numbers are written as gfortran's list-directed output writes them (REAL(8):
17 significant digits, G-style, 26 columns; INTEGER: 12 columns).  With
GPU_TRAJECTORIES n > 1 the files carry trajectory 0 and the energies are
averages over the trajectories.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

from . import keyfile as K
from .units import BOHR_ANGSTROM, angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from .units import EMASS_AMU, temperature_from_ekin

PRESCON = 290371576.61  # Hartree/bohr^3 -> atm (src/general.f90:263)


def fortran_real(x):
    """One REAL(8) item of gfortran list-directed output (26 columns)."""
    x = float(x)
    if x == 0.0:
        return "   0.0000000000000000     "
    if not math.isfinite(x):
        return f"{'NaN' if x != x else ('Infinity' if x > 0 else '-Infinity'):>21}     "
    s = f"{x:.16e}"                              # 17 significant digits, correctly rounded
    mant, ex = s.split("e")
    k = int(ex) + 1
    if 0 <= k <= 17 and abs(x) >= 0.1:
        body = f"{x:.{17 - k}f}"
        return f"{body:>21}     "
    e = int(ex)
    return f"{mant:>21}E{'-' if e < 0 else '+'}{abs(e):03d}"


def fortran_int(n):
    return f"{int(n):>12}"


def write_frame(f, names, xyz_ang, box_ang=None):
    """One xyz frame; under NpT the comment line holds the box edges
    (src/verlet.f90:669-673, 788-795)."""
    comment = "" if box_ang is None else "".join(fortran_real(v) for v in box_ang)
    f.write(fortran_int(len(names)) + "\n" + comment + "\n")
    for nm, r in zip(names, xyz_ang):
        f.write(" " + f"{nm:<3}" + "".join(fortran_real(v) for v in r) + "\n")
    f.flush()


def momenta_from_velocities(v, mass, shape):
    """READ_VEL start momenta of every trajectory: bead 1 p = -v m, others 0."""
    p = np.zeros(shape)
    p[:, 0] = -np.asarray(v)[None] * np.asarray(mass)[None, :, None]
    return p


def build_pes(d, nve):
    """The engine's PES argument (and the objects that must stay alive)."""
    if d.pes in K.ANALYTIC:
        return K.ANALYTIC[d.pes], []
    from . import qmdff as Q
    from .engine import EVBPair, QMDFFForceField
    kw = dict(zahn=True, coul_cut=10.0) if nve else dict(zahn=d.zahn, coul_cut=50.0)
    ffs = []
    for i, name in enumerate(d.ffnames):
        ff = Q.read_qmdff(os.path.join(d.directory, name))
        if i < len(d.eshift):
            ff.e_zero = d.eshift[i]
        ffs.append(QMDFFForceField(ff, **kw))
        if d.box:
            # set_periodic with the cutoffs of the key file (Angstrom)
            ffs[-1].set_periodic(d.box, 10.0 if nve else d.coul_cut, 10.0 if nve else d.vdw_cut)
    if d.pes == "QMDFF":
        return ffs[0], ffs
    if len(ffs) != 2:
        raise K.KeyError_("DE_EVB needs two force fields in FFNAMES")
    par = K.read_evb_pars(os.path.join(d.directory, "evb_pars.dat"), d.coupling)
    pair = EVBPair(ffs[0], ffs[1], d.coupling, **par)
    return pair, ffs + [pair]


def run(path, out_dir=None, quiet=False):
    from .engine import RPMDEngine
    d = K.read(path)
    out_dir = out_dir or os.getcwd()
    sym, xyz = K.read_xyz(os.path.join(d.directory, d.xyzstart))
    q0 = angstrom_to_bohr(np.array(xyz))
    mass = np.array([mass_au(s) for s in sym])
    nve = d.ensemble == "NVE"
    pes, keep = build_pes(d, nve)
    beta = None if nve or d.kelvin <= 0.0 else beta_from_kelvin(d.kelvin)
    thermo = "none" if nve else d.thermostat
    eng = RPMDEngine(pes, mass, d.nbeads, d.ntraj, dt_fs_to_au(d.dt_fs), beta=beta, thermostat=thermo,
                     andersen_step=d.andersen_step, transrot=True, precision="fp64", seed=d.seed,
                     nose_q_au=nose_q_to_au(d.nose_damp, d.dt_fs))
    npt = d.ensemble == "NPT"
    if npt:  # Berendsen barostat on the periodic force field's box
        eng.set_npt(d.pressure)
    eng.init_positions(q0, 0.0)
    eng.init_momenta(zero=nve)
    eng.compute_forces()
    if d.read_vel and not nve and d.thermostat == "andersen":
        # src/mdinit.f90:113-118: bead 1 gets p = -v m (sign as in the
        # reference); the reference leaves the other beads unset, here zero
        v = K.read_velocities(os.path.join(d.directory, "velocity_start.dat"), len(sym))
        q, p, f, _, _ = eng.get_state()
        eng.set_state(q, momenta_from_velocities(v, mass, p.shape), f)
    names = list(sym)
    P, N = d.nbeads, len(sym)
    traj = None if (d.output_sparse and P > 1) else open(os.path.join(out_dir, "trajectory.xyz"), "w")
    cen = open(os.path.join(out_dir, "traj_centroid.xyz"), "w") if P > 1 else None
    ener = open(os.path.join(out_dir, "md_energies.dat"), "w") if d.energycon else None
    if ener:
        ener.write(" #   MD step   pot.energy    kin.energy   total energy \n")
    iw = max(d.iwrite, 1)

    def dump(istep, q, p, epot, box=None, press_avg=None):
        ekin = float(np.mean(np.sum(p * p / (2.0 * mass[None, None, :, None]), axis=(1, 2, 3))))
        ep = float(np.mean(epot))
        b0 = None if box is None else box[0] * BOHR_ANGSTROM
        if traj:
            write_frame(traj, names * P, q[0].reshape(-1, 3) * BOHR_ANGSTROM, b0)
        if cen:
            write_frame(cen, names, q[0].mean(axis=0) * BOHR_ANGSTROM, b0)
        if ener:
            ener.write(fortran_int(istep) + fortran_real(ep / P) + fortran_real(ekin / P) +
                       fortran_real((ep + ekin) / P) + "\n")
        if not quiet and box is not None:
            # src/verlet.f90:1190-1197: volume (A^3), press_avg (atm), density
            # (g/cm^3; the REAL(4) literals 1.6605402E-24 and 1E-24 widened)
            t = temperature_from_ekin(ekin, N, P)
            vol = float(np.mean(np.prod(box, axis=1))) * BOHR_ANGSTROM ** 3
            dens = (float(np.sum(mass)) * float(np.float32(1.6605402e-24)) * EMASS_AMU) / (vol * float(np.float32(1e-24)))
            print(f"{istep:8d}{ep / P:12.5f}     {t:10.4f}  {vol:12.4f}{float(np.mean(press_avg)) * PRESCON:14.5f}"
                  f"    {dens:12.6f}")
        elif not quiet:
            if nve:
                print(f" Step: {istep:8d}  --  pot. energy: {ep / P:12.5f} Hartree ")
            else:
                t = temperature_from_ekin(ekin, N, P)
                print(f" Step: {istep:8d}  --  pot. energy: {ep / P:12.5f} Hartree  --  temperature: "
                      f"{t:10.4f} K")
        return False

    try:
        if npt:
            # every iwrite steps: the state, the boxes and the pressure sum
            done = 0
            while done + iw <= d.nstep:
                eng.run(iw)
                done += iw
                q, p, _, epot, _ = eng.get_state()
                box, _, psum = eng.npt_state(reset_sum=True)
                dump(done, q, p, epot, box, psum / iw)
            if done < d.nstep:
                eng.run(d.nstep - done)
        else:
            # frames are written from page-locked snapshots while the GPU steps on
            eng.run_dump_async(d.nstep, iw, dump)
    finally:
        for fh in (traj, cen, ener):
            if fh:
                fh.close()
        eng.close()
        for o in keep:
            o.close()
    return d


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m caracal_gb300.dynamic dynamic.key", file=sys.stderr)
        return 2
    try:
        d = run(argv[0])
    except K.KeyError_ as e:
        print(f" {e}", file=sys.stderr)
        return 1
    if d.unsupported:
        print(" keywords outside this engine's path were ignored: " + " ".join(d.unsupported), file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(main())
