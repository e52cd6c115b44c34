"""Caracal's `calc_rate` (BIMOLEC reactions, analytic surfaces) on the GPU engine:
``python -m caracal_gb300.calc_rate calc_rate.key``.

The parts of src/calc_rate.f90 and where they run here:

1. umbrella windows xi = BONDS lo .. hi in steps of DIST (UMBRELLA block), each
   with SAMPLE_TRAJS trajectories: all windows' trajectories are one engine
   (cr_engine_set_umbrella), equilibrated EQUI_STEPS steps with the bias
   BIAS * TEMP, then sampled SAMPLE_STEPS steps after unbiased forces
   (src/calc_rate.f90:1568-1700); per window the average and variance of xi
   are the means over its trajectories.  The windows' start structures are
   pulled along xi from TS_STRUC as Caracal generates them (GEN_STEPS steps
   per window with the bias of that window, outwards from the transition
   state, src/calc_rate.f90:860-1110).
2. the free-energy profile by umbrella integration over XI_RANGE with BINS
   points (PMF block; src/calc_rate.f90:1936-1998), written to
   pmf_integration.dat in kJ/mol; its maximum and the minimum before it.
3. the recrossing factor: a SHAKE/RATTLE parent on the dividing surface at
   the PMF maximum (cr_engine_set_parent), equilibrated EQUI_STEPS steps; every
   CHILD_INTERVAL steps CHILD_PERPOINT children (+-p pairs) run CHILD_STEPS
   NVE steps from the parent's ring polymer (cr_engine_init_children) until
   CHILD_TOTAL children; kappa(t) = sum of flux numerators / denominators
   (src/recross.f90:540-637), written to recross.dat.
4. k(T) by the BIMOLEC formula of src/calc_k_t.f90 (caracal_gb300.pmf).
"""
from __future__ import annotations

import os
import sys
from dataclasses import dataclass, field

import numpy as np

from . import keyfile as K
from .pmf import bimolecular_rate, umbrella_integration
from .units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au


@dataclass
class RateInput:
    ts_struc: str = ""
    nbeads: int = 1
    dt_fs: float = 0.1
    pes: str = ""
    kelvin: float = 0.0
    thermostat: str = "andersen"
    andersen_step: int = 70
    reac1: list = field(default_factory=list)
    reac2: list = field(default_factory=list)
    bond_form: tuple = (0, 0)
    bond_break: tuple = (0, 0)
    r_inf: float = 0.0
    npaths: int = 1
    bias: float = 0.0
    umbr_lo: float = 0.0
    umbr_hi: float = 1.0
    umbr_dist: float = 0.1
    gen_steps: int = 0
    equi_steps: int = 0
    sample_steps: int = 0
    sample_trajs: int = 1
    xi_lo: float = 0.0
    xi_hi: float = 1.0
    nbins: int = 100
    rc_equi: int = 0
    child_total: int = 0
    child_interval: int = 1
    child_perpoint: int = 2
    child_steps: int = 0
    seed: int = 0
    directory: str = "."


def parse(text, directory="."):
    lines = text.splitlines()
    r = RateInput(directory=directory)
    for ln in lines:
        w = ln.split()
        if not w:
            continue
        k = w[0].upper()
        if k == "TS_STRUC":
            r.ts_struc = w[1]
        elif k == "RPMD_BEADS":
            r.nbeads = int(w[1])
        elif k == "DELTAT":
            r.dt_fs = float(w[1])
        elif k == "PES":
            r.pes = w[1].upper()
        elif k == "SEED":
            r.seed = int(w[1])
    for ln in K._blocks(lines, "NVT"):
        w = ln.split()
        k = w[0].upper()
        if k == "TEMP":
            r.kelvin = float(w[1])
        elif k == "THERMOSTAT":
            r.thermostat = {"ANDERSEN": "andersen", "NOSE-HOOVER": "nhc"}.get(w[1].upper(), "andersen")
        elif k == "ANDERSEN_STEP":
            r.andersen_step = int(w[1])
    for ln in K._blocks(lines, "MECHA"):
        w = ln.split()
        k = w[0].upper()
        if k == "TYPE" and w[1].upper() != "BIMOLEC":
            raise K.KeyError_("only the BIMOLEC reaction type is on this engine's path")
        if k == "REACTANT1":
            r.reac1 = [int(x) for x in w[1:]]
        elif k == "REACTANT2":
            r.reac2 = [int(x) for x in w[1:]]
        elif k == "DIST_INF":
            r.r_inf = float(w[1])
        elif k == "N_PATHS":
            r.npaths = int(w[1])
        elif k == "BOND_FORM":
            r.bond_form = (int(w[1]), int(w[2]))
        elif k == "BOND_BREAK":
            r.bond_break = (int(w[1]), int(w[2]))
    for ln in K._blocks(lines, "UMBRELLA"):
        w = ln.split()
        k = w[0].upper()
        if k == "BIAS":
            r.bias = float(w[1])
        elif k == "BONDS":
            r.umbr_lo, r.umbr_hi = float(w[1]), float(w[2])
        elif k == "DIST":
            r.umbr_dist = float(w[1])
        elif k == "GEN_STEPS":
            r.gen_steps = int(w[1])
        elif k == "EQUI_STEPS":
            r.equi_steps = int(w[1])
        elif k == "SAMPLE_STEPS":
            r.sample_steps = int(w[1])
        elif k == "SAMPLE_TRAJS":
            r.sample_trajs = int(w[1])
    for ln in K._blocks(lines, "PMF"):
        w = ln.split()
        k = w[0].upper()
        if k == "XI_RANGE":
            r.xi_lo, r.xi_hi = float(w[1]), float(w[2])
        elif k == "BINS":
            r.nbins = int(w[1])
    for ln in K._blocks(lines, "RECROSS"):
        w = ln.split()
        k = w[0].upper()
        if k == "EQUI_STEPS":
            r.rc_equi = int(w[1])
        elif k == "CHILD_TOTAL":
            r.child_total = int(w[1])
        elif k == "CHILD_INTERVAL":
            r.child_interval = int(w[1])
        elif k == "CHILD_PERPOINT":
            r.child_perpoint = int(w[1])
        elif k == "CHILD_STEPS":
            r.child_steps = int(w[1])
    if r.pes not in K.ANALYTIC:
        raise K.KeyError_(f"PES {r.pes or '(none)'}: calc_rate runs on the analytic surfaces here")
    if r.kelvin <= 0.0:
        raise K.KeyError_("Give a positive temperature!")
    return r


def reference_bonds(q0, r):
    """MECHA reference bond lengths from the transition-state structure."""
    f, b = r.bond_form, r.bond_break
    return (float(np.linalg.norm(q0[f[0] - 1] - q0[f[1] - 1])), float(np.linalg.norm(q0[b[0] - 1] - q0[b[1] - 1])))


def generate_structures(r, pes, mass, beta, dt, q0, xw, kf, mech):
    """Start ring polymers of the windows: one trajectory pulled from the
    transition state outwards, GEN_STEPS steps in each window's bias."""
    from .engine import RPMDEngine
    out = np.zeros((len(xw), r.nbeads, len(mass), 3))
    up = [i for i in range(len(xw)) if xw[i] >= 1.0]
    down = [i for i in reversed(range(len(xw))) if xw[i] < 1.0]
    for seq in (up, down):
        if not seq:
            continue
        g = RPMDEngine(pes, mass, r.nbeads, 1, dt, beta=beta, thermostat=r.thermostat,
                       andersen_step=r.andersen_step, transrot=True, seed=r.seed + 7)
        g.init_positions(q0, 0.0)
        g.init_momenta()
        for i in seq:
            q, p, f, _, _ = g.get_state()
            g.set_umbrella(centers=[xw[i]], kforce=kf, **mech)
            g.set_state(q, p, f)
            g.run(max(r.gen_steps, 1))
            out[i] = g.get_state()[0][0]
        g.close()
    return out


def write_recross_restart(out_dir, bunches_done, num, den, qpar):
    """The recrossing restart files after a bunch of children
    (src/recross.f90:418-440): recross_num_tmp.dat (one numerator per child
    step), recross_denom_tmp.dat, recross_parent_pos.dat (the parent's beads,
    `x y z` bohr per atom) and recross_status (bunches done).  Caracal opens
    the parent file with status="replace" and then reads from it, so its file
    stays empty and its resume starts over; here the file holds the parent."""
    with open(os.path.join(out_dir, "recross_num_tmp.dat"), "w") as fh:
        for v in num:
            fh.write(f"{v:26.16E}\n")
    with open(os.path.join(out_dir, "recross_denom_tmp.dat"), "w") as fh:
        fh.write(f"{den:26.16E}\n")
    with open(os.path.join(out_dir, "recross_parent_pos.dat"), "w") as fh:
        for bead in qpar:
            for atom in bead:
                fh.write("".join(f"{v:26.16E}" for v in atom) + "\n")
    with open(os.path.join(out_dir, "recross_status"), "w") as fh:
        fh.write(f"{int(bunches_done):12d}\n")


def read_recross_restart(out_dir, child_steps, nbeads, natoms):
    """(bunches done, numerators, denominator, parent beads or None) from the
    restart files (src/recross.f90:124-228); missing or incomplete files give
    a fresh start (0, zeros, 0, None), an incomplete parent file None."""
    fresh = (0, np.zeros(child_steps), 0.0, None)
    try:
        with open(os.path.join(out_dir, "recross_status")) as fh:
            k = int(fh.read().split()[0])
        with open(os.path.join(out_dir, "recross_num_tmp.dat")) as fh:
            num = np.array([float(x.replace("D", "E")) for x in fh.read().split()])
        with open(os.path.join(out_dir, "recross_denom_tmp.dat")) as fh:
            den = float(fh.read().split()[0].replace("D", "E"))
    except (OSError, ValueError, IndexError):
        return fresh
    if k <= 0 or len(num) < child_steps:
        return fresh
    qpar = None
    try:
        with open(os.path.join(out_dir, "recross_parent_pos.dat")) as fh:
            vals = np.array([float(x.replace("D", "E")) for x in fh.read().split()])
        if len(vals) >= nbeads * natoms * 3:
            qpar = vals[:nbeads * natoms * 3].reshape(nbeads, natoms, 3)
    except (OSError, ValueError):
        qpar = None
    return k, num[:child_steps], den, qpar


def run(path, out_dir=None, quiet=False):
    from .engine import RPMDEngine
    with open(path) as fh:
        r = parse(fh.read(), directory=os.path.dirname(os.path.abspath(path)))
    out_dir = out_dir or os.getcwd()
    sym, xyz = K.read_xyz(os.path.join(r.directory, r.ts_struc))
    q0 = angstrom_to_bohr(np.array(xyz))
    mass = np.array([mass_au(s) for s in sym])
    beta = beta_from_kelvin(r.kelvin)
    dt = dt_fs_to_au(r.dt_fs)
    form_ref, break_ref = reference_bonds(q0, r)
    mech = dict(reac1=r.reac1, reac2=r.reac2, bond_form=r.bond_form, bond_break=r.bond_break,
                form_ref=form_ref, break_ref=break_ref, r_inf=r.r_inf)
    pes = K.ANALYTIC[r.pes]

    # 1. umbrella windows (n_all windows, src/calc_rate.f90:653-657)
    n_all = int(round((r.umbr_hi - r.umbr_lo) / r.umbr_dist)) + 1
    xw = r.umbr_lo + r.umbr_dist * np.arange(n_all)
    T = n_all * r.sample_trajs
    kf = r.bias * r.kelvin
    starts = generate_structures(r, pes, mass, beta, dt, q0, xw, kf, mech)
    eng = RPMDEngine(pes, mass, r.nbeads, T, dt, beta=beta, thermostat=r.thermostat,
                     andersen_step=r.andersen_step, transrot=True, seed=r.seed)
    eng.init_positions(q0, 0.0)
    eng.init_momenta()
    _, p0, _, _, _ = eng.get_state()
    eng.set_umbrella(centers=np.repeat(xw, r.sample_trajs), kforce=kf, **mech)
    eng.set_state(np.repeat(starts, r.sample_trajs, axis=0), p0)   # unbiased forces
    eng.run(r.equi_steps)
    eng.compute_forces()
    eng.umbrella_sampling(True)
    eng.run(r.sample_steps)
    xs, x2, _ = eng.umbrella_stats()
    eng.close()
    av_t = xs / r.sample_steps
    va_t = x2 / r.sample_steps - av_t * av_t
    average = av_t.reshape(n_all, r.sample_trajs).mean(axis=1)
    variance = va_t.reshape(n_all, r.sample_trajs).mean(axis=1)

    # 2. umbrella integration
    coord, pmf = umbrella_integration(xw, np.full(n_all, kf), average, variance, beta, r.xi_lo, r.xi_hi, r.nbins,
                                      r.sample_trajs * r.sample_steps)
    with open(os.path.join(out_dir, "pmf_integration.dat"), "w") as fh:
        fh.write(" # xi-value     PMF(kJ/mol)\n")
        for c, v in zip(coord, pmf):
            fh.write(f"{c:24.16f}{v * 2625.50:26.16f}\n")
    imax = int(np.argmax(pmf))
    imin = int(np.argmin(pmf[:imax + 1]))
    xi_barrier = float(coord[imax])

    # 3. recrossing: constrained parent at the PMF maximum, children from it
    kappa_num = np.zeros(r.child_steps)
    kappa_den = 0.0
    if r.child_total > 0 and r.child_steps > 0:
        nkids = max(2, r.child_perpoint - r.child_perpoint % 2)
        bunches = -(-r.child_total // nkids)
        point, kappa_num, kappa_den, qpar = read_recross_restart(out_dir, r.child_steps, r.nbeads, len(mass))
        if point >= bunches and qpar is None:
            point = bunches                    # every bunch done: the sums are final
        elif point > 0 and qpar is None:
            point, kappa_num, kappa_den = 0, np.zeros(r.child_steps), 0.0
        done = point * nkids
        par = RPMDEngine(pes, mass, r.nbeads, 1, dt, beta=beta, thermostat=r.thermostat,
                         andersen_step=r.andersen_step, transrot=False, seed=r.seed + 1)
        par.init_positions(q0, 0.0)
        par.init_momenta()
        if qpar is not None and point > 0:     # resume from the saved parent, fresh momenta
            _, p1, _, _, _ = par.get_state()
            par.set_state(qpar[None], p1)
        else:
            par.compute_forces()
        par.set_parent(xi_ideal=xi_barrier, **mech)
        if point == 0:
            par.run(max(r.rc_equi, 1))
        while done < r.child_total:
            par.run(r.child_interval)
            qp, _, _, _, _ = par.get_state()
            # children of this parent snapshot: their own momentum stream (traj0)
            kids = RPMDEngine(pes, mass, r.nbeads, nkids, dt, beta=beta, thermostat="none", transrot=False,
                              seed=r.seed + 2, traj0=point * nkids)
            kids.set_recross(xi_ideal=xi_barrier, max_steps=r.child_steps, **mech)
            kids.init_children(qp[0])
            kids.run(r.child_steps)
            num, den, _ = kids.kappa(r.child_steps)
            kids.close()
            kappa_num[:len(num)] += num
            kappa_den += den
            done += nkids
            point += 1
            write_recross_restart(out_dir, point, kappa_num, kappa_den, qp[0])
        par.close()
    kappa_t = kappa_num / kappa_den if kappa_den > 0 else np.ones(max(r.child_steps, 1))
    with open(os.path.join(out_dir, "recross.dat"), "w") as fh:
        fh.write(" # time (fs)      kappa(t)\n")
        for i, v in enumerate(kappa_t):
            fh.write(f"{(i + 1) * r.dt_fs:24.16f}{v:26.16f}\n")
    kappa = float(kappa_t[-1])
    with open(os.path.join(out_dir, "recross_finished"), "w") as fh:   # src/recross.f90:660-665
        fh.write(f"{kappa:26.16E}\n")
    if kappa < 0.002:   # src/calc_rate.f90:2237-2252
        kappa = 1.0

    # 4. rate constant
    m1 = float(sum(mass[a - 1] for a in r.reac1))
    m2 = float(sum(mass[a - 1] for a in r.reac2))
    k_t = bimolecular_rate(kappa, pmf[imax], pmf[imin], r.r_inf, beta, m1, m2, r.npaths)
    result = dict(xi_barrier=xi_barrier, pmf_max_kjmol=float(pmf[imax] * 2625.50),
                  pmf_min_kjmol=float(pmf[imin] * 2625.50), kappa=kappa, k_t=k_t, windows=n_all,
                  trajectories=T)
    if not quiet:
        print(f" Free energy barrier: {(pmf[imax] - pmf[imin]) * 2625.50:12.5f} kJ/mol at xi = {xi_barrier:10.5f}")
        print(f" Recrossing factor kappa: {kappa:12.6f}")
        print(f" Rate constant k(T): {k_t:16.8e} cm^3 mol^-1 s^-1")
    return result


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m caracal_gb300.calc_rate calc_rate.key", file=sys.stderr)
        return 2
    try:
        run(argv[0])
    except K.KeyError_ as e:
        print(f" {e}", file=sys.stderr)
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
