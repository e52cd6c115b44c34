"""Caracal's `calc_rate` (BIMOLEC reactions, analytic surfaces) on the GPU engine:
``python -m caracal_gb300.calc_rate rate.key``.

Reads Caracal's own calc_rate key files (src/calc_rate_read.f90) and runs
the parts of src/calc_rate.f90 in the reference's order:

1. start structures (src/calc_rate.f90:640-1110): ONE classical trajectory
   (Caracal sets nbeads = 1 here, :649) pulled through the umbrella windows,
   first upwards from the transition state through xi = 1, 1 + dist, ...,
   then from the structure at xi = 1 downwards through 1 - dist, ..., with
   mdinit (fresh Andersen momenta, biased forces) and GEN_STEPS steps in
   each window; the structures are shifted to their centre of mass.  Windows
   1 .. n_all - 1 of BONDS lo .. hi in steps of DIST are made and sampled,
   the window at `hi` never is (the loops stop at n_all - 1, :1359, :1957).
2. umbrella sampling (:1340-1700): SAMPLE_TRAJS ring polymers per window
   (all beads on the window's structure), mdinit, EQUI_STEPS biased steps,
   an unbiased force call, SAMPLE_STEPS steps accumulating xi; a trajectory
   whose xi variance exceeds 1e-2 is run again (:1681-1687).  Caracal runs
   the windows' trajectories one after another over MPI workers; here all
   windows and trajectories are one engine.
3. the free-energy profile by umbrella integration (:1936-1998) and its
   maximum; the minimum at xi = 0 (MINLOC ZERO, the default) or before the
   maximum (MINLOC PMF_MIN) (:2080-2093).
4. the recrossing factor (src/recross.f90:64-668): a SHAKE/RATTLE parent on
   the dividing surface at the PMF maximum, started from the generated
   structure nearest to it (:2180-2196), mdinit, EQUI_STEPS steps with
   ANDERSEN_STEP = int(sqrt(EQUI_STEPS)); then CHILD_TOTAL / CHILD_PERPOINT
   times: CHILD_PERPOINT children (+-p pairs) from the parent's ring polymer
   for CHILD_STEPS NVE steps, then mdinit and CHILD_INTERVAL parent steps
   with ANDERSEN_STEP = int(sqrt(CHILD_INTERVAL)) (:334-480).
   kappa(t) = sum of flux numerators / sum of denominators (:637-658).
5. k(T) by the BIMOLEC formula of src/calc_k_t.f90 (caracal_gb300.pmf).

Statistical errors (not printed by Caracal) come with the result: kappa(t)
by a jackknife over the child batches, the PMF maximum by a jackknife over
the SAMPLE_TRAJS trajectories of every window.

The pipeline takes the engine class as an argument (default: the CUDA
engine, :class:`caracal_gb300.engine.RPMDEngine`); anything with the same
methods can stand in for it.
"""
from __future__ import annotations

import math
import os
import sys
from dataclasses import dataclass, field

import numpy as np

from . import keyfile as K
from .pmf import bimolecular_rate, umbrella_integration
from .units import BOHR_ANGSTROM, angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au

KJMOL_PER_HARTREE = 2625.50   # src/calc_rate.f90:1992


def _nint(x):
    """Fortran NINT: nearest integer, halves away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def _real(w):
    return float(w.replace("d", "e").replace("D", "E"))


@dataclass
class RateInput:
    ts_struc: str = ""
    nbeads: int = 1
    dt_fs: float = 0.1
    pes: str = ""
    kelvin: float = 0.0
    thermostat: str = "andersen"
    andersen_step: int = 70
    umbr_type: str = ""
    reac1: list = field(default_factory=list)
    reac2: list = field(default_factory=list)
    bond_form: tuple = (0, 0)
    bond_break: tuple = (0, 0)
    r_inf: float = 0.0            # bohr (DIST_INF is given in Angstrom)
    npaths: int = 1
    bias: float = 0.0             # force constant per Kelvin (BIAS); k = BIAS * TEMP
    umbr_lo: float = 0.0
    umbr_hi: float = 1.0
    umbr_dist: float = 0.1
    gen_steps: int = 0
    equi_steps: int = 0
    sample_steps: int = 0
    sample_trajs: int = 1
    xi_lo: float = 0.0
    xi_hi: float = 1.0
    nbins: int = 0
    pmf_method: str = "INTEGRATION"
    minloc: str = "ZERO"
    rc_equi: int = 0
    child_total: int = 0
    child_interval: int = 0
    child_perpoint: int = 0
    child_steps: int = 0
    xi_manual: float | None = None
    print_poly: float = -5.0
    tdump_fs: float = 0.0
    seed: int = 0
    directory: str = "."
    # engine-only options (not Caracal keywords): the normal-mode transform
    # (0: Caracal's cosine transform, 1: orthonormal normal modes) and the
    # COM/rotation removal in the structure generation and the windows
    # (Caracal's verlet calls transrot there every step)
    nm_mode: int = 0
    transrot: bool = True


def _pair(tok):
    """An `a-b` atom pair of BOND_FORM / BOND_BREAK (src/calc_rate_read.f90:702-760)."""
    parts = [x for x in tok.replace("-", " ").split() if x]
    if len(parts) != 2:
        raise K.KeyError_(f"Correct format: BOND_FORM/BOND_BREAK [atom1-atom2], got {tok!r}")
    return int(parts[0]), int(parts[1])


def _atoms(words):
    """Atom indices of REACTANT1/2: every integer token (others are skipped,
    as src/calc_rate_read.f90:573-600 does)."""
    out = []
    for x in words:
        try:
            out.append(int(x))
        except ValueError:
            pass
    return out


def parse(text, directory="."):
    """RateInput from the text of a calc_rate key file."""
    lines = [ln.rstrip("\n") for ln in text.splitlines()]
    r = RateInput(directory=directory)
    blocks = {name: K._blocks(lines, name) for name in ("NVT", "MECHA", "UMBRELLA", "PMF", "RECROSS")}
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
            r.dt_fs = _real(w[1])
        elif k == "PES":
            r.pes = w[1].upper()
        elif k == "PRINT_POLYMER":
            r.print_poly = _real(w[1])
        elif k == "TDUMP":
            r.tdump_fs = _real(w[1])
        elif k in ("RANDOM_SEED", "SEED"):
            r.seed = int(w[1])
        elif k == "NM_TRANSFORM":              # engine-only keyword
            r.nm_mode = {"CARACAL": 0, "ORTHONORMAL": 1}[w[1].upper()]
        elif k == "WINDOW_TRANSROT":           # engine-only keyword
            r.transrot = w[1].upper() not in ("OFF", "NO", "FALSE", "0")
    if not blocks["NVT"]:
        raise K.KeyError_("Please add a NVT section with parameters to the keyfile!")
    for ln in blocks["NVT"]:
        w = ln.split()
        if not w:
            continue
        k = w[0].upper()
        if k == "TEMP":
            r.kelvin = _real(w[1])
        elif k == "THERMOSTAT":
            t = w[1].upper()
            if t not in ("ANDERSEN", "NOSE-HOOVER"):
                raise K.KeyError_(f"thermostat {w[1]} is not on this engine's calc_rate path")
            r.thermostat = "andersen" if t == "ANDERSEN" else "nhc"
        elif k == "ANDERSEN_STEP":
            r.andersen_step = int(w[1])
    if not blocks["MECHA"]:
        raise K.KeyError_("Please add a MECHA section with parameters to the keyfile!")
    for ln in blocks["MECHA"]:
        w = ln.split()
        if not w:
            continue
        k = w[0].upper()
        if k == "TYPE":
            r.umbr_type = w[1].upper()
        elif k == "REACTANT1":
            r.reac1 = _atoms(w[1:])
        elif k == "REACTANT2":
            r.reac2 = _atoms(w[1:])
        elif k == "DIST_INF":
            r.r_inf = _real(w[1]) / BOHR_ANGSTROM   # src/calc_rate_read.f90:686-693
        elif k == "N_PATHS":
            r.npaths = int(w[1])
        elif k in ("BOND_FORM", "BOND_BREAK"):
            # Caracal reads one `a-b` token per bond (form_num = break_num = 1
            # for BIMOLEC); `a b` as two tokens is accepted as well
            tok = w[1] if "-" in w[1] else " ".join(w[1:3])
            if k == "BOND_FORM":
                r.bond_form = _pair(tok)
            else:
                r.bond_break = _pair(tok)
    if r.umbr_type != "BIMOLEC":
        raise K.KeyError_(f"reaction type {r.umbr_type or '(none)'}: only BIMOLEC is on this engine's path")
    if not blocks["UMBRELLA"]:
        raise K.KeyError_("Please add an UMBRELLA section with parameters to the keyfile!")
    for ln in blocks["UMBRELLA"]:
        w = ln.split()
        if not w:
            continue
        k = w[0].upper()
        if k == "BIAS":
            r.bias = _real(w[1])
        elif k == "BIAS_LIST":
            raise K.KeyError_("BIAS_LIST (per-window force constants) is not on this engine's path")
        elif k == "BONDS":
            r.umbr_lo, r.umbr_hi = _real(w[1]), _real(w[2])
        elif k == "DIST":
            r.umbr_dist = _real(w[1])
        elif k == "GEN_STEPS":
            r.gen_steps = int(w[1])
        elif k == "EQUI_STEPS":
            r.equi_steps = int(w[1])
        elif k == "SAMPLE_STEPS":
            r.sample_steps = int(w[1])
        elif k == "SAMPLE_TRAJS":
            r.sample_trajs = int(w[1])
    if not blocks["PMF"]:
        raise K.KeyError_("Please add a PMF section with parameters to the keyfile!")
    for ln in blocks["PMF"]:
        w = ln.split()
        if not w:
            continue
        k = w[0].upper()
        if k == "XI_RANGE":
            r.xi_lo, r.xi_hi = _real(w[1]), _real(w[2])
        elif k == "BINS":
            r.nbins = int(w[1])
        elif k == "METHOD":
            r.pmf_method = w[1].upper()
        elif k == "MINLOC":
            r.minloc = w[1].upper()
    if not blocks["RECROSS"]:
        raise K.KeyError_("Please add a RECROSS section with parameters to the keyfile!")
    for ln in blocks["RECROSS"]:
        w = ln.split()
        if not w:
            continue
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
        elif k == "MANUAL_POS":
            r.xi_manual = _real(w[1])
        # MPI and NO_CHECK: the MPI layout and Caracal's trajectory checks
        # (rpmd_check) have no counterpart here; non-finite trajectories stop
        # the engine with an error status instead
    # checks of src/calc_rate_read.f90:1290-1420
    if r.pes not in K.ANALYTIC:
        raise K.KeyError_(f"PES {r.pes or '(none)'}: calc_rate runs on the analytic surfaces here")
    if r.kelvin <= 0.0:
        raise K.KeyError_("Give a positive temperature!")
    if r.npaths < 1:
        raise K.KeyError_("The number of reaction paths must be at least 1!")
    if r.nbins == 0:
        raise K.KeyError_("Please give the number of bins for the PMF calculation (BINS)!")
    if r.pmf_method not in ("INTEGRATION", "WHAM", "ALL"):
        r.pmf_method = "INTEGRATION"    # src/calc_rate_read.f90:1541-1552
    if r.minloc not in ("ZERO", "PMF_MIN"):
        raise K.KeyError_("The keyword PMF_MINLOC was found but no valid option was given!")
    if r.child_total > 0:
        if r.child_perpoint <= 0 or r.child_interval <= 0 or r.child_steps <= 0:
            raise K.KeyError_("Please give CHILD_INTERVAL, CHILD_PERPOINT and CHILD_STEPS!")
        if r.child_total % r.child_perpoint != 0:
            raise K.KeyError_("CHILD_TOTAL must be a multiple of CHILD_PERPOINT!")
        if r.child_perpoint % 2 != 0:
            raise K.KeyError_("CHILD_PERPOINT must be even (children come in +-p pairs)!")
    return r


def window_layout(r):
    """(n_all, xi of windows 1 .. n_all - 1, index order) as
    src/calc_rate.f90:650-663, 832-1000 number them: windows below 1 are
    1 - i dist (i = 1 .. n_samplings) at index n_samplings - i + 1, windows
    from 1 up are 1 + (i - 1) dist (i = 1 .. n_over) at n_all + i - n_over - 1."""
    n_over = _nint((r.umbr_hi - 1.0) / r.umbr_dist)
    n_samplings = _nint((1.0 - r.umbr_lo) / r.umbr_dist)
    n_all = _nint((r.umbr_hi - r.umbr_lo) / r.umbr_dist) + 1
    if n_over + n_samplings != n_all - 1:
        raise K.KeyError_("Total number of sampling windows unequal sum of windows > 1 and <= 1!")
    if n_over < 1:
        raise K.KeyError_("The umbrella windows must reach xi = 1 (BONDS upper value >= 1 + DIST)")
    xw = np.zeros(n_all - 1)
    for i in range(1, n_over + 1):
        xw[n_all + i - (n_over + 1) - 1] = 1.0 + (i - 1) * r.umbr_dist
    for i in range(1, n_samplings + 1):
        xw[n_samplings - i] = 1.0 - i * r.umbr_dist
    return n_all, n_over, n_samplings, xw


def reference_bonds(q0, r):
    """MECHA reference bond lengths from the transition-state structure
    (src/bonds_ref.f90:51-74)."""
    f, b = r.bond_form, r.bond_break
    return (float(np.linalg.norm(q0[f[0] - 1] - q0[f[1] - 1])), float(np.linalg.norm(q0[b[0] - 1] - q0[b[1] - 1])))


def generate_structures(r, Engine, pes, mass, beta, dt, q0, kf, mech, layout):
    """Start structures of the windows (part 1): one classical trajectory,
    GEN_STEPS steps per window with mdinit before each; returns (n_all - 1,
    natoms, 3) bohr, shifted to the centre of mass (src/calc_rate.f90:1118-1133)."""
    n_all, n_over, n_samplings, xw = layout
    natoms = len(mass)
    out = np.zeros((n_all - 1, natoms, 3))
    g = Engine(pes, mass, 1, 1, dt, beta=beta, thermostat=r.thermostat, andersen_step=r.andersen_step,
               transrot=r.transrot, seed=r.seed + 7, nm_mode=r.nm_mode)
    g.init_positions(q0, 0.0)
    draw = 0

    def window(idx, qstart=None):
        nonlocal draw
        if qstart is not None:
            g.set_state(qstart[None, None], np.zeros((1, 1, natoms, 3)))
        g.set_umbrella(centers=[xw[idx]], kforce=kf, **mech)
        g.mdinit(draw)
        draw += 1
        g.run(max(r.gen_steps, 1))
        out[idx] = g.get_state()[0][0, 0]

    for i in range(1, n_over + 1):            # xi = 1, 1 + dist, ... from the TS
        window(n_all + i - (n_over + 1) - 1)
    q1 = out[n_samplings].copy()              # the structure at xi = 1
    for i in range(1, n_samplings + 1):       # xi = 1 - dist, 1 - 2 dist, ...
        window(n_samplings - i, q1 if i == 1 else None)
    g.close()
    com = (out * mass[None, :, None]).sum(axis=1) / mass.sum()
    return out - com[:, None, :]


def sample_windows(r, Engine, pes, mass, beta, dt, kf, mech, xw, starts, max_redo=3):
    """Umbrella sampling of every window (part 2): per trajectory the mean
    and variance of xi over SAMPLE_STEPS steps, shape (windows, SAMPLE_TRAJS).
    Trajectories with a variance above 1e-2 run again with fresh momenta
    (Caracal's restart, src/calc_rate.f90:1681-1687), up to max_redo times."""
    nw, S, P, natoms = len(xw), r.sample_trajs, r.nbeads, len(mass)
    avg = np.zeros((nw, S))
    var = np.zeros((nw, S))
    todo = np.arange(nw * S)
    redo = 0
    for attempt in range(max_redo + 1):
        T = len(todo)
        win = todo // S
        eng = Engine(pes, mass, P, T, dt, beta=beta, thermostat=r.thermostat, andersen_step=r.andersen_step,
                     transrot=r.transrot, seed=r.seed + 101 * attempt, traj0=0, nm_mode=r.nm_mode)
        q = np.repeat(starts[win][:, None], P, axis=1)
        eng.set_state(q, np.zeros_like(q))
        eng.set_umbrella(centers=xw[win], kforce=kf, **mech)
        eng.mdinit(0)
        eng.run(r.equi_steps)
        eng.compute_forces()          # unbiased first sampling force (src/calc_rate.f90:1598-1602)
        eng.umbrella_sampling(True)
        eng.run(r.sample_steps)
        xs, x2, _ = eng.umbrella_stats()
        eng.close()
        a = xs / r.sample_steps
        v = x2 / r.sample_steps - a * a
        avg.flat[todo] = a
        var.flat[todo] = v
        bad = v > 1e-2
        if not bad.any():
            break
        todo = todo[bad]
        redo += int(bad.sum())
    return avg, var, redo


def pmf_profile(r, xw, kf, beta, avg, var):
    """(bin coordinates, PMF in Hartree) by umbrella integration of the
    window means/variances (averaged over each window's trajectories)."""
    return umbrella_integration(xw, np.full(len(xw), kf), avg.mean(axis=1), var.mean(axis=1), beta,
                                r.xi_lo, r.xi_hi, r.nbins, r.sample_trajs * r.sample_steps)


def pmf_extrema(r, coord, pmf):
    """(index of the maximum, index of the minimum) as src/calc_rate.f90:2060-2093."""
    imax = int(np.argmax(pmf))
    if r.minloc == "ZERO":
        # minlocate = -int(xi_min / ((xi_max - xi_min) / nbins)) + 1 (1-based)
        imin = -int(r.xi_lo / ((r.xi_hi - r.xi_lo) / r.nbins))
        imin = min(max(imin, 0), len(pmf) - 1)
    else:
        imin = int(np.argmin(pmf[:imax + 1]))
    return imax, imin


def jackknife(values):
    """Standard error from the leave-one-out estimates `values` (first axis:
    the left-out sample)."""
    v = np.asarray(values, dtype=float)
    n = len(v)
    if n < 2:
        return np.full(v.shape[1:], np.nan) if v.ndim > 1 else float("nan")
    err = np.sqrt((n - 1) / n * np.sum((v - v.mean(axis=0)) ** 2, axis=0))
    return err if v.ndim > 1 else float(err)


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


def recrossing(r, Engine, pes, mass, beta, dt, mech, xi_barrier, qstart, out_dir):
    """Part 4: (kappa(t) numerator sums, denominator sum, per-batch numerators
    (batches, CHILD_STEPS), per-batch denominators) of the constrained parent
    and its children (src/recross.f90:230-480)."""
    P, natoms = r.nbeads, len(mass)
    nkids = r.child_perpoint
    batches = r.child_total // nkids
    point, kappa_num, kappa_den, qpar = read_recross_restart(out_dir, r.child_steps, P, natoms)
    if point >= batches and qpar is None:
        point = batches                        # every batch done: the sums are final
    elif point > 0 and qpar is None:
        point, kappa_num, kappa_den = 0, np.zeros(r.child_steps), 0.0
    per_num, per_den = [], []
    par = Engine(pes, mass, P, 1, dt, beta=beta, thermostat=r.thermostat,
                 andersen_step=max(1, int(math.sqrt(r.rc_equi))), transrot=False, seed=r.seed + 1, nm_mode=r.nm_mode)
    q0 = qpar[None] if (qpar is not None and point > 0) else np.repeat(qstart[None, None], P, axis=1)
    par.set_state(q0, np.zeros_like(q0))
    par.set_parent(xi_ideal=xi_barrier, **mech)
    par.mdinit(0)
    par.run(r.rc_equi if point == 0 else 100)  # a resumed parent re-equilibrates 100 steps (:264-268)
    par.set_andersen_step(max(1, int(math.sqrt(r.child_interval))))
    while point < batches:
        qp = par.get_state()[0][0]
        # children of this parent snapshot, their own momentum stream (traj0)
        kids = Engine(pes, mass, P, nkids, dt, beta=beta, thermostat="none", transrot=False,
                      seed=r.seed + 2, traj0=point * nkids, nm_mode=r.nm_mode)
        kids.set_recross(xi_ideal=xi_barrier, max_steps=r.child_steps, **mech)
        kids.init_children(qp)
        kids.run(r.child_steps)
        num, den, _ = kids.kappa(r.child_steps)
        kids.close()
        kappa_num[:len(num)] += num
        kappa_den += den
        per_num.append(np.array(num))
        per_den.append(den)
        point += 1
        write_recross_restart(out_dir, point, kappa_num, kappa_den, qp)
        if point < batches:
            par.mdinit(point)                  # fresh parent momenta (src/recross.f90:462)
            par.run(r.child_interval)
    par.close()
    return kappa_num, kappa_den, np.array(per_num), np.array(per_den)


def run(path, out_dir=None, quiet=False, engine=None, **options):
    """Run the calc_rate key file `path`; writes Caracal's result files into
    out_dir and returns a dict of the results and their statistical errors.
    `options` set RateInput fields over the key file (e.g. nm_mode=1,
    transrot=False)."""
    if engine is None:
        from .engine import RPMDEngine as engine
    with open(path) as fh:
        r = parse(fh.read(), directory=os.path.dirname(os.path.abspath(path)))
    for k, v in options.items():
        if not hasattr(r, k):
            raise TypeError(f"unknown calc_rate option {k}")
        setattr(r, k, v)
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
    kf = r.bias * r.kelvin                     # src/calc_rate.f90:698

    # 1.-2. start structures and umbrella sampling
    layout = window_layout(r)
    n_all, _, _, xw = layout
    starts = generate_structures(r, engine, pes, mass, beta, dt, q0, kf, mech, layout)
    avg, var, redo = sample_windows(r, engine, pes, mass, beta, dt, kf, mech, xw, starts)
    with open(os.path.join(out_dir, "umbr_int.dat"), "w") as fh:
        fh.write(" # xi_position      average(xi)       variance(xi)\n")
        for x, a, v in zip(xw, avg.mean(axis=1), var.mean(axis=1)):
            fh.write(f"{x:24.16f}{a:26.16E}{v:26.16E}\n")

    # 3. free-energy profile
    coord, pmf = pmf_profile(r, xw, kf, beta, avg, var)
    with open(os.path.join(out_dir, "pmf_integration.dat"), "w") as fh:
        fh.write(" # xi-value     PMF(kJ/mol)\n")
        for c, v in zip(coord, pmf):
            fh.write(f"{c:24.16f}{v * KJMOL_PER_HARTREE:26.16f}\n")
    imax, imin = pmf_extrema(r, coord, pmf)
    xi_barrier = float(coord[imax]) if r.xi_manual is None else float(r.xi_manual)
    jk_max, jk_bar = [], []
    S = r.sample_trajs
    if S > 1:      # leave one trajectory of every window out
        for j in range(S):
            keep = [i for i in range(S) if i != j]
            _, pj = pmf_profile(r, xw, kf, beta, avg[:, keep], var[:, keep])
            a, b = pmf_extrema(r, coord, pj)
            jk_max.append(pj[a] * KJMOL_PER_HARTREE)
            jk_bar.append((pj[a] - pj[b]) * KJMOL_PER_HARTREE)
    max_err = jackknife(jk_max) if jk_max else float("nan")
    barrier_err = jackknife(jk_bar) if jk_bar else float("nan")

    # 4. recrossing
    kappa_t = np.ones(max(r.child_steps, 1))
    kappa_err = np.full(max(r.child_steps, 1), np.nan)
    if r.child_total > 0:
        ts_locate = int(np.argmin(np.abs(xw - xi_barrier)))
        num, den, per_num, per_den = recrossing(r, engine, pes, mass, beta, dt, mech, xi_barrier,
                                                starts[ts_locate], out_dir)
        kappa_t = num / den if den > 0 else np.ones(r.child_steps)
        B = len(per_den)
        if B > 1 and den > 0:
            loo = [(num - per_num[b]) / (den - per_den[b]) for b in range(B)]
            kappa_err = jackknife(np.array(loo))
    with open(os.path.join(out_dir, "recross.dat"), "w") as fh:
        fh.write(" # time (fs)      kappa(t)\n")
        for i, v in enumerate(kappa_t):
            fh.write(f"{(i + 1) * r.dt_fs:24.16f}{v:26.16f}\n")
    kappa = float(kappa_t[-1])
    with open(os.path.join(out_dir, "recross_finished"), "w") as fh:   # src/recross.f90:660-665
        fh.write(f"{kappa:26.16E}\n")
    kappa_used = 1.0 if kappa < 0.002 else kappa   # src/calc_rate.f90:2237-2252

    # 5. rate constant
    m1 = float(sum(mass[a - 1] for a in r.reac1))
    m2 = float(sum(mass[a - 1] for a in r.reac2))
    k_t = bimolecular_rate(kappa_used, pmf[imax], pmf[imin], r.r_inf, beta, m1, m2, r.npaths)
    result = dict(xi_barrier=xi_barrier, pmf_max_kjmol=float(pmf[imax] * KJMOL_PER_HARTREE),
                  pmf_max_stderr_kjmol=max_err, pmf_min_kjmol=float(pmf[imin] * KJMOL_PER_HARTREE),
                  barrier_kjmol=float((pmf[imax] - pmf[imin]) * KJMOL_PER_HARTREE),
                  barrier_stderr_kjmol=barrier_err, kappa=kappa,
                  kappa_stderr=float(np.atleast_1d(kappa_err)[-1]), kappa_t=kappa_t,
                  kappa_t_stderr=np.atleast_1d(kappa_err), k_t=k_t, windows=n_all - 1,
                  trajectories=(n_all - 1) * r.sample_trajs, redone=redo, coord=coord, pmf_kjmol=pmf * KJMOL_PER_HARTREE)
    if not quiet:
        print(f" Free energy barrier: {result['barrier_kjmol']:12.5f} kJ/mol at xi = {xi_barrier:10.5f}")
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
