"""ORACLE (test infrastructure only): ctypes view of the CPU restatement.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this module, and only as the checker.  The product path (the CUDA
library under ``caracal_gb300``) never loads it.

Arrays follow Caracal's Fortran layout ``q(3, natoms, nbeads)`` per
trajectory; numpy arrays of shape ``(ntraj, nbeads, natoms, 3)`` in C order
have exactly that memory layout.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

PES_IDS = {"h3": 1, "ch4h": 2, "ch4oh": 3, "qmdff": 4, "evb": 5, "water": 6, "oh3": 7, "geh4oh": 8, "brh2": 9}
EVB_BASES = {"const": 0, "1g": 1, "2g": 2, "3g": 3, "sp": 4, "sd": 5, "sd2": 6, "sp2d": 7}
THERMOSTATS = {"none": 0, "andersen": 1, "nose-hoover": 2, "nhc": 2, "pile": 3}
OPCOUNT_FIELDS = ("add", "mul", "div", "sqrt", "exp", "log", "pow", "sin", "cos",
                  "acos", "erf", "cmp", "tanh", "cosh")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc/g++ only)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    else:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class Cfg(C.Structure):
    _fields_ = [("pes", C.c_int), ("natoms", C.c_int), ("nbeads", C.c_int),
                ("thermostat", C.c_int), ("andersen_step", C.c_int), ("transrot", C.c_int),
                ("seed", C.c_uint32), ("dt", C.c_double), ("beta", C.c_double),
                ("pile_tau0", C.c_double), ("mass", C.POINTER(C.c_double)), ("nose_q", C.c_double),
                ("nm_mode", C.c_int)]


class QmdffDef(C.Structure):
    _fields_ = [("natoms", C.c_int), ("at", C.POINTER(C.c_int)), ("q", C.POINTER(C.c_double)),
                ("rad", C.POINTER(C.c_double)), ("nbond", C.c_int), ("nangl", C.c_int),
                ("ntors", C.c_int), ("nnci", C.c_int), ("bond", C.POINTER(C.c_int)),
                ("vbond", C.POINTER(C.c_double)), ("angl", C.POINTER(C.c_int)),
                ("vangl", C.POINTER(C.c_double)), ("tors", C.POINTER(C.c_int)),
                ("vtors", C.POINTER(C.c_double)), ("nci", C.POINTER(C.c_int)),
                ("pR0", C.POINTER(C.c_double)), ("pC6", C.POINTER(C.c_double)),
                ("pSr42", C.POINTER(C.c_double)), ("pZab", C.POINTER(C.c_double)),
                ("pAlpha", C.POINTER(C.c_double)), ("nhb", C.c_int), ("hb", C.POINTER(C.c_int)),
                ("vhb", C.POINTER(C.c_double)), ("eps1", C.c_double * 7), ("eps2", C.c_double * 7),
                ("coul_cut", C.c_double), ("zahn", C.c_int), ("zahn_a", C.c_double),
                ("zahn_par", C.c_double), ("e_zero", C.c_double)]


_keep = []


def set_evb(ff1, ff2, tables, basis="1g", par=None, **kw):
    """PES 5: dE-EVB of ff1 and ff2 (each with its own E_zero); par = dict of
    offa..offh, offm, offn (a..h, m, n)."""
    set_qmdff(ff2, tables, **kw)
    lib().orc_qmdff_set2(C.byref(_last_def[0]))
    _keep2[:] = list(_keep)
    set_qmdff(ff1, tables, **kw)
    p = np.zeros(10)
    for k, name in enumerate("abcdefghmn"):
        p[k] = float((par or {}).get(name, 0.0))
    lib().orc_evb_set(EVB_BASES[basis], _dp(p))


_keep2 = []
_last_def = [None]


def set_water(nwater, box=None, coul_cut=0.0, zahn=False, zahn_a=0.0, zahn_par=0.0):
    """PES 6: Caracal's flexible SPC water box of nwater molecules (O, H, H);
    box = (Lx, Ly, Lz) in bohr for periodic boundaries, None for none."""
    ln = (C.c_double * 3)(*(box if box is not None else (0.0, 0.0, 0.0)))
    lib().orc_water_set(int(nwater), int(box is not None), ln, float(coul_cut), int(zahn), float(zahn_a),
                        float(zahn_par))


def set_qmdff(ff, tables, coul_cut=50.0, zahn=False, zahn_a=0.0, zahn_par=0.0):
    """Load a caracal_gb300.qmdff.QMDFF (1-based atoms) as the oracle's PES 4."""
    from caracal_gb300 import qmdff as Q
    ip = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
    fp = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    hb = np.asarray(getattr(ff, "hb", np.zeros((0, 3), int))).reshape(-1, 3)
    arrs = dict(at=ip(ff.at), q=fp(ff.q), rad=fp(ff.rad_bohr()), bond=ip(ff.bond - 1),
                hb=ip(hb - 1 if len(hb) else hb), vhb=fp(Q.hb_parameters(ff) if len(hb) else np.zeros((0, 2))),
                vbond=fp(ff.vbond), angl=ip(ff.angl - 1), vangl=fp(ff.vangl),
                tors=ip(np.column_stack([ff.tors[:, :4] - 1, ff.tors[:, 4:]])), vtors=fp(ff.vtors),
                nci=ip(np.column_stack([ff.nci[:, :2] - 1, ff.nci[:, 2]])))
    pr = [fp(a) for a in Q.pair_parameters(ff, tables)]
    _keep[:] = [arrs, pr]
    e1, e2 = Q.eps_factors()
    d = QmdffDef()
    d.natoms = ff.n
    d.nbond, d.nangl, d.ntors, d.nnci = len(ff.bond), len(ff.angl), len(ff.tors), len(ff.nci)
    for k in ("q", "rad", "vbond", "vangl", "vtors"):
        setattr(d, k, arrs[k].ctypes.data_as(C.POINTER(C.c_double)))
    for k in ("at", "bond", "angl", "tors", "nci", "hb"):
        setattr(d, k, arrs[k].ctypes.data_as(C.POINTER(C.c_int)))
    d.vhb = arrs["vhb"].ctypes.data_as(C.POINTER(C.c_double))
    d.nhb = len(hb)
    for k, a in zip(("pR0", "pC6", "pSr42", "pZab", "pAlpha"), pr):
        setattr(d, k, a.ctypes.data_as(C.POINTER(C.c_double)))
    for i in range(7):
        d.eps1[i], d.eps2[i] = e1[i], e2[i]
    d.coul_cut, d.zahn, d.zahn_a, d.zahn_par, d.e_zero = coul_cut, int(zahn), zahn_a, zahn_par, ff.e_zero
    _last_def[0] = d
    lib().orc_qmdff_set(C.byref(d))


def set_qmdff_periodic(box_ang, coul_cut_ang=50.0, vdw_cut_ang=10.0):
    """set_periodic for the current QMDFF: returns (coul_cut, vdw_cut,
    zahn_a, zahn_par) in bohr as set."""
    box = np.ascontiguousarray(box_ang, dtype=np.float64)
    out = np.zeros(4)
    lib().orc_qmdff_set_periodic(_dp(box), float(coul_cut_ang), float(vdw_cut_ang), _dp(out))
    return tuple(out)


def qmdff_egrad_virial(q, box=None):
    """The current QMDFF on q (nbeads, n, 3) bohr: V, dV/dq and each bead's
    virial trace (the reference's vir_ten terms); box (nbeads, 3) bohr per
    bead, or None for the force field's own."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    nb = q.shape[0]
    V, g, w = np.zeros(nb), np.zeros_like(q), np.zeros(nb)
    bx = None if box is None else np.ascontiguousarray(np.broadcast_to(box, (nb, 3)), dtype=np.float64)
    rc = lib().orc_qmdff_egrad_virial(_dp(q), nb, None if bx is None else _dp(bx), _dp(V), _dp(g), _dp(w))
    if rc:
        raise ValueError("a box needs set_qmdff_periodic first")
    return V, g, w


# Berendsen barostat constants of mdinit (src/mdinit.f90:155-158) and the
# pressure unit (src/general.f90:263: Hartree/bohr^3 -> atm)
PRESCON = 290371576.61
BERENDSEN_TAUPRES = 2.0
BERENDSEN_COMPRESS = 0.000046 * PRESCON / 1000.0


def run_npt(cfg, q, p, f, nsteps, box, pressure_atm, istep0=0, traj0=0, nthreads=0):
    """run() under the Berendsen barostat (periodic QMDFF): box (ntraj, 3)
    bohr; returns (q, p, f, epot, status, box, press) with press in a.u."""
    q = np.array(q, dtype=np.float64)
    p = np.array(p, dtype=np.float64)
    f = np.array(f, dtype=np.float64)
    T = q.shape[0]
    bx = np.array(np.broadcast_to(box, (T, 3)), dtype=np.float64)
    e, pr = np.zeros(T), np.zeros(T)
    st = np.zeros(T, dtype=np.int32)
    rc = lib().orc_run_npt(C.byref(cfg.c), T, traj0, istep0, nsteps, _dp(q), _dp(p), _dp(f), _dp(e),
                           st.ctypes.data_as(C.POINTER(C.c_int)), _dp(bx), _dp(pr), pressure_atm / PRESCON,
                           BERENDSEN_COMPRESS, BERENDSEN_TAUPRES, nthreads)
    if rc:
        raise ValueError("run_npt needs the periodic QMDFF (PES 4)")
    return q, p, f, e, st, bx, pr


class XiDef(C.Structure):
    _fields_ = [("nreac1", C.c_int), ("reac1", C.c_int * 8), ("nreac2", C.c_int),
                ("reac2", C.c_int * 8), ("form", C.c_int * 2), ("brk", C.c_int * 2),
                ("form_ref", C.c_double), ("break_ref", C.c_double), ("r_inf", C.c_double),
                ("xi_ideal", C.c_double)]


def make_xidef(reac1, reac2, form, brk, form_ref, break_ref, r_inf, xi_ideal):
    """BIMOLEC definition from 0-based atom lists."""
    x = XiDef()
    x.nreac1, x.nreac2 = len(reac1), len(reac2)
    for i, a in enumerate(reac1):
        x.reac1[i] = a
    for i, a in enumerate(reac2):
        x.reac2[i] = a
    x.form[0], x.form[1] = form
    x.brk[0], x.brk[1] = brk
    x.form_ref, x.break_ref, x.r_inf, x.xi_ideal = form_ref, break_ref, r_inf, xi_ideal
    return x


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        d = C.POINTER(C.c_double)
        _lib.orc_egrad_h3.argtypes = [d, C.c_int, C.c_int, d, d, C.POINTER(C.c_int)]
        _lib.orc_h3_pote.argtypes = [d, d, d]
        _lib.orc_cos_transform.argtypes = [d, C.c_int]
        _lib.orc_egrad.argtypes = [C.c_int, d, C.c_int, C.c_int, d, d]
        _lib.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                                           C.POINTER(C.c_uint32)]
        _lib.orc_normal_pair.argtypes = [C.c_uint32] * 6 + [d]
        _lib.orc_transrot.argtypes = [C.POINTER(Cfg), d, d]
        _lib.orc_init_positions.argtypes = [C.POINTER(Cfg), C.c_int, C.c_uint32, d, C.c_double, d]
        _lib.orc_init_momenta.argtypes = [C.POINTER(Cfg), C.c_int, C.c_uint32, d]
        _lib.orc_init_momenta_draw.argtypes = [C.POINTER(Cfg), C.c_int, C.c_uint32, C.c_uint32, d]
        _lib.orc_d3_pair_c6.argtypes = [d, C.c_int, C.c_int, C.POINTER(C.c_int), d, d, d, d]
        _lib.orc_init_forces.argtypes = [C.POINTER(Cfg), C.c_int, d, d, d]
        _lib.orc_run.argtypes = [C.POINTER(Cfg), C.c_int, C.c_uint32, C.c_int, C.c_int, d, d, d, d,
                                 C.POINTER(C.c_int), C.c_int, d]
        _lib.orc_qmdff_set.argtypes = [C.POINTER(QmdffDef)]
        _lib.orc_qmdff_set2.argtypes = [C.POINTER(QmdffDef)]
        _lib.orc_qmdff_set_periodic.argtypes = [d, C.c_double, C.c_double, d]
        _lib.orc_qmdff_egrad_virial.argtypes = [d, C.c_int, d, d, d, d]
        _lib.orc_run_npt.argtypes = [C.POINTER(Cfg), C.c_int, C.c_uint32, C.c_int, C.c_int, d, d, d, d,
                                     C.POINTER(C.c_int), d, d, C.c_double, C.c_double, C.c_double, C.c_int]
        _lib.orc_evb_set.argtypes = [C.c_int, d]
        _lib.orc_nhc_half.argtypes = [C.POINTER(Cfg), d, d]
        _lib.orc_evb_fit.argtypes = [C.c_int, d, C.c_int, C.c_int, d, d, d, d, d]
        _lib.orc_run_parent.argtypes = [C.POINTER(Cfg), C.POINTER(XiDef), C.c_int, C.c_uint32, C.c_int, C.c_int,
                                        d, d, d, d, C.POINTER(C.c_int), d, d]
        _lib.orc_calc_xi.argtypes = [C.POINTER(XiDef), C.c_int, d, d, d]
        _lib.orc_calc_xi.restype = C.c_double
        _lib.orc_umbrella_bias.argtypes = [C.POINTER(Cfg), C.POINTER(XiDef), C.c_double, C.c_double, d, d]
        _lib.orc_umbrella_bias.restype = C.c_double
        _lib.orc_calc_xi_umbrella.argtypes = [C.POINTER(XiDef), C.c_int, d, d, d, d]
        _lib.orc_calc_xi_umbrella.restype = C.c_double
        _lib.orc_run_umbrella.argtypes = [C.POINTER(Cfg), C.POINTER(XiDef), C.c_int, C.c_uint32, C.c_int, C.c_int,
                                          d, d, d, d, d, d, C.POINTER(C.c_int), d, C.c_int, d, d, C.c_int,
                                          C.c_double, C.c_double, d]
        _lib.orc_recross_children.argtypes = [C.POINTER(Cfg), C.POINTER(XiDef), C.c_int, C.c_uint32, d,
                                              C.c_int, d, d, d, d, d, C.c_int]
        _lib.orc_pes_opcount.argtypes = [C.c_int, d, C.POINTER(C.c_uint64)]
        _lib.orc_water_set.argtypes = [C.c_int, C.c_int, d, C.c_double, C.c_int, C.c_double, C.c_double]
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Config:
    """Step configuration for the oracle (all quantities in atomic units)."""

    def __init__(self, pes, mass, nbeads, dt, beta, thermostat="none", andersen_step=70,
                 pile_tau0=0.0, transrot=True, seed=0, nose_q=0.0, nm_mode=0):
        self.mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.natoms = len(self.mass)
        self.nbeads = int(nbeads)
        self.thermostat = THERMOSTATS[thermostat]
        self.c = Cfg(PES_IDS[pes] if isinstance(pes, str) else int(pes), self.natoms,
                     self.nbeads, self.thermostat, int(andersen_step), int(bool(transrot)),
                     int(seed) & 0xFFFFFFFF, float(dt), float(beta), float(pile_tau0),
                     _dp(self.mass), float(nose_q), int(nm_mode))

    def shape(self, ntraj):
        return (ntraj, self.nbeads, self.natoms, 3)


def philox(ctr, k0, k1):
    c = (C.c_uint32 * 4)(*ctr)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k0, k1, o)
    return list(o)


def normal_pair(seed, traj, pair, bead, step, tag):
    out = np.zeros(2)
    lib().orc_normal_pair(seed, traj, pair, bead, step, tag, _dp(out))
    return out


def egrad_h3(q):
    """q: (nbeads, natoms=3, 3) -> V (nbeads,), dVdq (nbeads, 3, 3)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    nb = q.shape[0]
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    lib().orc_egrad_h3(_dp(q), 3, nb, _dp(V), _dp(g), C.byref(info))
    return V, g


def egrad(pes, q):
    """Any PES: q (nbeads, natoms, 3) bohr -> V (nbeads,), dVdq."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    V = np.zeros(q.shape[0])
    g = np.zeros_like(q)
    lib().orc_egrad(PES_IDS[pes] if isinstance(pes, str) else int(pes), _dp(q), q.shape[1],
                    q.shape[0], _dp(V), _dp(g))
    return V, g


def h3_pote(R):
    R = np.ascontiguousarray(R, dtype=np.float64)
    V = np.zeros(1)
    dV = np.zeros(3)
    lib().orc_h3_pote(_dp(R), _dp(V), _dp(dV))
    return V[0], dV


def cos_transform(x):
    x = np.array(x, dtype=np.float64)
    lib().orc_cos_transform(_dp(x), len(x))
    return x


def transrot(cfg: Config, q, p):
    q = np.ascontiguousarray(q, dtype=np.float64)
    p = np.array(p, dtype=np.float64)
    rc = lib().orc_transrot(C.byref(cfg.c), _dp(q), _dp(p))
    return rc, p


def init_positions(cfg: Config, ntraj, q0, sigma, traj0=0):
    q0 = np.ascontiguousarray(q0, dtype=np.float64)
    q = np.zeros(cfg.shape(ntraj))
    lib().orc_init_positions(C.byref(cfg.c), ntraj, traj0, _dp(q0), float(sigma), _dp(q))
    return q


def init_momenta(cfg: Config, ntraj, traj0=0, draw=0):
    p = np.zeros(cfg.shape(ntraj))
    lib().orc_init_momenta_draw(C.byref(cfg.c), ntraj, traj0, int(draw) & 0xFFFFFFFF, _dp(p))
    return p


def d3_pair_c6(pars, at, xyz, rcov):
    """prepare's pair C6 (n, n) and coordination numbers (n,) restated in C++
    from the D3 reference lines pars (nlines, 5)."""
    pars = np.ascontiguousarray(pars, dtype=np.float64)
    at = np.ascontiguousarray(at, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    rcov = np.ascontiguousarray(rcov, dtype=np.float64)
    n = len(at)
    c6 = np.zeros((n, n))
    cn = np.zeros(n)
    lib().orc_d3_pair_c6(_dp(pars), pars.shape[0], n, at.ctypes.data_as(C.POINTER(C.c_int)), _dp(xyz), _dp(rcov),
                         _dp(c6), _dp(cn))
    return c6, cn


def init_forces(cfg: Config, q):
    q = np.ascontiguousarray(q, dtype=np.float64)
    f = np.zeros_like(q)
    e = np.zeros(q.shape[0])
    lib().orc_init_forces(C.byref(cfg.c), q.shape[0], _dp(q), _dp(f), _dp(e))
    return f, e


def run(cfg: Config, q, p, f, nsteps, istep0=0, traj0=0, nthreads=0, vnh=None):
    """Advance copies of (q, p, f) by nsteps; returns (q, p, f, epot, status).
    For the Nose-Hoover chain, vnh (ntraj, 4) is the chain state, updated in
    place (zeros when None, as after mdinit)."""
    q = np.array(q, dtype=np.float64)
    p = np.array(p, dtype=np.float64)
    f = np.array(f, dtype=np.float64)
    T = q.shape[0]
    e = np.zeros(T)
    st = np.zeros(T, dtype=np.int32)
    if cfg.thermostat == 2 and vnh is None:
        vnh = np.zeros((T, 4))
    vp = None
    if vnh is not None:
        assert vnh.dtype == np.float64 and vnh.flags.c_contiguous and vnh.shape == (T, 4)
        vp = _dp(vnh)
    lib().orc_run(C.byref(cfg.c), T, traj0, istep0, nsteps, _dp(q), _dp(p), _dp(f), _dp(e),
                  st.ctypes.data_as(C.POINTER(C.c_int)), nthreads, vp)
    return q, p, f, e, st


def pes_opcount(pes, q):
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = (C.c_uint64 * 14)()
    lib().orc_pes_opcount(PES_IDS[pes] if isinstance(pes, str) else pes, _dp(q), out)
    return dict(zip(OPCOUNT_FIELDS, list(out)))


def calc_xi(xd, coords, mass):
    c = np.ascontiguousarray(coords, dtype=np.float64)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    dxi = np.zeros_like(c)
    xi = lib().orc_calc_xi(C.byref(xd), c.shape[0], _dp(c), _dp(m), _dp(dxi))
    return xi, dxi


def recross_children(cfg: Config, xd, ntraj, q_parent, nsteps, traj0=0, nthreads=0, states=False):
    """Returns (num (nsteps,), denom, w (ntraj,)[, q, p])."""
    qp = np.ascontiguousarray(q_parent, dtype=np.float64)
    num = np.zeros(nsteps)
    den = np.zeros(1)
    w = np.zeros(ntraj)
    q = np.zeros(cfg.shape(ntraj)) if states else None
    p = np.zeros(cfg.shape(ntraj)) if states else None
    lib().orc_recross_children(C.byref(cfg.c), C.byref(xd), ntraj, traj0, _dp(qp), nsteps, _dp(num),
                               _dp(den), _dp(w), _dp(q) if states else None,
                               _dp(p) if states else None, nthreads)
    return (num, den[0], w, q, p) if states else (num, den[0], w)


def nhc_half(cfg: Config, vnh, p):
    """One Nose-Hoover chain call on one trajectory: returns (vnh, p) updated."""
    v = np.array(vnh, dtype=np.float64)
    pp = np.array(p, dtype=np.float64)
    lib().orc_nhc_half(C.byref(cfg.c), _dp(v), _dp(pp))
    return v, pp


def run_parent(cfg: Config, xd, q, p, f, nsteps, istep0=0, traj0=0, dxi=None, vnh=None):
    """Constrained parent trajectories (SHAKE/RATTLE on xi = 0): returns
    (q, p, f, epot, status, dxi); dxi is the dxi_act state (zeros: start from
    the current centroid)."""
    q = np.array(q, dtype=np.float64)
    p = np.array(p, dtype=np.float64)
    f = np.array(f, dtype=np.float64)
    T = q.shape[0]
    e = np.zeros(T)
    st = np.zeros(T, dtype=np.int32)
    dxi = np.zeros((T, cfg.natoms * 3)) if dxi is None else np.array(dxi, dtype=np.float64)
    if cfg.thermostat == 2 and vnh is None:
        vnh = np.zeros((T, 4))
    vp = _dp(vnh) if vnh is not None else None
    lib().orc_run_parent(C.byref(cfg.c), C.byref(xd), T, traj0, istep0, nsteps, _dp(q), _dp(p), _dp(f), _dp(e),
                         st.ctypes.data_as(C.POINTER(C.c_int)), _dp(dxi), vp)
    return q, p, f, e, st, dxi


def run_umbrella(cfg: Config, xd, q, p, f, nsteps, centers, kforce, istep0=0, traj0=0, vnh=None, sampling=False,
                 stats=None, nbins=0, lo=0.0, hi=1.0):
    """Umbrella-window trajectories (bias towards centers[t] with kforce[t]):
    returns (q, p, f, epot, status, stats) with stats = dict(xsum, xsum2, hist)
    accumulated over the steps when sampling is set."""
    q = np.array(q, dtype=np.float64)
    p = np.array(p, dtype=np.float64)
    f = np.array(f, dtype=np.float64)
    T = q.shape[0]
    e = np.zeros(T)
    st = np.zeros(T, dtype=np.int32)
    if stats is None:
        stats = dict(xsum=np.zeros(T), xsum2=np.zeros(T), hist=np.zeros((T, max(nbins, 1))))
    if cfg.thermostat == 2 and vnh is None:
        vnh = np.zeros((T, 4))
    c = np.ascontiguousarray(centers, dtype=np.float64)
    k = np.ascontiguousarray(kforce, dtype=np.float64)
    lib().orc_run_umbrella(C.byref(cfg.c), C.byref(xd), T, traj0, istep0, nsteps, _dp(c), _dp(k), _dp(q), _dp(p),
                           _dp(f), _dp(e), st.ctypes.data_as(C.POINTER(C.c_int)),
                           _dp(vnh) if vnh is not None else None, int(bool(sampling)), _dp(stats["xsum"]),
                           _dp(stats["xsum2"]), int(nbins), float(lo), float(hi), _dp(stats["hist"]))
    return q, p, f, e, st, stats


def umbrella_bias(cfg: Config, xd, xi0, kforce, q, f):
    """f (nbeads, N, 3) plus the umbrella bias of the ring polymer q; returns (xi, f)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    f = np.array(f, dtype=np.float64)
    xi = lib().orc_umbrella_bias(C.byref(cfg.c), C.byref(xd), float(xi0), float(kforce), _dp(q), _dp(f))
    return xi, f


def calc_xi_umbrella(xd, coords, mass):
    """xi (calc_xi mode 1), dxi (N, 3) and the Hessian (3N, 3N)."""
    c = np.ascontiguousarray(coords, dtype=np.float64)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    n = c.shape[0]
    d = np.zeros((n, 3))
    h = np.zeros((3 * n, 3 * n))
    x = lib().orc_calc_xi_umbrella(C.byref(xd), n, _dp(c), _dp(m), _dp(d), _dp(h))
    return x, d, h


FIT_BASES = {"1g": 1, "2g": 2, "3g": 3, "sp": 4, "sd": 5, "sd2": 6, "sp2d": 7, "sp2d3": 8}


def evb_fit(basis, x, e1, e2, eref, jacobian=True):
    """lm_de_func residuals (and fdjac2's Jacobian, shape (npar, m))."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    e1, e2, eref = (np.ascontiguousarray(a, dtype=np.float64) for a in (e1, e2, eref))
    m = len(e1)
    fvec = np.zeros(m)
    fjac = np.zeros((len(x), m)) if jacobian else None
    lib().orc_evb_fit(FIT_BASES[basis], _dp(x), len(x), m, _dp(e1), _dp(e2), _dp(eref), _dp(fvec),
                      _dp(fjac) if jacobian else None)
    return (fvec, fjac) if jacobian else fvec
