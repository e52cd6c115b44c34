"""Python host mirror of the engine's C-ABI, named after Caracal's routines.

``egrad_h3`` mirrors ``subroutine egrad_h3(q,Natoms,Nbeads,V,dVdq,info)``
(src/egrad_h3.f:29); ``RPMDEngine`` batches the ``dynamic`` stepping loop
(src/dynamic.f90:1569-1579 -> ``verlet``, src/verlet.f90:65) over many
independent trajectories, with ``mdinit`` (src/mdinit.f90:40-173) as
``init_positions`` / ``init_momenta`` / ``compute_forces``.

Arrays are numpy float64 of shape (ntraj, nbeads, natoms, 3) in C order,
which is Caracal's q(3, natoms, nbeads) column-major layout per trajectory.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .units import beta_from_kelvin, dt_fs_to_au

PES = {"h3": L.CR_PES_H3, "ana_h3": L.CR_PES_H3, "oh3": L.CR_PES_OH3, "ana_oh3": L.CR_PES_OH3, "ch4h": L.CR_PES_CH4H, "ana_ch4h": L.CR_PES_CH4H,
       "ch4oh": L.CR_PES_CH4OH, "ana_ch4oh": L.CR_PES_CH4OH, "geh4oh": L.CR_PES_GEH4OH, "ana_geh4oh": L.CR_PES_GEH4OH,
       "brh2": L.CR_PES_BRH2, "ana_brh2": L.CR_PES_BRH2}
PES_NATOMS = {L.CR_PES_H3: 3, L.CR_PES_CH4H: 6, L.CR_PES_CH4OH: 7, L.CR_PES_OH3: 4, L.CR_PES_GEH4OH: 7, L.CR_PES_BRH2: 3}
THERMOSTAT = {"none": L.CR_THERMO_NONE, "nve": L.CR_THERMO_NONE, "andersen": L.CR_THERMO_ANDERSEN,
              "nose-hoover": L.CR_THERMO_NHC, "nhc": L.CR_THERMO_NHC, "pile": L.CR_THERMO_PILE}
PRECISION = {"fp64": L.CR_PREC_FP64, "plain": L.CR_PREC_FP64, "mixed": L.CR_PREC_MIXED}


def egrad_h3(q):
    """BKMP2 energies and gradients of q (nbeads, 3, 3) bohr -> (V (nbeads,), dVdq)."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (3, 3):
        raise ValueError("egrad_h3 expects q of shape (nbeads, 3, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_h3(L.dptr(q), 3, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_h3")
    return V, g


def egrad_ch4h(q):
    """CH4+H energies and gradients of q (nbeads, 6, 3) bohr, Caracal's atom order."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (6, 3):
        raise ValueError("egrad_ch4h expects q of shape (nbeads, 6, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_ch4h(L.dptr(q), 6, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_ch4h")
    return V, g


def egrad_ch4oh(q):
    """CH4+OH energies and gradients of q (nbeads, 7, 3) bohr, Caracal's atom order
    (H, C, H, H, H, O, H(O))."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (7, 3):
        raise ValueError("egrad_ch4oh expects q of shape (nbeads, 7, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_ch4oh(L.dptr(q), 7, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_ch4oh")
    return V, g


def egrad_geh4oh(q):
    """GeH4 + OH (ANA_GEH4OH) energies and gradients of q (nbeads, 7, 3) bohr,
    Caracal's atom order (H, Ge, H, H, H, O, H(O))."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (7, 3):
        raise ValueError("egrad_geh4oh expects q of shape (nbeads, 7, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_geh4oh(L.dptr(q), 7, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_geh4oh")
    return V, g


def egrad_brh2(q):
    """Br + H2 (DIM-3C, ANA_BRH2) energies and gradients of q (nbeads, 3, 3)
    bohr, atoms H, Br, H."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (3, 3):
        raise ValueError("egrad_brh2 expects q of shape (nbeads, 3, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_brh2(L.dptr(q), 3, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_brh2")
    return V, g


def egrad_oh3(q):
    """OH + H2 (Schatz-Elgersma, ANA_OH3) energies and gradients of q
    (nbeads, 4, 3) bohr, atoms O, H, H, H."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    if q.ndim == 2:
        q = q[None]
    nb = q.shape[0]
    if q.shape[1:] != (4, 3):
        raise ValueError("egrad_oh3 expects q of shape (nbeads, 4, 3)")
    V = np.zeros(nb)
    g = np.zeros_like(q)
    info = C.c_int(0)
    L.check(L.lib().cr_egrad_oh3(L.dptr(q), 4, nb, L.dptr(V), L.dptr(g), C.byref(info)), "egrad_oh3")
    return V, g


class WaterBox:
    """Caracal's flexible SPC water box on the device (cr_water,
    src/egrad_water.f90): ``nwater`` molecules, atoms ordered O, H, H.
    ``box`` (Angstrom) makes it periodic, with the Coulomb cutoff
    ``coul_cut`` (Angstrom) and the Zahn form set up as src/set_periodic.f90
    does (:func:`caracal_gb300.water.periodic_setup`); without a box every
    pair interacts."""

    def __init__(self, nwater, box=None, coul_cut=0.0, zahn=False):
        from . import water as W
        d = L.CrWaterDef()
        d.nwater = int(nwater)
        if box is not None:
            bb, cut, za, zp = W.periodic_setup(box, coul_cut, zahn)
            d.periodic = 1
            for k in range(3):
                d.box[k] = bb[k]
            d.coul_cut, d.zahn, d.zahn_a, d.zahn_par = cut, int(bool(zahn)), za, zp
        self.nwater = int(nwater)
        self.n = 3 * self.nwater
        self.box_bohr = tuple(d.box) if box is not None else None
        self.coul_cut = d.coul_cut
        self.zahn, self.zahn_a, self.zahn_par = bool(d.zahn), d.zahn_a, d.zahn_par
        h = C.c_void_p()
        L.check(L.lib().cr_water_create(C.byref(d), C.byref(h)), "cr_water_create")
        self._h = h

    @property
    def mass(self):
        from . import water as W
        return W.masses(self.nwater)

    def egrad(self, xyz, precision="fp64"):
        """Energies and gradients of xyz (nbeads, n, 3) bohr."""
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        if x.shape[1:] != (self.n, 3):
            raise ValueError(f"xyz must be (nbeads, {self.n}, 3)")
        V = np.zeros(x.shape[0])
        g = np.zeros_like(x)
        L.check(L.lib().cr_water_egrad(self._h, L.dptr(x), x.shape[0], L.dptr(V), L.dptr(g),
                                       PRECISION[precision] if isinstance(precision, str) else int(precision)),
                "cr_water_egrad")
        return V, g

    def close(self):
        if getattr(self, "_h", None):
            L.lib().cr_water_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class QMDFFForceField:
    """A QMDFF resident on the device (cr_qmdff): Caracal's ff_eg + ff_nonb +
    E_zero (src/gradient.f90:342-358) for one molecule, no H-bond terms.

    ``ff`` is a :class:`caracal_gb300.qmdff.QMDFF` (1-based topology, as read
    from a .qmdff file); ``tables`` the element-pair tables ff_nonb takes
    (:class:`caracal_gb300.qmdff.ElementTables`).  NVT runs use eps1-scaled
    Coulomb within 50 bohr; Caracal's NVE runs use ``zahn=True`` with
    ``coul_cut=10``, ``zahn_a = zahn_par = 0``.
    """

    def __init__(self, ff, tables=None, coul_cut=50.0, zahn=False, zahn_a=0.0, zahn_par=0.0):
        from . import qmdff as Q
        tables = tables if tables is not None else Q.ElementTables.caracal()
        ip = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        fp = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        self.n = int(ff.n)
        tors = np.asarray(ff.tors).reshape(-1, 6)
        self._arrs = dict(
            at=ip(ff.at), q=fp(ff.q), rad=fp(Q.element_radii()),
            bond=ip(np.asarray(ff.bond).reshape(-1, 2)), vbond=fp(np.asarray(ff.vbond).reshape(-1, 3)),
            angl=ip(np.asarray(ff.angl).reshape(-1, 3)), vangl=fp(np.asarray(ff.vangl).reshape(-1, 2)),
            tors=ip(tors), vtors=fp(np.asarray(ff.vtors).reshape(-1, 14)),
            nci=ip(np.asarray(ff.nci).reshape(-1, 3)),
            hb=ip(np.asarray(ff.hb).reshape(-1, 3)), vhb=fp(Q.hb_parameters(ff).reshape(-1, 2)),
            r0ab=fp(tables.r0ab[1:, 1:].T), zab=fp(tables.zab[1:, 1:].T),
            r0094=fp(tables.r094[1:, 1:].T), sr42=fp(tables.sr42[1:, 1:].T), c66ab=fp(np.asarray(ff.c6).T))
        a = self._arrs
        d = L.CrQmdffDef()
        d.natoms = self.n
        d.nbond, d.nangl, d.ntors, d.nnci = len(a["bond"]), len(a["angl"]), len(a["tors"]), len(a["nci"])
        for k in ("at", "bond", "angl", "tors", "nci", "hb"):
            setattr(d, k, L.iptr(a[k]))
        for k in ("q", "rad", "vbond", "vangl", "vtors", "r0ab", "zab", "r0094", "sr42", "c66ab", "vhb"):
            setattr(d, k, L.dptr(a[k]))
        d.nhb = len(a["hb"])
        e1, e2 = Q.eps_factors()
        for k in range(6):
            d.eps1[k], d.eps2[k] = e1[k + 1], e2[k + 1]
        d.coul_cut, d.zahn, d.zahn_a, d.zahn_par = float(coul_cut), int(bool(zahn)), float(zahn_a), float(zahn_par)
        d.e_zero = float(ff.e_zero)
        h = C.c_void_p()
        L.check(L.lib().cr_qmdff_create(C.byref(d), C.byref(h)), "cr_qmdff_create")
        self._h = h

    def egrad(self, xyz, precision="fp64"):
        """Energies (with E_zero) and gradients of xyz (nbeads, n, 3) bohr."""
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        if x.shape[1:] != (self.n, 3):
            raise ValueError(f"expected xyz of shape (nbeads, {self.n}, 3)")
        e = np.zeros(x.shape[0])
        g = np.zeros_like(x)
        prec = PRECISION[precision] if isinstance(precision, str) else int(precision)
        L.check(L.lib().cr_qmdff_egrad(self._h, L.dptr(x), x.shape[0], L.dptr(e), L.dptr(g), prec),
                "cr_qmdff_egrad")
        return e, g

    def egrad_virial(self, xyz, box_bohr=None, precision="fp64"):
        """Energies, gradients and each bead's virial trace (the reference's
        vir_ten terms, NpT) of xyz (nbeads, n, 3) bohr; box_bohr (nbeads, 3)
        or None for the force field's box (set_periodic first)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        if x.shape[1:] != (self.n, 3):
            raise ValueError(f"expected xyz of shape (nbeads, {self.n}, 3)")
        nb = x.shape[0]
        e, w = np.zeros(nb), np.zeros(nb)
        g = np.zeros_like(x)
        bx = None if box_bohr is None else np.ascontiguousarray(np.broadcast_to(box_bohr, (nb, 3)), dtype=np.float64)
        prec = PRECISION[precision] if isinstance(precision, str) else int(precision)
        L.check(L.lib().cr_qmdff_egrad_virial(self._h, L.dptr(x), nb, None if bx is None else L.dptr(bx), L.dptr(e),
                                              L.dptr(g), L.dptr(w), prec), "cr_qmdff_egrad_virial")
        return e, g, w

    def _piece(self, fn, xyz, e, g, precision):
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, self.n, 3)
        prec = PRECISION[precision] if isinstance(precision, str) else int(precision)
        L.check(fn(self._h, L.dptr(x), x.shape[0], L.dptr(e), L.dptr(g), prec), fn.__name__)

    def ff_eg(self, xyz, e, g, precision="fp64"):
        """Caracal's ff_eg: bonded terms into e (nbeads,), g (nbeads, n, 3), overwritten."""
        self._piece(L.lib().cr_qmdff_eg, xyz, e, g, precision)

    def ff_nonb(self, xyz, e, g, precision="fp64"):
        """Caracal's ff_nonb: the NCI-pair terms added to e, g."""
        self._piece(L.lib().cr_qmdff_nonb, xyz, e, g, precision)

    def ff_hb(self, xyz, e, g, precision="fp64"):
        """Caracal's ff_hb: the hydrogen- and halogen-bond terms added to e, g."""
        self._piece(L.lib().cr_qmdff_hb, xyz, e, g, precision)

    @classmethod
    def load(cls, path, tables=None, e_zero=0.0, zahn=False, coul_cut=50.0):
        """A device QMDFF read from a .qmdff file by the library's own reader
        with Caracal's set-up (cr_qmdff_load_d3: coordination numbers of the
        file's geometry, CN-interpolated D3 pair C6)."""
        from . import qmdff as Q
        tables = tables if tables is not None else Q.ElementTables.caracal()
        fp = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        c6ab, maxci = Q.d3_reference()
        arrs = dict(rad=fp(Q.element_radii()), r0ab=fp(tables.r0ab[1:, 1:].T), zab=fp(tables.zab[1:, 1:].T),
                    r0094=fp(tables.r094[1:, 1:].T), sr42=fp(tables.sr42[1:, 1:].T),
                    c6ref=fp(np.ravel(c6ab, order="F")), maxci=np.ascontiguousarray(maxci, dtype=np.int32),
                    rcov=fp(Q.element_data()["rcov"]))
        t = L.CrQmdffTables(*[L.dptr(arrs[k]) for k in ("rad", "r0ab", "zab", "r0094", "sr42")], None)
        d3 = L.CrD3Reference(L.dptr(arrs["c6ref"]), L.iptr(arrs["maxci"]), L.dptr(arrs["rcov"]))
        h = C.c_void_p()
        L.check(L.lib().cr_qmdff_load_d3(str(path).encode(), C.byref(t), C.byref(d3), float(e_zero),
                                         int(bool(zahn)), float(coul_cut), C.byref(h)), "cr_qmdff_load_d3")
        obj = cls.__new__(cls)
        obj._h = h
        obj._arrs = arrs
        counts = np.zeros(5, dtype=np.int32)
        n = C.c_int()
        L.check(L.lib().cr_qmdff_file_counts(str(path).encode(), C.byref(n), L.iptr(counts)), "file_counts")
        obj.n = n.value
        return obj

    @property
    def nparams(self):
        """Number of linear parameters (bond k, angle k, torsion V, pair qq)."""
        n = C.c_int()
        L.check(L.lib().cr_qmdff_nparams(self._h, C.byref(n)), "cr_qmdff_nparams")
        return n.value

    def hvp(self, xyz, w):
        """Energies, gradients and Hessian-vector products H w (plain FP64)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, self.n, 3)
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(x.shape)
        e = np.zeros(x.shape[0])
        g = np.zeros_like(x)
        hw = np.zeros_like(x)
        L.check(L.lib().cr_qmdff_hvp(self._h, L.dptr(x), L.dptr(w), x.shape[0], L.dptr(e), L.dptr(g), L.dptr(hw)),
                "cr_qmdff_hvp")
        return e, g, hw

    def param_vjp(self, xyz, v):
        """d/dtheta sum_b v_b . grad E(xyz_b) over the linear parameters
        (bond k, angle k, torsion V, pair qq, in that order)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, self.n, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(x.shape)
        grad = np.zeros(self.nparams)
        L.check(L.lib().cr_qmdff_param_vjp(self._h, L.dptr(x), L.dptr(v), x.shape[0], L.dptr(grad)),
                "cr_qmdff_param_vjp")
        return grad

    def schedule_info(self):
        b = np.zeros(5, dtype=np.int32)
        c = C.c_int()
        L.check(L.lib().cr_qmdff_schedule_info(self._h, L.iptr(b), C.byref(c)), "schedule_info")
        return {"batches": b.tolist(), "colors": c.value}

    def set_periodic(self, box_ang, coul_cut_ang=50.0, vdw_cut_ang=10.0):
        """Periodic box (edges in Angstrom) with set_periodic's cutoff rules;
        returns (coul_cut, vdw_cut, zahn_a, zahn_par) in bohr as set.  box_ang
        None switches it off.  Before creating an engine on the force field."""
        cuts = np.zeros(4)
        if box_ang is None:
            L.check(L.lib().cr_qmdff_set_periodic(self._h, None, 0.0, 0.0, None), "qmdff_set_periodic")
            return None
        box = np.ascontiguousarray(box_ang, dtype=np.float64)
        L.check(L.lib().cr_qmdff_set_periodic(self._h, L.dptr(box), float(coul_cut_ang), float(vdw_cut_ang),
                                              L.dptr(cuts)), "qmdff_set_periodic")
        return tuple(cuts)

    def tuning(self, precision="fp64"):
        """The autotuner's choice and timings of the force-kernel variants."""
        v = C.c_int()
        ms = (C.c_float * 3)()
        prec = PRECISION[precision] if isinstance(precision, str) else int(precision)
        L.check(L.lib().cr_qmdff_tuning(self._h, prec, C.byref(v), ms), "qmdff_tuning")
        return {"variant": v.value, "ms": list(ms)}

    def close(self):
        if getattr(self, "_h", None):
            L.lib().cr_qmdff_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


EVB_BASES = {"const": 0, "1g": 1, "2g": 2, "3g": 3, "sp": 4, "sd": 5, "sd2": 6, "sp2d": 7}


class EVBPair:
    """dE-EVB of two device QMDFFs (cr_evb): Caracal's two-QMDFF gradient
    branch (src/gradient.f90:361-386, 1228-1304).  Each force field carries
    its E_zero; ``basis`` is Caracal's off_basis and ``par`` the offa..offh,
    offm, offn values as a dict with keys a..h, m, n.  Both force fields must
    stay alive while the pair is used."""

    def __init__(self, ff1, ff2, basis="1g", **par):
        self.ff1, self.ff2 = ff1, ff2
        self.n = ff1.n
        d = L.CrEvbDef()
        d.basis = EVB_BASES[basis]
        for k in "abcdefghmn":
            setattr(d, k, float(par.get(k, 0.0)))
        h = C.c_void_p()
        L.check(L.lib().cr_evb_create(ff1._h, ff2._h, C.byref(d), C.byref(h)), "cr_evb_create")
        self._h = h

    def egrad(self, xyz, precision="fp64"):
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        if x.ndim == 2:
            x = x[None]
        e = np.zeros(x.shape[0])
        g = np.zeros_like(x)
        prec = PRECISION[precision] if isinstance(precision, str) else int(precision)
        L.check(L.lib().cr_evb_egrad(self._h, L.dptr(x), x.shape[0], L.dptr(e), L.dptr(g), prec), "cr_evb_egrad")
        return e, g

    def param_vjp(self, xyz, v, ff1=True):
        """d/dc sum_b v_b . grad E_EVB(xyz_b) over the coupling parameters
        (dict a..h, m, n) and, with ff1, over the first force field's linear
        parameters (plain FP64)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, self.n, 3)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(x.shape)
        gc = np.zeros(10)
        gf = np.zeros(max(self.ff1.nparams, 1)) if ff1 else None
        L.check(L.lib().cr_evb_param_vjp(self._h, L.dptr(x), L.dptr(v), x.shape[0], L.dptr(gc),
                                         L.dptr(gf) if ff1 else None), "cr_evb_param_vjp")
        out = dict(zip("abcdefghmn", gc))
        return (out, gf[:self.ff1.nparams]) if ff1 else out

    def close(self):
        if getattr(self, "_h", None):
            L.lib().cr_evb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


FIT_BASES = {"1g": 1, "2g": 2, "3g": 3, "sp": 4, "sd": 5, "sd2": 6, "sp2d": 7, "sp2d3": 8}


def evb_fit(basis, x, e1, e2, eref, jacobian=True):
    """Residuals of Caracal's dE-EVB coupling fit (lm_de_func) at parameters x
    and, optionally, MINPACK's forward-difference Jacobian (fdjac2), shape
    (npar, m); computed on the device."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    e1, e2, eref = (np.ascontiguousarray(a, dtype=np.float64) for a in (e1, e2, eref))
    m = len(e1)
    fvec = np.zeros(m)
    fjac = np.zeros((len(x), m)) if jacobian else None
    L.check(L.lib().cr_evb_fit(FIT_BASES[basis], L.dptr(x), len(x), m, L.dptr(e1), L.dptr(e2), L.dptr(eref),
                               L.dptr(fvec), L.dptr(fjac) if jacobian else None), "cr_evb_fit")
    return (fvec, fjac) if jacobian else fvec


def evb_fit_grad(basis, x, e1, e2, eref):
    """Analytic gradient of sum_i fvec_i of the dE-EVB fit (device, dual numbers)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    e1, e2, eref = (np.ascontiguousarray(a, dtype=np.float64) for a in (e1, e2, eref))
    grad = np.zeros(len(x))
    L.check(L.lib().cr_evb_fit_grad(FIT_BASES[basis], L.dptr(x), len(x), len(e1), L.dptr(e1), L.dptr(e2),
                                    L.dptr(eref), L.dptr(grad)), "cr_evb_fit_grad")
    return grad


class PinnedHost:
    """Page-lock numpy arrays the caller owns (cr_host_register) for the
    duration of a with-block, so host-buffer steps copy them at pinned speed."""

    def __init__(self, *arrays):
        self.arrays = [a for a in arrays if a is not None]

    def __enter__(self):
        done = []
        try:
            for a in self.arrays:
                if not a.flags.c_contiguous:
                    raise ValueError("only contiguous arrays can be registered")
                L.check(L.lib().cr_host_register(a.ctypes.data_as(C.c_void_p), a.nbytes), "cr_host_register")
                done.append(a)
        except Exception:
            for a in done:
                L.lib().cr_host_unregister(a.ctypes.data_as(C.c_void_p))
            raise
        return self

    def __exit__(self, *exc):
        for a in self.arrays:
            L.lib().cr_host_unregister(a.ctypes.data_as(C.c_void_p))


class RPMDEngine:
    """A batch of independent RPMD trajectories resident on one GPU.

    ``pes`` is an analytic surface name ("h3", "ch4h") or a
    :class:`QMDFFForceField`, which must stay alive while the engine runs."""

    def __init__(self, pes, mass, nbeads, ntraj, dt_au, beta=None, thermostat="none",
                 andersen_step=70, pile_tau0_au=0.0, transrot=True, precision="fp64", seed=0,
                 traj0=0, nose_q_au=0.0, nm_mode=0):
        self.ff = pes if isinstance(pes, (QMDFFForceField, EVBPair)) else None
        self.water = pes if isinstance(pes, WaterBox) else None
        if isinstance(pes, WaterBox):
            self.pes = L.CR_PES_WATER
        elif isinstance(pes, EVBPair):
            self.pes = L.CR_PES_EVB
        elif self.ff is not None:
            self.pes = L.CR_PES_QMDFF
        else:
            self.pes = PES[pes] if isinstance(pes, str) else int(pes)
        self.mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.natoms = len(self.mass)
        self.nbeads = int(nbeads)
        self.ntraj = int(ntraj)
        self.beta = float("inf") if beta is None else float(beta)
        self.cfg = L.CrConfig(self.pes, self.natoms, self.nbeads, self.ntraj,
                              THERMOSTAT[thermostat] if isinstance(thermostat, str) else int(thermostat),
                              int(andersen_step), int(bool(transrot)),
                              PRECISION[precision] if isinstance(precision, str) else int(precision),
                              int(seed) & 0xFFFFFFFF, int(traj0) & 0xFFFFFFFF, float(dt_au),
                              self.beta, float(pile_tau0_au), L.dptr(self.mass), float(nose_q_au), int(nm_mode))
        h = C.c_void_p()
        if self.water is not None:
            L.check(L.lib().cr_engine_create_water(C.byref(self.cfg), self.water._h, C.byref(h)),
                    "cr_engine_create_water")
        elif isinstance(self.ff, EVBPair):
            L.check(L.lib().cr_engine_create_evb(C.byref(self.cfg), self.ff._h, C.byref(h)),
                    "cr_engine_create_evb")
        elif self.ff is not None:
            L.check(L.lib().cr_engine_create_qmdff(C.byref(self.cfg), self.ff._h, C.byref(h)),
                    "cr_engine_create_qmdff")
        else:
            L.check(L.lib().cr_engine_create(C.byref(self.cfg), C.byref(h)), "cr_engine_create")
        self._h = h

    @classmethod
    def from_caracal_units(cls, pes, mass, nbeads, ntraj, dt_fs, kelvin=None, **kw):
        beta = None if not kelvin else beta_from_kelvin(kelvin)
        return cls(pes, mass, nbeads, ntraj, dt_fs_to_au(dt_fs), beta=beta, **kw)

    @property
    def shape(self):
        return (self.ntraj, self.nbeads, self.natoms, 3)

    def close(self):
        if getattr(self, "_h", None):
            L.lib().cr_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_positions(self, q0, sigma=0.0):
        q0 = np.ascontiguousarray(q0, dtype=np.float64).reshape(self.natoms, 3)
        L.check(L.lib().cr_engine_init_positions(self._h, L.dptr(q0), float(sigma)), "init_positions")

    def init_momenta(self, zero=False):
        L.check(L.lib().cr_engine_init_momenta(self._h, int(bool(zero))), "init_momenta")

    def compute_forces(self):
        L.check(L.lib().cr_engine_compute_forces(self._h), "compute_forces")

    def mdinit(self, draw=0):
        """Caracal's mdinit: forces (plus the umbrella bias where the engine
        has windows), momenta from Gaussian stream `draw` (NVT) or zero
        (NVE), chain at rest."""
        L.check(L.lib().cr_engine_mdinit(self._h, int(draw) & 0xFFFFFFFF), "mdinit")

    def set_andersen_step(self, n):
        L.check(L.lib().cr_engine_set_andersen_step(self._h, int(n)), "set_andersen_step")

    def set_npt(self, pressure_atm, box_bohr=None):
        """NpT with the Berendsen barostat (periodic QMDFF): target pressure
        in atm, each trajectory's starting box (ntraj, 3) bohr or None for
        the force field's."""
        bx = None
        if box_bohr is not None:
            bx = np.ascontiguousarray(np.broadcast_to(box_bohr, (self.ntraj, 3)), dtype=np.float64)
        L.check(L.lib().cr_engine_set_npt(self._h, float(pressure_atm), None if bx is None else L.dptr(bx)),
                "set_npt")

    def npt_state(self, reset_sum=False):
        """(box (ntraj, 3) bohr, the last step's pressure (ntraj,) a.u., the
        sum of the pressures since the last reset (ntraj,) a.u.)."""
        box = np.zeros((self.ntraj, 3))
        pr, ps = np.zeros(self.ntraj), np.zeros(self.ntraj)
        L.check(L.lib().cr_engine_get_npt(self._h, L.dptr(box), L.dptr(pr), L.dptr(ps), int(bool(reset_sum))),
                "get_npt")
        return box, pr, ps

    def set_launch(self, threads_per_block=0, threads_per_bead=1):
        """Threads per block and per bead of the persistent step kernel
        (threads_per_block 0: the built-in choice)."""
        L.check(L.lib().cr_engine_set_launch(self._h, int(threads_per_block), int(threads_per_bead)),
                "set_launch")

    def launch(self):
        """(threads per block, blocks, threads per bead) of the persistent step
        kernel; zeros on the graph path."""
        b, g, tpb = C.c_int(0), C.c_int(0), C.c_int(0)
        L.check(L.lib().cr_engine_get_launch(self._h, C.byref(b), C.byref(g), C.byref(tpb)), "get_launch")
        return b.value, g.value, tpb.value

    def autotune(self, nsteps=20):
        """Time nsteps steps at each launch shape from the same state (put
        back afterwards), keep the fastest; returns (threads per block,
        threads per bead, ms per step)."""
        b, tpb, ms = C.c_int(0), C.c_int(0), C.c_float(0.0)
        L.check(L.lib().cr_engine_autotune(self._h, int(nsteps), C.byref(b), C.byref(tpb), C.byref(ms)),
                "autotune")
        return b.value, tpb.value, ms.value

    def set_state(self, q, p, f=None):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.shape)
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(self.shape)
        fp = None
        if f is not None:
            f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.shape)
            fp = L.dptr(f)
        L.check(L.lib().cr_engine_set_state(self._h, L.dptr(q), L.dptr(p), fp), "set_state")

    def get_state(self):
        q = np.zeros(self.shape)
        p = np.zeros(self.shape)
        f = np.zeros(self.shape)
        e = np.zeros(self.ntraj)
        st = np.zeros(self.ntraj, dtype=np.int32)
        L.check(L.lib().cr_engine_get_state(self._h, L.dptr(q), L.dptr(p), L.dptr(f), L.dptr(e),
                                            L.iptr(st)), "get_state")
        return q, p, f, e, st

    def run(self, nsteps, check=True):
        rc = L.lib().cr_engine_run(self._h, int(nsteps))
        if check:
            L.check(rc, "run")
        return rc

    def run_dump(self, nsteps, every, callback):
        """Run nsteps steps; after every step whose index is a multiple of
        `every`, callback(istep, q, p, epot) gets the state (numpy views of
        host buffers, valid during the call); a truthy return stops the run."""
        q = np.zeros(self.shape)
        p = np.zeros(self.shape)
        e = np.zeros(self.ntraj)

        def cb(_user, istep, _q, _p, _e):
            return 1 if callback(istep, q, p, e) else 0
        fn = L.DUMP_FN(cb)
        L.check(L.lib().cr_engine_run_dump(self._h, int(nsteps), int(every), fn, None, L.dptr(q), L.dptr(p),
                                           L.dptr(e)), "run_dump")

    def run_dump_async(self, nsteps, every, callback):
        """run_dump with the frames copied out behind the stepping: the GPU
        runs on while callback(istep, q, p, epot) writes the previous frame.
        The arrays are views of the library's page-locked snapshot buffers,
        valid during the call only (copy what must be kept)."""
        n = int(np.prod(self.shape))

        def cb(_user, istep, q, p, e):
            qa = np.ctypeslib.as_array(q, shape=(n,)).reshape(self.shape)
            pa = np.ctypeslib.as_array(p, shape=(n,)).reshape(self.shape)
            ea = np.ctypeslib.as_array(e, shape=(self.ntraj,))
            return 1 if callback(istep, qa, pa, ea) else 0
        fn = L.DUMP_FN(cb)
        L.check(L.lib().cr_engine_run_dump_async(self._h, int(nsteps), int(every), fn, None), "run_dump_async")

    def step_host(self, q, p, f, epot=None):
        """One verlet step through host arrays (modified in place)."""
        ep = L.dptr(epot) if epot is not None else None
        L.check(L.lib().cr_engine_step_host(self._h, L.dptr(q), L.dptr(p), L.dptr(f), ep), "step_host")

    @staticmethod
    def _recross_def(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal):
        rc = L.CrRecross()
        rc.nreac1, rc.nreac2 = len(reac1), len(reac2)
        for i, a in enumerate(reac1):
            rc.reac1[i] = a
        for i, a in enumerate(reac2):
            rc.reac2[i] = a
        rc.bond_form[0], rc.bond_form[1] = bond_form
        rc.bond_break[0], rc.bond_break[1] = bond_break
        rc.form_ref, rc.break_ref, rc.r_inf, rc.xi_ideal = form_ref, break_ref, r_inf, xi_ideal
        return rc

    def set_parent(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal=1.0):
        """Constrained parent (SHAKE/RATTLE on xi = 0 of the BIMOLEC coordinate;
        1-based atoms as in Caracal's MECHA block); call after the initial state."""
        rc = self._recross_def(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal)
        L.check(L.lib().cr_engine_set_parent(self._h, C.byref(rc)), "set_parent")

    def set_umbrella(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, centers, kforce,
                     nbins=0, lo=0.0, hi=1.0, xi_ideal=1.0):
        """Umbrella windows: trajectory t biased towards xi = centers[t] with
        force constant kforce[t] (Eh), xi of calc_xi mode 1 on the MECHA
        definition (1-based atoms); nbins > 0 also histograms xi over [lo, hi)."""
        rc = self._recross_def(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal)
        c = np.ascontiguousarray(np.broadcast_to(centers, (self.ntraj,)), dtype=np.float64)
        k = np.ascontiguousarray(np.broadcast_to(kforce, (self.ntraj,)), dtype=np.float64)
        self._umb_nbins = int(nbins)
        L.check(L.lib().cr_engine_set_umbrella(self._h, C.byref(rc), L.dptr(c), L.dptr(k), int(nbins), float(lo),
                                               float(hi)), "set_umbrella")

    def umbrella_sampling(self, on=True):
        L.check(L.lib().cr_engine_umbrella_sampling(self._h, int(bool(on))), "umbrella_sampling")

    def umbrella_stats(self, reset=False):
        """(xsum, xsum2, hist) of xi over the sampled steps per trajectory."""
        xs = np.zeros(self.ntraj)
        x2 = np.zeros(self.ntraj)
        h = np.zeros((self.ntraj, max(getattr(self, "_umb_nbins", 0), 1)))
        L.check(L.lib().cr_engine_umbrella_stats(self._h, L.dptr(xs), L.dptr(x2), L.dptr(h), int(bool(reset))),
                "umbrella_stats")
        return xs, x2, h[:, :getattr(self, "_umb_nbins", 0)]

    def set_recross(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf,
                    xi_ideal=1.0, max_steps=1):
        """BIMOLEC recrossing bookkeeping; atom indices 1-based as in Caracal's MECHA block."""
        rc = L.CrRecross()
        rc.nreac1, rc.nreac2 = len(reac1), len(reac2)
        for i, a in enumerate(reac1):
            rc.reac1[i] = a
        for i, a in enumerate(reac2):
            rc.reac2[i] = a
        rc.bond_form[0], rc.bond_form[1] = bond_form
        rc.bond_break[0], rc.bond_break[1] = bond_break
        rc.form_ref, rc.break_ref, rc.r_inf, rc.xi_ideal = form_ref, break_ref, r_inf, xi_ideal
        L.check(L.lib().cr_engine_set_recross(self._h, C.byref(rc), int(max_steps)), "set_recross")

    def init_children(self, q_parent):
        qp = np.ascontiguousarray(q_parent, dtype=np.float64).reshape(self.nbeads, self.natoms, 3)
        L.check(L.lib().cr_engine_init_children(self._h, L.dptr(qp)), "init_children")

    def kappa(self, max_steps):
        num = np.zeros(max_steps)
        den = np.zeros(1)
        w = np.zeros(self.ntraj)
        ns = C.c_int(0)
        L.check(L.lib().cr_engine_kappa(self._h, L.dptr(num), L.dptr(den), L.dptr(w), C.byref(ns)),
                "kappa")
        return num[:ns.value], float(den[0]), w

    def last_kernel_ms(self):
        ms = C.c_float()
        L.check(L.lib().cr_engine_last_kernel_ms(self._h, C.byref(ms)), "last_kernel_ms")
        return ms.value

    def launch_info(self):
        g, b, s, n = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.check(L.lib().cr_engine_launch_info(self._h, C.byref(g), C.byref(b), C.byref(s), C.byref(n)),
                "launch_info")
        return {"grid": g.value, "block": b.value, "smem_bytes": s.value, "launches": n.value}


class RPMDBatch:
    """Several engines (trajectory classes of different surfaces, atom and
    bead counts or precisions) advanced together, one graph launch per chunk
    of steps (cr_batch).  run(n) gives every engine the state that its own
    run(n) would give."""

    def __init__(self, engines, chunk_steps=50):
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e._h for e in self.engines])
        h = C.c_void_p()
        L.check(L.lib().cr_batch_create(arr, len(self.engines), int(chunk_steps), C.byref(h)), "batch_create")
        self._h = h

    def run(self, nsteps, check=True):
        rc = L.lib().cr_batch_run(self._h, int(nsteps))
        if check:
            L.check(rc, "batch_run")
        return rc

    def info(self):
        n, g, ms = C.c_longlong(), C.c_int(), C.c_float()
        L.check(L.lib().cr_batch_info(self._h, C.byref(n), C.byref(g), C.byref(ms)), "batch_info")
        return {"launches": n.value, "graph_nodes": g.value, "ms": ms.value}

    def timeline(self):
        """Per engine (begin, end) in ms of its branch within the last graph
        launch; overlapping intervals ran concurrently."""
        n = len(self.engines)
        b, e = (C.c_float * n)(), (C.c_float * n)()
        L.check(L.lib().cr_batch_timeline(self._h, b, e), "batch_timeline")
        return [(b[i], e[i]) for i in range(n)]

    def close(self):
        if getattr(self, "_h", None):
            L.lib().cr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
