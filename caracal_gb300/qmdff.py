"""QMDFF force-field data on the host: `.qmdff` files, Caracal's element tables
and D3 dispersion set-up, and the synthetic alkane.

* ``read_qmdff`` / ``write_qmdff`` follow Caracal's file format: the reader of
  src/rdsolvff.f90:34-202 (header ``n q d``, method line, ``at x y z q mol``
  per atom, ``nbond nangl ntors nhb nnci``, the term lines, H-bond triples six
  per line, NCI triples eight per line; torsion phases are stored over pi) and
  the writer of src/main_gen.f90:825-847.
* ``prepare`` is Caracal's QMDFF set-up (src/prepare.f90:100-127): the D3
  reference C6 table as ``copyc6`` lays it out (src/copyc6.f90:35674-35744,
  element codes split by ``limit``, src/limit.f90:34-60), coordination numbers
  of the reference geometry (``ncoord_qmdff``, src/ncoord_qmdff.f90:36-76) and
  the CN-interpolated pair C6 (``getc6``, src/getc6.f90:35-83).
* ``ElementTables.caracal`` are the per-element-pair tables ``setnonb`` makes
  (src/setnonb.f90:35-192): sr42 = 3 s8 r2r4_i r2r4_j, r094 = a1 sqrt(3
  r2r4_i r2r4_j) + a2, zab = vz_i vz_j (``valel``, src/valel.f90:35-115),
  r0ab = 16.5 / R0AB^1.5 with the D3 cut-off radii of ``setr0``
  (src/setr0.f90), with Caracal's REAL(4) literals (a1 = 0.45, s8 = 2.7, the
  r2r4 / rcov / R0AB arrays, the valel factors).  The element data come from
  ``data/qmdff_tables.npz`` (made by ``data/make_qmdff_tables.py`` from the
  reference's source files).
* ``alkane`` builds the synthetic C_nH_2n+2 QMDFF of the benchmark: zig-zag
  chain, r(CC) = 1.53 A, r(CH) = 1.09 A, tetrahedral angles, bond / angle /
  torsion force constants drawn in +-20 % of 0.3 Eh/bohr^2, 0.1 Eh/rad^2,
  0.002 Eh from the seed, charges +-0.1 e with exact neutrality, NCI = all
  pairs three or more bonds apart (categories 3, 4, >=5 -> 5), C6 from
  Caracal's D3 set-up on its geometry.
"""
from __future__ import annotations

import functools
import math
import os
from dataclasses import dataclass, field

import numpy as np

from .units import BOHR_ANGSTROM

F32 = lambda x: float(np.float32(x))  # noqa: E731  (REAL(4) literal widened to REAL(8))
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "qmdff_tables.npz")

# H-bond / halogen-bond scaling of src/setnonb.f90:123-137 (REAL(4) literals)
SCALE_HB = {7: F32(0.8), 8: F32(0.3), 9: F32(0.1), 15: F32(2.0), 16: F32(2.0), 17: F32(2.0),
            34: F32(2.0), 35: F32(2.0)}
SCALE_XB = {17: F32(0.30), 35: F32(0.60), 53: F32(0.80), 85: F32(1.00)}


@functools.lru_cache(maxsize=1)
def element_data():
    """The element arrays of data/qmdff_tables.npz (read once)."""
    with np.load(DATA) as d:
        return {k: d[k].copy() for k in d.files}


def valence_charges():
    """vz(94) of valel (src/valel.f90:35-115), index 0 = element 1: the
    valence-shell counts times the REAL(4) fit factors, then the fitted
    group-1/2 values (REAL(4) literals widened)."""
    z = np.zeros(95)
    for i in range(1, 55):
        at = float(i)
        z[i] = at
        if 2 < i <= 10:
            z[i] = at - 2
        if 10 < i <= 13:
            z[i] = at - 10
        if 13 < i <= 18:
            z[i] = at - 10
        if (30 <= i <= 36) or i in (19, 20):
            z[i] = at - 18
            if i >= 30:
                z[i] = at - 28
        if 21 <= i <= 29:
            z[i] = at - 18
        if 37 <= i <= 47:
            z[i] = at - 36
        if 47 < i <= 54:
            z[i] = at - 46
    z[57:81] = 4.0
    for i in range(81, 87):
        z[i] = float(i) - 78.0
    z[1:3] *= F32(2.35)
    z[3:11] *= F32(0.95)
    z[11:19] *= F32(0.75)
    z[19:55] *= F32(0.65)
    z[55:95] *= F32(0.60)
    for i, v in ((3, 1.7), (11, 2.5), (19, 3.0), (37, 3.0), (55, 3.0), (87, 3.0), (4, 5.5), (12, 3.0), (20, 2.8),
                 (38, 2.6), (56, 2.4), (88, 2.4)):
        z[i] = F32(v)
    return z[1:]


def valence_charge(z):
    return float(valence_charges()[int(z) - 1])


def _limit(iat):
    """src/limit.f90: element code above 100 -> (element, CN-reference index)."""
    iadr = 1
    while iat > 100:
        iat -= 100
        iadr += 1
    return iat, iadr


@functools.lru_cache(maxsize=1)
def d3_reference():
    """(c6ab (94, 94, 5, 5, 3), maxci (94,)) as copyc6 leaves module qmdff:
    c6ab[i, j, a, b] = (C6, CN_i, CN_j) of the reference pair (element i+1,
    CN index a+1; element j+1, CN index b+1), -1 where none exists; the
    alkali and alkaline-earth C6 copied from the preceding rare gas."""
    pars = element_data()["d3_pars"]
    c6ab = np.full((94, 94, 5, 5, 3), -1.0)
    maxci = np.zeros(94, dtype=np.int64)
    for c6, a, b, cn1, cn2 in pars:
        iat, iadr = _limit(int(a))
        jat, jadr = _limit(int(b))
        maxci[iat - 1] = max(maxci[iat - 1], iadr)
        maxci[jat - 1] = max(maxci[jat - 1], jadr)
        c6ab[iat - 1, jat - 1, iadr - 1, jadr - 1] = (c6, cn1, cn2)
        c6ab[jat - 1, iat - 1, jadr - 1, iadr - 1] = (c6, cn2, cn1)
    for iat in (3, 11, 19, 37, 55, 87):       # src/copyc6.f90:35702-35740
        i, g = iat - 1, iat - 2               # 0-based alkali, rare gas
        for j in range(94):
            mj = maxci[j]
            for ii in range(maxci[i]):
                c6ab[i, j, ii, :mj, 0] = c6ab[g, j, 0, :mj, 0]
                c6ab[j, i, :mj, ii, 0] = c6ab[j, g, :mj, 0, 0]
            for ii in range(maxci[i + 1]):
                c6ab[i + 1, j, ii, :mj, 0] = c6ab[g, j, 0, :mj, 0]
                c6ab[j, i + 1, :mj, ii, 0] = c6ab[j, g, :mj, 0, 0]
    return c6ab, maxci


def ncoord(at, xyz, cn_thr=5000.0):
    """Coordination numbers (src/ncoord_qmdff.f90:36-76): sum over the other
    atoms of 1 / (1 + exp(-16 (rcov_i + rcov_j) / r - 1)), pairs with
    r^2 > cn_thr bohr^2 skipped; xyz in bohr."""
    rcov = element_data()["rcov"]
    n = len(at)
    cn = np.zeros(n)
    for i in range(n):
        xn = 0.0
        for j in range(n):
            if j == i:
                continue
            dx, dy, dz = xyz[j, 0] - xyz[i, 0], xyz[j, 1] - xyz[i, 1], xyz[j, 2] - xyz[i, 2]
            r2 = dx * dx + dy * dy + dz * dz
            if r2 > cn_thr:
                continue
            r = math.sqrt(r2)
            rr = (rcov[at[i] - 1] + rcov[at[j] - 1]) / r
            xn = xn + 1.0 / (1.0 + math.exp(-16.0 * (rr - 1.0)))
        cn[i] = xn
    return cn


def getc6(iat, jat, nci, ncj):
    """CN-interpolated C6 of elements iat, jat (src/getc6.f90:35-83): the
    exp(-4 r) weighted mean over the reference pairs, r = (CN1 - nci)^2 +
    (CN2 - ncj)^2; the nearest reference where every weight underflows."""
    c6ab, maxci = d3_reference()
    c6mem, rsum, csum, r_save = -1e99, 0.0, 0.0, 10000.0
    for i in range(maxci[iat - 1]):
        for j in range(maxci[jat - 1]):
            c6, cn1, cn2 = c6ab[iat - 1, jat - 1, i, j]
            if c6 > 0:
                r = (cn1 - nci) * (cn1 - nci) + (cn2 - ncj) * (cn2 - ncj)   # Fortran ** 2: a product
                if r < r_save:
                    r_save, c6mem = r, c6
                tmp1 = math.exp(-4.0 * r)
                rsum = rsum + tmp1
                csum = csum + tmp1 * c6
    return csum / rsum if rsum > 1e-99 else c6mem


def pair_c6(at, xyz):
    """c6xy (n, n) of prepare (src/prepare.f90:121-129) for the reference
    geometry xyz (bohr)."""
    at = np.asarray(at, dtype=int)
    cn = ncoord(at, np.asarray(xyz, dtype=float))
    n = len(at)
    c6 = np.zeros((n, n))
    for i1 in range(n):
        for i2 in range(i1 + 1):
            c6[i2, i1] = c6[i1, i2] = getc6(int(at[i1]), int(at[i2]), cn[i1], cn[i2])
    return c6


SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
           "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu").split()


def element_number(symbol):
    """Atomic number of an element symbol (case-insensitive)."""
    return SYMBOLS.index(symbol.strip().capitalize()) + 1


def read_xyz_frames(path):
    """Every frame of an xyz file, coordinates converted to bohr:
    (nframes, natoms, 3)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    frames, k = [], 0
    while k < len(lines) and lines[k].strip():
        n = int(lines[k].split()[0])
        frames.append([[float(x) for x in lines[k + 2 + i].split()[1:4]] for i in range(n)])
        k += n + 2
    return np.array(frames) / BOHR_ANGSTROM


def element_radii():
    """rad(94) of module qmdff after prepare: covalent radii (Mantina et al.,
    src/prepare.f90:177-192) converted to bohr."""
    return element_data()["rad_angstrom"] / BOHR_ANGSTROM


def hbpara(a, b, q):
    """src/hbpara.f90: exp(-a q) / (exp(-a q) + b)."""
    return np.exp(-a * q) / (np.exp(-a * q) + b)


def hb_parameters(ff):
    """vhb(2, nhb) as rdsolvff computes it (src/rdsolvff.f90:142-152): for an H
    bond (third atom H) ca, cb = hbpara(10, 5, q) * scalehb of atoms 1 and 2,
    for a halogen bond ca = scalexb(X) * hbpara(-6.5, 1, q(X))."""
    hb = np.asarray(ff.hb).reshape(-1, 3)
    v = np.zeros((len(hb), 2))
    for k, (a, b, h) in enumerate(hb):
        a, b, h = a - 1, b - 1, h - 1
        if ff.at[h] == 1:
            v[k, 0] = hbpara(10.0, 5.0, ff.q[a]) * SCALE_HB.get(int(ff.at[a]), 0.0)
            v[k, 1] = hbpara(10.0, 5.0, ff.q[b]) * SCALE_HB.get(int(ff.at[b]), 0.0)
        else:
            v[k, 0] = SCALE_XB.get(int(ff.at[h]), 0.0) * hbpara(-6.5, 1.0, ff.q[h])
    return v


@dataclass
class ElementTables:
    """Per-element-pair tables of ff_nonb, 1-based [iz1, iz2] as Caracal's
    arrays (iz1, iz2) (index 0 unused)."""
    r0ab: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))   # alpha of the repulsion
    zab: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))
    r094: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))
    sr42: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))

    @classmethod
    @functools.lru_cache(maxsize=1)
    def caracal(cls):
        """setnonb's tables (src/setnonb.f90:138-161), term by term in the
        reference's evaluation order: sr42(j,i) = 3 s8 r2r4(i) r2r4(j),
        r094(j,i) = a1 sqrt(3 r2r4(i) r2r4(j)) + a2, zab(j,i) = vz(i) vz(j),
        r0ab = 16.5 / (R0AB / 0.52917726)^1.5 (src/setr0.f90:810-819)."""
        d = element_data()
        r2r4 = d["r2r4"]
        vz = valence_charges()
        t = cls()
        a1, s8, a2 = F32(0.45), F32(2.7), 4.0
        for i in range(94):
            for j in range(94):
                t.sr42[j + 1, i + 1] = 3.0 * s8 * r2r4[i] * r2r4[j]
                t.r094[j + 1, i + 1] = a1 * math.sqrt(3.0 * r2r4[i] * r2r4[j]) + a2
                t.zab[j + 1, i + 1] = vz[i] * vz[j]
        r0 = d["r0ab_ref"]
        k = 0
        for i in range(94):
            for j in range(i + 1):
                v = 16.5 / (r0[k] / 0.52917726) ** 1.5
                t.r0ab[i + 1, j + 1] = t.r0ab[j + 1, i + 1] = v
                k += 1
        return t


@dataclass
class QMDFF:
    at: np.ndarray            # (n,) element numbers
    xyz: np.ndarray           # (n, 3) reference geometry, bohr
    q: np.ndarray             # (n,) charges
    bond: np.ndarray          # (nbond, 2) 1-based
    vbond: np.ndarray         # (nbond, 3): r0 (bohr), k, a
    angl: np.ndarray          # (nangl, 3) 1-based, centre first
    vangl: np.ndarray         # (nangl, 2): theta0 (rad), k
    tors: np.ndarray          # (ntors, 6): i j k l nt type (1-based atoms)
    vtors: np.ndarray         # (ntors, 14): phi0, V, (rn, phase*pi, Vn) x 4
    nci: np.ndarray           # (nnci, 3): i j category (1-based atoms)
    c6: np.ndarray            # (n, n) pair C6 (Caracal's c6xy)
    e_zero: float = 0.0
    method: str = "synthetic"
    hb: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), int))  # (nhb, 3) A B H, 1-based

    @property
    def n(self):
        return len(self.at)

    def rad_bohr(self):
        return element_radii()[np.asarray(self.at, dtype=int) - 1]

    @property
    def nhb(self):
        return len(np.asarray(self.hb).reshape(-1, 3))


def _fmt(x):
    return f"{x:18.12f}"


def write_qmdff(ff: QMDFF, path):
    """Caracal's .qmdff text format (src/main_gen.f90:825-847)."""
    with open(path, "w") as fh:
        fh.write(f"{ff.n:4d}{1.0:10.4f}{0.0:10.4f}\n{ff.method}\n")
        for i in range(ff.n):
            fh.write(f"{int(ff.at[i]):5d}" + "".join(_fmt(v) for v in ff.xyz[i]) + _fmt(ff.q[i]) + f"{0:5d}\n")
        fh.write("".join(f"{v:8d}" for v in (len(ff.bond), len(ff.angl), len(ff.tors), ff.nhb, len(ff.nci), 0))
                 + "\n")
        for b, v in zip(ff.bond, ff.vbond):
            fh.write(f"{b[0]:5d}{b[1]:5d}" + "".join(_fmt(x) for x in v) + "\n")
        for a, v in zip(ff.angl, ff.vangl):
            fh.write(f"{a[0]:5d}{a[1]:5d}{a[2]:5d}" + "".join(_fmt(x) for x in v) + "\n")
        for t, v in zip(ff.tors, ff.vtors):
            s = "".join(f"{x:4d}" for x in t[:4]) + "".join(f"{x:2d}" for x in t[4:6])
            s += f"{v[0]:16.12f}{v[1]:16.12f}"
            for j in range(int(t[4])):
                s += f"{v[2 + 3 * j]:4.1f}{v[3 + 3 * j] / np.pi:4.1f}{v[4 + 3 * j]:16.8E}"
            fh.write(s + "\n")
        htrip = [f"{a:4d}{b:4d}{c:4d}  " for a, b, c in np.asarray(ff.hb).reshape(-1, 3)]
        for k in range(0, len(htrip), 6):
            fh.write("".join(htrip[k:k + 6]) + "\n")
        trip = [f"{a:4d}{b:4d}{c:4d}  " for a, b, c in ff.nci]
        for k in range(0, len(trip), 8):
            fh.write("".join(trip[k:k + 8]) + "\n")


def _records(path):
    with open(path) as fh:
        return fh.read().splitlines()


def read_qmdff(path, c6=None):
    """Read a .qmdff file with the record semantics of Caracal's list-directed
    reads (each read starts on a new line and may continue over lines)."""
    lines = _records(path)
    pos = [0]

    def read(nvals, conv=float):
        vals = []
        while len(vals) < nvals:
            toks = lines[pos[0]].replace("D", "E").replace("d", "e").split()
            pos[0] += 1
            vals.extend(toks)
        return [conv(v) for v in vals[:nvals]]

    head = lines[0].split()
    n = int(float(head[0]))
    pos[0] = 2
    at, xyz, q = np.zeros(n, int), np.zeros((n, 3)), np.zeros(n)
    for i in range(n):
        v = read(6)
        at[i], xyz[i], q[i] = int(v[0]), v[1:4], v[4]
    nbond, nangl, ntors, nhb, nnci = [int(x) for x in read(5)]
    bond, vbond = np.zeros((nbond, 2), int), np.zeros((nbond, 3))
    for m in range(nbond):
        v = read(5)
        bond[m], vbond[m] = [int(v[0]), int(v[1])], v[2:5]
    angl, vangl = np.zeros((nangl, 3), int), np.zeros((nangl, 2))
    for m in range(nangl):
        v = read(5)
        angl[m], vangl[m] = [int(x) for x in v[:3]], v[3:5]
    tors, vtors = np.zeros((ntors, 6), int), np.zeros((ntors, 14))
    for m in range(ntors):
        line = lines[pos[0]].replace("D", "E").replace("d", "e")
        pos[0] += 1
        toks = line.split()
        tors[m] = [int(x) for x in toks[:6]]
        nt = tors[m, 4]
        vals = [float(x) for x in toks[6:6 + 2 + 3 * nt]]
        vtors[m, :2] = vals[:2]
        for j in range(nt):
            vtors[m, 2 + 3 * j] = vals[2 + 3 * j]
            vtors[m, 3 + 3 * j] = vals[3 + 3 * j] * np.pi
            vtors[m, 4 + 3 * j] = vals[4 + 3 * j]
    hb = np.array(read(3 * nhb, int), dtype=int).reshape(nhb, 3) if nhb else np.zeros((0, 3), int)
    nci = np.array(read(3 * nnci, int), dtype=int).reshape(nnci, 3) if nnci else np.zeros((0, 3), int)
    if c6 is None:
        c6 = pair_c6(at, xyz)
    return QMDFF(at=at, xyz=xyz, q=q, bond=bond, vbond=vbond, angl=angl, vangl=vangl, tors=tors,
                 vtors=vtors, nci=nci, c6=c6, hb=hb)


def alkane_geometry(nc=20, r_cc=1.53, r_ch=1.09):
    """Zig-zag C_nH_2n+2, Angstrom; returns (at, xyz, carbon neighbour list)."""
    th = np.arccos(-1.0 / 3.0)
    ux, uz = np.sin(th / 2.0), np.cos(th / 2.0)
    cpos = np.array([[k * r_cc * ux, 0.0, (k % 2) * r_cc * uz] for k in range(nc)])
    at, xyz = [6] * nc, [c for c in cpos]
    hs = []
    for k in range(nc):
        nbr = []
        if k > 0:
            nbr.append(cpos[k - 1] - cpos[k])
        if k < nc - 1:
            nbr.append(cpos[k + 1] - cpos[k])
        if len(nbr) == 1:   # terminal: continue the zig-zag for the in-plane H
            nbr.append(np.array([-nbr[0][0], 0.0, nbr[0][2]]))
            inplane = nbr[1] / np.linalg.norm(nbr[1])
            hs.append((k, inplane))
        b = -(nbr[0] / np.linalg.norm(nbr[0]) + nbr[1] / np.linalg.norm(nbr[1]))
        b /= np.linalg.norm(b)
        y = np.array([0.0, 1.0, 0.0])
        for s in (1.0, -1.0):
            d = np.cos(th / 2.0) * b + s * np.sin(th / 2.0) * y
            hs.append((k, d / np.linalg.norm(d)))
    for k, d in hs:
        at.append(1)
        xyz.append(cpos[k] + r_ch * d)
    return np.array(at), np.array(xyz)


def _topology(at, xyz_ang):
    n = len(at)
    bonds = []
    for i in range(n):
        for j in range(i + 1, n):
            d = np.linalg.norm(xyz_ang[i] - xyz_ang[j])
            cut = 1.7 if at[i] == 6 and at[j] == 6 else 1.2
            if d < cut:
                bonds.append((i, j))
    adj = [[] for _ in range(n)]
    for i, j in bonds:
        adj[i].append(j)
        adj[j].append(i)
    # topological distance by BFS
    dist = np.full((n, n), 99, dtype=int)
    for s in range(n):
        dist[s, s] = 0
        front = [s]
        while front:
            nxt = []
            for u in front:
                for v in adj[u]:
                    if dist[s, v] > dist[s, u] + 1:
                        dist[s, v] = dist[s, u] + 1
                        nxt.append(v)
            front = nxt
    return bonds, adj, dist


def _adjacency(n, bonds):
    adj = [[] for _ in range(n)]
    for i, j in bonds:
        adj[i].append(j)
        adj[j].append(i)
    dist = np.full((n, n), 99, dtype=int)
    for s in range(n):
        dist[s, s] = 0
        front = [s]
        while front:
            nxt = []
            for u in front:
                for v in adj[u]:
                    if dist[s, v] > dist[s, u] + 1:
                        dist[s, v] = dist[s, u] + 1
                        nxt.append(v)
            front = nxt
    return adj, dist


def from_topology(at, xyz, bonds, seed=20261203, k_bond=0.3, k_angle=0.1, v_tors=0.002, r0=None,
                  e_zero=0.0, charges=None, hb=None):
    """QMDFF terms for a bond list (0-based pairs) on geometry xyz (bohr): bond
    curvature k_bond, angle curvature k_angle, torsion barrier v_tors (each
    drawn in +-20 % from the seed), reference values from the geometry (or
    r0[(i, j)] for given bonds), charges +-0.1 e neutral, NCI = pairs three or
    more bonds apart."""
    rng = np.random.default_rng(seed)
    at = np.asarray(at)
    n = len(at)
    adj, dist = _adjacency(n, bonds)
    bond = np.array([[i + 1, j + 1] for i, j in bonds])
    vbond = np.zeros((len(bonds), 3))
    a_exp = 6.0
    for m, (i, j) in enumerate(bonds):
        rr = np.linalg.norm(xyz[i] - xyz[j]) if r0 is None or (i, j) not in r0 else r0[(i, j)]
        K = k_bond * rng.uniform(0.8, 1.2)          # curvature Eh/bohr^2
        vbond[m] = [rr, 2.0 * K * rr * rr / (a_exp * a_exp), a_exp]
    angl, vangl = [], []
    for j in range(n):
        nb = adj[j]
        for x in range(len(nb)):
            for y in range(x + 1, len(nb)):
                i, k = nb[x], nb[y]
                v1, v2 = xyz[i] - xyz[j], xyz[k] - xyz[j]
                th0 = np.arccos(np.clip(np.dot(v1, v2) / np.linalg.norm(v1) / np.linalg.norm(v2), -1, 1))
                if at[i] == 1 and at[k] == 1 or abs(th0 - np.arccos(-1 / 3)) > 0.6:
                    th0 = np.arccos(-1.0 / 3.0)       # tetrahedral reference for distorted centres
                K = k_angle * rng.uniform(0.8, 1.2)   # Eh/rad^2
                angl.append([j + 1, i + 1, k + 1])
                vangl.append([th0, K / (2.0 * np.sin(th0) ** 2)])
    tors, vtors = [], []
    for b, c in bonds:
        for a in adj[b]:
            if a == c:
                continue
            for d in adj[c]:
                if d == b or d == a:
                    continue
                v = np.zeros(14)
                v[0] = np.pi          # phi0 (staggered reference)
                v[1] = v_tors * rng.uniform(0.8, 1.2)
                v[2], v[3], v[4] = 3.0, np.pi, 1.0   # rn = 3, phase pi: minima at staggered
                tors.append([a + 1, b + 1, c + 1, d + 1, 1, 0])
                vtors.append(v)
    nci = []
    for i in range(n):
        for j in range(i + 1, n):
            if dist[i, j] >= 3:
                nci.append([i + 1, j + 1, min(int(dist[i, j]), 5)])
    if charges is None:
        q = np.where(at == 6, -0.1, 0.1).astype(float)
        q[at == 1] -= q.sum() / np.count_nonzero(at == 1)   # exact neutrality
    else:
        q = np.asarray(charges, dtype=float)
    hb = np.zeros((0, 3), int) if hb is None else np.asarray(hb, int).reshape(-1, 3)
    return QMDFF(at=at, xyz=xyz.copy(), q=q, bond=bond, vbond=vbond, angl=np.array(angl).reshape(-1, 3),
                 vangl=np.array(vangl).reshape(-1, 2), tors=np.array(tors).reshape(-1, 6),
                 vtors=np.array(vtors).reshape(-1, 14), nci=np.array(nci).reshape(-1, 3), c6=pair_c6(at, xyz),
                 e_zero=e_zero, hb=hb)


def water_dimer():
    """Synthetic QMDFF of a water dimer with one O-H...O hydrogen bond
    (hb triple: acceptor O, donor O, bridging H), bohr."""
    xa = np.array([[0.0, 0.0, 0.0], [0.96, 0.0, 0.0], [-0.24, 0.93, 0.0],
                   [2.91, 0.0, 0.0], [3.23, 0.76, 0.47], [3.23, -0.76, 0.47]])
    at = np.array([8, 1, 1, 8, 1, 1])
    return from_topology(at, xa / BOHR_ANGSTROM, [(0, 1), (0, 2), (3, 4), (3, 5)], seed=11,
                         charges=[-0.6, 0.3, 0.3, -0.6, 0.3, 0.3], hb=[[4, 1, 2]])


def chloromethane_ammonia():
    """Synthetic QMDFF of CH3Cl...NH3 with one C-Cl...N halogen bond (hb triple:
    C, N, Cl), bohr."""
    xa = np.array([[0.0, 0.0, 0.0], [-0.36, 1.03, 0.0], [-0.36, -0.51, 0.89], [-0.36, -0.51, -0.89],
                   [1.78, 0.0, 0.0], [4.88, 0.0, 0.0], [5.26, 0.94, 0.0], [5.26, -0.47, 0.81],
                   [5.26, -0.47, -0.81]])
    at = np.array([6, 1, 1, 1, 17, 7, 1, 1, 1])
    return from_topology(at, xa / BOHR_ANGSTROM, [(0, 1), (0, 2), (0, 3), (0, 4), (5, 6), (5, 7), (5, 8)],
                         seed=12, charges=[-0.2, 0.12, 0.12, 0.12, -0.16, -0.9, 0.3, 0.3, 0.3],
                         hb=[[1, 6, 5]])


def alkane(nc=20, seed=20261203, k_bond=0.3, k_angle=0.1, v_tors=0.002):
    """Synthetic C_nH_2n+2 QMDFF (bohr, Hartree)."""
    at, xa = alkane_geometry(nc)
    bonds, _, _ = _topology(at, xa)
    return from_topology(at, xa / BOHR_ANGSTROM, bonds, seed=seed, k_bond=k_bond, k_angle=k_angle,
                         v_tors=v_tors)


def alkane_evb_partner(ff: QMDFF, seed=20261207, e_zero=0.02):
    """EVB partner of an alkane QMDFF: the first hydrogen of carbon 0 is bonded
    to carbon 1 instead (a 1,2 H shift), with r(CH) = 1.09 A as the partner's
    reference bond length; same atoms, own parameters and E_zero."""
    n = ff.n
    bonds = [(int(i) - 1, int(j) - 1) for i, j in ff.bond]
    h = next(j for i, j in bonds if i == 0 and ff.at[j] == 1)
    bonds = [(i, j) for i, j in bonds if not (i == 0 and j == h)] + [(1, h)]
    r0 = {(1, h): 1.09 / BOHR_ANGSTROM}
    assert len(bonds) == n - 1
    return from_topology(ff.at, ff.xyz, bonds, seed=seed, r0=r0, e_zero=e_zero)


def pair_parameters(ff: QMDFF, tab: ElementTables):
    """Per-NCI-pair R0, C6, sr42, zab, alpha as ff_nonb reads them."""
    i1, i2 = ff.nci[:, 0] - 1, ff.nci[:, 1] - 1
    z1, z2 = ff.at[i1], ff.at[i2]
    return (tab.r094[z1, z2].copy(), ff.c6[i2, i1].copy(), tab.sr42[z1, z2].copy(),
            tab.zab[z1, z2].copy(), tab.r0ab[z1, z2].copy())


def eps_factors():
    """eps1, eps2 of src/setnonb.f90:164-190 (index = NCI category)."""
    eps1 = np.zeros(7)
    eps2 = np.zeros(7)
    eps1[3], eps1[4], eps1[5] = F32(0.85), 1.0, 1.0
    eps2[3], eps2[4], eps2[5], eps2[6] = 0.5, 0.5, 1.0, 1.0
    return eps1, eps2
