"""QMDFF force-field data on the host: `.qmdff` files and the synthetic alkane.

* ``read_qmdff`` / ``write_qmdff`` follow Caracal's file format: the reader of
  src/rdsolvff.f90:34-202 (header ``n q d``, method line, ``at x y z q mol``
  per atom, ``nbond nangl ntors nhb nnci``, the term lines, H-bond triples six
  per line, NCI triples eight per line; torsion phases are stored over pi) and
  the writer of src/main_gen.f90:825-847.
* ``ElementTables`` are the per-element-pair non-bonded tables Caracal's
  ``prepare`` hands to ``ff_nonb`` (src/setnonb.f90): sr42 = 3 s8 r2r4_i r2r4_j,
  r094 = a1 sqrt(3 r2r4_i r2r4_j) + a2, zab = vz_i vz_j, r0ab = 16.5/R0AB^1.5,
  with Caracal's REAL(4) literals (a1 = 0.45, s8 = 2.7, the valel factors).
  The engine takes these tables (and the C6 pair matrix) from its caller, as
  ff_nonb does.  For the synthetic alkane the C6 pair values and the D3 pair
  radii R0AB are D3-like constants chosen here (Caracal's D3 reference data is
  not reproduced), so that workload is "QMDFF-shaped", not a Caracal fit.
* ``alkane`` builds the synthetic C_nH_2n+2 QMDFF of the benchmark: zig-zag
  chain, r(CC) = 1.53 A, r(CH) = 1.09 A, tetrahedral angles, bond / angle /
  torsion force constants drawn in +-20 % of 0.3 Eh/bohr^2, 0.1 Eh/rad^2,
  0.002 Eh from the seed, charges +-0.1 e with exact neutrality, NCI = all
  pairs three or more bonds apart (categories 3, 4, >=5 -> 5).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .units import BOHR_ANGSTROM

F32 = lambda x: float(np.float32(x))  # noqa: E731  (REAL(4) literal widened to REAL(8))

# published D3 values Caracal keeps in src/setnonb.f90 (r2r4) for H, C, N, O, Cl
R2R4 = {1: F32(2.00734898), 6: F32(3.10492822), 7: F32(2.71175247), 8: F32(2.59361680),
        17: F32(3.72932356)}
# covalent radii, Angstrom (Caracal's rad table is in bohr, src/prepare.f90)
RAD_ANG = {1: 0.32, 6: 0.75, 7: 0.71, 8: 0.63, 17: 0.99}
# synthetic D3-like inputs (not Caracal's D3 tables)
C6_PAIR = {(1, 1): 3.0898, (1, 6): 7.5916, (6, 6): 18.1368, (1, 7): 5.5, (1, 8): 4.6, (6, 7): 14.0,
           (6, 8): 11.5, (7, 7): 11.0, (7, 8): 9.5, (8, 8): 8.0, (1, 17): 12.0, (6, 17): 30.0,
           (7, 17): 24.0, (8, 17): 20.0, (17, 17): 50.0}
R0AB_PAIR_ANG = {(1, 1): 2.1823, (1, 6): 2.5984, (6, 6): 2.9146, (1, 7): 2.47, (1, 8): 2.36,
                 (6, 7): 2.77, (6, 8): 2.66, (7, 7): 2.63, (7, 8): 2.52, (8, 8): 2.41, (1, 17): 2.80,
                 (6, 17): 3.10, (7, 17): 2.97, (8, 17): 2.86, (17, 17): 3.34}
# H-bond / halogen-bond scaling of src/setnonb.f90:123-137 (REAL(4) literals)
SCALE_HB = {7: F32(0.8), 8: F32(0.3), 9: F32(0.1), 15: F32(2.0), 16: F32(2.0), 17: F32(2.0),
            34: F32(2.0), 35: F32(2.0)}
SCALE_XB = {17: F32(0.30), 35: F32(0.60), 53: F32(0.80), 85: F32(1.00)}


def element_radii():
    """rad(94) of module qmdff: covalent radius per element in bohr (H and C set)."""
    r = np.zeros(94)
    for z, v in RAD_ANG.items():
        r[z - 1] = v / BOHR_ANGSTROM
    return r


def valence_charge(z):
    """valel (src/valel.f90) for rows 1-3: valence count times the REAL(4) fit factor."""
    if z <= 2:
        return float(z) * F32(2.35)
    if z <= 10:
        return 1.7 if z == 3 else 5.5 if z == 4 else float(z - 2) * F32(0.95)
    if z <= 18:
        return 2.5 if z == 11 else 3.0 if z == 12 else float(z - 10) * F32(0.75)
    raise ValueError("valence charges are tabulated up to Ar")


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
    r0ab: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))   # alpha of the repulsion
    zab: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))
    r094: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))
    sr42: np.ndarray = field(default_factory=lambda: np.zeros((95, 95)))

    @classmethod
    def d3_like(cls, elements=(1, 6, 7, 8, 17)):
        t = cls()
        a1, s8, a2 = F32(0.45), F32(2.7), 4.0
        for zi in elements:
            for zj in elements:
                t.sr42[zi, zj] = 3.0 * s8 * R2R4[zi] * R2R4[zj]
                t.r094[zi, zj] = a1 * np.sqrt(3.0 * R2R4[zi] * R2R4[zj]) + a2
                t.zab[zi, zj] = valence_charge(zi) * valence_charge(zj)
                key = (min(zi, zj), max(zi, zj))
                r0 = R0AB_PAIR_ANG[key] / BOHR_ANGSTROM
                t.r0ab[zi, zj] = F32(16.5) / r0 ** 1.5
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
        return np.array([RAD_ANG[int(z)] / BOHR_ANGSTROM for z in self.at])

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
        c6 = pair_c6(at)
    return QMDFF(at=at, xyz=xyz, q=q, bond=bond, vbond=vbond, angl=angl, vangl=vangl, tors=tors,
                 vtors=vtors, nci=nci, c6=c6, hb=hb)


def pair_c6(at):
    n = len(at)
    c6 = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            c6[i, j] = C6_PAIR[(min(at[i], at[j]), max(at[i], at[j]))]
    return c6


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
                 vtors=np.array(vtors).reshape(-1, 14), nci=np.array(nci).reshape(-1, 3), c6=pair_c6(at),
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
