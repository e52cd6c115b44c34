"""CPU: Caracal's QMDFF set-up on the host -- the D3 reference table as copyc6
lays it out, coordination numbers and CN-interpolated pair C6 (prepare), the
element tables of setnonb / setr0 / valel -- checked against the oracle's
separate C++ restatement, and the reference's own QMDFF inputs
(examples/dynamic/glutathione, examples/evbopt/dE-EVB) read with it."""
import os

import numpy as np
import pytest

from caracal_gb300 import keyfile as K
from caracal_gb300 import qmdff as Q
from conftest import ROOT
from oracle import oracle as orc

REF = os.path.join(ROOT, "tests", "golden", "reference")
GLUT = os.path.join(REF, "dynamic", "glutathione")
EVB = os.path.join(REF, "evbopt", "dE-EVB")
F32 = lambda x: float(np.float32(x))  # noqa: E731


def test_d3_reference_table_layout():
    c6ab, maxci = Q.d3_reference()
    d = Q.element_data()
    assert d["d3_pars"].shape == (32385, 5)
    # H has the free-atom and the H2 reference (CN 0 and 0.9118), C five references
    assert maxci[0] == 2 and maxci[5] == 5
    assert c6ab[0, 0, 0, 0, 0] == 3.0267 and c6ab[0, 0, 0, 0, 1] == 0.9118
    # symmetric: (i, a; j, b) = (j, b; i, a) with the CNs swapped
    for (i, j, a, b) in ((5, 0, 2, 1), (7, 6, 1, 0), (15, 5, 0, 3)):
        assert c6ab[i, j, a, b, 0] == c6ab[j, i, b, a, 0]
        assert c6ab[i, j, a, b, 1] == c6ab[j, i, b, a, 2]
    # alkali and alkaline-earth C6 taken from the preceding rare gas (CN index 1)
    assert c6ab[2, 5, 0, 1, 0] == c6ab[1, 5, 0, 1, 0]
    assert c6ab[3, 5, 0, 0, 0] == c6ab[1, 5, 0, 0, 0]


def test_element_tables_follow_setnonb():
    t = Q.ElementTables.caracal()
    d = Q.element_data()
    r2r4, vz = d["r2r4"], Q.valence_charges()
    # REAL(4) literals: r2r4, a1 = 0.45, s8 = 2.7, the valel factors
    assert r2r4[0] == F32(2.00734898) and d["rcov"][5] == F32(1.88972601)
    s8, a1 = F32(2.7), F32(0.45)
    assert t.sr42[1, 6] == 3.0 * s8 * r2r4[5] * r2r4[0]      # sr42(j,i) = 3 s8 r2r4(i) r2r4(j)
    assert t.r094[8, 6] == a1 * np.sqrt(3.0 * r2r4[5] * r2r4[7]) + 4.0
    assert vz[0] == 1.0 * F32(2.35) and vz[5] == 4.0 * F32(0.95) and vz[2] == F32(1.7) and vz[15] == 6.0 * F32(0.75)
    assert t.zab[6, 1] == vz[0] * vz[5]
    # r0ab = 16.5 / (R0AB / 0.52917726)^1.5, R0AB(H,H) = 2.1823 (REAL(4))
    assert t.r0ab[1, 1] == 16.5 / (F32(2.1823) / 0.52917726) ** 1.5
    assert np.array_equal(t.r0ab, t.r0ab.T) and np.array_equal(t.zab, t.zab.T)
    # covalent radii in bohr: O 0.64 A, Cl 1.00 A
    rad = Q.element_radii()
    assert rad[7] == 0.64 / 0.52917721092 and rad[16] == 1.00 / 0.52917721092


def test_pair_c6_matches_oracle_restatement():
    d = Q.element_data()
    for ff in (Q.read_qmdff(os.path.join(GLUT, "glutathione.qmdff")), Q.alkane()):
        c6o, cno = orc.d3_pair_c6(d["d3_pars"], ff.at, ff.xyz, d["rcov"])
        assert np.array_equal(Q.ncoord(ff.at, ff.xyz), cno)
        assert np.array_equal(ff.c6, c6o)
        assert np.all(ff.c6 > 0) and np.array_equal(ff.c6, ff.c6.T)


def test_reference_glutathione_inputs():
    ff = Q.read_qmdff(os.path.join(GLUT, "glutathione.qmdff"))
    assert (ff.n, len(ff.bond), len(ff.angl), len(ff.tors), ff.nhb, len(ff.nci)) == (37, 96, 60, 56, 148, 570)
    assert set(ff.at.tolist()) == {1, 6, 7, 8, 16}
    vhb = Q.hb_parameters(ff)
    assert vhb.shape == (148, 2) and np.all(np.isfinite(vhb)) and vhb.max() > 0
    d = K.read(os.path.join(GLUT, "glutathione.key"))
    assert (d.pes, d.nbeads, d.ensemble, d.kelvin, d.thermostat, d.dt_fs) == ("QMDFF", 1, "NVT", 500.0, "nhc", 1.0)
    assert d.ffnames == ["glutathione.qmdff"] and d.eshift == [-1403.0282384116763]
    assert "EVAL_COORD" in d.unsupported
    sym, xyz = K.read_xyz(os.path.join(GLUT, "start.xyz"))
    assert len(sym) == 37 and [Q.element_number(s) for s in sym] == ff.at.tolist()


def test_reference_glutathione_oracle_gradient():
    """The oracle's QMDFF with the real file (live H-bond terms) against
    central differences of its own energy."""
    ff = Q.read_qmdff(os.path.join(GLUT, "glutathione.qmdff"))
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    x = ff.xyz + np.random.default_rng(3).normal(0.0, 0.03, ff.xyz.shape)
    V, g = orc.egrad("qmdff", x)
    h = 1e-5
    for a in (0, 5, 17, 36):
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, c] += h
            xm[a, c] -= h
            fd = (orc.egrad("qmdff", xp)[0][0] - orc.egrad("qmdff", xm)[0][0]) / (2 * h)
            assert abs(fd - g[0][a, c]) < 2e-8


def test_reference_de_evb_inputs():
    ff1 = Q.read_qmdff(os.path.join(EVB, "min1.qmdff"))
    ff2 = Q.read_qmdff(os.path.join(EVB, "min2.qmdff"))
    assert ff1.n == ff2.n == 17 and np.array_equal(ff1.at, ff2.at)
    ref = np.loadtxt(os.path.join(EVB, "ref.dat"))
    frames = Q.read_xyz_frames(os.path.join(EVB, "struc.xyz"))
    assert frames.shape == (len(ref), 17, 3) and np.all(np.isfinite(ref))
    with open(os.path.join(EVB, "evbopt.key")) as fh:
        txt = fh.read().upper()
    assert "PES DE_EVB" in txt and "COUPLING SP" in txt
