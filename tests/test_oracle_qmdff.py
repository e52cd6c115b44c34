"""CPU: the QMDFF oracle (ff_eg + ff_nonb restatement) and the host-side
QMDFF data: topology of the synthetic C20H42, the .qmdff reader/writer, and
the oracle's analytic gradient against central differences (Caracal's own
NUM_GRAD check, src/gradient.f90)."""
import numpy as np
import pytest

from caracal_gb300 import qmdff as Q
from oracle import oracle as orc


@pytest.fixture(scope="module")
def alkane():
    ff = Q.alkane()
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    return ff


def test_alkane_topology(alkane):
    ff = alkane
    assert ff.n == 62 and int((ff.at == 6).sum()) == 20
    assert len(ff.bond) == 61 and len(ff.angl) == 120 and len(ff.tors) == 171
    # all pairs three or more bonds apart
    assert len(ff.nci) == 1710
    assert set(np.unique(ff.nci[:, 2])) <= {3, 4, 5}
    assert abs(ff.q.sum()) < 1e-12


def test_reference_geometry_is_valence_minimum(alkane):
    ff = alkane
    # bonds, angles and torsions sit at their reference values, so only the
    # non-bonded pairs contribute: a copy without NCI pairs has E = 0, g = 0
    ff0 = Q.QMDFF(at=ff.at, xyz=ff.xyz, q=ff.q, bond=ff.bond, vbond=ff.vbond, angl=ff.angl,
                  vangl=ff.vangl, tors=ff.tors, vtors=ff.vtors, nci=ff.nci[:0], c6=ff.c6)
    orc.set_qmdff(ff0, Q.ElementTables.caracal())
    V, g = orc.egrad("qmdff", ff.xyz)
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    assert abs(V[0]) < 1e-20
    assert np.max(np.abs(g)) < 1e-12


def test_gradient_matches_central_differences(alkane):
    rng = np.random.default_rng(5)
    x = alkane.xyz + rng.normal(0, 0.1, alkane.xyz.shape)
    V, g = orc.egrad("qmdff", x)
    h = 1e-5
    fd = np.zeros_like(x)
    for a in range(x.shape[0]):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, d] += h
            xm[a, d] -= h
            fd[a, d] = (orc.egrad("qmdff", xp)[0][0] - orc.egrad("qmdff", xm)[0][0]) / (2 * h)
    assert np.max(np.abs(fd - g[0])) / np.max(np.abs(g[0])) < 1e-7


def test_zahn_coulomb_gradient(alkane):
    # NVE form: q q (erfc(a r)/r - par (r - cut)) within 10 bohr
    ff = alkane
    orc.set_qmdff(ff, Q.ElementTables.caracal(), coul_cut=10.0, zahn=True)
    try:
        x = ff.xyz + np.random.default_rng(6).normal(0, 0.05, ff.xyz.shape)
        V, g = orc.egrad("qmdff", x)
        assert np.isfinite(V).all() and np.isfinite(g).all()
    finally:
        orc.set_qmdff(ff, Q.ElementTables.caracal())


def test_qmdff_file_round_trip(alkane, tmp_path):
    ff = alkane
    path = tmp_path / "c20h42.qmdff"
    Q.write_qmdff(ff, path)
    rd = Q.read_qmdff(path)
    assert np.array_equal(rd.at, ff.at)
    np.testing.assert_allclose(rd.xyz, ff.xyz, atol=1e-11)
    np.testing.assert_allclose(rd.q, ff.q, atol=1e-11)
    for k in ("bond", "angl", "tors", "nci"):
        assert np.array_equal(getattr(rd, k), getattr(ff, k)), k
    np.testing.assert_allclose(rd.vbond, ff.vbond, atol=1e-11)
    np.testing.assert_allclose(rd.vangl, ff.vangl, atol=1e-11)
    np.testing.assert_allclose(rd.vtors, ff.vtors, atol=1e-11)


def test_element_tables_real4_literals():
    t = Q.ElementTables.caracal()
    # setnonb's a1 = 0.45, s8 = 2.7 and the r2r4 array are REAL(4) literals widened to REAL(8)
    s8 = float(np.float32(2.7))
    r2r4 = Q.element_data()["r2r4"]
    assert r2r4[5] == float(np.float32(3.10492822))
    assert t.sr42[6, 6] == 3.0 * s8 * r2r4[5] * r2r4[5]
    assert Q.eps_factors()[0][3] == float(np.float32(0.85))
    r = Q.element_radii()
    assert r.shape == (94,) and r[0] > 0 and r[5] > 0


def test_hbond_gradient_central_differences():
    # eabhag (src/eabhag.f90) is analytic: its gradient is the derivative of
    # its energy; the synthetic water dimer has one O-H...O triple
    ff = Q.water_dimer()
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    x = ff.xyz + np.random.default_rng(0).normal(0, 0.03, ff.xyz.shape)
    V, g = orc.egrad("qmdff", x)
    ff0 = Q.QMDFF(**{**ff.__dict__, "hb": np.zeros((0, 3), int)})
    orc.set_qmdff(ff0, Q.ElementTables.caracal())
    V0, _ = orc.egrad("qmdff", x)
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    assert V[0] < V0[0] - 1e-4          # the H bond is attractive here
    h = 1e-5
    for a in range(ff.n):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, d] += h
            xm[a, d] -= h
            fd = (orc.egrad("qmdff", xp)[0][0] - orc.egrad("qmdff", xm)[0][0]) / (2 * h)
            assert abs(fd - g[0][a, d]) < 1e-9


def test_halogen_bond_reproduces_reference_quirk():
    # eabxag (src/eabxag.f90:111-134) assigns each scalar difference quotient
    # to the whole 3-vector inside its j loop: every component of each of the
    # three atoms' gradients equals that atom's z quotient
    ff = Q.chloromethane_ammonia()
    tab = Q.ElementTables.caracal()
    x = ff.xyz + np.random.default_rng(1).normal(0, 0.03, ff.xyz.shape)
    orc.set_qmdff(ff, tab)
    _, g = orc.egrad("qmdff", x)
    orc.set_qmdff(Q.QMDFF(**{**ff.__dict__, "hb": np.zeros((0, 3), int)}), tab)
    _, g0 = orc.egrad("qmdff", x)
    dg = g[0] - g0[0]
    for atom in (0, 4, 5):              # C, Cl, N of the triple
        assert np.allclose(dg[atom], dg[atom][2], rtol=0, atol=1e-15)
        assert abs(dg[atom][2]) > 1e-6
    others = [i for i in range(ff.n) if i not in (0, 4, 5)]
    assert np.max(np.abs(dg[others])) < 1e-15


def test_qmdff_file_round_trip_with_hbonds(tmp_path):
    ff = Q.water_dimer()
    path = tmp_path / "w2.qmdff"
    Q.write_qmdff(ff, path)
    rd = Q.read_qmdff(path)
    assert np.array_equal(rd.hb, ff.hb) and np.array_equal(rd.nci, ff.nci)
    np.testing.assert_allclose(Q.hb_parameters(rd), Q.hb_parameters(ff), atol=1e-10)


def test_periodic_rules_and_large_box_limit():
    """set_periodic's cutoff rules (src/set_periodic.f90:67-113), and a box
    far larger than the molecule with cutoffs beyond every pair: the same
    energy and gradient as the non-periodic force field."""
    from caracal_gb300 import qmdff as Q
    ff = Q.alkane()
    tab = Q.ElementTables.caracal()
    bohr = 0.52917721092
    x = ff.xyz[None] + np.random.default_rng(3).normal(0, 0.05, (4,) + ff.xyz.shape)
    orc.set_qmdff(ff, tab)
    e0, g0 = orc.egrad("qmdff", x)
    cuts = orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 150.0)
    assert cuts[0] == 150.0 / bohr and cuts[1] == 150.0 / bohr
    e1, g1 = orc.egrad("qmdff", x)
    assert np.array_equal(e0, e1) and np.array_equal(g0, g1)
    # a Coulomb cutoff beyond half the shortest edge: half of it minus 0.1 bohr;
    # one below 5 bohr: the same
    assert orc.set_qmdff_periodic([30.0, 24.0, 40.0], 50.0, 10.0)[0] == 12.0 / bohr - 0.1
    assert orc.set_qmdff_periodic([30.0, 24.0, 40.0], 2.0, 10.0)[0] == 12.0 / bohr - 0.1
    # the dispersion cutoff removes pairs: the energy changes
    orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 4.0)
    e2, _ = orc.egrad("qmdff", x)
    assert not np.allclose(e2, e0)
    # Zahn: the cutoff is fixed at 10 A with its parameters
    orc.set_qmdff(ff, tab, zahn=True)
    c = orc.set_qmdff_periodic([30.0, 30.0, 30.0], 50.0, 10.0)
    a = 0.2 * bohr
    rc = 10.0 / bohr
    from math import erfc, exp, pi, sqrt
    assert c[0] == rc and c[2] == a
    assert abs(c[3] - (erfc(a * rc) / rc ** 2 + 2 * a / sqrt(pi) * exp(-(a * rc) ** 2) / rc)) < 1e-15
    orc.set_qmdff(ff, tab)


def _no_torsions(ff):
    from caracal_gb300 import qmdff as Q
    return Q.QMDFF(**{**ff.__dict__, "tors": np.zeros((0, 6), int), "vtors": np.zeros((0, 14))})


def test_virial_bonds_angles_pairs_is_the_scaling_derivative():
    """The virial trace of the terms whose reference formula is the sum of
    (r - r_ref).g over the term's atoms (bonds, angles, NCI pairs and
    hydrogen bonds, src/ff_eg.f90:138-150, 270-281, src/ff_nonb.f90:180-190,
    405-415): for a whole molecule in a box with cutoffs beyond every pair it
    is dE/ds of the uniform scaling r -> s r at s = 1."""
    from caracal_gb300 import qmdff as Q
    ff = _no_torsions(Q.alkane())
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 150.0)
    x = ff.xyz[None] + np.random.default_rng(7).normal(0, 0.05, (3,) + ff.xyz.shape)
    _, g, w = orc.qmdff_egrad_virial(x)
    assert np.allclose(w, np.einsum("bij,bij->b", x, g), rtol=1e-12, atol=1e-12)
    h = 1e-6
    ep, _ = orc.egrad("qmdff", x * (1 + h))
    em, _ = orc.egrad("qmdff", x * (1 - h))
    assert np.allclose(w, (ep - em) / (2 * h), rtol=1e-6, atol=1e-9)


def test_virial_torsions_follow_the_reference_vectors():
    """With torsions the reference's formula vab.g_i + vcb.(g_k + g_l) +
    vdc.g_l (vcb = r_j - r_k, vdc = r_k - r_l, src/ff_eg.f90:317-320,
    420-440) differs from sum (r - r_j).g; the difference is
    -2 [(r_k - r_j).(g_k + g_l) + (r_l - r_k).g_l] per torsion, so the trace
    is not the scaling derivative (and the force field's total is)."""
    from caracal_gb300 import qmdff as Q
    ff = Q.alkane()
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 150.0)
    x = ff.xyz[None] + np.random.default_rng(8).normal(0, 0.05, (2,) + ff.xyz.shape)
    _, g, w = orc.qmdff_egrad_virial(x)
    orc.set_qmdff(_no_torsions(ff), Q.ElementTables.caracal())
    orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 150.0)
    _, g0, w0 = orc.qmdff_egrad_virial(x)
    gt = g - g0                                  # the torsions' gradient
    consistent = np.einsum("bij,bij->b", x, gt)  # sum r.g of the torsion terms = dE_tors/ds
    assert np.all(np.abs((w - w0) - consistent) > 1e-8 * np.abs(consistent).max())
    # a rigid translation leaves it unchanged (each term's vectors are differences)
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    orc.set_qmdff_periodic([400.0, 400.0, 400.0], 150.0, 150.0)
    _, _, wt = orc.qmdff_egrad_virial(x + np.array([0.3, -1.1, 2.0]))
    assert np.allclose(wt, w, rtol=1e-10, atol=1e-12)


def test_npt_berendsen_oracle_step():
    """One Berendsen step (src/verlet.f90:1111-1151): the pressure is
    -tr W / (3 V) from the step's virial, box and coordinates scale by
    (1 + dt compress / taupres (p - p0))^(1/3)."""
    from caracal_gb300 import qmdff as Q
    from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
    ff = Q.alkane(nc=3)
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    orc.set_qmdff_periodic([15.0, 15.0, 15.0], 50.0, 10.0)
    mass = [mass_au("C" if z == 6 else "H") for z in ff.at]
    dt = dt_fs_to_au(0.5)
    cfg = orc.Config("qmdff", mass, 2, dt, beta_from_kelvin(300.0), thermostat="andersen", andersen_step=5,
                     transrot=True, seed=3)
    q = orc.init_positions(cfg, 2, ff.xyz, 0.02)
    p = orc.init_momenta(cfg, 2)
    f, _ = orc.init_forces(cfg, q)
    box0 = np.full((2, 3), 15.0 / 0.52917721092)
    q1, p1, f1, e1, st, box1, pr = orc.run_npt(cfg, q, p, f, 1, box0, 1.0)
    # the pressure from the virial of the step's own forces: the pre-scaling
    # positions are q1 / scale
    scale = box1[:, 0] / box0[:, 0]
    _, _, w = orc.qmdff_egrad_virial((q1 / scale[:, None, None, None]).reshape(-1, ff.n, 3),
                                     np.repeat(box0, 2, axis=0))
    V = np.prod(box0, axis=1)
    assert np.allclose(pr, -w.reshape(2, 2).sum(axis=1) / (3 * V), rtol=1e-10)
    rate = dt * orc.BERENDSEN_COMPRESS / orc.BERENDSEN_TAUPRES
    assert np.allclose(scale, (1 + rate * (pr - 1.0 / orc.PRESCON)) ** (1 / 3), rtol=1e-14)
    assert np.allclose(box1, box0 * scale[:, None], rtol=1e-15) and not st.any()
