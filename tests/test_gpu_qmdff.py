"""GPU: the QMDFF force kernel and the large-molecule engine path against the
oracle, synthetic C20H42 (62 atoms).

Tolerances (norm-wise relative, max|a-b|/max|b|):
  plain FP64 form: energies and gradients <= 1e-12, single engine step
                   <= 1e-12, 20-step trajectories <= 1e-9;
  mixed form:      gradient error against FP64 bounded by 2e-6 on distorted
                   geometries, and by 1e-7 of the largest force component on
                   thermal ring polymers (the form's stated bound).
"""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300 import qmdff as Q
from caracal_gb300.engine import QMDFFForceField
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, nose_q_to_au
from caracal_gb300.workloads import qmdff_config
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def alkane():
    return Q.alkane()


@pytest.fixture(scope="module")
def gpu_ff(alkane, require_gpu):
    ff = QMDFFForceField(alkane)
    yield ff
    ff.close()


@pytest.fixture(autouse=True)
def oracle_ff(alkane):
    orc.set_qmdff(alkane, Q.ElementTables.caracal())


def geoms(ff, nb, sigma, seed):
    rng = np.random.default_rng(seed)
    return ff.xyz[None] + rng.normal(0, sigma, (nb,) + ff.xyz.shape)


def test_schedule_covers_every_term(gpu_ff):
    info = gpu_ff.schedule_info()
    b = info["batches"]
    # mixed form: NCI pairs in matchings of one colour (at most 31 terms on 62
    # atoms); bonds, angles, torsions with at most 3, 4, 6 colours per batch
    assert b[0] >= 2 and b[3] >= (1710 + 30) // 31
    assert b[1] >= 4 and b[2] >= 6
    assert sum(b) <= info["colors"] <= 3 * b[0] + 4 * b[1] + 6 * b[2] + b[3] + 2 * b[4]


def test_egrad_fp64_matches_oracle(gpu_ff, alkane):
    x = geoms(alkane, 256, 0.1, 1)
    e, g = gpu_ff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def test_autotuner_picks_a_variant_and_keeps_parity(alkane, require_gpu):
    ff = QMDFFForceField(alkane)
    assert ff.tuning("fp64")["variant"] == -1
    x = geoms(alkane, 2048, 0.1, 9)
    e, g = ff.egrad(x, "fp64")          # first launch of >= 2048 beads: tunes
    t = ff.tuning("fp64")
    e2, g2 = ff.egrad(x, "fp64")        # the chosen variant
    ff.close()
    assert t["variant"] in (0, 1, 2) and min(t["ms"]) > 0.0
    eo, go = orc.egrad("qmdff", x)
    assert rel_err(e2, eo) <= 1e-12 and rel_err(g2, go) <= 1e-12
    assert rel_err(e, eo) <= 1e-12 and rel_err(g, go) <= 1e-12


def test_egrad_mixed_error(gpu_ff, alkane):
    x = geoms(alkane, 256, 0.1, 2)
    e, g = gpu_ff.egrad(x, "mixed")
    e64, g64 = gpu_ff.egrad(x, "fp64")
    err = np.sqrt(np.sum((g - g64) ** 2) / np.sum(g64 ** 2))
    assert err <= 2e-6
    assert rel_err(e, e64) <= 2e-6


def test_mixed_force_error_within_1e7_on_thermal_ring_polymers(gpu_ff, alkane):
    """The mixed form's force error, max |g_mixed - g_fp64| / max |g_fp64|, on
    ring polymers from a thermal FP64 run (300 K, 64 beads): <= 1e-7."""
    eng, _ = make_pair(gpu_ff, alkane, 64, 8, "andersen", andersen_step=10)
    eng.init_positions(alkane.xyz, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    eng.run(150)
    q, _, _, _, st = eng.get_state()
    eng.close()
    assert not st.any()
    x = q.reshape(-1, alkane.n, 3)
    e64, g64 = gpu_ff.egrad(x, "fp64")
    em, gm = gpu_ff.egrad(x, "mixed")
    assert np.max(np.abs(gm - g64)) / np.max(np.abs(g64)) <= 1e-7
    assert np.max(np.abs(em - e64)) / np.max(np.abs(e64)) <= 2e-7


def test_egrad_zahn_matches_oracle(alkane, require_gpu):
    ff = QMDFFForceField(alkane, coul_cut=10.0, zahn=True)
    orc.set_qmdff(alkane, Q.ElementTables.caracal(), coul_cut=10.0, zahn=True)
    x = geoms(alkane, 64, 0.1, 3)
    e, g = ff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    ff.close()
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def make_pair(gpu_ff, alkane, nbeads, ntraj, thermostat, andersen_step=5, precision="fp64",
              transrot=True, kelvin=300.0, dt_fs=0.5, seed=77, nm_mode=0):
    mass = qmdff_config().mass
    beta = beta_from_kelvin(kelvin)
    dt = dt_fs_to_au(dt_fs)
    tau0 = dt_fs_to_au(100.0)
    eng = RPMDEngine(gpu_ff, mass, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0_au=tau0, transrot=transrot,
                     precision=precision, seed=seed, nm_mode=nm_mode)
    cfg = orc.Config("qmdff", mass, nbeads, dt, beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0=tau0, transrot=transrot, seed=seed,
                     nm_mode=nm_mode)
    return eng, cfg


def start(eng, cfg, alkane, sigma=0.02):
    eng.init_positions(alkane.xyz, sigma)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, eng.ntraj, alkane.xyz, sigma)
    p = orc.init_momenta(cfg, eng.ntraj)
    f, e = orc.init_forces(cfg, q)
    return q, p, f, e


def test_init_matches_oracle(gpu_ff, alkane):
    eng, cfg = make_pair(gpu_ff, alkane, 8, 2, "andersen")
    q, p, f, e = start(eng, cfg, alkane)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    assert rel_err(qg, q) <= 1e-15
    assert rel_err(pg, p) <= 1e-14
    assert rel_err(fg, f) <= 1e-12
    assert rel_err(eg, e) <= 1e-12


@pytest.mark.parametrize("thermostat", ["andersen", "pile", "none"])
@pytest.mark.parametrize("nbeads", [1, 2, 3, 4, 6, 8, 16, 32, 64])
def test_single_step_matches_oracle(gpu_ff, alkane, thermostat, nbeads):
    eng, cfg = make_pair(gpu_ff, alkane, nbeads, 2, thermostat, andersen_step=1)
    q, p, f, e = start(eng, cfg, alkane)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 1)
    assert rel_err(qg, qo) <= 1e-12
    assert rel_err(pg, po) <= 1e-12
    assert rel_err(fg, fo) <= 1e-12
    assert rel_err(eg, eo) <= 1e-12
    assert not st.any() and not sto.any()


@pytest.mark.parametrize("thermostat,nbeads", [("andersen", 8), ("pile", 6), ("none", 4)])
def test_orthonormal_modes_step_matches_oracle(gpu_ff, alkane, thermostat, nbeads):
    """nm_mode 1 on the graph path (circulant drift of split_drift_kernel)."""
    eng, cfg = make_pair(gpu_ff, alkane, nbeads, 2, thermostat, andersen_step=3, nm_mode=1)
    q, p, f, e = start(eng, cfg, alkane)
    eng.run(5)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 5)
    assert not st.any() and not sto.any()
    assert rel_err(qg, qo) <= 1e-11 and rel_err(pg, po) <= 1e-11 and rel_err(eg, eo) <= 1e-11


@pytest.mark.parametrize("thermostat,nbeads", [("andersen", 8), ("pile", 6), ("none", 4), ("andersen", 64),
                                               ("none", 32)])
def test_trajectory_matches_oracle(gpu_ff, alkane, thermostat, nbeads):
    """100 steps (two runs) against the oracle; P = 32 and 64 take the fast
    cosine-transform drift."""
    eng, cfg = make_pair(gpu_ff, alkane, nbeads, 2, thermostat, andersen_step=5)
    q, p, f, e = start(eng, cfg, alkane)
    eng.run(37)
    eng.run(63)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 100)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9
    assert rel_err(eg, eo) <= 1e-9


def test_step_host_matches_run(gpu_ff, alkane):
    eng, cfg = make_pair(gpu_ff, alkane, 8, 3, "andersen", andersen_step=2)
    start(eng, cfg, alkane)
    q, p, f, e, st = eng.get_state()
    eng.step_host(q, p, f)
    eng.step_host(q, p, f)
    eng2, _ = make_pair(gpu_ff, alkane, 8, 3, "andersen", andersen_step=2)
    start(eng2, cfg, alkane)
    eng2.run(2)
    q2, p2, f2, e2, st2 = eng2.get_state()
    eng.close()
    eng2.close()
    assert rel_err(q, q2) <= 1e-15
    assert rel_err(p, p2) <= 1e-15


@pytest.mark.parametrize("thermostat", ["andersen", "nhc", "pile"])
def test_step_host_pipelined_groups_match_run(gpu_ff, alkane, thermostat):
    # 384 trajectories x 8 beads x 62 atoms: 4.6 MB per state array, two
    # trajectory groups in the pipelined host step (step kernels on offset
    # trajectory ranges, noise keys of the global trajectory index)
    engs = []
    for _ in range(2):
        eng = RPMDEngine(gpu_ff, qmdff_config().mass, 8, 384, dt_fs_to_au(0.5), beta=beta_from_kelvin(300.0),
                         thermostat=thermostat, andersen_step=2, pile_tau0_au=dt_fs_to_au(100.0),
                         nose_q_au=nose_q_to_au(20.0, 0.5), seed=77)
        eng.init_positions(alkane.xyz, 0.02)
        eng.init_momenta()
        # twice: a first launch of >= 2048 beads may run the force kernel's
        # autotuner, whose register variants can differ in the last bit
        eng.compute_forces()
        eng.compute_forces()
        engs.append(eng)
    a, b = engs
    q, p, f, e, _ = a.get_state()
    for _ in range(3):
        a.step_host(q, p, f, e)
    # drift, forces, kick, moments, solve, transrot apply (+ 2 NHC)
    per_group = 6 + (2 if thermostat == "nhc" else 0)
    assert a.launch_info()["launches"] == 2 * per_group + 1
    b.run(3)
    qb, pb, fb, eb, st = b.get_state()
    a.close()
    b.close()
    assert not st.any()
    assert rel_err(q, qb) <= 1e-15 and rel_err(p, pb) <= 1e-15
    assert rel_err(f, fb) <= 1e-15 and rel_err(e, eb) <= 1e-15


def test_mixed_engine_tracks_fp64(gpu_ff, alkane):
    a, cfg = make_pair(gpu_ff, alkane, 16, 4, "none", precision="fp64")
    b, _ = make_pair(gpu_ff, alkane, 16, 4, "none", precision="mixed")
    for eng in (a, b):
        start(eng, cfg, alkane)
        eng.run(10)
    qa, pa, fa, ea, _ = a.get_state()
    qb, pb, fb, eb, _ = b.get_state()
    a.close()
    b.close()
    assert rel_err(qb, qa) <= 1e-8
    assert rel_err(fb, fa) <= 1e-5


def test_recross_unsupported_on_qmdff(gpu_ff, alkane):
    from caracal_gb300 import CaracalError
    eng, _ = make_pair(gpu_ff, alkane, 4, 2, "none")
    with pytest.raises(CaracalError):
        eng.set_recross([1], [2], (1, 2), (1, 3), 2.0, 2.0, 10.0, max_steps=4)
    eng.close()


@pytest.mark.parametrize("system,tol", [("water_dimer", 1e-12), ("chloromethane_ammonia", 1e-9)])
def test_hbond_terms_match_oracle(require_gpu, system, tol):
    # halogen bonds carry Caracal's difference-quotient gradient (step 1e-6):
    # rounding differences of the two energies are amplified by 5e5, so their
    # parity bound is 1e-9; hydrogen bonds are analytic (1e-12)
    ff = getattr(Q, system)()
    tab = Q.ElementTables.caracal()
    orc.set_qmdff(ff, tab)
    gff = QMDFFForceField(ff, tab)
    assert gff.schedule_info()["batches"][4] == 1
    x = ff.xyz[None] + np.random.default_rng(4).normal(0, 0.03, (64,) + ff.xyz.shape)
    e, g = gff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    em, gm = gff.egrad(x, "mixed")
    gff.close()
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= tol
    assert np.sqrt(np.sum((gm - g) ** 2) / np.sum(g ** 2)) <= 5e-6


@pytest.mark.parametrize("which", ["alkane", "water_dimer", "chloromethane_ammonia"])
def test_qmdff_load_matches_python_reader(require_gpu, tmp_path, which):
    """The library's own .qmdff reader (cr_qmdff_load) gives the force field
    the Python reader builds: identical energies and gradients."""
    ff = Q.alkane(nc=5) if which == "alkane" else getattr(Q, which)()
    path = tmp_path / "x.qmdff"
    Q.write_qmdff(ff, path)
    a = QMDFFForceField.load(path, e_zero=-0.3)
    ref = Q.read_qmdff(path)
    ref.e_zero = -0.3
    b = QMDFFForceField(ref)
    x = ff.xyz[None] + np.random.default_rng(3).normal(0, 0.05, (8,) + ff.xyz.shape)
    for prec in ("fp64", "mixed"):
        ea, ga = a.egrad(x, prec)
        eb, gb = b.egrad(x, prec)
        assert np.array_equal(ea, eb) and np.array_equal(ga, gb)
    a.close()
    b.close()


# ---- the reference's own QMDFF inputs -------------------------------------
import os  # noqa: E402

from conftest import ROOT  # noqa: E402

REF = os.path.join(ROOT, "tests", "golden", "reference")
GLUT = os.path.join(REF, "dynamic", "glutathione")
EVB = os.path.join(REF, "evbopt", "dE-EVB")
GLUT_ESHIFT = -1403.0282384116763   # ESHIFT of examples/dynamic/glutathione/glutathione.key


@pytest.fixture(scope="module")
def glutathione():
    ff = Q.read_qmdff(os.path.join(GLUT, "glutathione.qmdff"))
    ff.e_zero = GLUT_ESHIFT
    return ff


def test_glutathione_egrad_matches_oracle(require_gpu, glutathione):
    """examples/dynamic/glutathione/glutathione.qmdff with Caracal's set-up
    (D3 pair C6 from the coordination numbers of its geometry, 148 H-bond
    terms): the device force field against the oracle; the library's own
    reader (cr_qmdff_load_d3) against the Python reader."""
    ff = glutathione
    tab = Q.ElementTables.caracal()
    orc.set_qmdff(ff, tab)
    gff = QMDFFForceField(ff, tab)
    x = ff.xyz[None] + np.random.default_rng(21).normal(0, 0.05, (64,) + ff.xyz.shape)
    x[0] = ff.xyz
    e, g = gff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    assert rel_err(e, eo) <= 1e-12
    # Per geometry, the gradient agrees to 1e-12 of max|g| unless Caracal's
    # formula is itself ill-conditioned there: a torsion whose dihedral sits
    # next to 0 or pi (the carboxyl H-O-C-O of this file has phi0 = 0.004 rad)
    # goes through acos, whose derivative amplifies one rounding of the
    # cosine.  The oracle's own change under a one-ulp perturbation of the
    # coordinates measures that amplification; such geometries are held to
    # four times it instead, and there may be only a few of them.
    rng = np.random.default_rng(4)
    sens = np.zeros(len(x))
    for _ in range(2):
        _, gp = orc.egrad("qmdff", x * (1.0 + rng.uniform(-1.0, 1.0, x.shape) * 2.2e-16))
        sens = np.maximum(sens, np.abs(gp - go).max(axis=(1, 2)))
    scale = np.abs(go).max()
    err = np.abs(g - go).max(axis=(1, 2)) / scale
    bound = np.maximum(1e-12, 4.0 * sens / scale)
    assert np.all(err <= bound), (err.max(), np.argmax(err / bound))
    assert np.count_nonzero(bound > 1e-12) <= 4
    em, gm = gff.egrad(x, "mixed")
    assert rel_err(gm, g) <= 1e-6
    ld = QMDFFForceField.load(os.path.join(GLUT, "glutathione.qmdff"), e_zero=GLUT_ESHIFT)
    el, gl = ld.egrad(x, "fp64")
    ld.close()
    gff.close()
    assert np.array_equal(el, e) and np.array_equal(gl, g)


def test_glutathione_nvt_100_steps_matches_oracle(require_gpu, glutathione):
    """glutathione.key's dynamics (1 bead, NVT 500 K, Nose-Hoover chain with
    the default NOSE_DAMP 100, dt 1 fs) from start.xyz: 100 steps of 4
    trajectories against the oracle."""
    from caracal_gb300 import keyfile as K
    from caracal_gb300.units import angstrom_to_bohr, mass_au
    ff = glutathione
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    gff = QMDFFForceField(ff)
    sym, xyz = K.read_xyz(os.path.join(GLUT, "start.xyz"))
    q0 = angstrom_to_bohr(np.array(xyz))
    mass = np.array([mass_au(s) for s in sym])
    dt, beta, nq = dt_fs_to_au(1.0), beta_from_kelvin(500.0), nose_q_to_au(100.0, 1.0)
    eng = RPMDEngine(gff, mass, 1, 4, dt, beta=beta, thermostat="nhc", nose_q_au=nq, seed=5)
    eng.init_positions(q0, 0.0)
    eng.init_momenta()
    eng.compute_forces()
    cfg = orc.Config("qmdff", mass, 1, dt, beta, thermostat="nhc", nose_q=nq, seed=5)
    q = orc.init_positions(cfg, 4, q0, 0.0)
    p = orc.init_momenta(cfg, 4)
    f, _ = orc.init_forces(cfg, q)
    eng.run(60)
    eng.run(40)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    gff.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 100)
    assert not st.any() and not sto.any()
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9
    assert rel_err(eg, eo) <= 1e-9


def test_reference_de_evb_example_evaluates(require_gpu):
    """examples/evbopt/dE-EVB: both QMDFFs (with the ESHIFT energies of
    evbopt.key) on every reference structure, and the SP-coupling fit
    residuals and fdjac2 Jacobian at a starting guess, device against
    oracle."""
    from caracal_gb300.engine import evb_fit
    e1s, e2s = -272.22659664700754, -272.16798367875066
    ff1 = Q.read_qmdff(os.path.join(EVB, "min1.qmdff"))
    ff2 = Q.read_qmdff(os.path.join(EVB, "min2.qmdff"))
    ff1.e_zero, ff2.e_zero = e1s, e2s
    x = Q.read_xyz_frames(os.path.join(EVB, "struc.xyz"))
    eref = np.loadtxt(os.path.join(EVB, "ref.dat"))
    tab = Q.ElementTables.caracal()
    es = []
    for ff in (ff1, ff2):
        orc.set_qmdff(ff, tab)
        gff = QMDFFForceField(ff, tab)
        e, _ = gff.egrad(x, "fp64")
        eo, _ = orc.egrad("qmdff", x)
        gff.close()
        assert rel_err(e, eo) <= 1e-12
        es.append(e)
    par = np.array([0.02, 0.5, 0.01, 0.1])           # SP basis: a, b, c, d
    fv, fj = evb_fit("sp", par, es[0], es[1], eref)
    fvo, fjo = orc.evb_fit("sp", par, es[0], es[1], eref)
    assert rel_err(fv, fvo) <= 1e-12
    # fdjac2 divides a residual difference by h = sqrt(epsmch) |x_j| ~ 1.5e-8
    # |x_j|, so a one-ulp difference between the device's and the oracle's
    # residuals (exp and sqrt of two libraries) shows up about 1e8 times
    # larger in the Jacobian: ~1e-8 relative is the formula's own floor.
    assert rel_err(fj, fjo) <= 2e-7
    assert np.all(np.isfinite(fv)) and fv.shape == eref.shape


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("mixed", 1e-6)])
def test_call_site_pieces_sum_to_egrad(require_gpu, glutathione, prec, tol):
    """cr_qmdff_eg (overwrite) + cr_qmdff_nonb + cr_qmdff_hb (accumulate) +
    E_zero, the pieces of Caracal's call site (src/gradient.f90:341-358),
    against the fused cr_qmdff_egrad."""
    gff = QMDFFForceField(glutathione)
    x = glutathione.xyz[None] + np.random.default_rng(9).normal(0, 0.05, (16,) + glutathione.xyz.shape)
    e = np.full(16, np.nan)
    g = np.full_like(x, np.nan)
    gff.ff_eg(x, e, g, prec)
    e_cov = e.copy()
    gff.ff_nonb(x, e, g, prec)
    gff.ff_hb(x, e, g, prec)
    ef, gf = gff.egrad(x, prec)
    gff.close()
    assert np.all(np.isfinite(e)) and np.all(np.isfinite(g))
    assert not np.allclose(e_cov, e)                       # the non-bonded pieces add
    # the fused entry adds E_zero (-1403 Eh) inside, so its result carries
    # that number's rounding (2.3e-13 Eh per ulp); beyond it the pieces agree
    # to tol of the force-field energy
    ez = glutathione.e_zero
    assert np.abs(e + ez - ef).max() <= tol * np.abs(e).max() + 4.0 * np.spacing(abs(ez))
    assert rel_err(g, gf) <= tol


@pytest.mark.parametrize("zahn", [False, True])
def test_periodic_box_matches_oracle(require_gpu, glutathione, zahn):
    """PERIODIC: glutathione (about 15 A long) in a 24 A box with a 6 A
    dispersion cutoff (Coulomb at half the box, or the Zahn form at 10 A), so
    long intramolecular pairs take their nearest image: the device against
    the oracle (Caracal's box_image at its call sites); the same geometries
    with atoms moved by box edges: the device unchanged (every vector is
    imaged; Caracal's raw-coordinate dihedrals would not be)."""
    ff = glutathione
    tab = Q.ElementTables.caracal()
    box = np.array([24.0, 24.0, 24.0])
    orc.set_qmdff(ff, tab, zahn=zahn)
    oc = orc.set_qmdff_periodic(box, 50.0, 6.0)
    gff = QMDFFForceField(ff, tab, zahn=zahn)
    dc = gff.set_periodic(box, 50.0, 6.0)
    assert np.allclose(dc, oc, rtol=0, atol=0)
    x = ff.xyz[None] + np.random.default_rng(8).normal(0, 0.05, (16,) + ff.xyz.shape)
    e, g = gff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    assert rel_err(e, eo) <= 1e-12 and rel_err(g, go) <= 1e-11
    gff.set_periodic(None)
    en, _ = gff.egrad(x, "fp64")
    assert np.abs(en - e).min() > 1e-6                 # the cutoffs and images act
    gff.set_periodic(box, 50.0, 6.0)
    L = box / 0.52917721092
    xw = x.copy()
    shift = np.random.default_rng(9).integers(-1, 2, xw.shape[:2] + (3,))
    shift[:, 0] = 0                                    # atom 0 stays
    xw += shift * L
    ew, gw = gff.egrad(xw, "fp64")
    assert rel_err(ew, e) <= 1e-12 and rel_err(gw, g) <= 1e-11
    em, gm = gff.egrad(xw, "mixed")
    assert rel_err(gm, g) <= 1e-6 and rel_err(em, e) <= 1e-6
    gff.close()
    orc.set_qmdff(ff, tab)
