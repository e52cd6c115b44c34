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
    orc.set_qmdff(alkane, Q.ElementTables.d3_like())


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
    orc.set_qmdff(alkane, Q.ElementTables.d3_like(), coul_cut=10.0, zahn=True)
    x = geoms(alkane, 64, 0.1, 3)
    e, g = ff.egrad(x, "fp64")
    eo, go = orc.egrad("qmdff", x)
    ff.close()
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def make_pair(gpu_ff, alkane, nbeads, ntraj, thermostat, andersen_step=5, precision="fp64",
              transrot=True, kelvin=300.0, dt_fs=0.5, seed=77):
    mass = qmdff_config().mass
    beta = beta_from_kelvin(kelvin)
    dt = dt_fs_to_au(dt_fs)
    tau0 = dt_fs_to_au(100.0)
    eng = RPMDEngine(gpu_ff, mass, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0_au=tau0, transrot=transrot,
                     precision=precision, seed=seed)
    cfg = orc.Config("qmdff", mass, nbeads, dt, beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0=tau0, transrot=transrot, seed=seed)
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
@pytest.mark.parametrize("nbeads", [1, 2, 3, 4, 6, 8, 16, 64])
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
def test_trajectory_matches_oracle(gpu_ff, alkane, thermostat, nbeads):
    eng, cfg = make_pair(gpu_ff, alkane, nbeads, 2, thermostat, andersen_step=5)
    q, p, f, e = start(eng, cfg, alkane)
    eng.run(12)
    eng.run(8)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 20)
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
    tab = Q.ElementTables.d3_like()
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
