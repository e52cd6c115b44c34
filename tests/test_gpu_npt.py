"""GPU: NpT with the Berendsen barostat on a periodic QMDFF against the
oracle.  The virial trace per bead (the reference's vir_ten terms, torsion,
inversion and halogen-bond forms included) <= 1e-11 of the largest |W| in
FP64, the mixed form <= 1e-5; engine steps with per-trajectory boxes:
one step <= 1e-12 (q, p, f, box, pressure), 100 steps <= 1e-9."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300 import qmdff as Q
from caracal_gb300.engine import QMDFFForceField
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

BOX_ANG = 18.0
BOHR = 0.52917721092


@pytest.fixture(scope="module")
def chain():
    return Q.alkane(nc=8)


@pytest.fixture
def periodic_pair(chain, require_gpu):
    tab = Q.ElementTables.caracal()
    orc.set_qmdff(chain, tab)
    orc.set_qmdff_periodic([BOX_ANG] * 3, 50.0, 8.0)
    ff = QMDFFForceField(chain, tab)
    ff.set_periodic([BOX_ANG] * 3, 50.0, 8.0)
    yield ff
    ff.close()
    orc.set_qmdff(chain, tab)


def test_virial_matches_oracle(periodic_pair, chain):
    rng = np.random.default_rng(4)
    x = chain.xyz[None] + rng.normal(0, 0.08, (64,) + chain.xyz.shape)
    box = (BOX_ANG / BOHR) * (1.0 + rng.uniform(-0.2, 0.2, (64, 3)))  # each bead its own box
    e, g, w = periodic_pair.egrad_virial(x, box, "fp64")
    eo, go, wo = orc.qmdff_egrad_virial(x, box)
    assert rel_err(e, eo) <= 1e-12 and rel_err(g, go) <= 1e-12
    assert np.abs(w - wo).max() <= 1e-11 * np.abs(wo).max()
    # the force field's own box where none is given
    e1, _, w1 = periodic_pair.egrad_virial(x[:4])
    eo1, _, wo1 = orc.qmdff_egrad_virial(x[:4])
    assert rel_err(e1, eo1) <= 1e-12 and np.abs(w1 - wo1).max() <= 1e-11 * np.abs(wo1).max()
    em, gm, wm = periodic_pair.egrad_virial(x, box, "mixed")
    assert np.abs(wm - wo).max() <= 1e-5 * np.abs(wo).max() and rel_err(gm, go) <= 1e-6


def make_npt(ff, chain, nbeads, ntraj, thermostat="andersen", seed=21, pressure=1.0, box=None,
             oracle_thermostat=None):
    mass = [mass_au("C" if z == 6 else "H") for z in chain.at]
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(0.5)
    eng = RPMDEngine(ff, mass, nbeads, ntraj, dt, beta=beta, thermostat=thermostat, andersen_step=5,
                     transrot=True, seed=seed, nose_q_au=nose_q_to_au(100.0, 0.5))
    cfg = orc.Config("qmdff", mass, nbeads, dt, beta, thermostat=oracle_thermostat or thermostat, andersen_step=5,
                     transrot=True, seed=seed)
    eng.set_npt(pressure, box)
    eng.init_positions(chain.xyz, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, ntraj, chain.xyz, 0.02)
    p = orc.init_momenta(cfg, ntraj)
    # mdinit's forces, each trajectory in its own box
    bx = np.broadcast_to(BOX_ANG / BOHR if box is None else box, (ntraj, 3))
    _, f, _ = orc.qmdff_egrad_virial(q.reshape(-1, chain.n, 3), np.repeat(bx, nbeads, axis=0))
    return eng, cfg, q, p, f.reshape(q.shape)


@pytest.mark.parametrize("nbeads", [1, 4, 16])
def test_npt_single_step(periodic_pair, chain, nbeads):
    T = 3
    box0 = np.full((T, 3), BOX_ANG / BOHR) * np.array([[1.0], [0.95], [1.1]])
    eng, cfg, q, p, f = make_npt(periodic_pair, chain, nbeads, T, box=box0, pressure=500.0)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    bg, pr, _ = eng.npt_state()
    eng.close()
    qo, po, fo, eo, so, bo, pro = orc.run_npt(cfg, q, p, f, 1, box0, 500.0)
    assert not st.any() and not so.any()
    assert rel_err(qg, qo) <= 1e-12 and rel_err(pg, po) <= 1e-12 and rel_err(fg, fo) <= 1e-12
    assert rel_err(eg, eo) <= 1e-12
    assert rel_err(bg, bo) <= 1e-14 and rel_err(pr, pro) <= 1e-11
    assert not np.allclose(bg, box0)              # the boxes moved, each its own way


@pytest.mark.parametrize("thermostat", ["andersen", "none", "nhc"])
def test_npt_100_steps(periodic_pair, chain, thermostat):
    """100 steps: q, p, boxes and pressures against the oracle.  With the
    Nose-Hoover chain the reference applies no thermostat under the
    Berendsen barostat: the trajectory equals the one without."""
    eng, cfg, q, p, f = make_npt(periodic_pair, chain, 8, 2, thermostat=thermostat,
                                 oracle_thermostat="none" if thermostat == "nhc" else None)
    eng.run(100)
    qg, pg, fg, eg, st = eng.get_state()
    bg, pr, _ = eng.npt_state()
    eng.close()
    qo, po, fo, eo, so, bo, pro = orc.run_npt(cfg, q, p, f, 100, BOX_ANG / BOHR, 1.0)
    assert not st.any()
    assert rel_err(qg, qo) <= 1e-9 and rel_err(pg, po) <= 1e-9 and rel_err(eg, eo) <= 1e-9
    assert rel_err(bg, bo) <= 1e-9 and rel_err(pr, pro) <= 1e-8


def test_npt_refused_without_periodic_qmdff(chain, require_gpu):
    tab = Q.ElementTables.caracal()
    ff = QMDFFForceField(chain, tab)
    mass = [mass_au("C" if z == 6 else "H") for z in chain.at]
    eng = RPMDEngine(ff, mass, 2, 1, dt_fs_to_au(0.5), beta=beta_from_kelvin(300.0), thermostat="andersen")
    with pytest.raises(Exception, match="periodic QMDFF"):
        eng.set_npt(1.0)
    eng.close()
    with pytest.raises(Exception, match="periodic"):
        ff.egrad_virial(chain.xyz[None])
    ff.close()


def test_npt_pressure_sum(periodic_pair, chain):
    """The running sum Caracal prints as press_avg (src/verlet.f90:1171-1210):
    the per-step pressures of 6 steps add up; a reset zeroes it."""
    eng, cfg, q, p, f = make_npt(periodic_pair, chain, 2, 2)
    steps = []
    for _ in range(6):
        eng.run(1)
        steps.append(eng.npt_state()[1])
    box, last, psum = eng.npt_state(reset_sum=True)
    assert np.allclose(psum, np.sum(steps, axis=0), rtol=1e-14, atol=0) and np.array_equal(last, steps[-1])
    assert not eng.npt_state()[2].any()
    eng.close()
