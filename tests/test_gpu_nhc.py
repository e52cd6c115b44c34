"""GPU: the Nose-Hoover chain thermostat (src/nhc.f90, applied before the
first and after the second half kick, src/verlet.f90:186-208, 1085-1106) in
both step paths against the oracle.  Plain FP64 tolerances: one step
<= 1e-12, 40 steps <= 1e-9 (norm-wise relative)."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300 import qmdff as Q
from caracal_gb300.engine import QMDFFForceField
from caracal_gb300.units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from caracal_gb300.workloads import h3_collinear, qmdff_config
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

DT_FS = 0.1


def pair_h3(nbeads, ntraj, nose_steps=20.0, kelvin=300.0, seed=11):
    mass = [mass_au("H")] * 3
    beta, dt = beta_from_kelvin(kelvin), dt_fs_to_au(DT_FS)
    nq = nose_q_to_au(nose_steps, DT_FS)
    eng = RPMDEngine("h3", mass, nbeads, ntraj, dt, beta=beta, thermostat="nhc", nose_q_au=nq, seed=seed)
    cfg = orc.Config("h3", mass, nbeads, dt, beta, thermostat="nhc", nose_q=nq, seed=seed)
    sigma = float(angstrom_to_bohr(0.01))
    eng.init_positions(h3_collinear(), sigma)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, ntraj, h3_collinear(), sigma)
    p = orc.init_momenta(cfg, ntraj)
    f, _ = orc.init_forces(cfg, q)
    return eng, cfg, q, p, f


@pytest.mark.parametrize("nbeads", [1, 3, 16, 32, 64])
def test_nhc_single_step_h3(require_gpu, nbeads):
    eng, cfg, q, p, f = pair_h3(nbeads, 6)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 1)
    assert rel_err(qg, qo) <= 1e-12
    assert rel_err(pg, po) <= 1e-12
    assert rel_err(eg, eo) <= 1e-12


def test_nhc_trajectory_h3_state_carries_over(require_gpu):
    eng, cfg, q, p, f = pair_h3(16, 8, nose_steps=5.0)
    eng.run(25)
    eng.run(15)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 40)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9


def test_nhc_needs_nose_q(require_gpu):
    from caracal_gb300 import CaracalError
    with pytest.raises(CaracalError):
        RPMDEngine("h3", [mass_au("H")] * 3, 4, 2, dt_fs_to_au(DT_FS), beta=beta_from_kelvin(300.0),
                   thermostat="nhc", nose_q_au=0.0)


@pytest.mark.parametrize("nbeads", [4, 8])
def test_nhc_qmdff_path(require_gpu, nbeads):
    ff = Q.alkane()
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    gff = QMDFFForceField(ff)
    mass = qmdff_config().mass
    dt_fs = 0.5
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(dt_fs)
    nq = nose_q_to_au(10.0, dt_fs)
    eng = RPMDEngine(gff, mass, nbeads, 2, dt, beta=beta, thermostat="nhc", nose_q_au=nq, seed=5)
    cfg = orc.Config("qmdff", mass, nbeads, dt, beta, thermostat="nhc", nose_q=nq, seed=5)
    eng.init_positions(ff.xyz, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, 2, ff.xyz, 0.02)
    p = orc.init_momenta(cfg, 2)
    f, _ = orc.init_forces(cfg, q)
    eng.run(1)
    q1, p1, _, e1, _ = eng.get_state()
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 1)
    assert rel_err(q1, qo) <= 1e-12
    assert rel_err(p1, po) <= 1e-12
    eng.run(9)
    q10, p10, _, _, _ = eng.get_state()
    eng.close()
    gff.close()
    vnh = np.zeros((2, 4))
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 10, vnh=vnh)
    assert rel_err(q10, qo) <= 1e-9
    assert rel_err(p10, po) <= 1e-9
