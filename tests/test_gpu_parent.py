"""GPU: the constrained parent (SHAKE/RATTLE on the BIMOLEC dividing
surface, src/constrain_q.f90, src/constrain_p.f90) through the engine's
graph path against the oracle: one step <= 1e-12, 30 steps <= 1e-9."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300.workloads import ch4h_config, ch4h_recross_definition
from conftest import rel_err
from oracle import oracle as orc
from test_oracle_parent import _xd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("thermostat,nbeads", [("andersen", 8), ("none", 4), ("pile", 16)])
def test_parent_matches_oracle(require_gpu, thermostat, nbeads):
    wl = ch4h_config(ntraj=3, nbeads=nbeads)
    rd = ch4h_recross_definition(wl.q0)
    xd = _xd(rd)
    eng = RPMDEngine("ch4h", wl.mass, nbeads, 3, wl.dt_au, beta=wl.beta, thermostat=thermostat,
                     andersen_step=7, pile_tau0_au=wl.pile_tau0_au, transrot=False, seed=21)
    cfg = orc.Config("ch4h", wl.mass, nbeads, wl.dt_au, wl.beta, thermostat=thermostat, andersen_step=7,
                     pile_tau0=wl.pile_tau0_au, transrot=False, seed=21)
    eng.init_positions(wl.q0, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    eng.set_parent(**rd)
    q = orc.init_positions(cfg, 3, wl.q0, 0.02)
    p = orc.init_momenta(cfg, 3)
    f, _ = orc.init_forces(cfg, q)
    eng.run(1)
    q1, p1, f1, e1, st = eng.get_state()
    qo, po, fo, eo, so, dxi = orc.run_parent(cfg, xd, q, p, f, 1)
    assert not st.any() and not so.any()
    assert rel_err(q1, qo) <= 1e-12 and rel_err(p1, po) <= 1e-12 and rel_err(e1, eo) <= 1e-12
    eng.run(29)
    q30, p30, _, e30, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, so, dxi = orc.run_parent(cfg, xd, qo, po, fo, 29, istep0=1, dxi=dxi)
    assert rel_err(q30, qo) <= 1e-9 and rel_err(p30, po) <= 1e-9
    for t in range(3):
        assert abs(orc.calc_xi(xd, q30[t].mean(axis=0), wl.mass)[0]) < 1e-8
