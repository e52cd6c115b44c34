"""CPU: the constrained parent of calc_rate (verlet with constrain = 1:
SHAKE, src/constrain_q.f90; RATTLE, src/constrain_p.f90) in the oracle."""
import numpy as np

from caracal_gb300.workloads import ch4h_config, ch4h_recross_definition
from oracle import oracle as orc


def _xd(rd):
    return orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                          (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                          (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                          rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])


def test_parent_stays_on_the_dividing_surface():
    wl = ch4h_config(ntraj=2, nbeads=8)
    xd = _xd(ch4h_recross_definition(wl.q0))
    cfg = orc.Config("ch4h", wl.mass, 8, wl.dt_au, wl.beta, thermostat="andersen", andersen_step=1000,
                     transrot=False, seed=3)
    q = orc.init_positions(cfg, 2, wl.q0, 0.02)
    p = orc.init_momenta(cfg, 2)
    f, _ = orc.init_forces(cfg, q)
    q1, p1, f1, e1, st, dxi = orc.run_parent(cfg, xd, q, p, f, 40)
    assert not st.any()
    for t in range(2):
        xi, dx = orc.calc_xi(xd, q1[t].mean(axis=0), wl.mass)
        assert abs(xi) < 1e-9
        # RATTLE (no Andersen resample in these steps): the centroid momentum
        # along the stored dxi vanishes
        v = sum(float(np.sum(dxi[t].reshape(6, 3) * p1[t, k] / wl.mass[:, None])) for k in range(8))
        assert abs(v) < 1e-10 * np.abs(p1[t]).max()
