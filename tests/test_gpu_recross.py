"""GPU: recrossing children (calc_rate part 4) through the C-ABI against the oracle.

The child states after n steps match the oracle to <= 1e-9 (FP64 form), the
flux weights vs/fs to <= 1e-12, and kappa(t) = num(t)/denom to <= 1e-9
(a child whose xi sits within rounding of 0 could flip a side; the seeds used
here have none).
"""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300.workloads import ch4h_config, ch4h_recross_definition
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def run_pair(ntraj, nbeads, nsteps, precision="fp64"):
    wl = ch4h_config(ntraj=ntraj, nbeads=nbeads)
    rd = ch4h_recross_definition(wl.q0)
    eng = RPMDEngine("ch4h", wl.mass, nbeads, ntraj, wl.dt_au, beta=wl.beta, thermostat="none",
                     transrot=False, precision=precision, seed=wl.seed)
    eng.set_recross(max_steps=nsteps, **rd)
    qpar = np.repeat(wl.q0[None], nbeads, axis=0)
    eng.init_children(qpar)
    eng.run(nsteps)
    num, den, w = eng.kappa(nsteps)
    q, p, f, e, st = eng.get_state()
    cfg = orc.Config("ch4h", wl.mass, nbeads, wl.dt_au, wl.beta, transrot=False, seed=wl.seed)
    xd = orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                        (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                        (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                        rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])
    onum, oden, ow, oq, op = orc.recross_children(cfg, xd, ntraj, qpar, nsteps, states=True)
    return (num, den, w, q, p, st), (onum, oden, ow, oq, op)


def test_children_match_oracle(require_gpu):
    (num, den, w, q, p, st), (onum, oden, ow, oq, op) = run_pair(16, 8, 80)
    assert not st.any()
    assert rel_err(w, ow) <= 1e-12
    assert abs(den - oden) <= 1e-12 * abs(oden)
    assert rel_err(q, oq) <= 1e-9 and rel_err(p, op) <= 1e-9
    assert rel_err(num / den, onum / oden) <= 1e-9


def test_pairs_have_opposite_momenta_and_one_positive_flux(require_gpu):
    (num, den, w, q, p, st), _ = run_pair(8, 4, 1)
    assert np.allclose(w[0::2], -w[1::2], rtol=0, atol=1e-14)
    assert den > 0 and np.isclose(den, np.abs(w).sum() / 2)


def test_run_beyond_capacity_is_rejected(require_gpu):
    wl = ch4h_config(ntraj=2, nbeads=4)
    eng = RPMDEngine("ch4h", wl.mass, 4, 2, wl.dt_au, beta=wl.beta, transrot=False, seed=1)
    eng.set_recross(max_steps=5, **ch4h_recross_definition(wl.q0))
    eng.init_children(np.repeat(wl.q0[None], 4, axis=0))
    assert eng.run(6, check=False) != 0
