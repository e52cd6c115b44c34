"""GPU: Caracal's ANA_BRH2 surface (Br + H2, src/egrad_brh2.f) through the
C-ABI and in the persistent step kernel against the oracle.  Tolerances
(norm-wise relative): energies and gradients <= 1e-12; one step <= 1e-12;
100 steps <= 1e-9.  The surface has one (FP64) form: the mixed engine's
forces equal the plain engine's."""
import ctypes as C

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from caracal_gb300 import RPMDEngine, egrad_brh2
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MASS = [mass_au(s) for s in ("H", "Br", "H")]
Q0 = np.array([[0.0, 0.0, -3.6], [0.0, 0.0, 2.673], [0.0, 0.2, 0.0]])   # H ... H-Br, bohr


def test_egrad_matches_oracle(require_gpu):
    rng = np.random.default_rng(3)
    q = Q0[None] + rng.normal(0, 0.15, (4096, 3, 3))
    V, g = egrad_brh2(q)
    Vo, go = orc.egrad("brh2", q)
    assert rel_err(V, Vo) <= 1e-12 and rel_err(g, go) <= 1e-12
    lib = L.lib()
    assert lib.cr_initialize_brh2() == 0
    info = C.c_int(0)
    z = np.zeros((1, 4, 3))
    assert lib.cr_egrad_brh2(L.dptr(z), 4, 1, L.dptr(np.zeros(1)), L.dptr(z), C.byref(info)) == L.CR_ERR_ARG


def pair(nbeads, ntraj, thermostat, precision="fp64", seed=9):
    beta, dt, tau0 = beta_from_kelvin(300.0), dt_fs_to_au(0.1), dt_fs_to_au(100.0)
    eng = RPMDEngine("brh2", MASS, nbeads, ntraj, dt, beta=beta, thermostat=thermostat, andersen_step=1,
                     pile_tau0_au=tau0, transrot=True, precision=precision, seed=seed)
    cfg = orc.Config("brh2", MASS, nbeads, dt, beta, thermostat=thermostat, andersen_step=1, pile_tau0=tau0,
                     transrot=True, seed=seed)
    eng.init_positions(Q0, 0.05)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, ntraj, Q0, 0.05)
    p = orc.init_momenta(cfg, ntraj)
    f, _ = orc.init_forces(cfg, q)
    return eng, cfg, q, p, f


@pytest.mark.parametrize("nbeads", [1, 8, 16])
@pytest.mark.parametrize("thermostat", ["none", "andersen", "pile"])
def test_single_step(require_gpu, nbeads, thermostat):
    eng, cfg, q, p, f = pair(nbeads, 8, thermostat)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    eng.close()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st.any()
    assert rel_err(qg, qo) <= 1e-12 and rel_err(pg, po) <= 1e-12
    assert rel_err(fg, fo) <= 1e-12 and rel_err(eg, eo) <= 1e-12


def test_100_steps_and_mixed_form(require_gpu):
    eng, cfg, q, p, f = pair(16, 32, "none")
    eng.run(100)
    qg, pg, _, eg, st = eng.get_state()
    eng.close()
    qo, po, _, eo, _ = orc.run(cfg, q, p, f, 100)
    assert not st.any()
    assert rel_err(qg, qo) <= 1e-9 and rel_err(pg, po) <= 1e-9 and rel_err(eg, eo) <= 1e-9
    e64, *_ = pair(16, 32, "none")
    emx, *_ = pair(16, 32, "none", precision="mixed")
    _, _, f64, v64, _ = e64.get_state()
    _, _, fmx, vmx, _ = emx.get_state()
    e64.close()
    emx.close()
    assert np.array_equal(fmx, f64) and np.array_equal(vmx, v64)
