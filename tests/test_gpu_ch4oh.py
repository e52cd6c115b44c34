"""GPU: CH4 + OH (egrad_ch4oh) through the C-ABI against the oracle.

Plain FP64 form: forces <= 1e-12, one NVE step <= 1e-12, 100 steps <= 1e-9
(norm-wise relative); mixed form: force error against FP64 <= 1.5e-7, the
energy (summed in FP32) <= 1.5e-6.
"""
import ctypes as C

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from caracal_gb300 import RPMDEngine, egrad_ch4oh
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
from caracal_gb300.workloads import ch4oh_geometry
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MASS = [mass_au(s) for s in ("H", "C", "H", "H", "H", "O", "H")]


def pair(nbeads, ntraj, thermostat="none", kelvin=500.0, precision="fp64", transrot=False,
         andersen_step=20, seed=7):
    beta = beta_from_kelvin(kelvin)
    dt = dt_fs_to_au(0.1)
    tau0 = dt_fs_to_au(100.0)
    eng = RPMDEngine("ch4oh", MASS, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0_au=tau0, transrot=transrot,
                     precision=precision, seed=seed)
    cfg = orc.Config("ch4oh", MASS, nbeads, dt, beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0=tau0, transrot=transrot, seed=seed)
    return eng, cfg


def start(eng, cfg, sigma=0.02):
    q0 = ch4oh_geometry()
    eng.init_positions(q0, sigma)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, eng.ntraj, q0, sigma)
    p = orc.init_momenta(cfg, eng.ntraj)
    f, e = orc.init_forces(cfg, q)
    return q, p, f, e


def test_egrad_ch4oh_matches_oracle(require_gpu):
    rng = np.random.default_rng(5)
    q = ch4oh_geometry()[None] + rng.normal(0, 0.1, (2048, 7, 3))
    V, g = egrad_ch4oh(q)
    Vo, go = orc.egrad("ch4oh", q)
    assert rel_err(V, Vo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def test_initialize_ch4oh_and_wrong_natoms(require_gpu):
    lib = L.lib()
    assert lib.cr_initialize_ch4oh() == 0
    q = np.zeros((1, 3, 3))
    info = C.c_int(0)
    assert lib.cr_egrad_ch4oh(L.dptr(q), 3, 1, L.dptr(np.zeros(1)), L.dptr(q), C.byref(info)) == L.CR_ERR_ARG


@pytest.mark.parametrize("nbeads", [1, 8, 32])
@pytest.mark.parametrize("thermostat,transrot", [("none", False), ("andersen", True), ("pile", True)])
def test_ch4oh_single_step(require_gpu, nbeads, thermostat, transrot):
    eng, cfg = pair(nbeads, 4, thermostat=thermostat, transrot=transrot, andersen_step=1)
    q, p, f, e = start(eng, cfg)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st.any()
    assert rel_err(qg, qo) <= 1e-12
    assert rel_err(pg, po) <= 1e-12
    assert rel_err(fg, fo) <= 1e-12
    assert rel_err(eg, eo) <= 1e-12


def test_ch4oh_100_steps_nve(require_gpu):
    eng, cfg = pair(32, 6)
    q, p, f, e = start(eng, cfg)
    eng.run(100)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 100)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9
    assert rel_err(eg, eo) <= 1e-9


def test_ch4oh_mixed_force_error(require_gpu):
    rng = np.random.default_rng(6)
    q = ch4oh_geometry()[None] + rng.normal(0, 0.1, (256 * 32, 7, 3))
    q = q.reshape(256, 32, 7, 3)
    e64, _ = pair(32, 256, precision="fp64")
    e32, _ = pair(32, 256, precision="mixed")
    z = np.zeros_like(q)
    e64.set_state(q, z)
    e32.set_state(q, z)
    _, _, f64, v64, _ = e64.get_state()
    _, _, f32, v32, _ = e32.get_state()
    err = rel_err(f32, f64)
    print(f"CH4OH mixed-form force error {err:.3e}, energy error {rel_err(v32, v64):.3e}")
    # the O-H Morse, the stretches and the bends in float pairs: 3.6e-8 on
    # the host restatement of the mixed form
    assert err < 1.5e-7 and rel_err(v32, v64) < 1.5e-6
