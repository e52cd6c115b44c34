"""GPU: CH4 + OH (egrad_ch4oh) and GeH4 + OH (egrad_geh4oh, the same surface
code with its own constants) through the C-ABI against the oracle.

Plain FP64 form: forces <= 1e-12, one NVE step <= 1e-12, 100 steps <= 1e-9
(norm-wise relative); mixed form: force error against FP64 <= 1.5e-7, the
energy (summed in FP32) <= 1.5e-6.
"""
import ctypes as C

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from caracal_gb300 import RPMDEngine, egrad_ch4oh, egrad_geh4oh
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
from caracal_gb300.workloads import ch4oh_geometry, geh4oh_geometry
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SURF = {"ch4oh": (egrad_ch4oh, ch4oh_geometry, [mass_au(s) for s in ("H", "C", "H", "H", "H", "O", "H")]),
        "geh4oh": (egrad_geh4oh, geh4oh_geometry, [mass_au(s) for s in ("H", "Ge", "H", "H", "H", "O", "H")])}
PES = pytest.mark.parametrize("pes", ["ch4oh", "geh4oh"])


def pair(nbeads, ntraj, thermostat="none", kelvin=500.0, precision="fp64", transrot=False,
         andersen_step=20, seed=7, pes="ch4oh"):
    mass = SURF[pes][2]
    beta = beta_from_kelvin(kelvin)
    dt = dt_fs_to_au(0.1)
    tau0 = dt_fs_to_au(100.0)
    eng = RPMDEngine(pes, mass, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0_au=tau0, transrot=transrot,
                     precision=precision, seed=seed)
    cfg = orc.Config(pes, mass, nbeads, dt, beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0=tau0, transrot=transrot, seed=seed)
    return eng, cfg


def start(eng, cfg, sigma=0.02, pes="ch4oh"):
    q0 = SURF[pes][1]()
    eng.init_positions(q0, sigma)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, eng.ntraj, q0, sigma)
    p = orc.init_momenta(cfg, eng.ntraj)
    f, e = orc.init_forces(cfg, q)
    return q, p, f, e


@PES
def test_egrad_matches_oracle(require_gpu, pes):
    rng = np.random.default_rng(5)
    q = SURF[pes][1]()[None] + rng.normal(0, 0.1, (2048, 7, 3))
    V, g = SURF[pes][0](q)
    Vo, go = orc.egrad(pes, q)
    assert rel_err(V, Vo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def test_initialize_and_wrong_natoms(require_gpu):
    lib = L.lib()
    assert lib.cr_initialize_ch4oh() == 0 and lib.cr_initialize_geh4oh() == 0
    q = np.zeros((1, 3, 3))
    info = C.c_int(0)
    assert lib.cr_egrad_ch4oh(L.dptr(q), 3, 1, L.dptr(np.zeros(1)), L.dptr(q), C.byref(info)) == L.CR_ERR_ARG
    assert lib.cr_egrad_geh4oh(L.dptr(q), 3, 1, L.dptr(np.zeros(1)), L.dptr(q), C.byref(info)) == L.CR_ERR_ARG


@PES
@pytest.mark.parametrize("nbeads", [1, 8, 32])
@pytest.mark.parametrize("thermostat,transrot", [("none", False), ("andersen", True), ("pile", True)])
def test_single_step(require_gpu, nbeads, thermostat, transrot, pes):
    eng, cfg = pair(nbeads, 4, thermostat=thermostat, transrot=transrot, andersen_step=1, pes=pes)
    q, p, f, e = start(eng, cfg, pes=pes)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st.any()
    assert rel_err(qg, qo) <= 1e-12
    assert rel_err(pg, po) <= 1e-12
    assert rel_err(fg, fo) <= 1e-12
    assert rel_err(eg, eo) <= 1e-12


@PES
def test_100_steps_nve(require_gpu, pes):
    eng, cfg = pair(32, 6, pes=pes)
    q, p, f, e = start(eng, cfg, pes=pes)
    eng.run(100)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 100)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9
    assert rel_err(eg, eo) <= 1e-9


@PES
def test_mixed_force_error(require_gpu, pes):
    rng = np.random.default_rng(6)
    q = SURF[pes][1]()[None] + rng.normal(0, 0.1, (256 * 32, 7, 3))
    q = q.reshape(256, 32, 7, 3)
    e64, _ = pair(32, 256, precision="fp64", pes=pes)
    e32, _ = pair(32, 256, precision="mixed", pes=pes)
    z = np.zeros_like(q)
    e64.set_state(q, z)
    e32.set_state(q, z)
    _, _, f64, v64, _ = e64.get_state()
    _, _, f32, v32, _ = e32.get_state()
    err = rel_err(f32, f64)
    print(f"{pes} mixed-form force error {err:.3e}, energy error {rel_err(v32, v64):.3e}")
    # the O-H Morse, the stretches and the bends in float pairs: 3.6e-8 on
    # the host restatement of the mixed form
    assert err < 1.5e-7 and rel_err(v32, v64) < 1.5e-6


def test_geh4oh_departing_h_matches_oracle(require_gpu):
    """GeH4 + OH evaluates switchf's sphi at every Ge-H distance (CH4 + OH cuts
    it at 3.8 A): one methane H pulled out to 4-20 A, FP64 against the oracle,
    and the mixed form stays finite where exp(bphi (r - cphi)^3) passes the
    float range (r > 17.9 A)."""
    q0 = geh4oh_geometry()
    u = q0[2] - q0[1]
    u /= np.linalg.norm(u)
    qs = []
    for r_ang in np.linspace(4.0, 20.0, 64):
        q = q0.copy()
        q[2] = q0[1] + u * r_ang / 0.52917721092
        qs.append(q)
    q = np.array(qs)
    V, g = egrad_geh4oh(q)
    Vo, go = orc.egrad("geh4oh", q)
    assert np.isfinite(V).all() and rel_err(V, Vo) <= 1e-12 and rel_err(g, go) <= 1e-12
    e32, _ = pair(1, 64, precision="mixed", pes="geh4oh")
    e32.set_state(q[:, None], np.zeros_like(q[:, None]))
    _, _, f32, v32, _ = e32.get_state()
    assert np.isfinite(f32).all() and np.isfinite(v32).all()
    # the engine's f is Caracal's derivs (dV/dq)
    assert rel_err(f32[:, 0], go) < 1.5e-6
