"""GPU: the CUDA engine (through its C-ABI) against the oracle, H3 / BKMP2.

Tolerances (norm-wise relative, max|a-b|/max|b|):
  plain FP64 form: single-step forces and positions <= 1e-12,
                   100-step trajectories <= 1e-9;
  mixed form:      force error against FP64 reported and bounded below.
"""
import ctypes as C

import numpy as np
import pytest

from caracal_gb300 import _lib as L
from caracal_gb300 import RPMDEngine, egrad_h3
from caracal_gb300.units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from caracal_gb300.workloads import h3_collinear
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MH = mass_au("H")


def make_pair(nbeads, ntraj, thermostat="andersen", kelvin=300.0, andersen_step=20,
              transrot=True, precision="fp64", seed=20261203, dt_fs=0.1, nm_mode=0):
    beta = beta_from_kelvin(kelvin) if kelvin else float("inf")
    dt = dt_fs_to_au(dt_fs)
    tau0 = dt_fs_to_au(100.0)
    eng = RPMDEngine("h3", [MH] * 3, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0_au=tau0, transrot=transrot,
                     precision=precision, seed=seed, nm_mode=nm_mode)
    cfg = orc.Config("h3", [MH] * 3, nbeads, dt, beta, thermostat=thermostat,
                     andersen_step=andersen_step, pile_tau0=tau0, transrot=transrot, seed=seed,
                     nm_mode=nm_mode)
    return eng, cfg


def start(eng, cfg, sigma=None, zero_p=False):
    sigma = float(angstrom_to_bohr(0.01)) if sigma is None else sigma
    q0 = h3_collinear()
    eng.init_positions(q0, sigma)
    eng.init_momenta(zero=zero_p)
    eng.compute_forces()
    q = orc.init_positions(cfg, eng.ntraj, q0, sigma)
    p = np.zeros(cfg.shape(eng.ntraj)) if zero_p else orc.init_momenta(cfg, eng.ntraj)
    f, e = orc.init_forces(cfg, q)
    return q, p, f, e


def test_egrad_h3_matches_oracle(require_gpu):
    rng = np.random.default_rng(1)
    q = h3_collinear()[None] + rng.normal(0, 0.3, (4096, 3, 3))
    q[:64] = np.array([[0, 0, 0], [0, 0, 1.0], [0.8, 0, 0.5]]) + rng.normal(0, 0.05, (64, 3, 3))
    V, g = egrad_h3(q)
    Vo, go = orc.egrad_h3(q)
    assert rel_err(V, Vo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


def test_egrad_h3_zero_beads_and_info(require_gpu):
    lib = L.lib()
    info = C.c_int(5)
    z = np.zeros(1)
    assert lib.cr_egrad_h3(L.dptr(z), 3, 0, L.dptr(z), L.dptr(z), C.byref(info)) == 0
    assert info.value == 0


def test_init_matches_oracle(require_gpu):
    eng, cfg = make_pair(16, 8)
    q, p, f, e = start(eng, cfg)
    qg, pg, fg, eg, st = eng.get_state()
    assert rel_err(qg, q) <= 1e-15
    assert rel_err(pg, p) <= 1e-14
    assert rel_err(fg, f) <= 1e-12
    assert rel_err(eg, e) <= 1e-12


@pytest.mark.parametrize("thermostat", ["andersen", "pile", "none"])
@pytest.mark.parametrize("nbeads", [1, 3, 16, 32, 64, 128])
def test_single_step_matches_oracle(require_gpu, thermostat, nbeads):
    ntraj = 5
    eng, cfg = make_pair(nbeads, ntraj, thermostat=thermostat, andersen_step=1)
    q, p, f, e = start(eng, cfg)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st.any() and not so.any()
    assert rel_err(qg, qo) <= 1e-12
    assert rel_err(pg, po) <= 1e-12
    # forces of the step at its own new positions; against the oracle's step
    # the positions may differ in the last bit, which moves BKMP2's gradient
    # by ~1e-14 of its largest component (the bound's size at P = 3)
    _, g_at = orc.egrad("h3", qg.reshape(-1, 3, 3))
    assert rel_err(fg, g_at.reshape(fg.shape)) <= 1e-12
    assert rel_err(fg, fo) <= 1e-11
    assert rel_err(eg, eo) <= 1e-12


@pytest.mark.parametrize("thermostat", ["andersen", "pile"])
@pytest.mark.parametrize("nbeads", [16, 64])
def test_100_steps_match_oracle(require_gpu, thermostat, nbeads):
    eng, cfg = make_pair(nbeads, 6, thermostat=thermostat, andersen_step=20)
    q, p, f, e = start(eng, cfg)
    eng.run(60)
    eng.run(40)  # the step counter continues across runs
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 100)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(pg, po) <= 1e-9
    assert rel_err(eg, eo) <= 1e-9


@pytest.mark.parametrize("thermostat,nbeads", [("andersen", 4), ("andersen", 8), ("pile", 16), ("none", 32),
                                               ("andersen", 64), ("andersen", 3)])
def test_orthonormal_modes_match_oracle(require_gpu, thermostat, nbeads):
    """nm_mode 1 (orthonormal normal modes, the circulant propagator): one
    step <= 1e-12 and 100 steps <= 1e-9 against the oracle's transform-based
    restatement."""
    eng, cfg = make_pair(nbeads, 5, thermostat=thermostat, andersen_step=7, nm_mode=1)
    q, p, f, e = start(eng, cfg)
    eng.run(1)
    qg, pg, _, _, st = eng.get_state()
    q1, p1, f1, _, so = orc.run(cfg, q, p, f, 1)
    assert not st.any() and not so.any()
    assert rel_err(qg, q1) <= 1e-12 and rel_err(pg, p1) <= 1e-12
    eng.run(99)
    qg, pg, _, eg, st = eng.get_state()
    eng.close()
    qo, po, _, eo, so = orc.run(cfg, q1, p1, f1, 99, istep0=1)
    assert not st.any() and not so.any()
    assert rel_err(qg, qo) <= 1e-9 and rel_err(pg, po) <= 1e-9 and rel_err(eg, eo) <= 1e-9
    # the orthonormal transform keeps beads j and P - j distinct; Caracal's does not
    if nbeads >= 4:
        assert np.max(np.abs(qg[:, 1] - qg[:, nbeads - 1])) > 1e-6


def test_step_host_equals_device_run(require_gpu):
    eng, cfg = make_pair(16, 4, thermostat="pile")
    q, p, f, e = start(eng, cfg)
    qh, ph, fh = q.copy(), p.copy(), f.copy()
    eh = np.zeros(4)
    for _ in range(3):
        eng.step_host(qh, ph, fh, eh)
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 3)
    assert rel_err(qh, qo) <= 1e-12 and rel_err(ph, po) <= 1e-12 and rel_err(eh, eo) <= 1e-12


@pytest.mark.parametrize("thermostat", ["pile", "andersen", "nhc"])
def test_step_host_pipelined_groups_equal_device_run(require_gpu, thermostat):
    # 8192 trajectories x 16 beads: 9.4 MB per state array, so the host step
    # runs as 4 trajectory groups whose copies overlap the other groups' steps
    engs = []
    for _ in range(2):
        eng = RPMDEngine("h3", [MH] * 3, 16, 8192, dt_fs_to_au(0.1), beta=beta_from_kelvin(300.0),
                         thermostat=thermostat, andersen_step=2, pile_tau0_au=dt_fs_to_au(100.0),
                         nose_q_au=nose_q_to_au(20.0, 0.1), seed=20261203)
        eng.init_positions(h3_collinear(), float(angstrom_to_bohr(0.01)))
        eng.init_momenta()
        eng.compute_forces()
        engs.append(eng)
    a, b = engs
    q, p, f, e, _ = a.get_state()
    for _ in range(3):
        a.step_host(q, p, f, e)
    assert a.launch_info()["launches"] == 4
    b.run(3)
    qb, pb, fb, eb, st = b.get_state()
    a.close()
    b.close()
    assert not st.any()
    assert rel_err(q, qb) <= 1e-15 and rel_err(p, pb) <= 1e-15
    assert rel_err(f, fb) <= 1e-15 and rel_err(e, eb) <= 1e-15


def test_nve_classical_energy_drift_no_larger_than_oracle(require_gpu):
    # P = 1, NVE, transrot on (src/verlet.f90:1300-1306); compare drift of E = K + V
    eng, cfg = make_pair(1, 4, thermostat="none", kelvin=None)
    q, p, f, e = start(eng, cfg, sigma=0.05, zero_p=True)
    rng = np.random.default_rng(2)
    p = rng.normal(0, 3.0, p.shape)
    eng.set_state(q, p, f)
    def energy(p_, e_):
        return (p_ ** 2).sum(axis=(1, 2, 3)) / (2 * MH) + e_
    E0 = energy(p, e)
    eng.run(2000)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 2000)
    drift_gpu = np.abs(energy(pg, eg) - E0).max()
    drift_orc = np.abs(energy(po, eo) - E0).max()
    assert drift_gpu <= 1.01 * drift_orc + 1e-12


def test_nonfinite_trajectory_is_flagged_not_fatal(require_gpu):
    eng, cfg = make_pair(8, 3, thermostat="andersen")
    q, p, f, e = start(eng, cfg)
    qn = q.copy()
    qn[1, 2, 0, 0] = np.nan            # a poisoned bead in trajectory 1 (host data)
    eng.set_state(qn, p, f)
    rc = eng.run(2, check=False)
    assert rc == L.CR_ERR_TRAJECTORY
    qg, pg, fg, eg, st = eng.get_state()
    assert st[1] & L.CR_TRAJ_NONFINITE
    assert st[0] == 0 and st[2] == 0
    qo, po, fo, eo, so = orc.run(cfg, q[[0, 2]], p[[0, 2]], f[[0, 2]], 2, traj0=0)
    # trajectory 0 is unaffected by its poisoned neighbour
    assert rel_err(qg[0], qo[0]) <= 1e-12


def test_mixed_form_force_error(require_gpu):
    rng = np.random.default_rng(4)
    q = h3_collinear()[None] + rng.normal(0, 0.2, (8192, 3, 3))
    # the mixed form through the engine: one force evaluation at the same positions
    eng64, cfg = make_pair(16, 512, thermostat="none", kelvin=300.0, precision="fp64")
    eng32, _ = make_pair(16, 512, thermostat="none", kelvin=300.0, precision="mixed")
    qq = q.reshape(512, 16, 3, 3)
    zeros = np.zeros_like(qq)
    eng64.set_state(qq, zeros)
    eng32.set_state(qq, zeros)
    _, _, f64, e64, _ = eng64.get_state()
    _, _, f32, e32, _ = eng32.get_state()
    err_f = rel_err(f32, f64)
    err_e = rel_err(e32, e64)
    print(f"mixed-form force error {err_f:.3e}, energy error {err_e:.3e}")
    # stated bound of the mixed form on this distribution (measured ~2e-7)
    assert err_f < 1e-6 and err_e < 1e-6


@pytest.mark.parametrize("thermostat", ["andersen", "pile"])
def test_mixed_single_step_close_to_oracle(require_gpu, thermostat):
    eng, cfg = make_pair(16, 8, thermostat=thermostat, precision="mixed", andersen_step=1)
    q, p, f, e = start(eng, cfg)
    eng.run(1)
    qg, pg, fg, eg, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    # the mixed form's forces carry ~1e-6 norm-wise error (FP32 surface)
    assert rel_err(qg, qo) <= 1e-9
    assert rel_err(fg, fo) <= 5e-6
    assert rel_err(pg, po) <= 5e-6
