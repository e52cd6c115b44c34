"""GPU: Caracal's ANA_OH3 surface (OH + H2, src/egrad_oh3.f) through the
C-ABI and in the persistent step kernel against the oracle.  Tolerances
(norm-wise relative): FP64 energies and gradients <= 1e-12; one step
<= 1e-12 (forces at the step's own positions), 100 steps <= 1e-9; mixed
form force error <= 1.5e-7 of the largest force (the R1 Morse and the H2
LEPS term in float pairs, the rest FP32; FP64 distances and gradient
assembly)."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine, egrad_oh3
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

Q0 = np.array([[0, 0, 0], [1.83, 0, 0], [-0.6, 2.9, 0.1], [-0.8, 4.3, 0.2]], float)
MASS = [mass_au("O"), mass_au("H"), mass_au("H"), mass_au("H")]


def test_egrad_matches_oracle(require_gpu):
    rng = np.random.default_rng(3)
    q = Q0[None] + rng.normal(0, 0.2, (2048, 4, 3))
    V, g = egrad_oh3(q)
    Vo, go = orc.egrad("oh3", q)
    assert rel_err(V, Vo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


@pytest.mark.parametrize("nbeads", [8, 16, 3])
def test_engine_steps_match_oracle(require_gpu, nbeads):
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(0.1)
    eng = RPMDEngine("oh3", MASS, nbeads, 4, dt, beta=beta, thermostat="andersen", andersen_step=5, seed=11)
    cfg = orc.Config("oh3", MASS, nbeads, dt, beta, thermostat="andersen", andersen_step=5, seed=11)
    eng.init_positions(Q0, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, 4, Q0, 0.02)
    p = orc.init_momenta(cfg, 4)
    f, e = orc.init_forces(cfg, q)
    eng.run(1)
    q1, p1, f1, e1, st = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st.any()
    assert rel_err(q1, qo) <= 1e-12 and rel_err(p1, po) <= 1e-12
    _, g_at = orc.egrad("oh3", q1.reshape(-1, 4, 3))
    assert rel_err(f1, g_at.reshape(f1.shape)) <= 1e-12
    eng.run(99)
    q100, p100, _, e100, _ = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 100)
    eng.close()
    assert rel_err(q100, qo) <= 1e-9 and rel_err(p100, po) <= 1e-9 and rel_err(e100, eo) <= 1e-9


def test_mixed_force_error(require_gpu):
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(0.1)
    out = {}
    for prec in ("fp64", "mixed"):
        eng = RPMDEngine("oh3", MASS, 16, 64, dt, beta=beta, thermostat="andersen", seed=5, precision=prec)
        eng.init_positions(Q0, 0.05)
        eng.init_momenta()
        eng.compute_forces()
        out[prec] = eng.get_state()[2]
        eng.close()
    err = np.max(np.abs(out["mixed"] - out["fp64"])) / np.max(np.abs(out["fp64"]))
    print(f"oh3 mixed force error {err:.3e}")
    assert err <= 1.5e-7           # 4.3e-8 over the 4096 x 32 bench ensemble
