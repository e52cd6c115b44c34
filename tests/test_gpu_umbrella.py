"""GPU: umbrella windows (calc_rate's umbrella sampling, src/umbrella.f90 mode
0) through the engine's graph path against the oracle: one step <= 1e-12,
30 steps <= 1e-9, the sampled xi sums and histograms; and the per-window
statistics feeding umbrella integration."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300.pmf import umbrella_integration
from caracal_gb300.workloads import ch4h_config, ch4h_recross_definition
from conftest import rel_err
from oracle import oracle as orc
from test_oracle_parent import _xd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("thermostat,nbeads,transrot", [("andersen", 8, True), ("pile", 4, False)])
def test_umbrella_matches_oracle(require_gpu, thermostat, nbeads, transrot):
    T = 4
    wl = ch4h_config(ntraj=T, nbeads=nbeads)
    rd = ch4h_recross_definition(wl.q0)
    xd = _xd(rd)
    centers = np.array([0.9, 0.95, 1.0, 1.05])
    kforce = np.array([0.3, 0.4, 0.5, 0.6])
    eng = RPMDEngine("ch4h", wl.mass, nbeads, T, wl.dt_au, beta=wl.beta, thermostat=thermostat,
                     andersen_step=5, pile_tau0_au=wl.pile_tau0_au, transrot=transrot, seed=33)
    cfg = orc.Config("ch4h", wl.mass, nbeads, wl.dt_au, wl.beta, thermostat=thermostat, andersen_step=5,
                     pile_tau0=wl.pile_tau0_au, transrot=transrot, seed=33)
    eng.init_positions(wl.q0, 0.02)
    eng.init_momenta()
    eng.set_umbrella(centers=centers, kforce=kforce, nbins=40, lo=0.8, hi=1.2, **rd)
    eng.compute_forces()
    q = orc.init_positions(cfg, T, wl.q0, 0.02)
    p = orc.init_momenta(cfg, T)
    f, _ = orc.init_forces(cfg, q)
    eng.run(1)
    q1, p1, f1, e1, st = eng.get_state()
    qo, po, fo, eo, so, _ = orc.run_umbrella(cfg, xd, q, p, f, 1, centers, kforce)
    assert not st.any() and not so.any()
    for a, b in ((q1, qo), (p1, po), (f1, fo), (e1, eo)):
        assert rel_err(a, b) <= 1e-12
    eng.umbrella_sampling(True)
    eng.run(29)
    q30, p30, f30, _, st = eng.get_state()
    xs, x2, hist = eng.umbrella_stats()
    eng.close()
    qo, po, fo, eo, so, stats = orc.run_umbrella(cfg, xd, qo, po, fo, 29, centers, kforce, istep0=1,
                                                 sampling=True, nbins=40, lo=0.8, hi=1.2)
    assert rel_err(q30, qo) <= 1e-9 and rel_err(p30, po) <= 1e-9
    assert rel_err(xs, stats["xsum"]) <= 1e-9 and rel_err(x2, stats["xsum2"]) <= 1e-9
    # identical bins unless a xi falls within rounding of a bin edge
    assert np.abs(hist - stats["hist"][:, :40]).sum() <= 2
    assert 0 < hist.sum() <= 29 * T


def test_umbrella_windows_give_a_profile(require_gpu):
    """Windows across the dividing surface: means follow the window centres,
    positive variances, and umbrella integration returns a finite profile."""
    T = 16
    wl = ch4h_config(ntraj=T, nbeads=4)
    rd = ch4h_recross_definition(wl.q0)
    centers = np.linspace(0.95, 1.05, T)
    k = np.full(T, 20.0)      # xi fluctuates by 1/sqrt(beta k) ~ 0.009 against a spacing of 0.0067
    eng = RPMDEngine("ch4h", wl.mass, 4, T, wl.dt_au, beta=wl.beta, thermostat="andersen", andersen_step=20,
                     transrot=True, seed=5)
    eng.init_positions(wl.q0, 0.01)
    eng.init_momenta()
    eng.set_umbrella(centers=centers, kforce=k, **rd)
    eng.compute_forces()
    eng.run(200)              # equilibration
    eng.compute_forces()      # unbiased forces before sampling (src/calc_rate.f90:1612-1617)
    eng.umbrella_sampling(True)
    n = 400
    eng.run(n)
    xs, x2, _ = eng.umbrella_stats(reset=True)
    eng.close()
    av = xs / n
    va = x2 / n - av * av
    assert np.all(va > 0)
    assert np.corrcoef(av, centers)[0, 1] > 0.9
    coord, pmf = umbrella_integration(centers, k, av, va, wl.beta, 0.96, 1.04, 41, n)
    assert np.all(np.isfinite(pmf)) and pmf.min() >= 0.0   # shifted by the min over all bins (last one 0)
