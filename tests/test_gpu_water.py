"""GPU: Caracal's flexible SPC water box (src/egrad_water.f90) through the
C-ABI against the oracle.

Tolerances (norm-wise relative, max|a-b|/max|b|): plain FP64 energies and
gradients <= 1e-12; engine step <= 1e-12, 20 steps <= 1e-9.  Mixed form
(FP32 pairs, FP64 sums and intramolecular terms): force error <= 4e-6 of the
largest force, energy <= 2e-6 (measured 0.8-1.9e-6 and 0.5-0.9e-6): each
atom's force sums ~95 FP32 Coulomb pair forces of ~0.02 Eh/bohr, so the
FP32 rounding of the pairs sets the error, not the sums.
Parity is unpinned against the reference itself (no reference outputs for
this surface); the oracle follows src/egrad_water.f90 statement by statement.
"""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine, WaterBox
from caracal_gb300 import water as W
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def boxes(nw, nb, sigma, seed, periodic, zahn=False, cut=4.0):
    x, length = W.water_box(nw, seed=seed)
    rng = np.random.default_rng(seed)
    xs = x[None] + rng.normal(0, sigma, (nb,) + x.shape)
    if periodic:
        wb = WaterBox(nw, box=[length] * 3, coul_cut=cut, zahn=zahn)
        xs = xs + rng.normal(0, 5.0, (nb, 1, 3))  # whole-box shifts: the images matter
        orc.set_water(nw, wb.box_bohr, wb.coul_cut, zahn, wb.zahn_a, wb.zahn_par)
    else:
        wb = WaterBox(nw)
        orc.set_water(nw)
    return wb, xs


@pytest.mark.parametrize("periodic,zahn", [(False, False), (True, False), (True, True)])
def test_egrad_fp64_matches_oracle(require_gpu, periodic, zahn):
    wb, x = boxes(32, 64, 0.05, 1, periodic, zahn)
    e, g = wb.egrad(x, "fp64")
    eo, go = orc.egrad("water", x)
    wb.close()
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= 1e-12


@pytest.mark.parametrize("periodic,nw,nb,cut", [(False, 32, 64, 4.0), (True, 32, 64, 4.0), (True, 64, 1024, 6.0)])
def test_mixed_force_error(require_gpu, periodic, nw, nb, cut):
    # the last case has ~2e7 pair evaluations: some pairs sit within FP32
    # rounding of the cutoff, where the mixed form must decide as FP64 does
    wb, x = boxes(nw, nb, 0.1, 2, periodic, cut=cut)
    e64, g64 = wb.egrad(x, "fp64")
    em, gm = wb.egrad(x, "mixed")
    wb.close()
    ferr = np.max(np.abs(gm - g64)) / np.max(np.abs(g64))
    eerr = np.max(np.abs(em - e64)) / np.max(np.abs(e64))
    print(f"water mixed: force error {ferr:.3e}, energy error {eerr:.3e}")
    assert ferr <= 4e-6 and eerr <= 2e-6


def make_pair(wb, nbeads, ntraj, thermostat="andersen", andersen_step=5, seed=9):
    mass = W.masses(wb.nwater)
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(0.25)
    eng = RPMDEngine(wb, mass, nbeads, ntraj, dt, beta=beta, thermostat=thermostat,
                     andersen_step=andersen_step, seed=seed)
    cfg = orc.Config("water", mass, nbeads, dt, beta, thermostat=thermostat, andersen_step=andersen_step,
                     seed=seed)
    return eng, cfg


@pytest.mark.parametrize("nbeads", [8, 32, 6])
def test_engine_steps_match_oracle(require_gpu, nbeads):
    wb, x = boxes(16, 1, 0.0, 4, True)
    eng, cfg = make_pair(wb, nbeads, 3)
    eng.init_positions(x[0], 0.02)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, 3, x[0], 0.02)
    p = orc.init_momenta(cfg, 3)
    f, e = orc.init_forces(cfg, q)
    eng.run(1)
    q1, p1, f1, e1, st1 = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 1)
    assert not st1.any()
    assert rel_err(q1, qo) <= 1e-12 and rel_err(p1, po) <= 1e-12 and rel_err(f1, fo) <= 1e-12
    eng.run(19)
    q20, p20, _, e20, _ = eng.get_state()
    qo, po, fo, eo, so = orc.run(cfg, q, p, f, 20)
    eng.close()
    wb.close()
    assert rel_err(q20, qo) <= 1e-9 and rel_err(p20, po) <= 1e-9 and rel_err(e20, eo) <= 1e-9
