"""GPU: the calc_rate pipeline on H + H2 (start structures, umbrella windows,
umbrella integration, constrained parent, recrossing children, k(T)).

* A small case run through the CUDA engine and through the oracle from the
  same seeds: the profile and kappa(t) agree.
* The reference's own examples/calc_rate/h+h2/rate.key, unmodified, against
  the values the reference publishes for it (manual/figures/kappa_h3.png and
  pmf_h3.png, read off the plots): kappa(t = 50 fs) = 0.767 and a PMF
  maximum of 48.5 kJ/mol at xi = 1.0.  The tolerance is three jackknife
  standard errors of this run plus the reading error of the plots
  (0.005 in kappa, 0.5 kJ/mol in the PMF).
"""
import os
import shutil

import numpy as np
import pytest

from caracal_gb300.calc_rate import run
from conftest import ROOT

pytestmark = pytest.mark.gpu

KEY = """TS_STRUC ts.xyz
RPMD_BEADS 4
DELTAT 0.1
PES ANA_H3
RANDOM_SEED 11
NVT {
 TEMP 300
 THERMOSTAT ANDERSEN
 ANDERSEN_STEP 20
}
MECHA {
 TYPE BIMOLEC
 REACTANT1 1 2
 REACTANT2 3
 DIST_INF 10.0
 BOND_FORM 2-3
 BOND_BREAK 1-2
}
UMBRELLA {
 BIAS 0.05
 BONDS -0.1 1.1
 DIST 0.1
 GEN_STEPS 40
 EQUI_STEPS 60
 SAMPLE_STEPS 120
 SAMPLE_TRAJS 2
}
PMF {
 XI_RANGE -0.1 1.1
 BINS 60
}
RECROSS {
 EQUI_STEPS 40
 CHILD_TOTAL 8
 CHILD_INTERVAL 20
 CHILD_PERPOINT 4
 CHILD_STEPS 50
}
"""

H_H2 = os.path.join(ROOT, "tests", "golden", "reference", "calc_rate", "h+h2")


def write_inputs(d):
    """The small case: a symmetric H-H-H transition state (r = 0.93 A)."""
    xyz = np.array([[0.0, 0.0, -0.93], [0.0, 0.0, 0.0], [0.0, 0.0, 0.93]])
    (d / "ts.xyz").write_text("3\n\n" + "".join(f"H {a} {b} {c}\n" for a, b, c in xyz))
    (d / "calc_rate.key").write_text(KEY)
    return str(d / "calc_rate.key")


@pytest.mark.parametrize("options", [{}, {"nm_mode": 1, "transrot": False}])
def test_calc_rate_gpu_matches_oracle(require_gpu, tmp_path, options):
    from oracle_engine import OracleEngine
    dg, do = tmp_path / "gpu", tmp_path / "oracle"
    dg.mkdir()
    do.mkdir()
    rg = run(write_inputs(dg), out_dir=str(dg), quiet=True, **options)
    ro = run(write_inputs(do), out_dir=str(do), quiet=True, engine=OracleEngine, **options)
    pg, po = np.loadtxt(dg / "pmf_integration.dat"), np.loadtxt(do / "pmf_integration.dat")
    kg, ko = np.loadtxt(dg / "recross.dat"), np.loadtxt(do / "recross.dat")
    assert pg.shape == po.shape == (59, 2)
    # a few hundred steps of chaotic dynamics amplify 1e-16 roundings: 1e-7
    assert np.max(np.abs(pg[:, 1] - po[:, 1])) <= 1e-7 * max(1.0, np.abs(po[:, 1]).max())
    assert np.max(np.abs(kg[:, 1] - ko[:, 1])) <= 1e-7
    assert rg["xi_barrier"] == ro["xi_barrier"]
    assert rg["k_t"] == pytest.approx(ro["k_t"], rel=1e-6)


def test_h_h2_reference_example(require_gpu, tmp_path):
    """examples/calc_rate/h+h2/rate.key end to end (110 windows x 10 ring
    polymers x 30 000 steps, 8 beads; 100 parent snapshots x 100 children x
    500 steps) with the algorithm the published values were made with: the
    orthonormal normal-mode transform and no COM/rotation removal in the
    windows.  (Caracal's current source applies its cosine transform and
    transrot every window step; transrot removes the total angular
    momentum, which drops the 2 kT ln R rise of the profile.)"""
    for n in ("rate.key", "ts.xyz"):
        shutil.copyfile(os.path.join(H_H2, n), tmp_path / n)
    res = run(str(tmp_path / "rate.key"), out_dir=str(tmp_path), quiet=True, nm_mode=1, transrot=False)
    kap, kerr = res["kappa_t"][-1], res["kappa_t_stderr"][-1]
    pmax, perr = res["pmf_max_kjmol"], res["pmf_max_stderr_kjmol"]
    print(f"kappa(50 fs) = {kap:.4f} +- {kerr:.4f}; PMF max = {pmax:.2f} +- {perr:.2f} kJ/mol "
          f"at xi = {res['xi_barrier']:.4f}; k(T) = {res['k_t']:.4e} cm^3/mol/s")
    # The figures are one run of Caracal with the example's sample sizes, so
    # their statistical error equals this run's: the difference of the two
    # estimates has sqrt(2) times this run's standard error, held here to 3 of
    # those, plus the reading error of the figure (0.005 in kappa, 0.5 kJ/mol).
    z = 3.0 * np.sqrt(2.0)
    assert len(res["kappa_t"]) == 500
    assert abs(kap - 0.767) <= z * kerr + 0.005
    assert abs(pmax - 48.5) <= z * perr + 0.5
    assert abs(res["xi_barrier"] - 1.0) <= 0.02
    # the whole curves (digitised): kappa(t) against this run's error at each
    # time, the PMF against the error of its maximum (the integrated error
    # grows along xi)
    fk = np.loadtxt(os.path.join(ROOT, "tests", "golden", "reference", "figure_kappa_h3.txt"))
    fp = np.loadtxt(os.path.join(ROOT, "tests", "golden", "reference", "figure_pmf_h3.txt"))
    dt_fs = 0.1
    rows = []
    for t in (2.5, 5.0, 10.0, 20.0, 30.0, 40.0):
        i = int(round(t / dt_fs)) - 1
        rows.append((t, res["kappa_t"][i], np.interp(t, fk[:, 0], fk[:, 1]), res["kappa_t_stderr"][i]))
    pm = [(xi, np.interp(xi, res["coord"], res["pmf_kjmol"]), np.interp(xi, fp[:, 0], fp[:, 1]))
          for xi in (0.2, 0.4, 0.6, 0.8, 0.9)]
    print("kappa(t): t, run, figure, stderr", rows)
    print("PMF(xi): xi, run, figure", pm)
    for t, got, want, err in rows:
        assert abs(got - want) <= z * err + 0.005, (t, got, want, err)
    for xi, got, want in pm:
        assert abs(got - want) <= z * perr + 0.5, (xi, got, want)
