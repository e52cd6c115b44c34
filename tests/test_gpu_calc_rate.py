"""GPU: the calc_rate pipeline on H + H2 (umbrella windows, umbrella
integration, constrained parent, recrossing children, k(T)) on a small
input: every stage runs and writes Caracal's files with finite values."""
import numpy as np
import pytest

from caracal_gb300.calc_rate import run
from caracal_gb300.units import BOHR_ANGSTROM

pytestmark = pytest.mark.gpu

KEY = """TS_STRUC ts.xyz
RPMD_BEADS 4
DELTAT 0.1
PES ANA_H3
SEED 11
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
 BOND_FORM 2 3
 BOND_BREAK 1 2
}
UMBRELLA {
 BIAS 0.15
 BONDS -0.05 1.05
 DIST 0.1
 GEN_STEPS 100
 EQUI_STEPS 100
 SAMPLE_STEPS 200
 SAMPLE_TRAJS 2
}
PMF {
 XI_RANGE 0.0 1.0
 BINS 50
}
RECROSS {
 EQUI_STEPS 50
 CHILD_TOTAL 8
 CHILD_INTERVAL 20
 CHILD_PERPOINT 4
 CHILD_STEPS 60
}
"""


def test_calc_rate_h3(require_gpu, tmp_path):
    # symmetric H-H-H transition state, r = 0.93 Angstrom
    xyz = np.array([[0.0, 0.0, -0.93], [0.0, 0.0, 0.0], [0.0, 0.0, 0.93]])
    (tmp_path / "ts.xyz").write_text("3\n\n" + "".join(f"H {a} {b} {c}\n" for a, b, c in xyz))
    (tmp_path / "calc_rate.key").write_text(KEY)
    res = run(str(tmp_path / "calc_rate.key"), out_dir=str(tmp_path), quiet=True)
    pmf = np.loadtxt(tmp_path / "pmf_integration.dat")
    kap = np.loadtxt(tmp_path / "recross.dat")
    assert pmf.shape == (49, 2) and np.all(np.isfinite(pmf)) and pmf[:, 1].min() == 0.0
    assert kap.shape == (60, 2) and np.all(np.isfinite(kap))
    assert res["windows"] == 12 and res["trajectories"] == 24
    assert np.isfinite(res["k_t"]) and res["k_t"] > 0.0
    assert 0.0 < res["kappa"] <= 1.5
