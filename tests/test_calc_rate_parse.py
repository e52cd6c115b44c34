"""CPU: calc_rate key input (MECHA, UMBRELLA, PMF, RECROSS blocks) including
the reference's own examples/calc_rate/h+h2/rate.key, the window layout, the
BIMOLEC rate formula of calc_k_t, and the whole calc_rate pipeline run on
the oracle (a small case)."""
import os

import numpy as np
import pytest

from caracal_gb300 import keyfile as K
from caracal_gb300.calc_rate import parse, window_layout
from caracal_gb300.pmf import bimolecular_rate
from caracal_gb300.units import BOHR_ANGSTROM
from conftest import ROOT
from test_gpu_calc_rate import KEY

H_H2 = os.path.join(ROOT, "tests", "golden", "reference", "calc_rate", "h+h2")


def test_parse_calc_rate_key():
    r = parse(KEY)
    assert (r.nbeads, r.pes, r.kelvin, r.andersen_step) == (4, "ANA_H3", 300.0, 20)
    assert (r.reac1, r.reac2, r.bond_form, r.bond_break) == ([1, 2], [3], (2, 3), (1, 2))
    assert r.r_inf == 10.0 / BOHR_ANGSTROM        # DIST_INF is read in Angstrom
    assert (r.bias, r.umbr_lo, r.umbr_hi, r.umbr_dist) == (0.05, -0.1, 1.1, 0.1)
    assert (r.gen_steps, r.equi_steps, r.sample_steps, r.sample_trajs) == (40, 60, 120, 2)
    assert (r.xi_lo, r.xi_hi, r.nbins) == (-0.1, 1.1, 60)
    assert (r.rc_equi, r.child_total, r.child_interval, r.child_perpoint, r.child_steps) == (40, 8, 20, 4, 50)


def test_parse_reference_h_h2_rate_key():
    """The unmodified examples/calc_rate/h+h2/rate.key of the reference."""
    with open(os.path.join(H_H2, "rate.key")) as fh:
        r = parse(fh.read(), directory=H_H2)
    assert (r.ts_struc, r.pes, r.nbeads, r.dt_fs, r.print_poly, r.tdump_fs) == ("ts.xyz", "ANA_H3", 8, 0.1, 1.0, 1.0)
    assert (r.kelvin, r.thermostat, r.andersen_step) == (300.0, "andersen", 80)
    assert (r.umbr_type, r.reac1, r.reac2, r.bond_form, r.bond_break, r.npaths) == ("BIMOLEC", [1, 2], [3], (2, 3),
                                                                                    (1, 2), 2)
    assert r.r_inf == pytest.approx(16.0 / BOHR_ANGSTROM, rel=1e-15)
    assert (r.bias, r.umbr_lo, r.umbr_hi, r.umbr_dist) == (0.05, -0.05, 1.05, 0.01)
    assert (r.gen_steps, r.equi_steps, r.sample_steps, r.sample_trajs) == (10000, 10000, 20000, 10)
    assert (r.xi_lo, r.xi_hi, r.nbins, r.pmf_method, r.minloc) == (-0.05, 1.05, 5000, "INTEGRATION", "ZERO")
    assert (r.rc_equi, r.child_total, r.child_interval, r.child_perpoint, r.child_steps) == (50000, 10000, 1000,
                                                                                            100, 500)
    n_all, n_over, n_samp, xw = window_layout(r)
    # 111 window positions, 110 sampled: -0.05 .. 1.04 (src/calc_rate.f90:650-663)
    assert (n_all, n_over, n_samp, len(xw)) == (111, 5, 105, 110)
    assert xw[0] == pytest.approx(-0.05, abs=1e-12) and xw[-1] == pytest.approx(1.04, abs=1e-12)
    assert np.all(np.diff(xw) > 0.0099)


def test_window_layout_rejects_misfit_steps():
    r = parse(KEY)
    r.umbr_lo, r.umbr_hi, r.umbr_dist = -0.05, 1.05, 0.1   # 0.05 / 0.1 does not fit (Caracal stops)
    with pytest.raises(K.KeyError_):
        window_layout(r)


def test_calc_rate_refuses_other_paths():
    with pytest.raises(K.KeyError_):
        parse(KEY.replace("ANA_H3", "QMDFF"))
    with pytest.raises(K.KeyError_):
        parse(KEY.replace("TYPE BIMOLEC", "TYPE ATOM_SHIFT"))


def test_bimolecular_rate_formula():
    beta = 1.0 / (300.0 * 0.316679e-5)
    m1, m2 = 2 * 1837.0, 1837.0
    k1 = bimolecular_rate(1.0, 0.01, 0.0, 10.0, beta, m1, m2)
    # kappa and n_paths scale it; the barrier enters as exp(-beta dW)
    assert bimolecular_rate(0.5, 0.01, 0.0, 10.0, beta, m1, m2, npaths=2) == pytest.approx(k1, rel=1e-15)
    assert bimolecular_rate(1.0, 0.02, 0.0, 10.0, beta, m1, m2) == pytest.approx(k1 * np.exp(-beta * 0.01),
                                                                                 rel=1e-12)
    mu = m1 * m2 / (m1 + m2)
    au = 4 * np.pi * 100.0 * np.sqrt(1 / (2 * np.pi * beta * mu)) * np.exp(-beta * 0.01)
    assert k1 / au == pytest.approx(1e6 * 5.2917721092e-11 ** 3 / 2.418884326505e-17 * 6.02214179e23, rel=1e-6)


def test_recross_restart_files_round_trip(tmp_path):
    from caracal_gb300.calc_rate import read_recross_restart, write_recross_restart
    num = np.linspace(0.1, 0.9, 7)
    q = np.arange(2 * 3 * 3, dtype=float).reshape(2, 3, 3) * 0.1
    write_recross_restart(str(tmp_path), 4, num, 2.5, q)
    k, n2, d2, q2 = read_recross_restart(str(tmp_path), 7, 2, 3)
    assert k == 4 and d2 == 2.5 and np.array_equal(n2, num) and np.array_equal(q2, q)
    # an incomplete parent file: sums kept, no parent
    (tmp_path / "recross_parent_pos.dat").write_text(" 1.0 2.0 3.0\n")
    k, n2, d2, q2 = read_recross_restart(str(tmp_path), 7, 2, 3)
    assert k == 4 and q2 is None
    # too few numerators: a fresh start
    (tmp_path / "recross_num_tmp.dat").write_text(" 0.5\n")
    k, n2, d2, q2 = read_recross_restart(str(tmp_path), 7, 2, 3)
    assert k == 0 and d2 == 0.0 and not n2.any() and q2 is None
    assert read_recross_restart(str(tmp_path / "nothing"), 7, 2, 3)[0] == 0


def test_calc_rate_pipeline_on_oracle(tmp_path):
    """The whole pipeline (structures, windows, PMF, parent, children, k(T))
    with the oracle standing in for the engine."""
    from caracal_gb300.calc_rate import run
    from oracle_engine import OracleEngine
    from test_gpu_calc_rate import write_inputs
    key = write_inputs(tmp_path)
    res = run(key, out_dir=str(tmp_path), quiet=True, engine=OracleEngine)
    pmf = np.loadtxt(tmp_path / "pmf_integration.dat")
    kap = np.loadtxt(tmp_path / "recross.dat")
    assert pmf.shape == (59, 2) and np.all(np.isfinite(pmf)) and pmf[:, 1].min() == 0.0
    assert kap.shape == (50, 2) and np.all(np.isfinite(kap))
    assert res["windows"] == 12 and res["trajectories"] == 24
    assert np.isfinite(res["k_t"]) and res["k_t"] > 0.0
    assert np.isfinite(res["kappa_stderr"]) and np.isfinite(res["pmf_max_stderr_kjmol"])
