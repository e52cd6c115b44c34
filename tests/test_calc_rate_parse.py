"""CPU: calc_rate key input (MECHA, UMBRELLA, PMF, RECROSS blocks) and the
BIMOLEC rate formula of calc_k_t."""
import numpy as np
import pytest

from caracal_gb300 import keyfile as K
from caracal_gb300.calc_rate import parse
from caracal_gb300.pmf import bimolecular_rate
from test_gpu_calc_rate import KEY


def test_parse_calc_rate_key():
    r = parse(KEY)
    assert (r.nbeads, r.pes, r.kelvin, r.andersen_step) == (4, "ANA_H3", 300.0, 20)
    assert (r.reac1, r.reac2, r.bond_form, r.bond_break, r.r_inf) == ([1, 2], [3], (2, 3), (1, 2), 10.0)
    assert (r.bias, r.umbr_lo, r.umbr_hi, r.umbr_dist) == (0.15, -0.05, 1.05, 0.1)
    assert (r.gen_steps, r.equi_steps, r.sample_steps, r.sample_trajs) == (100, 100, 200, 2)
    assert (r.xi_lo, r.xi_hi, r.nbins) == (0.0, 1.0, 50)
    assert (r.rc_equi, r.child_total, r.child_interval, r.child_perpoint, r.child_steps) == (50, 8, 20, 4, 60)


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
