"""CPU: the oracle's recrossing pieces.

calc_xi (mode 2, BIMOLEC) against central differences; kappa bookkeeping:
pairs carry opposite flux weights, kappa(0+) = 1 when every positive-flux
child crosses in the first step, and the denominator is half of sum |w|.
"""
import numpy as np

from caracal_gb300.workloads import ch4h_config, ch4h_recross_definition
from oracle import oracle as orc


def xidef(rd):
    return orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                          (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                          (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                          rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])


def test_calc_xi_gradient_central_differences():
    wl = ch4h_config(ntraj=2, nbeads=2)
    rng = np.random.default_rng(9)
    for xi_ideal in (1.0, 0.7):
        rd = ch4h_recross_definition(wl.q0)
        rd["xi_ideal"] = xi_ideal
        xd = xidef(rd)
        q = wl.q0 + rng.normal(0, 0.1, wl.q0.shape)
        xi, dxi = orc.calc_xi(xd, q, wl.mass)
        h = 1e-6
        g = np.zeros_like(q)
        for i in range(q.shape[0]):
            for d in range(3):
                a, b = q.copy(), q.copy()
                a[i, d] += h
                b[i, d] -= h
                g[i, d] = (orc.calc_xi(xd, a, wl.mass)[0] - orc.calc_xi(xd, b, wl.mass)[0]) / (2 * h)
        assert np.max(np.abs(g - dxi)) < 1e-8


def test_xi_is_zero_on_the_reference_geometry():
    wl = ch4h_config(ntraj=2, nbeads=2)
    xi, _ = orc.calc_xi(xidef(ch4h_recross_definition(wl.q0)), wl.q0, wl.mass)
    assert abs(xi) < 1e-14


def test_child_pairs_and_kappa_bookkeeping():
    wl = ch4h_config(ntraj=8, nbeads=4)
    rd = ch4h_recross_definition(wl.q0)
    cfg = orc.Config("ch4h", wl.mass, 4, wl.dt_au, wl.beta, transrot=False, seed=wl.seed)
    qpar = np.repeat(wl.q0[None], 4, axis=0)
    num, den, w = orc.recross_children(cfg, xidef(rd), 8, qpar, 3)
    assert np.allclose(w[0::2], -w[1::2], atol=1e-14)
    assert np.isclose(den, np.abs(w).sum() / 2)
    assert abs(num[0] / den - 1.0) < 1e-12
