"""CPU: the parameter vector of the fitting harness and its chain rule."""
import numpy as np

from caracal_gb300 import qmdff as Q
from caracal_gb300.fit import QMDFFParams


def test_theta_round_trip():
    ff = Q.alkane(nc=3)
    p = QMDFFParams(ff)
    th = p.theta()
    assert th.shape == (p.size,)
    f2 = p.with_theta(th * 2.0)
    assert np.allclose(QMDFFParams(f2).theta(), th * 2.0)
    assert np.allclose(np.asarray(ff.vbond)[:, 1], th[:p.nbond])   # original untouched


def test_charge_chain_rule_matches_pair_products():
    ff = Q.alkane(nc=3)
    for zahn in (False, True):
        p = QMDFFParams(ff, zahn=zahn)
        rng = np.random.default_rng(0)
        graw = rng.normal(size=p.nbond + p.nangl + p.ntors + len(p.pi))
        th = p.theta()
        g = p.chain(graw)
        nv = p.nbond + p.nangl + p.ntors
        assert np.array_equal(g[:nv], graw[:nv])

        # S(q) = sum_p graw_p f_p q_i q_j: its gradient by central differences
        def S(q):
            return float(np.sum(graw[nv:] * p.pf * q[p.pi] * q[p.pj]))
        q = th[nv:]
        for i in range(0, p.natoms, 3):
            e = np.zeros_like(q)
            e[i] = 1e-6
            assert abs((S(q + e) - S(q - e)) / 2e-6 - g[nv + i]) <= 1e-8 * max(1.0, abs(g[nv + i]))
