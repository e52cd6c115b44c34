"""GPU: dE-EVB of two QMDFFs (cr_evb, src/gradient.f90:361-386, 1228-1304)
and the EVB engine against the oracle.  Plain FP64: energies and gradients
<= 1e-12, one step <= 1e-12, 10 steps <= 1e-9 (norm-wise relative)."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300 import qmdff as Q
from caracal_gb300.engine import EVBPair, QMDFFForceField
from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au
from caracal_gb300.workloads import qmdff_config
from conftest import rel_err
from oracle import oracle as orc
from test_oracle_evb import BASES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fields(require_gpu):
    ff = Q.alkane()
    ff2 = Q.alkane_evb_partner(ff)
    g1, g2 = QMDFFForceField(ff), QMDFFForceField(ff2)
    yield ff, ff2, g1, g2
    g1.close()
    g2.close()


@pytest.mark.parametrize("basis", list(BASES))
def test_evb_egrad_matches_oracle(fields, basis):
    ff, ff2, g1, g2 = fields
    orc.set_evb(ff, ff2, Q.ElementTables.caracal(), basis, BASES[basis])
    pair = EVBPair(g1, g2, basis, **BASES[basis])
    x = ff.xyz[None] + np.random.default_rng(3).normal(0, 0.05, (96,) + ff.xyz.shape)
    e, g = pair.egrad(x, "fp64")
    eo, go = orc.egrad("evb", x)
    em, gm = pair.egrad(x, "mixed")
    pair.close()
    assert rel_err(e, eo) <= 1e-12
    assert rel_err(g, go) <= 1e-12
    assert np.sqrt(np.sum((gm - g) ** 2) / np.sum(g ** 2)) <= 2e-6


def test_evb_engine_matches_oracle(fields):
    ff, ff2, g1, g2 = fields
    par = BASES["1g"]
    orc.set_evb(ff, ff2, Q.ElementTables.caracal(), "1g", par)
    pair = EVBPair(g1, g2, "1g", **par)
    mass = qmdff_config().mass
    beta, dt = beta_from_kelvin(300.0), dt_fs_to_au(0.5)
    eng = RPMDEngine(pair, mass, 8, 2, dt, beta=beta, thermostat="andersen", andersen_step=4, seed=9)
    cfg = orc.Config("evb", mass, 8, dt, beta, thermostat="andersen", andersen_step=4, seed=9)
    eng.init_positions(ff.xyz, 0.02)
    eng.init_momenta()
    eng.compute_forces()
    q = orc.init_positions(cfg, 2, ff.xyz, 0.02)
    p = orc.init_momenta(cfg, 2)
    f, e0 = orc.init_forces(cfg, q)
    _, _, fg0, eg0, _ = eng.get_state()
    assert rel_err(fg0, f) <= 1e-12 and rel_err(eg0, e0) <= 1e-12
    eng.run(1)
    q1, p1, f1, e1, _ = eng.get_state()
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 1)
    assert rel_err(q1, qo) <= 1e-12 and rel_err(p1, po) <= 1e-12 and rel_err(e1, eo) <= 1e-12
    eng.run(9)
    q10, p10, _, e10, _ = eng.get_state()
    eng.close()
    pair.close()
    qo, po, fo, eo, _ = orc.run(cfg, q, p, f, 10)
    assert rel_err(q10, qo) <= 1e-9 and rel_err(p10, po) <= 1e-9 and rel_err(e10, eo) <= 1e-9


@pytest.mark.parametrize("basis", ["1g", "2g", "3g", "sp", "sd", "sd2", "sp2d", "sp2d3"])
def test_evb_fit_matches_oracle(require_gpu, basis):
    from caracal_gb300.engine import evb_fit
    from test_oracle_evb import FIT, fit_data
    e1, e2, eref = fit_data(m=4096)
    fv, fj = evb_fit(basis, FIT[basis], e1, e2, eref)
    fo, fjo = orc.evb_fit(basis, FIT[basis], e1, e2, eref)
    assert rel_err(fv, fo) <= 1e-12
    # forward differences with fdjac2's h = sqrt(eps) |x_j| amplify last-bit
    # differences of the residuals by 1/h
    x = np.asarray(FIT[basis])
    for j in range(len(x)):
        hj = np.sqrt(np.finfo(float).eps) * abs(x[j])
        noise = 1e-15 * np.max(np.abs(eref)) ** 2 / hj
        assert np.max(np.abs(fj[j] - fjo[j])) <= 1e-10 * np.max(np.abs(fjo[j])) + noise


@pytest.mark.parametrize("basis", ["1g", "2g", "sp", "sp2d3"])
def test_evb_fit_gradient_matches_fdjac2(require_gpu, basis):
    """The analytic fit gradient against the reference's own route: MINPACK
    fdjac2 columns (forward differences) summed over the points, and central
    differences of the loss."""
    from caracal_gb300.engine import evb_fit_grad
    from test_oracle_evb import FIT, fit_data
    e1, e2, eref = fit_data(m=2048)
    x = np.asarray(FIT[basis])
    grad = evb_fit_grad(basis, x, e1, e2, eref)
    _, fjac = orc.evb_fit(basis, x, e1, e2, eref)
    fd2 = fjac.sum(axis=1)
    for j in range(len(x)):
        hj = np.sqrt(np.finfo(float).eps) * abs(x[j])
        noise = 1e-15 * np.max(np.abs(eref)) ** 2 / hj * len(e1)
        assert abs(grad[j] - fd2[j]) <= 1e-5 * abs(grad[j]) + noise
        h = 1e-6 * abs(x[j])
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        cd = (orc.evb_fit(basis, xp, e1, e2, eref, jacobian=False).sum() -
              orc.evb_fit(basis, xm, e1, e2, eref, jacobian=False).sum()) / (2 * h)
        assert abs(grad[j] - cd) <= 1e-7 * abs(grad[j]) + noise


@pytest.mark.parametrize("basis", ["1g", "sp"])
def test_evb_param_vjp_matches_finite_differences(fields, basis):
    from caracal_gb300.fit import QMDFFParams
    ff, ff2, g1, g2 = fields
    par = dict(BASES[basis])
    x = ff.xyz[None] + np.random.default_rng(61).normal(0, 0.05, (12,) + ff.xyz.shape)
    v = np.random.default_rng(62).normal(0, 1.0, x.shape)
    pair = EVBPair(g1, g2, basis, **par)
    gc, gf = pair.param_vjp(x, v)
    pair.close()

    def S_coupling(p):
        pr = EVBPair(g1, g2, basis, **p)
        _, g = pr.egrad(x)
        pr.close()
        return float(np.sum(v * g))
    for k in ("a", "b"):
        h = 1e-6 * abs(par[k])
        pp, pm = dict(par), dict(par)
        pp[k] += h
        pm[k] -= h
        fd = (S_coupling(pp) - S_coupling(pm)) / (2 * h)
        assert abs(fd - gc[k]) <= 1e-6 * abs(fd) + 1e-12
    params = QMDFFParams(ff)
    theta = params.theta()
    grad = params.chain(gf)

    def S_ff1(th):
        f1 = QMDFFForceField(params.with_theta(th))
        pr = EVBPair(f1, g2, basis, **par)
        _, g = pr.egrad(x)
        pr.close()
        f1.close()
        return float(np.sum(v * g))
    d = np.random.default_rng(63).normal(0, 1.0, theta.shape) * np.abs(theta)
    h = 1e-6
    fd = (S_ff1(theta + h * d) - S_ff1(theta - h * d)) / (2 * h)
    assert abs(fd - grad @ d) <= 1e-6 * abs(fd)
