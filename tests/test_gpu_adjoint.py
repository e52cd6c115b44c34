"""GPU: derivative kernels for parameter fitting and adjoints.

Hessian-vector products (dual numbers on the plain-form term formulas) and
parameter gradients of v . grad E are checked against central finite
differences of the device's own FP64 gradient and of the oracle's; the
force-matching loss gradient against finite differences of the loss
(h = 1e-6 relative), in numpy and through the torch.autograd.Function.
"""
import numpy as np
import pytest

from caracal_gb300 import qmdff as Q
from caracal_gb300.engine import QMDFFForceField
from caracal_gb300.fit import QMDFFParams, force_matching, torch_force_matching
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def thermal(ff, nb, sigma=0.08, seed=1):
    rng = np.random.default_rng(seed)
    return ff.xyz[None] + rng.normal(0.0, sigma, (nb,) + ff.xyz.shape)


@pytest.mark.parametrize("zahn", [False, True])
def test_hvp_matches_finite_differences(require_gpu, zahn):
    ff = Q.alkane(nc=4)
    gff = QMDFFForceField(ff, zahn=zahn, coul_cut=10.0 if zahn else 50.0)
    x = thermal(ff, 6)
    w = np.random.default_rng(2).normal(0.0, 1.0, x.shape)
    e, g, hw = gff.hvp(x, w)
    e0, g0 = gff.egrad(x)
    assert rel_err(g, g0) <= 1e-12
    assert rel_err(e, e0) <= 1e-12
    h = 1e-5
    _, gp = gff.egrad(x + h * w)
    _, gm = gff.egrad(x - h * w)
    assert rel_err(hw, (gp - gm) / (2 * h)) <= 1e-7
    gff.close()


def test_hvp_matches_oracle_finite_differences(require_gpu):
    ff = Q.alkane(nc=3)
    orc.set_qmdff(ff, Q.ElementTables.caracal())
    gff = QMDFFForceField(ff)
    x = thermal(ff, 3, seed=4)
    w = np.random.default_rng(5).normal(0.0, 1.0, x.shape)
    _, _, hw = gff.hvp(x, w)
    h = 1e-5
    _, gp = orc.egrad("qmdff", x + h * w)
    _, gm = orc.egrad("qmdff", x - h * w)
    assert rel_err(hw, (gp - gm) / (2 * h)) <= 1e-7
    gff.close()


def test_param_vjp_matches_finite_differences(require_gpu):
    ff = Q.alkane(nc=4)
    params = QMDFFParams(ff)
    x = thermal(ff, 5, seed=7)
    v = np.random.default_rng(8).normal(0.0, 1.0, x.shape)
    theta = params.theta()
    gff = QMDFFForceField(ff)
    grad = params.chain(gff.param_vjp(x, v))
    gff.close()

    def s(th):
        f = QMDFFForceField(params.with_theta(th))
        _, g = f.egrad(x)
        f.close()
        return float(np.sum(v * g))

    rng = np.random.default_rng(9)
    for _ in range(3):
        d = rng.normal(0.0, 1.0, theta.shape) * np.abs(theta)
        h = 1e-6
        fd = (s(theta + h * d) - s(theta - h * d)) / (2 * h)
        assert abs(fd - grad @ d) <= 1e-7 * max(abs(fd), 1e-12)
    # single parameters of every kind (bond, angle, torsion, charge)
    nb, na, nt = params.nbond, params.nangl, params.ntors
    for k in (0, nb + 1, nb + na + 2, nb + na + nt + 3):
        d = np.zeros_like(theta)
        d[k] = 1.0
        h = 1e-6 * max(abs(theta[k]), 1e-3)
        fd = (s(theta + h * d) - s(theta - h * d)) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 * max(abs(fd), 1e-10)


def test_force_matching_gradient(require_gpu):
    ff = Q.alkane(nc=4)
    params = QMDFFParams(ff)
    x = thermal(ff, 16, seed=11)
    f = QMDFFForceField(ff)
    _, g = f.egrad(x)
    f.close()
    f_ref = -g
    theta = params.theta() * np.random.default_rng(12).uniform(0.9, 1.1, params.size)
    loss, grad = force_matching(params, theta, x, f_ref)
    assert loss > 0
    rng = np.random.default_rng(13)
    d = rng.normal(0.0, 1.0, theta.shape) * np.abs(theta)
    h = 1e-6
    lp, _ = force_matching(params, theta + h * d, x, f_ref)
    lm, _ = force_matching(params, theta - h * d, x, f_ref)
    assert abs((lp - lm) / (2 * h) - grad @ d) <= 1e-6 * abs(grad @ d)
    # unperturbed parameters: the reference forces, zero loss and gradient
    l0, g0 = force_matching(params, params.theta(), x, f_ref)
    assert l0 == 0.0 and np.all(g0 == 0.0)


def test_force_matching_torch_function(require_gpu):
    torch = pytest.importorskip("torch")
    ff = Q.alkane(nc=3)
    params = QMDFFParams(ff)
    x = thermal(ff, 8, seed=21)
    f = QMDFFForceField(ff)
    _, g = f.egrad(x)
    f.close()
    theta0 = params.theta() * np.random.default_rng(22).uniform(0.9, 1.1, params.size)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    fn = torch_force_matching()
    loss = fn.apply(theta, params, x, -g)
    loss.backward()
    _, grad = force_matching(params, theta0, x, -g)
    assert np.allclose(theta.grad.numpy(), grad, rtol=0, atol=0)


def trajectory_case(nc=3, nbeads=4, ntraj=2, seed=31):
    from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
    ff = Q.alkane(nc=nc)
    params = QMDFFParams(ff)
    mass = np.array([mass_au("C" if z == 6 else "H") for z in ff.at])
    beta = beta_from_kelvin(300.0)
    rng = np.random.default_rng(seed)
    shape = (ntraj, nbeads, ff.n, 3)
    q0 = ff.xyz[None, None] + rng.normal(0.0, 0.05, shape)
    p0 = rng.normal(0.0, 1.0, shape) * np.sqrt(mass[None, None, :, None] * nbeads / beta)
    return params, mass, beta, dt_fs_to_au(0.5), q0, p0


def run_loss(params, theta, mass, beta, dt, q0, p0, a, b, nsteps):
    from caracal_gb300.fit import trajectory_engine
    eng, gff = trajectory_engine(params, theta, mass, q0.shape[1], q0.shape[0], dt, beta, q0, p0)
    eng.run(nsteps)
    q, p, _, _, _ = eng.get_state()
    eng.close()
    gff.close()
    return float(np.sum(a * q) + np.sum(b * p))


@pytest.mark.parametrize("every", [7, 40])
def test_trajectory_adjoint_matches_finite_differences(require_gpu, every):
    from caracal_gb300.fit import TrajectoryAdjoint, trajectory_engine
    params, mass, beta, dt, q0, p0 = trajectory_case()
    K = 30
    rng = np.random.default_rng(41)
    a = rng.normal(0.0, 1.0, q0.shape)
    b = rng.normal(0.0, 1.0, q0.shape) / np.sqrt(mass[None, None, :, None])
    theta = params.theta()
    eng, gff = trajectory_engine(params, theta, mass, q0.shape[1], q0.shape[0], dt, beta, q0, p0)
    adj = TrajectoryAdjoint(eng, K, every)
    adj.forward()
    raw, dq0, dp0 = adj.backward(a, b)
    grad = params.chain(raw, theta)
    # the engine ends in its state after step K, equal to a plain run
    qk, pk, _, _, _ = eng.get_state()
    e2, g2 = trajectory_engine(params, theta, mass, q0.shape[1], q0.shape[0], dt, beta, q0, p0)
    e2.run(K)
    q2, p2, _, _, _ = e2.get_state()
    assert np.array_equal(qk, q2) and np.array_equal(pk, p2)
    for x in (adj, eng, gff, e2, g2):
        x.close()
    # parameters: central differences along random directions
    for trial in range(2):
        d = rng.normal(0.0, 1.0, theta.shape) * np.abs(theta)
        h = 1e-5
        fd = (run_loss(params, theta + h * d, mass, beta, dt, q0, p0, a, b, K) -
              run_loss(params, theta - h * d, mass, beta, dt, q0, p0, a, b, K)) / (2 * h)
        assert abs(fd - grad @ d) <= 2e-6 * abs(fd), (trial, fd, grad @ d)
    # initial state
    dq = rng.normal(0.0, 1e-3, q0.shape)
    dp = rng.normal(0.0, 1e-3, q0.shape) * np.sqrt(mass[None, None, :, None] * q0.shape[1] / beta)
    h = 1e-4
    fd = (run_loss(params, theta, mass, beta, dt, q0 + h * dq, p0 + h * dp, a, b, K) -
          run_loss(params, theta, mass, beta, dt, q0 - h * dq, p0 - h * dp, a, b, K)) / (2 * h)
    assert abs(fd - (np.sum(dq0 * dq) + np.sum(dp0 * dp))) <= 2e-6 * abs(fd)


def test_trajectory_torch_function(require_gpu):
    torch = pytest.importorskip("torch")
    from caracal_gb300.fit import torch_trajectory
    params, mass, beta, dt, q0, p0 = trajectory_case(seed=51)
    spec = dict(params=params, mass=mass, nbeads=q0.shape[1], ntraj=q0.shape[0], dt_au=dt, beta=beta,
                nsteps=20, every=5)
    theta = torch.tensor(params.theta(), dtype=torch.float64, requires_grad=True)
    q0t = torch.tensor(q0, requires_grad=True)
    p0t = torch.tensor(p0, requires_grad=True)
    qk, pk = torch_trajectory().apply(theta, q0t, p0t, spec)
    ref = torch.tensor(q0)
    loss = 0.5 * ((qk - ref) ** 2).sum() + 1e-3 * (pk ** 2).sum()
    loss.backward()
    d = np.random.default_rng(52).normal(0.0, 1.0, params.size) * np.abs(params.theta())
    h = 1e-5

    def L(th):
        from caracal_gb300.fit import trajectory_engine
        eng, gff = trajectory_engine(params, th, mass, q0.shape[1], q0.shape[0], dt, beta, q0, p0)
        eng.run(20)
        q, p, _, _, _ = eng.get_state()
        eng.close()
        gff.close()
        return 0.5 * np.sum((q - q0) ** 2) + 1e-3 * np.sum(p ** 2)
    fd = (L(params.theta() + h * d) - L(params.theta() - h * d)) / (2 * h)
    assert abs(fd - theta.grad.numpy() @ d) <= 2e-6 * abs(fd)
    assert q0t.grad is not None and p0t.grad is not None
