"""Parameter gradients of QMDFF and dE-EVB losses on the device.

Caracal fits dE-EVB couplings with MINPACK's Levenberg-Marquardt on finite
differences (src/optimize_de.f90, src/lm_good.f `fdjac2`) and has no
gradient with respect to QMDFF force constants.  Here the loss gradients come
from hand-written derivative kernels:

* force matching, L = (1/G) sum_g |F_g(theta) - F_ref,g|^2 over G geometries,
  through ``cr_qmdff_param_vjp`` (every QMDFF term is linear in its force
  constant, so dF/dtheta is the term's gradient at unit constant);
* trajectories, through the adjoint of the ring-polymer velocity-Verlet step
  (:class:`TrajectoryAdjoint`, ``cr_adjoint_*``), which also needs
  Hessian-vector products (``cr_qmdff_hvp``, dual numbers on the term
  formulas).

theta, for a :class:`caracal_gb300.qmdff.QMDFF`, is the vector
[bond k (nbond), angle k (nangl), torsion V (ntors), charges q (natoms)].
The device works with the NCI pair products qq = eps1 q_i q_j (q_i q_j in the
Zahn form); :meth:`QMDFFParams.chain` maps their gradient to the charges.
"""
from __future__ import annotations

import copy

import numpy as np

from . import qmdff as Q


class QMDFFParams:
    """The linear parameters of a QMDFF as one vector."""

    def __init__(self, ff, zahn=False):
        self.ff = ff
        self.zahn = bool(zahn)
        self.nbond, self.nangl, self.ntors = len(ff.vbond), len(ff.vangl), len(ff.vtors)
        self.natoms = ff.n
        nci = np.asarray(ff.nci).reshape(-1, 3)
        self.pi, self.pj = nci[:, 0] - 1, nci[:, 1] - 1
        eps1, _ = Q.eps_factors()
        self.pf = np.ones(len(nci)) if self.zahn else eps1[nci[:, 2]]

    @property
    def size(self):
        return self.nbond + self.nangl + self.ntors + self.natoms

    def theta(self):
        f = self.ff
        return np.concatenate([np.asarray(f.vbond)[:, 1], np.asarray(f.vangl)[:, 1], np.asarray(f.vtors)[:, 1],
                               np.asarray(f.q, dtype=float)])

    def with_theta(self, theta):
        """A copy of the force field with the parameters theta."""
        t = np.asarray(theta, dtype=np.float64)
        if t.shape != (self.size,):
            raise ValueError(f"theta must have {self.size} entries")
        f = copy.deepcopy(self.ff)
        a, b, c = self.nbond, self.nbond + self.nangl, self.nbond + self.nangl + self.ntors
        f.vbond = np.array(f.vbond, dtype=float)
        f.vangl = np.array(f.vangl, dtype=float)
        f.vtors = np.array(f.vtors, dtype=float)
        f.vbond[:, 1] = t[:a]
        f.vangl[:, 1] = t[a:b]
        f.vtors[:, 1] = t[b:c]
        f.q = t[c:].copy()
        return f

    def chain(self, raw, theta=None):
        """Gradient over theta from the device's gradient over
        [bond k, angle k, torsion V, pair qq]: qq_p = f_p q_i q_j."""
        raw = np.asarray(raw, dtype=np.float64)
        q = np.asarray(self.ff.q if theta is None else theta[-self.natoms:], dtype=float)
        nv = self.nbond + self.nangl + self.ntors
        gq = np.zeros(self.natoms)
        gp = raw[nv:] * self.pf
        np.add.at(gq, self.pi, gp * q[self.pj])
        np.add.at(gq, self.pj, gp * q[self.pi])
        return np.concatenate([raw[:nv], gq])


def force_matching(params, theta, xyz, f_ref, tables=None, coul_cut=50.0):
    """Loss L = (1/G) sum_g |F_g - F_ref,g|^2 (F = -grad E, plain FP64) and
    dL/dtheta for G geometries xyz (G, n, 3)."""
    from .engine import QMDFFForceField
    gff = QMDFFForceField(params.with_theta(theta), tables, coul_cut=coul_cut, zahn=params.zahn)
    try:
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        _, g = gff.egrad(x)
        G = x.shape[0]
        d = -g - f_ref
        loss = float(np.sum(d * d) / G)
        # dL/dtheta = (2/G) sum (F - F_ref) . dF/dtheta = d/dtheta sum v . grad E
        v = (2.0 / G) * (g + f_ref)
        raw = gff.param_vjp(x, v)
    finally:
        gff.close()
    return loss, params.chain(raw, theta)


def torch_force_matching():
    """A torch.autograd.Function: loss = F.apply(theta, params, xyz, f_ref)
    with theta a float64 tensor; backward returns dL/dtheta from the device."""
    import torch

    class ForceMatchingLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, params, xyz, f_ref):
            loss, grad = force_matching(params, theta.detach().cpu().numpy(), xyz, f_ref)
            ctx.save_for_backward(torch.as_tensor(grad, dtype=theta.dtype))
            return theta.new_tensor(loss)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout * grad.to(gout.device), None, None, None

    return ForceMatchingLoss


class TrajectoryAdjoint:
    """Gradients of a loss of the final state of an NVE run (plain FP64,
    QMDFF engine, no transrot) by the adjoint of the step (cr_adjoint):
    ``forward()`` runs ``nsteps`` steps from the engine's state with
    checkpoints every ``every`` steps; ``backward(dl_dq, dl_dp)`` returns
    (dL/dtheta over the device's linear parameters, dL/dq0, dL/dp0)."""

    def __init__(self, engine, nsteps, every=20):
        import ctypes as C
        from . import _lib as L
        self._L, self.engine = L, engine
        h = C.c_void_p()
        L.check(L.lib().cr_adjoint_create(engine._h, int(nsteps), int(every), C.byref(h)), "cr_adjoint_create")
        self._h = h
        self.nlin = engine.ff.nparams

    def forward(self):
        self._L.check(self._L.lib().cr_adjoint_forward(self._h), "cr_adjoint_forward")

    def backward(self, dl_dq, dl_dp):
        L = self._L
        shape = self.engine.shape
        lq = np.ascontiguousarray(dl_dq, dtype=np.float64).reshape(shape)
        lp = np.ascontiguousarray(dl_dp, dtype=np.float64).reshape(shape)
        grad = np.zeros(max(self.nlin, 1))
        q0 = np.zeros(shape)
        p0 = np.zeros(shape)
        L.check(L.lib().cr_adjoint_backward(self._h, L.dptr(lq), L.dptr(lp), L.dptr(grad), L.dptr(q0), L.dptr(p0)),
                "cr_adjoint_backward")
        return grad[:self.nlin], q0, p0

    def close(self):
        if getattr(self, "_h", None):
            self._L.lib().cr_adjoint_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def trajectory_engine(params, theta, mass, nbeads, ntraj, dt_au, beta, q0, p0, tables=None):
    """An NVE plain-FP64 engine on the force field with parameters theta,
    started from (q0, p0) with its forces."""
    from .engine import QMDFFForceField, RPMDEngine
    gff = QMDFFForceField(params.with_theta(theta), tables, zahn=params.zahn,
                          coul_cut=10.0 if params.zahn else 50.0)
    eng = RPMDEngine(gff, mass, nbeads, ntraj, dt_au, beta=beta, thermostat="none", transrot=False,
                     precision="fp64")
    eng.set_state(q0, p0)
    return eng, gff


def torch_trajectory():
    """A torch.autograd.Function: (qK, pK) = F.apply(theta, q0, p0, spec) runs
    spec["nsteps"] NVE steps (checkpoints every spec["every"]) on the force
    field spec["params"].with_theta(theta); backward is the adjoint."""
    import torch

    class Trajectory(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, q0, p0, spec):
            th = theta.detach().cpu().numpy()
            eng, gff = trajectory_engine(spec["params"], th, spec["mass"], spec["nbeads"], spec["ntraj"],
                                         spec["dt_au"], spec["beta"], q0.detach().cpu().numpy(),
                                         p0.detach().cpu().numpy())
            adj = TrajectoryAdjoint(eng, spec["nsteps"], spec.get("every", 20))
            adj.forward()
            q, p, _, _, _ = eng.get_state()
            ctx.adj, ctx.keep, ctx.spec, ctx.theta = adj, (eng, gff), spec, th
            return theta.new_tensor(q), theta.new_tensor(p)

        @staticmethod
        def backward(ctx, gq, gp):
            gq = np.zeros(ctx.adj.engine.shape) if gq is None else gq.detach().cpu().numpy()
            gp = np.zeros(ctx.adj.engine.shape) if gp is None else gp.detach().cpu().numpy()
            raw, dq0, dp0 = ctx.adj.backward(gq, gp)
            grad = ctx.spec["params"].chain(raw, ctx.theta)
            ctx.adj.close()
            ctx.keep[0].close()
            ctx.keep[1].close()
            t = torch.as_tensor
            return t(grad), t(dq0), t(dp0), None

    return Trajectory
