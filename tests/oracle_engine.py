"""Test helper: the oracle (CPU restatement) behind the engine interface that
caracal_gb300.calc_rate drives, so the calc_rate pipeline can run on the
oracle and on the CUDA engine from the same seeds and be compared.

Only the methods calc_rate uses are provided; every call maps onto the
oracle's restatement of the same Caracal routine (init_positions, mdinit
with umbrella mode 0, run / run_umbrella / run_parent, recross_children).
"""
import numpy as np

from oracle import oracle as orc


class OracleEngine:
    def __init__(self, pes, mass, nbeads, ntraj, dt_au, beta=None, thermostat="none", andersen_step=70,
                 pile_tau0_au=0.0, transrot=True, precision="fp64", seed=0, traj0=0, nose_q_au=0.0, nm_mode=0):
        self.pes = pes
        self.mass = np.ascontiguousarray(mass, dtype=np.float64)
        self.P, self.T, self.N = int(nbeads), int(ntraj), len(self.mass)
        self.kw = dict(thermostat=thermostat, andersen_step=andersen_step, pile_tau0=pile_tau0_au,
                       transrot=transrot, seed=seed, nose_q=nose_q_au, nm_mode=nm_mode)
        self.dt, self.beta = float(dt_au), float("inf") if beta is None else float(beta)
        self.traj0 = int(traj0)
        self._cfg()
        shape = (self.T, self.P, self.N, 3)
        self.q, self.p, self.f = np.zeros(shape), np.zeros(shape), np.zeros(shape)
        self.e = np.zeros(self.T)
        self.st = np.zeros(self.T, dtype=np.int32)
        self.istep = 0
        self.mode = "plain"
        self.umb = None
        self.sampling = False
        self.stats = None
        self.dxi = None
        self.xd = None
        self.qpar = None
        self.nrun = 0

    def _cfg(self):
        self.cfg = orc.Config(self.pes, self.mass, self.P, self.dt, self.beta, **self.kw)

    def close(self):
        pass

    def init_positions(self, q0, sigma=0.0):
        self.q = orc.init_positions(self.cfg, self.T, np.asarray(q0, dtype=np.float64).reshape(self.N, 3), sigma,
                                    traj0=self.traj0)

    def set_state(self, q, p, f=None):
        self.q = np.array(q, dtype=np.float64).reshape(self.q.shape)
        self.p = np.array(p, dtype=np.float64).reshape(self.q.shape)
        self.f = orc.init_forces(self.cfg, self.q)[0] if f is None else np.array(f, dtype=np.float64)

    def get_state(self):
        return self.q.copy(), self.p.copy(), self.f.copy(), self.e.copy(), self.st.copy()

    def compute_forces(self):
        self.f, self.e = orc.init_forces(self.cfg, self.q)

    def mdinit(self, draw=0):
        self.f, self.e = orc.init_forces(self.cfg, self.q)
        if self.mode == "umbrella":
            c, k = self.umb
            for t in range(self.T):
                _, self.f[t] = orc.umbrella_bias(self.cfg, self.xd, c[t], k[t], self.q[t], self.f[t])
        if self.kw["thermostat"] == "none":
            self.p = np.zeros_like(self.q)
        else:
            self.p = orc.init_momenta(self.cfg, self.T, traj0=self.traj0, draw=draw)

    def set_andersen_step(self, n):
        self.kw["andersen_step"] = int(n)
        self._cfg()

    @staticmethod
    def _xd(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal):
        return orc.make_xidef([a - 1 for a in reac1], [a - 1 for a in reac2],
                              (bond_form[0] - 1, bond_form[1] - 1), (bond_break[0] - 1, bond_break[1] - 1),
                              form_ref, break_ref, r_inf, xi_ideal)

    def set_umbrella(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, centers, kforce,
                     nbins=0, lo=0.0, hi=1.0, xi_ideal=1.0):
        self.xd = self._xd(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal)
        c = np.ascontiguousarray(np.broadcast_to(centers, (self.T,)), dtype=np.float64)
        k = np.ascontiguousarray(np.broadcast_to(kforce, (self.T,)), dtype=np.float64)
        self.umb = (c, k)
        self.mode = "umbrella"
        self.sampling = False
        self.stats = dict(xsum=np.zeros(self.T), xsum2=np.zeros(self.T), hist=np.zeros((self.T, 1)))

    def umbrella_sampling(self, on=True):
        self.sampling = bool(on)

    def umbrella_stats(self, reset=False):
        s = self.stats
        out = (s["xsum"].copy(), s["xsum2"].copy(), np.zeros((self.T, 0)))
        if reset:
            for v in s.values():
                v[...] = 0.0
        return out

    def set_parent(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal=1.0):
        self.xd = self._xd(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal)
        self.mode = "parent"
        self.dxi = None

    def set_recross(self, reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal=1.0,
                    max_steps=1):
        self.xd = self._xd(reac1, reac2, bond_form, bond_break, form_ref, break_ref, r_inf, xi_ideal)
        self.mode = "children"

    def init_children(self, q_parent):
        self.qpar = np.array(q_parent, dtype=np.float64).reshape(self.P, self.N, 3)
        self.nrun = 0

    def run(self, nsteps, check=True):
        if self.mode == "children":
            self.nrun += int(nsteps)
        elif self.mode == "umbrella":
            c, k = self.umb
            self.q, self.p, self.f, self.e, self.st, self.stats = orc.run_umbrella(
                self.cfg, self.xd, self.q, self.p, self.f, nsteps, c, k, istep0=self.istep, traj0=self.traj0,
                sampling=self.sampling, stats=self.stats)
        elif self.mode == "parent":
            self.q, self.p, self.f, self.e, self.st, self.dxi = orc.run_parent(
                self.cfg, self.xd, self.q, self.p, self.f, nsteps, istep0=self.istep, traj0=self.traj0,
                dxi=self.dxi)
        else:
            self.q, self.p, self.f, self.e, self.st = orc.run(self.cfg, self.q, self.p, self.f, nsteps,
                                                             istep0=self.istep, traj0=self.traj0)
        self.istep += int(nsteps)
        if check and self.st.any():
            raise RuntimeError("oracle trajectory failed")
        return 0

    def kappa(self, max_steps):
        num, den, w = orc.recross_children(self.cfg, self.xd, self.T, self.qpar, self.nrun, traj0=self.traj0)
        return num, den, w
