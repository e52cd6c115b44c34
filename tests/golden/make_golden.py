"""Regenerate the golden fixtures of this directory from the oracle.

Caracal ships no expected outputs, so these fixtures freeze the oracle's
results (themselves pinned by central differences, published BKMP2
properties and Philox known answers) for regression and cross-machine
checks.  Run: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as orc  # noqa: E402
from caracal_gb300.workloads import ch4h_dividing_surface, ch4oh_geometry, geh4oh_geometry, h3_collinear  # noqa: E402
from caracal_gb300.units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au  # noqa: E402


def h3_egrad():
    rng = np.random.default_rng(20261203)
    geoms = [h3_collinear() + rng.normal(0, 0.05, (3, 3)) for _ in range(8)]
    geoms += [np.array([[0, 0, 0], [0, 0, 1.0], [0.8, 0, 0.5]]) + rng.normal(0, 0.02, (3, 3))
              for _ in range(4)]                     # compact: R < 1.15 bohr terms active
    geoms += [np.array([[0, 0, 0], [2.0, 0, 0], [1.0, 1.7320508, 0.0]]),   # equilateral
              np.array([[0, 0, 0], [0, 0, 1.757], [0, 0, 3.514]]),         # collinear saddle
              np.array([[0, 0, 0], [0, 0, 0.9], [0, 0, 1.8]])]             # R <= 0.95: Johnson branch
    q = np.array(geoms)
    V, g = orc.egrad_h3(q)
    return {"q": q.tolist(), "V": V.tolist(), "dVdq": g.tolist()}


def h3_traj(thermostat):
    mass = [mass_au("H")] * 3
    c = dict(mass=mass, nbeads=4, ntraj=2, nsteps=60, dt=dt_fs_to_au(0.1),
             beta=beta_from_kelvin(300.0), thermostat=thermostat, andersen_step=20,
             pile_tau0=dt_fs_to_au(100.0), seed=20261203,
             sigma=float(angstrom_to_bohr(0.01)))
    cfg = orc.Config("h3", mass, c["nbeads"], c["dt"], c["beta"], thermostat=thermostat,
                     andersen_step=c["andersen_step"], pile_tau0=c["pile_tau0"], seed=c["seed"])
    q0 = h3_collinear()
    q = orc.init_positions(cfg, c["ntraj"], q0, c["sigma"])
    p = orc.init_momenta(cfg, c["ntraj"])
    f, _ = orc.init_forces(cfg, q)
    q1, p1, f1, e1, st = orc.run(cfg, q, p, f, c["nsteps"])
    return {"config": c, "q0": q0.tolist(), "q": q1.tolist(), "p": p1.tolist(), "epot": e1.tolist()}


def ch4h_egrad():
    rng = np.random.default_rng(20261204)
    q = np.array([ch4h_dividing_surface() + rng.normal(0, 0.08, (6, 3)) for _ in range(12)])
    V, g = orc.egrad("ch4h", q)
    return {"q": q.tolist(), "V": V.tolist(), "dVdq": g.tolist()}


def ch4oh_egrad():
    rng = np.random.default_rng(20261205)
    q = np.array([ch4oh_geometry() + rng.normal(0, 0.08, (7, 3)) for _ in range(12)])
    V, g = orc.egrad("ch4oh", q)
    return {"q": q.tolist(), "V": V.tolist(), "dVdq": g.tolist()}


def geh4oh_egrad():
    rng = np.random.default_rng(20261206)
    q = np.array([geh4oh_geometry() + rng.normal(0, 0.08, (7, 3)) for _ in range(12)])
    V, g = orc.egrad("geh4oh", q)
    return {"q": q.tolist(), "V": V.tolist(), "dVdq": g.tolist()}


if __name__ == "__main__":
    with open(os.path.join(HERE, "h3_egrad.json"), "w") as fh:
        json.dump(h3_egrad(), fh)
    with open(os.path.join(HERE, "h3_traj.json"), "w") as fh:
        json.dump(h3_traj("andersen"), fh)
    with open(os.path.join(HERE, "h3_traj_pile.json"), "w") as fh:
        json.dump(h3_traj("pile"), fh)
    with open(os.path.join(HERE, "ch4h_egrad.json"), "w") as fh:
        json.dump(ch4h_egrad(), fh)
    with open(os.path.join(HERE, "ch4oh_egrad.json"), "w") as fh:
        json.dump(ch4oh_egrad(), fh)
    with open(os.path.join(HERE, "geh4oh_egrad.json"), "w") as fh:
        json.dump(geh4oh_egrad(), fh)
    print("golden fixtures written")
