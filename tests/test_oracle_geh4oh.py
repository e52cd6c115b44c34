"""CPU: the GeH4 + OH oracle (src/egrad_geh4oh.f, the CH4 + OH surface code
with its own constants) against its pins: central differences with
Caracal's 0.0201723 / 0.0201723416 gradient factor (as for CH4 + OH), the
equivalence of the three spectator H, the far-OH limit, and the two
routines where it departs from CH4 + OH (the pyramid angle 0.678 pi in
refangles, sphi at every Ge-H distance in switchf).  Parity unpinned
beyond these: Caracal ships no GeH4 + OH outputs."""
import json
import os

import numpy as np
import pytest

from caracal_gb300.workloads import geh4oh_geometry
from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
UNIT_RATIO = 0.03812 * 0.52918 / 0.0201723
ANG = 1.0 / 0.52917721092


def fd_grad(q, h):
    g = np.zeros_like(q)
    for i in range(q.shape[0]):
        for d in range(3):
            a, b = q.copy(), q.copy()
            a[i, d] += h
            b[i, d] -= h
            g[i, d] = (orc.egrad("geh4oh", a)[0][0] - orc.egrad("geh4oh", b)[0][0]) / (2 * h)
    return g


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_geh4oh_central_differences(seed):
    rng = np.random.default_rng(seed)
    q = geh4oh_geometry() + rng.normal(0, 0.08, (7, 3))
    _, g = orc.egrad("geh4oh", q)
    gn = fd_grad(q, 1e-5)
    assert np.max(np.abs(g[0] * UNIT_RATIO - gn)) < 1e-8 * max(1.0, np.max(np.abs(g)))


def test_geh4oh_symmetry_and_far_oh():
    # the Ge-O Morse range (acb = 0.676 / A against CH4 + OH's 2.987) makes
    # GeH4 + OH decay slowly: at 20 A the net force on OH is 1e-8
    q = geh4oh_geometry(r_ho_ang=20.0)
    V, g = orc.egrad("geh4oh", q)
    assert abs(g[0][5] + g[0][6]).max() < 1e-7
    perm = q[[0, 1, 3, 4, 2, 5, 6]]
    assert abs(orc.egrad("geh4oh", perm)[0][0] - V[0]) < 1e-12
    # a rigid rotation leaves V unchanged
    c, s = np.cos(0.7), np.sin(0.7)
    rot = np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])
    assert abs(orc.egrad("geh4oh", q @ rot.T)[0][0] - V[0]) < 1e-12


def test_geh4oh_departs_from_ch4oh_where_the_sources_differ():
    # with every Ge-H at the CH4 + OH cut-off's far side the CH4 + OH code
    # has sphi = 0, GeH4 + OH still evaluates it: a methane H pulled from 3.5
    # to 6 A changes the GeH4 + OH energy smoothly (no step at 3.8 A) and the
    # gradient stays the derivative of the energy across 3.8 A
    q0 = geh4oh_geometry()
    u = (q0[2] - q0[1]) / np.linalg.norm(q0[2] - q0[1])
    def at(r):
        q = q0.copy()
        q[2] = q0[1] + u * r * ANG
        return q
    for r in (3.79, 3.8, 3.81):
        q = at(r)
        _, g = orc.egrad("geh4oh", q)
        gn = fd_grad(q, 1e-5)
        assert np.max(np.abs(g[0] * UNIT_RATIO - gn)) < 1e-8 * max(1.0, np.max(np.abs(g)))
    e = [orc.egrad("geh4oh", at(r))[0][0] for r in np.linspace(3.7, 3.9, 21)]
    d2 = np.diff(e, 2)
    assert np.max(np.abs(d2)) < 1e-6
    # finite out to the float range of the switch's exp and beyond (FP64)
    V, g = orc.egrad("geh4oh", np.array([at(r) for r in (10.0, 15.0, 20.0)]))
    assert np.isfinite(V).all() and np.isfinite(g).all()


def test_geh4oh_golden():
    with open(os.path.join(GOLDEN, "geh4oh_egrad.json")) as fh:
        gold = json.load(fh)
    V, g = orc.egrad("geh4oh", np.array(gold["q"]))
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 1e-13 * np.max(np.abs(gold["V"]))
    assert np.max(np.abs(g - np.array(gold["dVdq"]))) <= 1e-12 * np.max(np.abs(gold["dVdq"]))
