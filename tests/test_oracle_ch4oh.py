"""CPU: the CH4+OH oracle against its pins.

As for CH4+H, Caracal's POTLIB surface scales the energy by 0.03812 but the
gradient by 0.0201723 instead of 0.03812 * 0.52918 (src/egrad_ch4oh.f:263-
279), so its analytic gradient is the derivative of its energy times
0.0201723 / 0.0201723416; the central-difference check (Caracal's NUM_GRAD
method) applies that factor.
"""
import json
import os

import numpy as np
import pytest

from caracal_gb300.workloads import ch4oh_geometry
from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
UNIT_RATIO = 0.03812 * 0.52918 / 0.0201723


def fd_grad(q, h):
    g = np.zeros_like(q)
    for i in range(q.shape[0]):
        for d in range(3):
            a, b = q.copy(), q.copy()
            a[i, d] += h
            b[i, d] -= h
            g[i, d] = (orc.egrad("ch4oh", a)[0][0] - orc.egrad("ch4oh", b)[0][0]) / (2 * h)
    return g


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ch4oh_central_differences(seed):
    rng = np.random.default_rng(seed)
    q = ch4oh_geometry() + rng.normal(0, 0.08, (7, 3))
    _, g = orc.egrad("ch4oh", q)
    gn = fd_grad(q, 1e-5)
    scale = np.max(np.abs(g))
    assert np.max(np.abs(g[0] * UNIT_RATIO - gn)) < 1e-8 * max(1.0, scale)


def test_ch4oh_far_oh_and_symmetry():
    q = ch4oh_geometry(r_ho_ang=12.0)
    V, g = orc.egrad("ch4oh", q)
    # CH4 + OH far apart: the O-H stretch and H-O-H bends vanish with distance
    # and the H(i)-O switch, so the forces on OH come from the O-H bond alone
    assert abs(g[0][5] + g[0][6]).max() < 1e-6
    # relabelling the three spectator methane H (atoms 3,4,5) leaves V unchanged
    perm = q[[0, 1, 3, 4, 2, 5, 6]]
    assert abs(orc.egrad("ch4oh", perm)[0][0] - V[0]) < 1e-12


def test_ch4oh_oh_bond_minimum():
    # the O-H Morse term alone has its minimum at r0hh = 0.9706 A: stretching
    # the far hydroxyl raises the energy on both sides
    e = [orc.egrad("ch4oh", ch4oh_geometry(r_ho_ang=12.0, r_oh_ang=r))[0][0] for r in (0.90, 0.9706, 1.05)]
    assert e[1] < e[0] and e[1] < e[2]


def test_ch4oh_golden():
    with open(os.path.join(GOLDEN, "ch4oh_egrad.json")) as fh:
        gold = json.load(fh)
    V, g = orc.egrad("ch4oh", np.array(gold["q"]))
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 1e-13 * np.max(np.abs(gold["V"]))
    assert np.max(np.abs(g - np.array(gold["dVdq"]))) <= 1e-12 * np.max(np.abs(gold["dVdq"]))
