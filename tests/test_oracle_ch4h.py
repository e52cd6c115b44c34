"""CPU: the CH4+H oracle against its pins.

Caracal's POTLIB surface is checked by central differences (Caracal's own
NUM_GRAD method).  The reference scales the energy by 0.03812 but the
gradient by 0.0201723 instead of 0.03812 * 0.52918 = 0.0201723416
(src/egrad_ch4h.f:263-279), so its analytic gradient is the derivative of its
energy times 0.0201723 / 0.0201723416; the check applies that factor, and the
raw 2.06e-6 mismatch is asserted as the reference's behaviour.
"""
import json
import os

import numpy as np
import pytest

from caracal_gb300.workloads import ch4h_dividing_surface
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
            g[i, d] = (orc.egrad("ch4h", a)[0][0] - orc.egrad("ch4h", b)[0][0]) / (2 * h)
    return g


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_ch4h_central_differences(seed):
    rng = np.random.default_rng(seed)
    q = ch4h_dividing_surface() + rng.normal(0, 0.08, (6, 3))
    _, g = orc.egrad("ch4h", q)
    gn = fd_grad(q, 1e-5)
    scale = np.max(np.abs(g))
    assert np.max(np.abs(g[0] * UNIT_RATIO - gn)) < 1e-8 * max(1.0, scale)
    # the unscaled mismatch is the reference's unit-factor inconsistency, not noise
    assert abs(np.max(np.abs(g[0] - gn)) / scale - (UNIT_RATIO - 1.0)) < 1e-6


def test_ch4h_reactant_asymptote_and_symmetry():
    q = ch4h_dividing_surface()
    far = q.copy()
    far[5] = q[0] * 30.0
    V_far, g_far = orc.egrad("ch4h", far)
    # CH4 at r(CH) = 1.09 A close to its minimum, H_b far: small forces on H_b
    assert abs(g_far[0][5]).max() < 1e-6
    # relabelling the three spectator methane H (atoms 3,4,5) leaves V unchanged
    perm = far[[0, 1, 3, 4, 2, 5]]
    assert abs(orc.egrad("ch4h", perm)[0][0] - V_far[0]) < 1e-12


def test_ch4h_golden():
    with open(os.path.join(GOLDEN, "ch4h_egrad.json")) as fh:
        gold = json.load(fh)
    V, g = orc.egrad("ch4h", np.array(gold["q"]))
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 1e-13 * np.max(np.abs(gold["V"]))
    assert np.max(np.abs(g - np.array(gold["dVdq"]))) <= 1e-12 * np.max(np.abs(gold["dVdq"]))
