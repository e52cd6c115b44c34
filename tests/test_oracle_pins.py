"""CPU: the oracle against its pins.

Caracal has no test suite and ships no expected outputs, and its Fortran
cannot be built here, so the oracle is pinned by (a) the Random123
known-answer vectors of Philox4x32-10, (b) Caracal's own gradient check
method -- central differences, NUM_GRAD (src/read_pes.f90:120-150,
src/gradient.f90:214-239) -- (c) published properties of the BKMP2
surface, (d) algebraic identities of Caracal's cosine transform, and
(e) the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py) that freeze it against regressions.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers():
    # Random123 kat_vectors, philox4x32_10
    assert orc.philox([0, 0, 0, 0], 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox([0xFFFFFFFF] * 4, 0xFFFFFFFF, 0xFFFFFFFF) == [0x408F276D, 0x41C83B0E,
                                                                    0xA20BC7C6, 0x6D5451FD]
    assert orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], 0xA4093822,
                      0x299F31D0) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_normals_are_standard():
    z = np.array([orc.normal_pair(7, t, i, b, 3, 1) for t in range(40) for i in range(10)
                  for b in range(40)]).ravel()
    n = len(z)
    assert abs(z.mean()) < 4 / np.sqrt(n) and abs(z.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    assert abs(np.mean(z ** 4) - 3.0) < 5 * np.sqrt(96.0 / n)          # Gaussian kurtosis


def test_normals_follow_box_muller_of_the_philox_words():
    """Each deviate pair is Box-Muller of 24-bit uniforms from two Philox
    words: u = (w0 >> 8) + 1, v = w1 >> 8 (times 2^-24); the FP32 polynomial
    log and sin/cos agree with FP64 libm to a few float ulps."""
    worst = 0.0
    for pair in range(64):
        w = orc.philox([pair >> 1, 5, 9, 2], 11, 3)
        wa, wb = (w[2], w[3]) if pair & 1 else (w[0], w[1])
        u = ((wa >> 8) + 1) * 2.0 ** -24
        v = (wb >> 8) * 2.0 ** -24
        r = np.sqrt(-2.0 * np.log(u))
        ref = np.array([r * np.cos(2 * np.pi * v), r * np.sin(2 * np.pi * v)])
        z = orc.normal_pair(11, 3, pair, 5, 9, 2)
        worst = max(worst, np.abs(z - ref).max() / max(1.0, r))
    assert worst < 1e-6


def test_bkmp2_published_properties():
    # H2 well: Schwenke curve minimum near r = 1.401 bohr, De ~ 0.1745 Eh
    v_h2, _ = orc.h3_pote([1.401, 40.0, 41.401])
    assert abs(v_h2 - (-0.17449577)) < 2e-6
    # collinear symmetric saddle at R1 = R2 = 1.757 bohr, barrier 9.61 kcal/mol
    v_ts, dv = orc.h3_pote([1.757, 1.757, 3.514])
    barrier_kcal = (v_ts - v_h2) * 627.5094743
    assert abs(barrier_kcal - 9.61) < 0.01
    assert abs(dv[0] - dv[1]) < 1e-12


def _fd_grad(q, h=1e-5):
    g = np.zeros_like(q)
    for i in range(q.shape[0]):
        for d in range(3):
            qp, qm = q.copy(), q.copy()
            qp[i, d] += h
            qm[i, d] -= h
            g[i, d] = (orc.egrad_h3(qp[None])[0][0] - orc.egrad_h3(qm[None])[0][0]) / (2 * h)
    return g


@pytest.mark.parametrize("geom", ["reactant", "compact", "bent", "equilateral"])
def test_egrad_h3_central_differences(geom):
    rng = np.random.default_rng(11)
    base = {
        "reactant": np.array([[0, 0, 0], [0, 0, 1.40], [0, 0, 6.1]]),
        "compact": np.array([[0, 0, 0], [0, 0, 1.0], [0.8, 0, 0.5]]),   # R < 1.15: CBEND/CSYM/CASYM on
        "bent": np.array([[0, 0, 0], [0, 0, 1.6], [1.5, 0, 2.5]]),
        "equilateral": np.array([[0, 0, 0], [2.0, 0, 0], [1.0, 1.7320508, 0]]),
    }[geom] + rng.normal(0, 0.02, (3, 3))
    _, g = orc.egrad_h3(base[None])
    gn = _fd_grad(base)
    # central-difference truncation error is O(h^2); near the equilateral cusp
    # of the London term it is ~1e-8 at h = 1e-5 bohr
    assert np.max(np.abs(g[0] - gn)) < 2e-8 * max(1.0, np.max(np.abs(g)))


def test_cos_transform_identity():
    # C.C = (I + R)/2: Caracal's rfft followed by irfft symmetrises over j -> -j
    rng = np.random.default_rng(3)
    for P in (1, 2, 3, 8, 16, 17, 32):
        x = rng.normal(size=P)
        y = orc.cos_transform(orc.cos_transform(x))
        xr = x[(-np.arange(P)) % P]
        assert np.max(np.abs(y - 0.5 * (x + xr))) < 1e-13


def test_transrot_removes_scaled_com_velocity():
    # with one bead the quirk vanishes (P^2 = 1): COM momentum and angular momentum go to 0
    mass = np.array([1837.0, 1837.0, 1837.0])
    cfg = orc.Config("h3", mass, 1, 1.0, 1.0)
    rng = np.random.default_rng(5)
    q = rng.normal(size=(1, 3, 3))
    p = rng.normal(size=(1, 3, 3))
    rc, p2 = orc.transrot(cfg, q, p)
    assert rc == 0
    assert np.max(np.abs(p2[0].sum(axis=0))) < 1e-12
    com = (q[0] * mass[:, None]).sum(0) / mass.sum()
    L = np.cross(q[0] - com, p2[0]).sum(0)
    assert np.max(np.abs(L)) < 1e-10
    # with P beads the total mass is P^2 sum(m) (src/transrot.f90:72-79): a
    # second, vectorised restatement of the same formulas must agree
    P = 4
    cfg = orc.Config("h3", mass, P, 1.0, 1.0)
    q = rng.normal(size=(1, P, 3, 3))
    p = rng.normal(size=(1, P, 3, 3))
    _, p2 = orc.transrot(cfg, q, p)
    m = mass[None, :, None]
    v = p[0] / m
    tm = P * P * mass.sum()
    vt = (v * m).sum(axis=(0, 1)) / tm
    xt = (q[0] * m).sum(axis=(0, 1)) / tm
    L = (np.cross(q[0], v) * m).sum(axis=(0, 1)) - np.cross(xt, vt) * tm
    xd = q[0] - xt
    I = (m[..., None] * (np.einsum("kia,kia->ki", xd, xd)[..., None, None] * np.eye(3)
                         - np.einsum("kia,kib->kiab", xd, xd))).sum(axis=(0, 1))
    w = np.linalg.solve(I, L)
    v2 = v - vt - np.cross(w, xd)
    assert np.max(np.abs(p2[0] - v2 * m)) < 1e-10 * np.max(np.abs(p2))


def test_golden_h3_fixtures():
    with open(os.path.join(GOLDEN, "h3_egrad.json")) as fh:
        gold = json.load(fh)
    q = np.array(gold["q"])
    V, g = orc.egrad_h3(q)
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 1e-13 * np.max(np.abs(gold["V"]))
    assert np.max(np.abs(g - np.array(gold["dVdq"]))) <= 1e-12 * np.max(np.abs(gold["dVdq"]))


def test_golden_h3_trajectory():
    with open(os.path.join(GOLDEN, "h3_traj.json")) as fh:
        gold = json.load(fh)
    c = gold["config"]
    cfg = orc.Config("h3", c["mass"], c["nbeads"], c["dt"], c["beta"], thermostat=c["thermostat"],
                     andersen_step=c["andersen_step"], pile_tau0=c["pile_tau0"], seed=c["seed"])
    q0 = np.array(gold["q0"])
    T = c["ntraj"]
    q = orc.init_positions(cfg, T, q0, c["sigma"])
    p = orc.init_momenta(cfg, T)
    f, _ = orc.init_forces(cfg, q)
    q1, p1, f1, e1, st = orc.run(cfg, q, p, f, c["nsteps"])
    assert np.max(np.abs(q1 - np.array(gold["q"]))) <= 1e-12 * np.max(np.abs(gold["q"]))
    assert np.max(np.abs(p1 - np.array(gold["p"]))) <= 1e-11 * np.max(np.abs(gold["p"]))
    assert not st.any()
