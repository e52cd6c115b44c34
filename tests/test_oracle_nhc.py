"""CPU: the oracle's Nose-Hoover chain (src/nhc.f90) against a second,
independent transcription of the reference loop, and the chain's effect."""
import math

import numpy as np

from caracal_gb300.units import K_BOLTZMANN_AU, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from oracle import oracle as orc


def nhc_reference(p, mass, nbeads, dt, kelvin, nose_q, vnh):
    """Line by line after src/nhc.f90:47-171 and src/mdinit.f90:128-147."""
    natoms = len(mass)
    nfree = 3 * natoms
    qterm = K_BOLTZMANN_AU * kelvin * nose_q * nose_q
    qnh = [nfree * qterm, qterm, qterm, qterm]
    gnh = [0.0] * 4
    vnh = list(vnh)
    ekt = float(np.float32(np.float32(1.380649e-23) / np.float32(4.3597447e-18))) * kelvin
    nc, ns = 5, 3
    dtc = dt / nc
    w1 = 1.0 / (2.0 - 2.0 ** (1.0 / 3.0))
    w = [w1, 1.0 - 2.0 * w1, w1]
    scale = 1.0
    eksum = 0.0
    for i in range(natoms):
        for j in range(nbeads):
            v = p[j, i]
            eksum = eksum + float(v @ v) / (2.0 * mass[i]) / nbeads / nbeads
    for _ in range(nc):
        for j in range(ns):
            dts = w[j] * dtc
            dt2, dt4, dt8 = 0.5 * dts, 0.25 * dts, 0.125 * dts
            gnh[3] = (qnh[2] * vnh[2] * vnh[2] - ekt) / qnh[3]
            vnh[3] = vnh[3] + gnh[3] * dt4
            gnh[2] = (qnh[1] * vnh[1] * vnh[1] - ekt) / qnh[2]
            e = math.exp(-vnh[3] * dt8)
            vnh[2] = e * (vnh[2] * e + gnh[2] * dt4)
            gnh[1] = (qnh[0] * vnh[0] * vnh[0] - ekt) / qnh[1]
            e = math.exp(-vnh[2] * dt8)
            vnh[1] = e * (vnh[1] * e + gnh[1] * dt4)
            gnh[0] = (2.0 * eksum - nfree * ekt) / qnh[0]
            e = math.exp(-vnh[1] * dt8)
            vnh[0] = e * (vnh[0] * e + gnh[0] * dt4)
            e = math.exp(-vnh[0] * dt2)
            scale = scale * e
            eksum = eksum * e * e
            gnh[0] = (2.0 * eksum - nfree * ekt) / qnh[0]
            e = math.exp(-vnh[1] * dt8)
            vnh[0] = e * (vnh[0] * e + gnh[0] * dt4)
            gnh[1] = (qnh[0] * vnh[0] * vnh[0] - ekt) / qnh[1]
            e = math.exp(-vnh[2] * dt8)
            vnh[1] = e * (vnh[1] * e + gnh[1] * dt4)
            gnh[2] = (qnh[1] * vnh[1] * vnh[1] - ekt) / qnh[2]
            e = math.exp(-vnh[3] * dt8)
            vnh[2] = e * (vnh[2] * e + gnh[2] * dt4)
            gnh[3] = (qnh[2] * vnh[2] * vnh[2] - ekt) / qnh[3]
            vnh[3] = vnh[3] + gnh[3] * dt4
    return np.array(vnh), scale * p


def test_nhc_matches_second_transcription():
    mass = np.array([mass_au("H")] * 3)
    P, kelvin, dt_fs = 8, 300.0, 0.1
    dt = dt_fs_to_au(dt_fs)
    nq = nose_q_to_au(100.0, dt_fs)
    cfg = orc.Config("h3", mass, P, dt, beta_from_kelvin(kelvin), thermostat="nhc", nose_q=nq)
    rng = np.random.default_rng(3)
    p = rng.normal(0, 30.0, (P, 3, 3))   # hot: the chain must cool it
    vnh = np.array([1e-4, -2e-4, 3e-5, 0.0])
    for _ in range(4):
        v_ref, p_ref = nhc_reference(p, mass, P, dt, 1.0 / (beta_from_kelvin(kelvin) * K_BOLTZMANN_AU), nq, vnh)
        v_or, p_or = orc.nhc_half(cfg, vnh, p)
        np.testing.assert_allclose(v_or, v_ref, rtol=1e-13, atol=1e-300)
        np.testing.assert_allclose(p_or, p_ref, rtol=1e-13)
        vnh, p = v_or, p_or


def test_nhc_drives_kinetic_energy_down_when_hot():
    mass = np.array([mass_au("H")] * 3)
    P, dt_fs = 4, 0.5
    dt = dt_fs_to_au(dt_fs)
    cfg = orc.Config("h3", mass, P, dt, beta_from_kelvin(300.0), thermostat="nhc",
                     nose_q=nose_q_to_au(10.0, dt_fs))
    p = np.random.default_rng(4).normal(0, 60.0, (P, 3, 3))
    vnh = np.zeros(4)
    ek0 = sum(float(p[j, i] @ p[j, i]) / (2 * mass[i]) for i in range(3) for j in range(P))
    for _ in range(200):
        vnh, p = orc.nhc_half(cfg, vnh, p)
    ek1 = sum(float(p[j, i] @ p[j, i]) / (2 * mass[i]) for i in range(3) for j in range(P))
    assert ek1 < ek0 and vnh[0] > 0.0
