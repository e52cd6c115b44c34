"""GPU: batches of trajectory classes (cr_batch) against the same engines run
one after another.

A batch launches every class's kernels from one graph per chunk of steps; the
kernels and their order within a class are those of cr_engine_run, so the
states must be bit-identical to separate runs.
"""
import numpy as np
import pytest

from caracal_gb300 import RPMDBatch, RPMDEngine
from caracal_gb300 import workloads as W
from caracal_gb300.engine import QMDFFForceField

pytestmark = pytest.mark.gpu


def small_classes():
    return [W.h3_config(ntraj=24, nbeads=8, thermostat="pile"),
            W.ch4h_md_config(ntraj=6, nbeads=32),
            W.ch4oh_md_config(ntraj=3, nbeads=64),
            W.qmdff_config(ntraj=2, nbeads=128, nc=4)]


def build(wl, precision, ff=None, andersen_step=None):
    pes = ff if wl.pes == "qmdff" else wl.pes
    eng = RPMDEngine(pes, wl.mass, wl.nbeads, wl.ntraj, wl.dt_au, beta=wl.beta, thermostat=wl.thermostat,
                     andersen_step=andersen_step or wl.andersen_step, pile_tau0_au=wl.pile_tau0_au,
                     transrot=wl.transrot, precision=precision, seed=wl.seed)
    eng.init_positions(wl.q0, wl.sigma_bohr)
    eng.init_momenta()
    eng.compute_forces()
    return eng


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_equals_separate_runs(require_gpu, precision):
    classes = small_classes()
    ff = QMDFFForceField(classes[3].extra["ff"])
    a = [build(wl, precision, ff, andersen_step=3) for wl in classes]
    b = [build(wl, precision, ff, andersen_step=3) for wl in classes]
    batch = RPMDBatch(a, chunk_steps=3)
    batch.run(7)           # two chunk graphs and a remainder of one step
    batch.run(2)
    for e in b:
        e.run(7)
        e.run(2)
    for ea, eb in zip(a, b):
        sa, sb = ea.get_state(), eb.get_state()
        for x, y in zip(sa, sb):
            assert np.array_equal(x, y)
        assert not sa[4].any()
    info = batch.info()
    assert info["launches"] > 0 and info["graph_nodes"] > 0
    # each class branch's first and last node of the last graph launch
    tl = batch.timeline()
    assert len(tl) == len(a)
    assert all(0.0 <= t0 <= t1 <= info["ms"] + 1e-3 for t0, t1 in tl), tl
    batch.close()


def test_batch_continues_engine_runs(require_gpu):
    wl = W.h3_config(ntraj=16, nbeads=8, thermostat="andersen")
    a = build(wl, "fp64", andersen_step=2)
    b = build(wl, "fp64", andersen_step=2)
    a.run(3)
    batch = RPMDBatch([a], chunk_steps=4)
    batch.run(5)
    a.run(2)
    b.run(10)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
    batch.close()


def test_batch_rejects_duplicates(require_gpu):
    from caracal_gb300 import CaracalError
    wl = W.h3_config(ntraj=4, nbeads=8)
    a = build(wl, "fp64")
    with pytest.raises(CaracalError):
        RPMDBatch([a, a])
