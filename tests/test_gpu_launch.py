"""GPU: launch shapes of the persistent step kernel and the autotuner.

A trajectory's beads live on one group of G = next_pow2(P) threads (times
the threads per bead) and all its sums stay inside that group, so the
number of trajectories per block changes where the work runs but not one
bit of the result.  Threads per bead split each bead's atoms between 2 or 4
threads: the per-coordinate work and the bead sums are the same operations
(the sums over beads combine in the same tree), except the kinetic and
moment sums of NHC and transrot, whose per-thread partial sums over atoms
regroup; those runs are held to the oracle at the one-thread-per-bead bar.
Separately compiled variants may contract a multiply-add differently, so
the other runs agree to rounding rather than bit for bit.
The autotuner's trial runs start from a saved state that is put back, so a
run after it is the run without it."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300.units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from caracal_gb300.workloads import h3_collinear, oh3_geometry
from conftest import rel_err
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def engine(nbeads, ntraj, thermostat, pes="h3", transrot=True, seed=77):
    mass = [mass_au("H")] * 3 if pes == "h3" else [mass_au(s) for s in ("O", "H", "H", "H")]
    e = RPMDEngine(pes, mass, nbeads, ntraj, dt_fs_to_au(0.1), beta=beta_from_kelvin(300.0),
                   thermostat=thermostat, andersen_step=7, pile_tau0_au=dt_fs_to_au(100.0), seed=seed,
                   nose_q_au=nose_q_to_au(100.0, 0.1), transrot=transrot)
    e.init_positions(h3_collinear() if pes == "h3" else oh3_geometry(), float(angstrom_to_bohr(0.01)))
    e.init_momenta()
    e.compute_forces()
    return e


@pytest.mark.parametrize("nbeads,thermostat", [(16, "pile"), (8, "andersen"), (6, "nhc")])
def test_launch_shapes_give_identical_trajectories(require_gpu, nbeads, thermostat):
    ref = engine(nbeads, 37, thermostat)
    ref.run(25)
    want = ref.get_state()
    g = 1 << (nbeads - 1).bit_length()
    for b in sorted({g, 32, 64, 128, 256}):
        e = engine(nbeads, 37, thermostat)
        e.set_launch(b)
        assert e.launch() == (b, (37 + b // g - 1) // (b // g), 1)
        e.run(25)
        got = e.get_state()
        e.close()
        assert all(np.array_equal(x, y) for x, y in zip(got, want)), b
    with pytest.raises(Exception):
        ref.set_launch(g + 1)
    ref.close()


@pytest.mark.parametrize("pes,nbeads,thermostat", [("h3", 16, "pile"), ("h3", 8, "andersen"), ("oh3", 8, "pile")])
@pytest.mark.parametrize("tpb", [2, 4])
def test_threads_per_bead_without_transrot_matches_one_thread(require_gpu, pes, nbeads, thermostat, tpb):
    """The same operations on every coordinate; separately compiled kernel
    variants may contract a multiply-add differently, so the trajectories
    agree to rounding (1e-13 after 30 steps), not bit for bit."""
    ref = engine(nbeads, 21, thermostat, pes, transrot=False)
    ref.run(30)
    want = ref.get_state()
    ref.close()
    g = 1 << (nbeads - 1).bit_length()
    e = engine(nbeads, 21, thermostat, pes, transrot=False)
    e.set_launch(max(32, g * tpb), tpb)
    assert e.launch()[2] == tpb
    e.run(30)
    got = e.get_state()
    e.close()
    errs = [rel_err(x, y) for x, y in zip(got[:4], want[:4])]
    print("threads per bead", tpb, "q p f epot rel. difference", errs)
    assert max(errs) <= 1e-13 and np.array_equal(got[4], want[4])


@pytest.mark.parametrize("thermostat", ["pile", "nhc", "andersen"])
def test_threads_per_bead_with_transrot_matches_oracle(require_gpu, thermostat):
    """H3, 16 beads, transrot on, 4 threads per bead: 100 steps against the
    oracle at the trajectory bar (1e-9)."""
    P, T = 16, 8
    dt, beta = dt_fs_to_au(0.1), beta_from_kelvin(300.0)
    kw = dict(thermostat=thermostat, andersen_step=7, pile_tau0_au=dt_fs_to_au(100.0), seed=5,
              nose_q_au=nose_q_to_au(100.0, 0.1), transrot=True)
    e = RPMDEngine("h3", [mass_au("H")] * 3, P, T, dt, beta=beta, **kw)
    e.set_launch(64, 4)
    sig = float(angstrom_to_bohr(0.01))
    e.init_positions(h3_collinear(), sig)
    e.init_momenta()
    e.compute_forces()
    cfg = orc.Config("h3", [mass_au("H")] * 3, P, dt, beta, thermostat=thermostat, andersen_step=7,
                     pile_tau0=dt_fs_to_au(100.0), transrot=True, seed=5, nose_q=nose_q_to_au(100.0, 0.1))
    q = orc.init_positions(cfg, T, h3_collinear(), sig)
    p = orc.init_momenta(cfg, T)
    f, _ = orc.init_forces(cfg, q)
    e.run(100)
    qg, pg, fg, eg, st = e.get_state()
    e.close()
    qo, po, fo, eo, sto = orc.run(cfg, q, p, f, 100)
    assert not st.any() and not sto.any()
    assert rel_err(qg, qo) <= 1e-9 and rel_err(pg, po) <= 1e-9 and rel_err(eg, eo) <= 1e-9


def test_autotune_leaves_the_run_unchanged(require_gpu):
    a, b = engine(16, 64, "pile"), engine(16, 64, "pile")
    a.run(3)
    b.run(3)
    tpb_block, tpb, ms = b.autotune(10)
    assert tpb in (1, 2, 4) and ms > 0.0 and b.launch()[0] == tpb_block and b.launch()[2] == tpb
    a.run(20)
    b.run(20)
    qa, qb = a.get_state(), b.get_state()
    if tpb == 1:
        assert all(np.array_equal(x, y) for x, y in zip(qa, qb))
    else:           # transrot's sums regroup across the sub-threads
        assert all(rel_err(y, x) <= 1e-10 for x, y in zip(qa[:4], qb[:4]))
    a.close()
    b.close()
