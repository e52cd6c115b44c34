"""GPU: launch shapes of the persistent step kernel and the autotuner.

A trajectory's beads live on one group of G = next_pow2(P) threads and all
its sums stay inside that group, so the number of trajectories per block
changes where the work runs but not one bit of the result.  The autotuner's
trial runs start from a saved state that is put back, so a run after it is
the run without it."""
import numpy as np
import pytest

from caracal_gb300 import RPMDEngine
from caracal_gb300.units import angstrom_to_bohr, beta_from_kelvin, dt_fs_to_au, mass_au, nose_q_to_au
from caracal_gb300.workloads import h3_collinear

pytestmark = pytest.mark.gpu


def engine(nbeads, ntraj, thermostat):
    e = RPMDEngine("h3", [mass_au("H")] * 3, nbeads, ntraj, dt_fs_to_au(0.1), beta=beta_from_kelvin(300.0),
                   thermostat=thermostat, andersen_step=7, pile_tau0_au=dt_fs_to_au(100.0), seed=77,
                   nose_q_au=nose_q_to_au(100.0, 0.1))
    e.init_positions(h3_collinear(), float(angstrom_to_bohr(0.01)))
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
        assert e.launch() == (b, (37 + b // g - 1) // (b // g))
        e.run(25)
        got = e.get_state()
        e.close()
        assert all(np.array_equal(x, y) for x, y in zip(got, want)), b
    with pytest.raises(Exception):
        ref.set_launch(g + 1)
    ref.close()


def test_autotune_leaves_the_run_unchanged(require_gpu):
    a, b = engine(16, 64, "pile"), engine(16, 64, "pile")
    a.run(3)
    b.run(3)
    tpb, ms = b.autotune(10)
    assert tpb in (16, 32, 64, 128, 256) and ms > 0.0 and b.launch()[0] == tpb
    a.run(20)
    b.run(20)
    assert all(np.array_equal(x, y) for x, y in zip(a.get_state(), b.get_state()))
    a.close()
    b.close()
