"""CPU, two processes over gloo: replicas of a recrossing batch.  Each rank
runs its share of the children (disjoint trajectory keys, traj0 = rank * T)
on the oracle and the kappa sums are combined with one all-reduce; the
result equals one process running all 2 T children."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

T, P, NSTEPS = 4, 4, 30


def _problem():
    sys.path.insert(0, ROOT)
    from caracal_gb300.units import beta_from_kelvin, dt_fs_to_au, mass_au
    from caracal_gb300.workloads import ch4h_dividing_surface, ch4h_recross_definition
    from oracle import oracle as orc
    q0 = ch4h_dividing_surface()
    rd = ch4h_recross_definition(q0)
    mass = [mass_au(s) for s in ("H", "C", "H", "H", "H", "H")]
    cfg = orc.Config("ch4h", mass, P, dt_fs_to_au(0.1), beta_from_kelvin(500.0), seed=7)
    xd = orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                        (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                        (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                        rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])
    qpar = np.repeat(q0[None], P, axis=0)
    return orc, cfg, xd, qpar


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from caracal_gb300.replicas import allreduce_kappa, replica_traj0
    orc, cfg, xd, qpar = _problem()
    num, den, _ = orc.recross_children(cfg, xd, T, qpar, NSTEPS, traj0=replica_traj0(rank, T), nthreads=1)
    num, den = allreduce_kappa(num, den, dist)
    if rank == 0:
        np.save(out, np.concatenate([num, [den]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_sum_to_one_batch(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "kappa.npy")
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    got = np.load(out)
    orc, cfg, xd, qpar = _problem()
    num, den, _ = orc.recross_children(cfg, xd, 2 * T, qpar, NSTEPS, traj0=0, nthreads=1)
    assert got[-1] == pytest.approx(den, rel=1e-14)
    assert np.allclose(got[:-1], num, rtol=1e-14, atol=1e-14 * abs(den))
    assert den > 0.0
