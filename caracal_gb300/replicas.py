"""Independent replicas of one workload over several processes, one GPU each.

Trajectories are independent, so N processes each advance their own share
of the batch with disjoint trajectory keys (``traj0 = rank * ntraj``: the
Gaussian streams of replica r are those trajectories r*T .. r*T+T-1 would
have in one big batch) and exchange nothing while stepping.  The only
cross-rank data are the recrossing sums of calc_rate's children, which
Caracal collects over MPI from its workers (src/recross.f90:381-415): the
flux numerators of every child step and the denominator, summed here with
one all-reduce.
"""
from __future__ import annotations

import numpy as np


def replica_traj0(rank, ntraj):
    """First global trajectory index of replica `rank` with `ntraj` trajectories."""
    return int(rank) * int(ntraj)


def allreduce_kappa(num, den, dist=None):
    """(num, den) summed over the ranks of the default process group; with
    no group (or one rank) the inputs come back unchanged.  Works on gloo
    (CPU tensors) and NCCL (the current CUDA device)."""
    num = np.asarray(num, dtype=np.float64)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return num.copy(), float(den)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(np.concatenate([num, [float(den)]])).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    out = t.cpu().numpy()
    return out[:-1].copy(), float(out[-1])
