"""Sharding of an SPPM iteration across ranks (one process per GPU).

Photon paths are independent: path i of iteration k draws from its own
stream (seed i + 135 + k * P, SPPM.cpp:520), so ranks that each run a
contiguous range of the P paths produce, together, exactly the photons of
the unsharded iteration.  Every rank holds all hitpoints (the eye pass is
cheap and seeded per pixel).  Each rank gathers its own photons into partial
per-hitpoint counts M_r and flux sums Phi_r; one all-reduce (sum) of
M (int32) and Phi (3 x float32), 16 bytes per hitpoint, gives every rank the
full M and Phi, after which each applies the same N/tau/R update
(fr_update).  The counts reduce exactly; the flux sums differ from the
unsharded ones only by FP32 summation order.

Every box of this deployment has one GPU, so bench.py runs replicas; the
partition and the reduction are exercised on CPU ranks (gloo) in tests.
"""
from __future__ import annotations

import numpy as np


def path_range(rank, world, paths):
    """Contiguous range [lo, hi) of the photon paths that rank `rank` runs."""
    if not 0 <= rank < world:
        raise ValueError('rank %d outside world %d' % (rank, world))
    base, extra = divmod(int(paths), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def reduce_partials(m, phi, group=None):
    """All-reduce (sum) of per-hitpoint photon counts (int32, H) and flux
    sums (float32, H x 3) over the process group; returns numpy arrays."""
    import torch
    import torch.distributed as dist
    tm = torch.from_numpy(np.ascontiguousarray(m, np.int32))
    tp = torch.from_numpy(np.ascontiguousarray(phi, np.float32))
    dist.all_reduce(tm, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(tp, op=dist.ReduceOp.SUM, group=group)
    return tm.numpy(), tp.numpy()
