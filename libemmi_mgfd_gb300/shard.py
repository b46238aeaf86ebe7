"""Shot sharding across ranks and the path's one exchange step.

The reference runs one shot per MPI rank (``shot_idx[iproc]``, or the
``shots=`` list, src/acq_init_free.c:120-138) and sums the misfit, the
gradient and the pseudo-Hessian over ranks with MPI_Allreduce
(src/fg_fwi.c:107, 231, 265-268).  Here one rank drives one GPU and holds a
block of shots; all frequencies of a shot, forward and adjoint, stay on its
rank (they share the shot's operator).  The rank solves its shots as one
batch, sums the gradient over them on the device (emmi_build_gradient), and
the ranks then add their partial sums once.  There is no exchange inside
the solves.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np


def shots_of_rank(nshots: int, rank: int, world: int,
                  shots: Optional[Sequence[int]] = None) -> List[int]:
    """1-based shot numbers of `rank`: a contiguous block of the shot list
    (1..nshots, or `shots` as the reference's shots= parameter gives it);
    the first nshots % world ranks take one more shot."""
    lst = list(range(1, nshots + 1)) if shots is None else [int(s) for s in shots]
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    for s in lst:
        if s < 1 or s > nshots:
            raise ValueError(f"shot {s} out of range [1, {nshots}]")
    q, r = divmod(len(lst), world)
    start = rank * q + min(rank, r)
    return lst[start:start + q + (1 if rank < r else 0)]


def allreduce_sum(arrays, pg=None):
    """Sum float32 host arrays over the ranks of `pg` (a torch.distributed
    module with an initialised process group, gloo for host memory), in
    place, as the reference's MPI_Allreduce(MPI_FLOAT, MPI_SUM).  With
    pg = None (one rank) the arrays are returned unchanged."""
    if pg is None:
        return arrays
    import torch
    out = []
    for a in arrays:
        a = np.ascontiguousarray(a, np.float32)
        t = torch.from_numpy(a)
        pg.all_reduce(t, op=pg.ReduceOp.SUM)
        out.append(a)
    return out


class ShardedObjective:
    """The data part of fg_fwi over ranks: this rank's evaluator (gpu.Fg
    built over shots_of_rank's shots, or anything with the same eval)
    computes its shots' misfits, gradient and pseudo-Hessian in one device
    pass, and the partial sums are added over the ranks once -- the
    reference's MPI_Allreduce of the misfit, the pseudo-Hessian and the
    gradient (src/fg_fwi.c:231, 265, 268).  Every rank returns the same
    totals: (fcost_dat, grad, phess)."""

    def __init__(self, evaluator, pg=None):
        self.ev = evaluator
        self.pg = pg

    def __call__(self, model):
        fcost, grad, phess = self.ev.eval(model)[:3]
        f = np.zeros(1, np.float32)
        for v in np.asarray(fcost, np.float32):  # the shots in order, as the reference sums
            f[0] = np.float32(f[0] + v)
        f, grad, phess = allreduce_sum([f, grad, phess], self.pg)
        return float(f[0]), grad, phess
