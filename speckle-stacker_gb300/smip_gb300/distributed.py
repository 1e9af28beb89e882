"""Multi-GPU layout of the SMIP workload.

Two ways the work divides, both without a data-path collective in the common
case:

* Independent stacks (jobs) -> one rank per GPU runs its own stacks
  ("replicas"); throughput adds up, nothing is exchanged.
* One stack sharded by frames -> the accumulation is additive, so each rank
  accumulates a contiguous block of frames against the stack's frame 0 and a
  single reduce-sum of the partial accumulators (bispectrum + compensation,
  power spectrum, shift-and-add sum, frame count) gives the full result.  On
  one GPU the same merge is ``Stack.merge``.

The host logic (frame partition, reduction order) is written here once and is
exercised by multi-process gloo tests on CPU.
"""
from __future__ import annotations

import numpy as np


def shard_range(nframes: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous block of frames for ``rank``; rank 0 holds frame 0 (the reference)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("invalid world/rank")
    base, extra = divmod(nframes, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of the independent stack a replica rank processes."""
    return int(base_seed) + 7919 * int(rank)


def allreduce_partials(arrays: dict, group=None) -> dict:
    """Sum numpy partial accumulators over all ranks (torch.distributed).

    Complex arrays are reduced as float64 pairs, integer arrays as int64, so
    the shift-and-add sum stays exact.  Returns new arrays.
    """
    import torch
    import torch.distributed as dist

    out = {}
    for k in sorted(arrays):
        a = np.asarray(arrays[k])
        if np.iscomplexobj(a):
            t = torch.from_numpy(np.ascontiguousarray(a.astype(np.complex128)).view(np.float64).copy())
        elif np.issubdtype(a.dtype, np.integer):
            t = torch.from_numpy(np.ascontiguousarray(a.astype(np.int64)))
        else:
            t = torch.from_numpy(np.ascontiguousarray(a.astype(np.float64)))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        r = t.numpy()
        if np.iscomplexobj(a):
            r = r.view(np.complex128).reshape(a.shape)
        out[k] = r.astype(a.dtype) if not np.iscomplexobj(a) else r.astype(np.complex128)
    return out
