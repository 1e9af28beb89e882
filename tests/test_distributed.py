"""Frame-sharded accumulation across ranks (gloo, world_size 2, CPU): each
rank accumulates its block of frames against frame 0 with the oracle; one
all-reduce of the partial accumulators equals the single-process result."""
import os
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp
from conftest import ROOT

from smip_gb300.distributed import replica_seed, shard_range


def test_shard_range_partition():
    for n in (1, 5, 40, 2001):
        for w in (1, 2, 3, 8):
            spans = [shard_range(n, w, r) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(e - s for s, e in spans) - min(e - s for s, e in spans) <= 1
    assert replica_seed(10, 0) != replica_seed(10, 1)
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _worker(rank, world, port, frames, depth, out_q):
    sys.path.insert(0, os.path.join(ROOT, "speckle-stacker_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    from oracle import Oracle, bispec_desc
    from smip_gb300.distributed import allreduce_partials, shard_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    O = Oracle()
    n, nr, nc = frames.shape
    s, e = shard_range(n, world, rank)
    d = bispec_desc(nc, nr, depth)
    B = np.zeros(d["base_size"], np.complex64)
    P = np.zeros(nr * nc, np.float64)
    Ssum = np.zeros(nr * nc, np.float64)
    ref = frames[0].astype(np.float64)
    shifts = O.accumulate_frames(frames[s:e], depth, ref, B, P, Ssum)
    red = allreduce_partials({"B": B, "P": P, "S": Ssum, "n": np.array([e - s])})
    if rank == 0:
        out_q.put((red["B"], red["P"], red["S"], int(red["n"][0]), shifts))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_reduce_matches_single(oracle):
    from smip_gb300 import synthetic as Sy

    spec = Sy.StackSpec(n=32, nframes=9, kind="binary", dtype="uint8", d_over_r0=4.0, bdepth=8, seed=77)
    frames = Sy.make_stack(spec)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, frames, 8, q)) for r in range(2)]
    for p in procs:
        p.start()
    B, P, S, n, _ = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    single = oracle.run_stack(frames, 8, 12)
    assert n == len(frames)
    # shift-and-add: integer sums, exact after normalisation
    assert np.array_equal(S.reshape(32, 32) / n, single["sum"])
    # power: FP64 sums in a different order
    assert np.abs(P.reshape(32, 32) / (n * 1024) - single["power"].real).max() <= 1e-12 * single["power"].real.max()
    # bispectrum: FP32 partials summed in FP64
    b = B / n
    rel = np.linalg.norm(b - single["bispec"].astype(np.complex128)) / np.linalg.norm(single["bispec"].astype(np.complex128))
    assert rel <= 1e-6
