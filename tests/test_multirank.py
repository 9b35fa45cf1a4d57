"""The multi-GPU path on CPU: two gloo ranks shard an ensemble the way
bench.py shards it under torchrun, and reduce timing and events the way it
does.  Trajectories never cross ranks, so the gathered shards must equal the
unsharded ensemble bit for bit."""

import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    import torch.distributed as dist

    import bench
    from oracle import oracle as O

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = bench.shard_seeds(rank, 0, 24)
        out, ev, tot, _ = O.sir_net().run_ensemble([999, 1, 0], seeds, 60.0, 6, n_threads=1)
        seconds = 1.0 + rank  # stand-in per-rank device time
        max_s, all_ev = bench.reduce_over_ranks(dist, seconds, float(tot), "cpu")
        shards = [None] * world
        dist.all_gather_object(shards, (rank, out, ev))
        if rank == 0:
            q.put((max_s, all_ev, shards))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import bench
    from oracle import oracle as O

    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    max_s, all_ev, shards = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert max_s == 2.0
    shards.sort(key=lambda x: x[0])
    # each rank's shard equals the same seeds run in one process
    total = 0
    for rank, out, ev in shards:
        ref, rev, rtot, _ = O.sir_net().run_ensemble([999, 1, 0], bench.shard_seeds(rank, 0, 24), 60.0, 6)
        np.testing.assert_array_equal(out, ref)
        np.testing.assert_array_equal(ev, rev)
        total += rtot
    assert all_ev == total
    # and the concatenated shards equal one ensemble over both ranks' seeds
    seeds = np.concatenate([bench.shard_seeds(r, 0, 24) for r in range(2)])
    full = O.sir_net().run_ensemble([999, 1, 0], seeds, 60.0, 6)[0]
    np.testing.assert_array_equal(np.concatenate([s[1] for s in shards], axis=2), full)
