"""
The multi-GPU mode of ``bench.py`` is independent replicas (one batch per
rank, no collective on the data path): every rank times its own steps, the
ranks meet at barriers around the timed region, and rank 0 reports the
maximum time over the ranks. Two CPU ranks over gloo exercise that host
logic (the environment torchrun sets, the barrier, the max reduction) and
check that each rank's work is independent of the other's.
"""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    import torch.distributed as dist

    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + rank, w)  # rank-dependent "step time"
    # each rank builds the same seeded workload by itself (no data exchange)
    from dxtb_gb300.workloads import config_molecules

    mols = config_molecules(2, count=3)
    out[rank] = (t, sum(len(m[0]) for m in mols))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_over_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 2.0  # max over the ranks
    assert out[0][1] == out[1][1]  # the same seeded workload on every rank
