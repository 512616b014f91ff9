"""CPU, world size 2 (gloo): the replica aggregation bench.py uses for N > 1
reports the slowest rank's time and the sum of the ranks' units, and the
reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from sgldbench_gb300 import replicas

    replicas.init("gloo")
    replicas.barrier()
    t, u = replicas.aggregate(1.0 + rank, 10.0 * (rank + 1))
    out[rank] = (t, u, replicas.dist_env())
    replicas.shutdown()


def test_aggregate_two_ranks():
    port = _free_port()
    world = 2
    # the manager's server process is spawned too: forking a process that already
    # runs threads (torch's) can deadlock the child
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        t, u, env = res[rank]
        assert t == pytest.approx(2.0) and u == pytest.approx(30.0)
        assert env == (rank, world, rank)


def test_single_process_passthrough():
    from sgldbench_gb300 import replicas

    assert replicas.aggregate(1.5, 7.0) == (1.5, 7.0)
