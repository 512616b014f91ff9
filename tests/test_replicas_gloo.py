"""CPU, world size 2 (gloo): the replica aggregation bench.py uses for N > 1
reports the slowest rank's time and the sum of the ranks' units, and the
reference arm runs on rank 0 only.  A rank that dies between steps, or stays
alive but never joins the next step, is detected by the others on the host:
their next collective raises (at once when the dead peer's connections close,
else at the group's timeout) instead of waiting forever.  The failures are
made on the host; no GPU is involved."""
import os
import socket
import time

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


def _worker_dies(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from sgldbench_gb300 import replicas

    replicas.init("gloo", timeout_s=20)
    replicas.barrier()          # step 1 completes on both ranks
    if rank == 1:
        os._exit(3)             # rank 1 dies between steps, with no collective in flight
    t0 = time.time()
    try:
        replicas.aggregate(1.0, 1.0)   # step 2's collective
        out[rank] = ("completed", time.time() - t0)
    except Exception as e:  # the waiting rank learns of the failure here
        out[rank] = (type(e).__name__, time.time() - t0)


def test_dead_rank_detected():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_worker_dies, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        alive = [p for p in procs if p.is_alive()]
        for p in alive:   # only the processes this test started
            p.kill()
            p.join()
        res = dict(out)
    assert not alive
    assert procs[1].exitcode == 3
    name, waited = res[0]
    assert name != "completed" and waited < 30.0


def _worker_stalls(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from sgldbench_gb300 import replicas

    replicas.init("gloo", timeout_s=5)
    replicas.barrier()
    if rank == 1:
        time.sleep(15)          # alive, but never joins step 2's collective
        out[rank] = ("stalled", 0.0)
        os._exit(0)
    t0 = time.time()
    try:
        replicas.aggregate(1.0, 1.0)
        out[rank] = ("completed", time.time() - t0)
    except Exception as e:  # the group's timeout ends the wait
        out[rank] = (type(e).__name__, time.time() - t0)
    os._exit(0)


def test_stalled_rank_times_out():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_worker_stalls, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        alive = [p for p in procs if p.is_alive()]
        for p in alive:   # only the processes this test started
            p.kill()
            p.join()
        res = dict(out)
    assert not alive
    name, waited = res[0]
    assert name != "completed" and 4.0 <= waited < 14.0
    assert res[1][0] == "stalled"
