"""Multi-process path of bench.py (replicas only): world size 2 over gloo on
the CPU.  Each rank runs its own realisation; the job time is the slowest
rank's and the throughput counts every rank's particles."""
import os
import pathlib
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r: 10*(r+1) ms for 1000*(r+1) particles
    ms, value = bench.replica_throughput(10.0 * (rank + 1), 1000 * (rank + 1))
    q.put((rank, ms, value, bench.dist_env()))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, env in out:
        assert ms == pytest.approx(20.0)                 # slowest rank
        assert value == pytest.approx(3000 / 0.020)      # all particles / max time
        assert env[0] == rank and env[1] == 2


def test_replica_throughput_single_process():
    sys.path.insert(0, str(ROOT))
    import bench
    ms, value = bench.replica_throughput(5.0, 500)
    assert ms == 5.0 and value == pytest.approx(100000.0)
