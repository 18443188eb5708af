"""Multi-GPU is replicas only: each rank runs the whole workload on its own
GPU with no collective on the data path; the bench reports the slowest
rank's time and the summed work. This checks that reduction with two gloo
ranks on the CPU (the GPU path uses the same code over NCCL)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup()
        # rank r "took" (r + 1) ms for 10 units of work
        ms, units = bench.replica_reduce(1.0 + r, 10.0, dist)
        out.put((r, w, local, ms, units))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_reduce_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for r, (rank, world, local, ms, units) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert ms == 2.0 and units == 20.0   # slowest rank's time, summed work


def test_replica_reduce_single_process():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_reduce(3.5, 7, None) == (3.5, 7.0)
