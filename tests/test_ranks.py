"""The bench's multi-GPU path without a GPU: two gloo ranks on the CPU
check that every rank draws its own curves (weak scaling, no data-path
collective) and that the step time reported is the slowest rank's."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    from triplelens_gb300 import workloads
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lenses, trajs, _ = workloads.config2(bench.rank_seed(2024, rank), n_curves=2, n_points=10)
    step_ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    worst = bench.max_over_ranks(step_ms, dist, "cpu")
    import torch
    mine = torch.tensor(lenses.ravel())
    gathered = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine)
    out.put((rank, worst, [g.numpy() for g in gathered]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_curves_and_take_the_slowest_time():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, worst, gathered in res:
        assert worst == 150.0
        assert not np.array_equal(gathered[0], gathered[1])   # distinct curves per rank
