"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The updates of one panel are independent, so each rank takes a contiguous
share of the update list with no collective on the data path; the only
collectives are the timing reductions (max of the per-rank times, sum of the
per-rank update counts)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    updates = [(i, j) for j in range(1, 64) for i in range(j + 1, 64)][:n]
    mine = bench.shard(updates, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t_max = bench.max_over_ranks(float(rank + 1), world)
    total = bench.sum_over_ranks(float(len(mine)), world)
    if rank == 0:
        flat = [u for part in gathered for u in part]
        out.put((flat == updates, t_max, total, [len(p) for p in gathered]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("n", [1953, 7])
def test_shard_covers_update_list_once(n):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    ok, t_max, total, sizes = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ok                                   # concatenated shards == the update list
    assert t_max == 2.0                         # max over ranks
    assert total == n                           # every update counted once
    assert abs(sizes[0] - sizes[1]) <= 1        # equal shares
