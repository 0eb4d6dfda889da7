"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The updates of one panel are independent, so each rank takes a share of the
update list with no collective on the data path.  The shares are balanced
by cost (longest processing time first on the per-update FP64 cost model,
hcore_gb300/shard.py), and each rank builds only the tiles its share reads.
The collectives are the set-up reduction of the tile ranks and the timing
reductions (max of the per-rank times, sum of the per-rank update counts)."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = dict(n_points=4096, nb=256)          # 16 tiles per dimension, 105 updates


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    from hcore_gb300 import panel as pnl

    dist.init_process_group("gloo", rank=rank, world_size=world)
    share, parts, imb = pnl.build_panel_share(rank, world, lambda v: bench.all_sum_ints(v, world),
                                              device="cpu", workers=2, **SMALL)
    facs = {t: (share.U[int(share.offset[s]):int(share.offset[s + 1])].numpy().copy(),
                int(share.rank[s])) for s, t in enumerate(share.tiles)}
    gathered = [None] * world
    dist.all_gather_object(gathered, (share.updates, sorted(share.tiles), facs, parts, imb))
    t_max = bench.max_over_ranks(float(rank + 1), world)
    total = bench.sum_over_ranks(float(len(share.updates)), world)
    if rank == 0:
        out.put((gathered, t_max, total))
    dist.barrier()
    dist.destroy_process_group()


def test_rank_balanced_shares_over_gloo():
    from hcore_gb300 import panel as pnl
    from hcore_gb300 import shard as sh

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, t_max, total = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    full = pnl.build_panel(device="cpu", workers=2, **SMALL)
    assert t_max == 2.0                                   # max over ranks
    assert total == len(full.updates)                     # every update counted once
    parts = gathered[0][3]
    assert parts == gathered[1][3]                        # same partition on every rank
    ups = [u for g in gathered for u in g[0]]
    assert sorted(ups) == sorted(full.updates)            # disjoint cover of the update list
    for upd, tiles, facs, _, _ in gathered:
        assert set(tiles) == sh.tiles_read(upd)           # only the tiles the share reads
        for t, (u, r) in facs.items():                    # same factors as the full build
            s = full.index[t]
            assert r == int(full.rank[s])
            np.testing.assert_array_equal(
                u, full.U[int(full.offset[s]):int(full.offset[s + 1])].numpy())
    # every rank's share is a strict subset of the tiles
    assert all(len(g[1]) < len(full.tiles) for g in gathered)


@pytest.mark.parametrize("world", [2, 4, 8])
def test_lpt_balances_the_benchmark_panel(world):
    """On the 1953 updates of the 65,536-point panel (k = a + c from 13 to
    70), the cost-balanced partition stays within 5% of the mean load, while
    contiguous equal shares of the list do not."""
    from hcore_gb300 import shard as sh

    with open(os.path.join(ROOT, "tests", "golden", "panel_ranks.json")) as f:
        d = json.load(f)
    costs = [sh.update_cost(d["nb"], a, b, c) for a, b, c in d["abc"]]
    parts = sh.lpt_partition(costs, world)
    assert sorted(u for p in parts for u in p) == list(range(len(costs)))
    assert sh.imbalance(costs, parts) <= 0.05
    n = len(costs)
    contiguous = [list(range(r * n // world, (r + 1) * n // world)) for r in range(world)]
    assert sh.imbalance(costs, contiguous) > sh.imbalance(costs, parts)


def test_lpt_edge_cases():
    from hcore_gb300 import shard as sh

    assert sh.lpt_partition([], 3) == [[], [], []]
    assert sh.lpt_partition([5.0], 2) == [[0], []]
    parts = sh.lpt_partition([3, 3, 2, 2, 2], 2)          # LPT: {3,2,2}=7 vs {3,2}=5
    assert sorted(len(p) for p in parts) == [2, 3]
    with pytest.raises(ValueError):
        sh.lpt_partition([1.0], 0)
