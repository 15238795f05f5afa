"""Multi-rank logic on CPU (gloo, world size 2): batched cells are spread over
ranks by pair work with no exchange (pbe_gb300.batch.shard_cells), and the
bench reduces its timings with a max over ranks. No GPU involved."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import pbe_gb300 as pg


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, cell_n, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = pg.batch.shard_cells(cell_n, rank, world)
    n = np.asarray(cell_n, dtype=np.float64)[mine]
    work = torch.tensor([float((n * (n + 1) / 2).sum()), float(len(mine))], dtype=torch.float64)
    gathered = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, work)
    t = torch.tensor([1.0 + rank], dtype=torch.float64)      # a per-rank "elapsed time"
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ids = torch.tensor(mine, dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([len(mine)], dtype=torch.int64))
    # all_gather needs equal sizes: pad to the largest
    m = max(int(s.item()) for s in sizes)
    padded = torch.full((m,), -1, dtype=torch.int64)
    padded[:len(mine)] = ids
    bufs = [torch.zeros(m, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(bufs, padded)
    if rank == 0:
        out.put((np.concatenate([b.numpy()[b.numpy() >= 0] for b in bufs]).tolist(),
                 [g.tolist() for g in gathered], float(t.item())))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_cells_shard_over_ranks_without_overlap(world):
    cfg_n = pg.grids.config_batched_cells(n_cells=500)["cell_n"]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, list(map(int, cfg_n)), q))
             for r in range(world)]
    for p in procs:
        p.start()
    ids, works, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(ids) == list(range(len(cfg_n)))            # every cell exactly once
    w = np.array([g[0] for g in works])
    assert w.max() / w.mean() < 1.05                        # balanced pair work
    assert tmax == float(world)                             # max over ranks


def test_shard_cells_edge_cases():
    assert list(pg.batch.shard_cells([10], 0, 1)) == [0]
    parts = [pg.batch.shard_cells([5, 5, 5], r, 4) for r in range(4)]
    assert sorted(np.concatenate(parts).tolist()) == [0, 1, 2]
    with pytest.raises(ValueError):
        pg.batch.shard_cells([5], 2, 2)
