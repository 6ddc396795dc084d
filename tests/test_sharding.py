"""The batched form's sharding across ranks (no GPU): contiguous world ranges balanced
by body count, every world on exactly one rank, and the max-over-ranks timing
reduction, exercised with two gloo ranks on CPU."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

from crashcat_gb300 import scenes, sharding


def test_world_ranges_partition_and_balance():
    counts = np.random.default_rng(0).integers(8, 512, size=4096)
    for ws in (1, 2, 3, 8):
        r = sharding.world_ranges(counts, ws)
        assert r[0][0] == 0 and r[-1][1] == len(counts)
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        loads = [counts[lo:hi].sum() for lo, hi in r]
        assert max(loads) - min(loads) <= 2 * counts.max()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world_size, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    sc = scenes.batched_worlds(num_worlds=64, seed=4)
    local = sharding.local_scene(sc, rank, world_size)
    mine = torch.tensor([local.num_worlds, local.n], dtype=torch.int64)
    gathered = [torch.zeros(2, dtype=torch.int64) for _ in range(world_size)]
    dist.all_gather(gathered, mine)
    t = sharding.max_over_ranks(1.0 + rank)
    out[rank] = (tuple(int(x) for g in gathered for x in g), t, int(local.bodies["world"].max()))
    dist.destroy_process_group()


def test_two_gloo_ranks_cover_every_world_once():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, ws, port, out)) for r in range(ws)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    sc = scenes.batched_worlds(num_worlds=64, seed=4)
    g0 = res[0][0]
    assert g0 == res[1][0]
    assert g0[0] + g0[2] == 64 and g0[1] + g0[3] == sc.n
    assert res[0][1] == res[1][1] == 2.0
    assert res[0][2] == g0[0] - 1 and res[1][2] == g0[2] - 1
