"""The multi-rank host logic on CPU with the gloo backend (world size 2):
the slowest-rank timing of bench.py and the cost-balanced sharding of the
ensemble across ranks (no data-path collective; only the timing and a final
gather of statistics cross ranks)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import importlib
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = importlib.import_module("bench")
        ens = importlib.import_module("3d_droplet_simulation_2007_gb300.ensemble")
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
        cfgs = ens.study_configs(64)
        mine = ens.shard(cfgs, rank, world)
        load = sum(ens.member_cost(cfgs[i]) for i in mine)
        gathered = [None] * world
        dist.all_gather_object(gathered, {"mine": mine, "load": load})
        if rank == 0:
            out.put({"ms": ms, "shards": gathered})
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_ranks_on_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res["ms"] == 15.0  # the slowest rank's time
    shards = res["shards"]
    members = sorted(i for s in shards for i in s["mine"])
    assert members == list(range(64))  # every member exactly once
    loads = [s["load"] for s in shards]
    assert max(loads) - min(loads) <= 0.1 * sum(loads) / world

