"""Sharding of the tank ensemble over ranks (host logic, CPU only).

The ensemble's tanks are independent, so ranks share no data while they
run; the partition must cover every tank once, in contiguous blocks whose
estimated work is balanced, and the final gather must return every tank's
summary on rank 0 in tank order.  The multi-rank part runs as two `gloo`
processes on the CPU."""
import math
import os
import socket

import pytest

import ensemble
import workloads


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_covers_every_tank_once():
    for costs in ([5.0], [1.0] * 7, [3.0, 1.0, 4.0, 1.0, 5.0, 9.0, 2.0, 6.0], [0.0, 0.0, 1.0], []):
        for world in (1, 2, 3, 4, 8):
            blocks = ensemble.partition(costs, world)
            assert len(blocks) == world
            assert blocks[0][0] == 0 and blocks[-1][1] == len(costs)
            for (a, b), (c, d) in zip(blocks, blocks[1:]):
                assert b == c and a <= b
            if len(costs) >= world:
                assert all(b > a for a, b in blocks)


def test_partition_balances_the_ensemble():
    specs = workloads.ensemble()
    costs = [ensemble.tank_cost(s, 1.0) for s in specs]
    total = sum(costs)
    for world in (2, 4, 8):
        blocks = ensemble.partition(costs, world)
        loads = [sum(costs[a:b]) for a, b in blocks]
        # a contiguous split can miss the even share by at most the largest tank
        assert max(loads) <= total / world + max(costs)
        assert sum(loads) == pytest.approx(total)


def test_cost_follows_size_and_order():
    base = workloads.ensemble(n_tanks=1)[0]
    small = dict(base, n1=257, mHOS=3)
    big = dict(base, n1=1025, mHOS=3)
    high = dict(base, n1=257, mHOS=7)
    assert ensemble.tank_cost(big, 1.0) > 4 * ensemble.tank_cost(small, 1.0)
    assert ensemble.tank_cost(high, 1.0) == pytest.approx(ensemble.tank_cost(small, 1.0) * 49 / 9)
    # the reference's x-mode stability limit: dt = 0.95 sqrt(8/pi^2) (xlen/h)/(n1-1)
    dt = 0.95 * math.sqrt(8 / math.pi ** 2) * 10.0 / 1024
    assert ensemble.tank_steps(big, 1.0) == pytest.approx(1.0 / (dt * math.sqrt(5.0 / 9.81)))


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        specs = workloads.ensemble()
        start, stop = ensemble.shard(specs, rank, world, 1.0)
        # stand-in for the tanks' results: what each rank would report
        local = [{"tank": k, "rank": rank, "n1": specs[k]["n1"]} for k in range(start, stop)]
        full = ensemble.gather_summaries(local, start, len(specs))
        if rank == 0:
            with open(os.path.join(out_dir, "gathered.txt"), "w") as f:
                for s in full:
                    f.write(f"{s['tank']} {s['rank']} {s['n1']}\n")
        else:
            assert full is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_gather_in_tank_order(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    rows = [l.split() for l in open(tmp_path / "gathered.txt")]
    specs = workloads.ensemble()
    assert [int(r[0]) for r in rows] == list(range(len(specs)))
    assert [int(r[2]) for r in rows] == [s["n1"] for s in specs]
    blocks = ensemble.partition([ensemble.tank_cost(s, 1.0) for s in specs], 2)
    for k, r in enumerate(rows):
        assert int(r[1]) == (0 if k < blocks[0][1] else 1)
