"""Multi-GPU dispatch of the batched and served configurations, tested with CPU ranks.

Two gloo ranks (world size 2) each take their share of a batch of small grids, run it with a
CPU runner (the oracle, standing in for one GPU per rank) on a fake per-rank device list, and
gather their totals; the shares must cover every instance once, and every instance's result
must equal the one-process run.
"""
import json
import os
import socket

import numpy as np
import pytest

from fvleg_2d_gb300 import dispatch, ic


def test_partition_is_deterministic_complete_and_balanced():
    rng = np.random.default_rng(3)
    sides = ic.batch_sides(256, rng)
    costs = [dispatch.batch_cost(nx, ny, 500) for nx, ny in sides]
    for world in (1, 2, 4, 8):
        owner = dispatch.partition(costs, world)
        assert owner == dispatch.partition(costs, world)
        assert sorted(i for r in range(world) for i in dispatch.shard(owner, r)) == list(range(256))
        loads = [sum(costs[i] for i in dispatch.shard(owner, r)) for r in range(world)]
        # longest-processing-time-first: within the largest item of the mean load
        assert max(loads) - sum(loads) / world <= max(costs)
        if world > 1:
            assert max(loads) / min(loads) < 1.1


def test_route_stream_goes_to_the_least_loaded_rank():
    costs = [dispatch.request_cost(n, t) for n, t in [(128, 0.1), (2048, 0.3), (256, 0.05),
                                                       (512, 0.2), (128, 0.3)]]
    owner = dispatch.route_stream(costs, 2)
    assert owner[:3] == [0, 1, 0]  # the third goes to rank 0, which holds only the small one
    load = [0.0, 0.0]
    for c, r in zip(costs, owner):
        assert load[r] == min(load)
        load[r] += c


def _instances():
    rng = np.random.default_rng(11)
    out = []
    for _ in range(6):
        n = int(rng.integers(12, 24))
        cfg, prims = ic.random_circles(n, n + 4, rng, flux_solver="HLLC", limiter="minmod")
        out.append((cfg, prims))
    return out


def _oracle_runner(steps):
    def run(device, share):
        import oracle as O

        codes, sums = [], []
        for cfg, prims in share:
            f = O.OracleFluid(cfg)
            f.set_primitive(*prims)
            ec = 0
            for _ in range(steps):
                ec = f.integrate()
                if ec:
                    break
            codes.append(ec)
            sums.append(float(f.state()["rho"].sum()))
        return {"cell_updates": sum(c.ni * c.nj * steps for c, _ in share), "seconds": 1.0,
                "device_seen": device, "codes": codes, "rho_sums": sums}
    return run


def _rank_main(rank, world, port, out_path):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist

    from fvleg_2d_gb300 import dispatch as D

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    items = _instances()
    owner = D.partition([D.batch_cost(c.ni, c.nj, 5) for c, _ in items], world)
    res = D.run_sharded(items, owner, rank, devices=[3, 5], runner=_oracle_runner(5), dist=dist)
    if rank == 0:
        res["owner"] = owner
        with open(out_path, "w") as f:
            json.dump(res, f)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_batch_over_two_gloo_ranks(oracle, tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    out = tmp_path / "sharded.json"
    mp.start_processes(_rank_main, args=(2, _free_port(), str(out)), nprocs=2, join=True,
                       start_method="spawn")
    res = json.loads(out.read_text())
    items = _instances()
    owner = res["owner"]
    per = res["per_rank"]
    assert [r["device_seen"] for r in per] == [3, 5]
    assert sum(r["items"] for r in per) == len(items) and all(r["items"] for r in per)
    assert res["cell_updates"] == sum(c.ni * c.nj * 5 for c, _ in items)
    # every instance's result equals the one-process run
    alone = _oracle_runner(5)(0, items)
    for rank, r in enumerate(per):
        idx = dispatch.shard(owner, rank)
        assert r["codes"] == [alone["codes"][i] for i in idx]
        assert r["rho_sums"] == [alone["rho_sums"][i] for i in idx]
