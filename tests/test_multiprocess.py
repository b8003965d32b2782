"""The multi-rank host path on CPU: two gloo ranks over 127.0.0.1 (no GPU involved).

* ensemble sharding: every system lands on exactly one rank, ranks agree on the assignment, the
  longest-processing-time bound holds;
* the barrier / max-over-ranks / sum-over-ranks helpers that bench.py's replica mode uses.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, outdir):
    import json

    import torch.distributed as dist

    from autopas_gb300 import sharding, workloads
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    systems = workloads.ensemble(64, nmin=500, nmax=50_000, seed=11)
    costs = [sharding.pair_work(len(s["pos"]), s["rho"], 2.8) for s in systems]
    ranks, loads = sharding.lpt_assign(costs, world)
    mine = ranks[rank]
    # every rank computes the same assignment: compare a checksum of the whole table
    table = torch.tensor([sum((k + 1) * (r + 1) for r, idxs in enumerate(ranks) for k in idxs)], dtype=torch.float64)
    gathered = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(gathered, table)
    sharding.barrier(dist)
    tmax = sharding.max_over_ranks(dist, float(rank + 1))
    tsum = sharding.sum_over_ranks(dist, float(len(mine)))
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"mine": mine, "loads": loads, "tables": [float(g.item()) for g in gathered], "tmax": tmax,
                   "tsum": tsum, "n": len(systems), "maxcost": max(costs)}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_an_ensemble(tmp_path):
    import json

    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    allidx = sorted(res[0]["mine"] + res[1]["mine"])
    assert allidx == list(range(res[0]["n"]))
    assert res[0]["tables"][0] == res[0]["tables"][1] == res[1]["tables"][0]
    assert res[0]["tmax"] == res[1]["tmax"] == 2.0
    assert res[0]["tsum"] == res[1]["tsum"] == res[0]["n"]
    loads = res[0]["loads"]
    # LPT: the heaviest rank exceeds the average by at most the largest single system
    assert max(loads) <= sum(loads) / world + res[0]["maxcost"] + 1e-9


def test_lpt_assignment_is_balanced_and_deterministic():
    from autopas_gb300 import sharding
    costs = [5, 9, 1, 3, 7, 2, 8, 4, 6]
    a1, l1 = sharding.lpt_assign(costs, 3)
    a2, l2 = sharding.lpt_assign(costs, 3)
    assert a1 == a2 and l1 == l2
    assert sorted(sum(a1, [])) == list(range(len(costs)))
    assert max(l1) - min(l1) <= max(costs)
