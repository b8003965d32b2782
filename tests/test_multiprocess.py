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


# ------------------------------------------------------------------------------------------------------------
# slab decomposition of one periodic system (RegularGridDecomposition.cpp:159-300) on two gloo ranks, with the
# CPU oracle as each rank's force function
# ------------------------------------------------------------------------------------------------------------
RC, SKIN = 2.5, 0.3


def _slab_system():
    import numpy as np

    from oracle import oracle as orc
    ell = 12.0
    bmin, bmax = np.zeros(3), np.array([3 * ell, ell, ell])
    n = int(0.7 * 3 * ell ** 3)
    pos = orc.gen_rsa(n, bmin, bmax, bmin, bmax, 0.8, seed=31)
    rng = np.random.default_rng(31)
    vel = rng.normal(0.0, 1.0, (n, 3))
    vel -= vel.mean(0)
    return pos, vel, bmin, bmax


def _rows(pos, vel, F, ids):
    import numpy as np
    return np.concatenate([pos, vel, F, ids[:, None].astype(np.float64)], axis=1)


def _slab_rank_main(rank, world, port, outdir):
    import json

    import numpy as np
    import torch
    import torch.distributed as dist

    from autopas_gb300 import decomposition as D
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pos, vel, bmin, bmax = _slab_system()
    ids = np.arange(len(pos))
    out = {}
    for w in (world, 1):  # the decomposed run, then every rank alone as the one-domain run
        dec = D.SlabDecomposition(rank if w == world else 0, w, bmin, bmax, RC, SKIN)
        comm = D.Comm(dist if w > 1 else None)
        mine = dec.inside(pos)
        rows = _rows(pos[mine], vel[mine], np.zeros((mine.sum(), 3)), ids[mine])
        halos = dec.exchange_halos(comm, rows[:, [0, 1, 2, 9]])
        forces = D.oracle_forces(orc, RC)
        F, glob = forces(rows[:, 0:3], halos[:, 0:3])
        rows[:, 6:9] = F
        # forces and globals of the first evaluation, then 15 velocity-Verlet steps with migration
        first = (rows[:, 9].tolist(), F.tolist(), glob.tolist(), len(halos))
        for _ in range(15):
            rows, glob_step = D.step_velocity_verlet(rows, forces, dec, comm, 0.001)
        out[w] = {"first": first, "final": rows.tolist()}
        if w > 1:
            g = torch.tensor(glob, dtype=torch.float64)
            dist.all_reduce(g)
            out["glob_sum"] = g.tolist()
    with open(os.path.join(outdir, f"slab{rank}.json"), "w") as f:
        json.dump({str(k): v for k, v in out.items()}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_decompose_a_periodic_slab(tmp_path, orc):
    """Two ranks, each owning half of a 3:1:1 periodic box along x, exchange halos with each other (x) and with
    themselves (y, z): the union of their forces equals the one-domain oracle's forces (md-flexible halo images,
    FP64) within 1e-12 of the largest force, the summed Upot and virial within 1e-12 relative, the summed pair
    counts exactly; fifteen velocity-Verlet steps with migration every step give the one-domain trajectory within
    1e-10 (the force sums differ in order only)."""
    import json

    import numpy as np
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_slab_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    res = [json.load(open(tmp_path / f"slab{r}.json")) for r in range(world)]
    pos, vel, bmin, bmax = _slab_system()
    n = len(pos)
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, RC, SKIN)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(RC), own=own)
    R = R[:n]
    oo, oh, _ = orc.count_interacting(allpos, RC, own=own)
    F = np.zeros((n, 3))
    seen = np.zeros(n, bool)
    for r in res:
        ids, f, _, nh = r[str(world)]["first"]
        ids = np.array(ids, int)
        assert not seen[ids].any(), "a particle is owned by two ranks"
        seen[ids] = True
        F[ids] = np.array(f)
        assert nh > 0
    assert seen.all()
    np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * np.abs(R).max())
    gs = res[0]["glob_sum"]
    assert gs == res[1]["glob_sum"]
    assert gs[0] == pytest.approx(glob[0], rel=1e-12)
    assert gs[1] == pytest.approx(glob[1], rel=1e-12)
    assert gs[2] == oo + oh / 2
    # the decomposed trajectory against the one-domain one (each rank ran the one-domain run too)
    final2 = np.concatenate([np.array(r[str(world)]["final"]) for r in res])
    final1 = np.array(res[0]["1"]["final"])
    final2 = final2[np.argsort(final2[:, 9])]
    final1 = final1[np.argsort(final1[:, 9])]
    assert np.array_equal(final2[:, 9], final1[:, 9])
    d = final2[:, 0:3] - final1[:, 0:3]
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    assert np.abs(d).max() < 1e-10
    assert np.abs(final2[:, 3:6] - final1[:, 3:6]).max() < 1e-8


def _ensemble_rank_main(rank, world, port, outdir):
    import json

    import numpy as np
    import torch.distributed as dist

    from autopas_gb300 import sharding, workloads
    from oracle import oracle as orc
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    systems = workloads.ensemble(10, nmin=300, nmax=1500, seed=17)
    costs = [sharding.pair_work(len(s["pos"]), s["rho"], RC + SKIN) for s in systems]
    ranks, _ = sharding.lpt_assign(costs, world)
    lj = orc.LJ(RC)
    out = {}
    for k in ranks[rank]:
        s = systems[k]
        p, v, _, e = orc.md_run(s["pos"], s["vel"], None, [1.0], s["bmin"], s["bmax"], SKIN, lj, 0.002, 8)
        out[k] = {"pos": p.tolist(), "vel": v.tolist(), "energy": e.tolist()}
    sharding.barrier(dist)
    with open(os.path.join(outdir, f"ens{rank}.json"), "w") as f:
        json.dump(out, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_step_their_ensemble_shares(tmp_path, orc):
    """Ensemble sharding with a data path: each rank steps its own systems (here with the oracle's md-flexible
    integrator); together they cover every system once, each exactly as one process stepping it alone."""
    import json

    import numpy as np
    import torch.multiprocessing as mp

    from autopas_gb300 import workloads
    world = 2
    mp.start_processes(_ensemble_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    res = {}
    for r in range(world):
        part = json.load(open(tmp_path / f"ens{r}.json"))
        assert not set(part) & set(res)
        res.update(part)
    systems = workloads.ensemble(10, nmin=300, nmax=1500, seed=17)
    assert sorted(int(k) for k in res) == list(range(len(systems)))
    lj = orc.LJ(RC)
    for k, s in enumerate(systems):
        p, v, _, e = orc.md_run(s["pos"], s["vel"], None, [1.0], s["bmin"], s["bmax"], SKIN, lj, 0.002, 8)
        assert np.array_equal(np.array(res[str(k)]["pos"]), p)
        assert np.array_equal(np.array(res[str(k)]["energy"]), e)


def test_slab_decomposition_halos_match_the_single_rank_images(orc):
    """One rank: the dimension-by-dimension exchange with itself forms exactly md-flexible's periodic images (the
    oracle's restatement), as a multiset of positions."""
    import numpy as np

    from autopas_gb300 import decomposition as D
    pos, vel, bmin, bmax = _slab_system()
    dec = D.SlabDecomposition(0, 1, bmin, bmax, RC, SKIN)
    halos = dec.exchange_halos(D.Comm(None), np.concatenate([pos, np.arange(len(pos))[:, None]], 1))
    hpos, owner, _ = orc.make_halos(pos, bmin, bmax, RC, SKIN)
    a = halos[np.lexsort(halos[:, [2, 1, 0]].T)][:, :3]
    b = hpos[np.lexsort(hpos[:, [2, 1, 0]].T)]
    assert a.shape == b.shape and np.array_equal(a, b)
