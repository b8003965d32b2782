"""The newton3 force path (traversal 2, pair-group half lists) against the CPU oracle and the full-list path.

Tolerances as in the other parity tests: pair sets bit-exact; mixed-form force RMS error relative to the RMS
force <= 1e-6; Upot and virial within 1e-6 relative; interacting-pair counts exact.  The newton3 path adds the
reactions on j with vector float reductions in arrival order, so its forces are not bitwise reproducible from
run to run (the reductions' order varies); the tests use tolerances accordingly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng_mod():
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine
    return engine


def liquid(n_cells=6, rho=0.8442, seed=0, jitter=0.08):
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(n_cells, rho, 0.72, seed=seed)
    rng = np.random.default_rng(seed)
    pos = np.mod(pos + rng.normal(0, jitter, pos.shape), bmax)
    return pos, vel, bmin, bmax


def rel_rms(F, R):
    return float(np.sqrt(((F - R) ** 2).sum(1).mean()) / np.sqrt((R ** 2).sum(1).mean()))


def canonical_oracle_pairs(orc, pos, bmin, bmax, rc, skin, which):
    allpos, own, allt, owner, code = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n = len(pos)
    if which == 0:
        a, b = orc.pair_set(allpos, rc + skin, own=own)
    else:
        a, b = orc.interacting_set(allpos, rc, own=own)
    halo_b = b >= n
    bb = np.where(halo_b, owner[np.where(halo_b, b - n, 0)], b)
    cc = np.where(halo_b, code[np.where(halo_b, b - n, 0)], 13)
    return np.unique(np.stack([a, bb, cc], 1), axis=0)


@pytest.mark.parametrize("C", [4, 8])
def test_newton3_pair_set_bit_exact(eng_mod, orc, C):
    """Every pair within rc+skin (and every interacting pair) is covered by exactly one group's list: the device
    pair set, both halo views of each periodic-image pair, equals the oracle's bit for bit."""
    pos, vel, bmin, bmax = liquid(6, seed=5)
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=C, traversal=2, newton3=1)
    e.set_particles(pos, vel)
    e.rebuild()
    assert e.info()["traversal"] == 2 and e.info()["newton3"] == 1
    for which in (0, 1):
        a, b, c = e.pair_set(which)
        dev = np.unique(np.stack([a, b, c], 1), axis=0)
        assert len(dev) == len(a), "a pair is covered by two groups"
        ref = canonical_oracle_pairs(orc, pos, bmin, bmax, rc, skin, which)
        assert np.array_equal(dev, ref)
    e.close()


@pytest.mark.parametrize("C", [4, 8])
def test_newton3_cluster_lists_are_half_of_the_full_lists(eng_mod, C):
    """The newton3 cluster-pair lists keep forward neighbours only (VerletClusterListsTest.cpp:215-256 checks the
    same halving): every entry of the full lists but a cluster's self entry appears in exactly two lists there,
    once here."""
    pos, vel, bmin, bmax = liquid(6, seed=7)
    rc, skin = 2.5, 0.3
    info = {}
    for t, n3 in ((1, 0), (2, 1)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=C, traversal=t, newton3=n3)
        e.set_particles(pos, vel)
        e.rebuild()
        info[t] = e.info()
        e.close()
    assert info[1]["num_clusters"] == info[2]["num_clusters"]
    assert info[1]["num_cluster_pairs"] == 2 * info[2]["num_cluster_pairs"] - info[2]["num_clusters"]


@pytest.mark.parametrize("C", [4, 8])
def test_newton3_forces_and_globals_match_oracle(eng_mod, orc, C):
    pos, vel, bmin, bmax = liquid(8, seed=11)
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=C, traversal=2, newton3=1)
    e.set_particles(pos, vel)
    g = e.compute_forces()[0]
    F = e.forces()
    e.close()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    R = R[: len(pos)]
    assert rel_rms(F, R) <= 1e-6
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-6)
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    n = len(pos)
    assert g["num_pairs"] == int(np.sum(ib < n)) + int(np.sum(ib >= n)) // 2
    # forces sum to zero (every reaction was delivered)
    assert np.abs(F.sum(0)).max() <= 1e-5 * np.sqrt((R ** 2).sum(1).mean()) * np.sqrt(n)


def test_newton3_mixture_with_shift(eng_mod, orc):
    from autopas_gb300 import workloads
    rng = np.random.default_rng(21)
    bmin, bmax = np.zeros(3), np.full(3, 14.0)
    pos = workloads.rsa(1800, bmin, bmax, bmin, bmax, 0.85, seed=5)
    types = rng.choice(4, size=len(pos), p=[0.4, 0.3, 0.2, 0.1]).astype(np.int32)
    eps, sig = [1.0, 0.8, 1.2, 0.6], [1.0, 1.1, 0.9, 1.2]
    rc, skin = 3.0, 0.3
    lj = orc.LJ(rc, epsilon=eps, sigma=sig, shift=True)
    allpos, own, allt, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin, types=types)
    R, glob, _ = orc.lj_forces(allpos, lj, own=own, types=allt)
    R = R[: len(pos)]
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1, 1, 1, 1],
                           shift=True, traversal=2, newton3=1)
    e.set_particles(pos, types=types)
    g = e.compute_forces()[0]
    F = e.forces()
    e.close()
    assert rel_rms(F, R) <= 1e-6
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)


@pytest.mark.parametrize("pieces", [0, 4])
def test_newton3_md_steps_follow_the_full_list_path(eng_mod, pieces):
    """Forty velocity-Verlet steps with rebuilds, CUDA-graph replay and the fused position update: the newton3
    trajectory stays within FP32 rounding of the full-list one, with the evaluation in one piece or in four
    (force pieces on two streams, each piece's finish on a third after the force pieces up to it)."""
    pos, vel, bmin, bmax = liquid(6, seed=13, jitter=0.02)
    rc, skin, dt = 2.5, 0.3, 0.002
    out = {}
    for t, n3 in ((1, 0), (2, 1)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, traversal=t, newton3=n3, rebuild_frequency=10,
                               n3_pieces=pieces)
        e.set_particles(pos, vel)
        e.compute_forces()
        g = e.step(dt, 40)[0]
        P, V = e.state()
        out[t] = (P, V, g)
        e.close()
    (P1, V1, g1), (P2, V2, g2) = out[1], out[2]
    d = P1 - P2
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    assert np.abs(d).max() < 1e-6
    assert np.abs(V1 - V2).max() < 1e-4
    assert g2["upot"] == pytest.approx(g1["upot"], rel=1e-6)
    assert g2["num_pairs"] == g1["num_pairs"]


def test_newton3_ensemble(eng_mod, orc):
    from autopas_gb300 import workloads
    systems = workloads.ensemble(4, nmin=600, nmax=4000, seed=4)
    rc, skin = 2.5, 0.3
    boxes = [(s["bmin"], s["bmax"]) for s in systems]
    pos = np.concatenate([s["pos"] for s in systems])
    sysid = np.concatenate([np.full(len(s["pos"]), k, np.int32) for k, s in enumerate(systems)])
    e = eng_mod.PairEngine(rc, skin, boxes, periodic=True, traversal=2, newton3=1)
    e.set_particles(pos, system=sysid)
    gs = e.compute_forces()
    F = e.forces()
    e.close()
    for k, s in enumerate(systems):
        allpos, own, _, _, _ = orc.periodic_system(s["pos"], s["bmin"], s["bmax"], rc, skin)
        R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
        R = R[: len(s["pos"])]
        assert rel_rms(F[sysid == k], R) <= 1e-6
        assert gs[k]["upot"] == pytest.approx(glob[0], rel=1e-6)


def test_newton3_configuration_rules(eng_mod):
    """Newton3 serves the mixed form: the FP64 form and a full-list traversal with newton3 required are refused;
    systems with explicit halo particles are accepted."""
    box = ([0, 0, 0], [12, 12, 12])
    e = eng_mod.PairEngine(2.5, 0.3, box, periodic=False, traversal=2, newton3=1)
    assert e.info()["traversal"] == 2 and e.info()["newton3"] == 1
    e.close()
    for kw in (dict(newton3=1, precision=eng_mod.PRECISION_FP64), dict(newton3=1, traversal=1),
               dict(traversal=2, newton3=0), dict(traversal=2, newton3=1, n3_pieces=9),
               dict(traversal=2, newton3=1, n3_pieces=-1)):
        args = dict(periodic=True, traversal=-1)
        args.update(kw)
        with pytest.raises(eng_mod.EngineError) as ei:
            eng_mod.PairEngine(2.5, 0.3, box, **args)
        assert ei.value.code == -1, kw


@pytest.mark.parametrize("C", [4, 8])
def test_newton3_sorted_variant(eng_mod, orc, C):
    """Kernel variant 3 takes each block's groups in decreasing order of list length; a group's accumulation does
    not depend on its lane, and the block sums a cluster's groups in the butterflies' order, so Upot, virial and the
    pair count are the unsorted variant's bit for bit, and the forces are the oracle's."""
    pos, vel, bmin, bmax = liquid(8, seed=17)
    rc, skin = 2.5, 0.3
    out = {}
    for v in (0, 3):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=C, traversal=2, newton3=1,
                               kernel_variant=v)
        e.set_particles(pos, vel)
        out[v] = (e.compute_forces()[0], e.forces())
        e.close()
    (g0, F0), (g3, F3) = out[0], out[3]
    assert (g3["upot"], g3["virial"], g3["num_pairs"]) == (g0["upot"], g0["virial"], g0["num_pairs"])
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    R = R[: len(pos)]
    assert rel_rms(F3, R) <= 1e-6
    assert g3["upot"] == pytest.approx(glob[0], rel=1e-6)


@pytest.mark.parametrize("C", [4, 8])
def test_newton3_explicit_halo_matches_oracle(eng_mod, orc, C):
    """Container mode with newton3 (the caller hands owned + halo particles, AutoPas addHaloParticle semantics):
    every pair with an owned endpoint is covered by exactly one group (pairs of two halos are not pairs of the
    container), a pair's energy and virial weigh its owned endpoints (LJFunctor.h:327-345), the forces on owned
    particles are the oracle's, halo particles get none, and the pair count is the oracle's."""
    pos, vel, bmin, bmax = liquid(6, seed=3)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n = len(pos)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, cluster_size=C, traversal=2, newton3=1)
    e.set_particles(allpos, ownership=own)
    g = e.compute_forces()[0]
    F = e.forces()
    for which in (0, 1):
        a, b, c = e.pair_set(which)
        assert np.all(c == 13)
        dev = np.unique(np.stack([np.minimum(a, b), np.maximum(a, b)], 1), axis=0)
        assert len(dev) == len(a), "a pair is covered by two groups"
        if which == 0:
            ra, rb = orc.pair_set(allpos, rc + skin, own=own)
        else:
            ra, rb = orc.interacting_set(allpos, rc, own=own)
        ref = np.unique(np.stack([np.minimum(ra, rb), np.maximum(ra, rb)], 1), axis=0)
        assert np.array_equal(dev, ref)
    e.close()
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    assert rel_rms(F[:n], R[:n]) <= 1e-6
    assert np.all(F[n:] == 0)
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-6)
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    assert g["num_pairs"] == len(ia)


def test_newton3_explicit_halo_md_follows_the_full_list_path(eng_mod, orc):
    """Steps with explicit halos (fused position update, rebuilds): the halos stay where the caller put them and
    the newton3 trajectory stays within FP32 rounding of the full-list one."""
    pos, vel, bmin, bmax = liquid(5, seed=37, jitter=0.02)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n = len(pos)
    allvel = np.zeros_like(allpos)
    allvel[:n] = vel * 0.1
    out = {}
    for t, n3 in ((1, 0), (2, 1)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, traversal=t, newton3=n3, rebuild_frequency=5)
        e.set_particles(allpos, allvel, ownership=own)
        e.compute_forces()
        g = e.step(0.002, 18)[0]
        P, V = e.state()
        e.close()
        assert np.array_equal(P[n:], allpos[n:])
        out[t] = (P, V, g)
    (P1, V1, g1), (P2, V2, g2) = out[1], out[2]
    assert np.abs(P1 - P2).max() < 1e-6
    assert np.abs(V1 - V2).max() < 1e-4
    assert g2["upot"] == pytest.approx(g1["upot"], rel=1e-6)
    assert g2["num_pairs"] == g1["num_pairs"]


@pytest.mark.parametrize("traversal,n3", [(1, 0), (2, 1)])
def test_ownership_changes_in_place(eng_mod, orc, traversal, n3):
    """pe_update_ownership (updateContainer with kept lists, updateHaloParticle): owned and halo particles that
    become dummies keep the lists valid and drop out of the forces and globals; a halo that becomes owned (it has
    no list of its own, and a group of halos has no entries towards other halos) makes the next evaluation
    rebuild.  Forces on owned particles, Upot and the pair count follow the oracle for each ownership state."""
    pos, vel, bmin, bmax = liquid(5, seed=41)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n, m = len(pos), len(allpos)
    rng = np.random.default_rng(3)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, traversal=traversal, newton3=n3)
    e.set_particles(allpos, ownership=own)
    e.compute_forces()
    r0 = e.stats(reset=False)["rebuilds"]

    def check(o):
        g = e.compute_forces()[0]
        F = e.forces()
        R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=o)
        real = o == 1
        assert rel_rms(F[real], R[real]) <= 1e-6
        assert np.all(F[~real] == 0)
        assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
        ia, _ = orc.interacting_set(allpos, rc, own=o)
        assert g["num_pairs"] == len(ia)

    o1 = own.copy()
    o1[rng.choice(n, 25, replace=False)] = 0
    o1[n + rng.choice(m - n, 40, replace=False)] = 0
    assert e.update_ownership(o1)
    check(o1)
    assert e.stats(reset=False)["rebuilds"] == r0
    o2 = o1.copy()
    halos = np.flatnonzero(o1 == 2)
    o2[halos[rng.choice(len(halos), 10, replace=False)]] = 1
    assert not e.update_ownership(o2)
    check(o2)
    assert e.stats(reset=False)["rebuilds"] == r0 + 1
    e.close()
