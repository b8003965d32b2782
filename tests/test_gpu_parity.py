"""Parity of the CUDA engine (through the C ABI) with the CPU oracle.

Tolerances:
* FP64 form: forces within 1e-12 of the largest force magnitude (the per-pair arithmetic is the reference's
  operation order; only the summation order differs), Upot and virial within 1e-12 relative.
* mixed form: force RMS error relative to the RMS force <= 1e-6 (the stated accuracy target), Upot within 1e-6.
* pair sets (rc+skin Verlet rule and the rc interacting set): bit-exact set equality.
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


def canonical_oracle_pairs(orc, pos, bmin, bmax, rc, skin, which, dist_mode=0):
    allpos, own, allt, owner, code = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n = len(pos)
    if which == 0:
        a, b = orc.pair_set(allpos, rc + skin, own=own, dist_mode=dist_mode)
    else:
        a, b = orc.interacting_set(allpos, rc, own=own, dist_mode=dist_mode)
    halo_b = b >= n
    bb = np.where(halo_b, owner[np.where(halo_b, b - n, 0)], b)
    cc = np.where(halo_b, code[np.where(halo_b, b - n, 0)], 13)
    return np.unique(np.stack([a, bb, cc], 1), axis=0)


def rel_rms(F, R):
    return float(np.sqrt(((F - R) ** 2).sum(1).mean()) / np.sqrt((R ** 2).sum(1).mean()))


@pytest.mark.parametrize("traversal", [0, 1])
@pytest.mark.parametrize("C", [4, 8])
def test_fp64_periodic_forces_match_oracle(eng_mod, orc, C, traversal):
    pos, vel, bmin, bmax = liquid()
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_FP64,
                           cluster_size=C, traversal=traversal)
    e.set_particles(pos, vel)
    g = e.compute_forces()[0]
    F = e.forces()
    lj = orc.LJ(rc)
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, lj, own=own)
    R = R[: len(pos)]
    scale = np.abs(R).max()
    np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * scale)
    assert g["upot"] == pytest.approx(glob[0], rel=1e-12)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-12)
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    n = len(pos)
    # unique physical pairs: owned-owned once, owned-halo pairs come in mirrored couples
    n_oo = int(np.sum(ib < n))
    n_oh = int(np.sum(ib >= n))
    assert g["num_pairs"] == n_oo + n_oh // 2


@pytest.mark.parametrize("traversal", [0, 1])
def test_fp64_explicit_halo_forces_match_oracle(eng_mod, orc, traversal):
    """Container mode: the caller hands owned + halo particles (AutoPas addHaloParticle semantics)."""
    pos, vel, bmin, bmax = liquid(5, seed=3)
    rc, skin = 2.5, 0.3
    allpos, own, allt, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=eng_mod.PRECISION_FP64,
                           traversal=traversal)
    e.set_particles(allpos, ownership=own)
    g = e.compute_forces()[0]
    F = e.forces()
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    n = len(pos)
    scale = np.abs(R[:n]).max()
    np.testing.assert_allclose(F[:n], R[:n], rtol=0, atol=1e-12 * scale)
    assert np.all(F[n:] == 0)
    assert g["upot"] == pytest.approx(glob[0], rel=1e-12)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-12)
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    assert g["num_pairs"] == len(ia)


@pytest.mark.parametrize("traversal", [0, 1])
@pytest.mark.parametrize("dist_mode", [0, 1])
@pytest.mark.parametrize("C", [4, 8])
def test_pair_set_bit_exact_periodic(eng_mod, orc, dist_mode, C, traversal):
    pos, vel, bmin, bmax = liquid(6, seed=5)
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=C, dist_mode=dist_mode,
                           traversal=traversal)
    e.set_particles(pos, vel)
    e.rebuild()
    for which in (0, 1):
        a, b, c = e.pair_set(which)
        dev = np.unique(np.stack([a, b, c], 1), axis=0)
        assert len(dev) == len(a), "device reported a pair twice"
        ref = canonical_oracle_pairs(orc, pos, bmin, bmax, rc, skin, which, dist_mode)
        assert len(dev) == len(ref)
        assert np.array_equal(dev, ref)


@pytest.mark.parametrize("traversal", [0, 1])
def test_pair_set_bit_exact_explicit_halo(eng_mod, orc, traversal):
    pos, vel, bmin, bmax = liquid(5, seed=9)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, traversal=traversal)
    e.set_particles(allpos, ownership=own)
    e.rebuild()
    a, b, c = e.pair_set(0)
    assert np.all(c == 13)
    dev = np.unique(np.stack([a, b], 1), axis=0)
    ra, rb = orc.pair_set(allpos, rc + skin, own=own)
    ref = np.unique(np.stack([ra, rb], 1), axis=0)
    assert np.array_equal(dev, ref)


@pytest.mark.parametrize("traversal", [0, 1])
@pytest.mark.parametrize("C", [4, 8])
def test_mixed_precision_error_bound(eng_mod, orc, C, traversal):
    pos, vel, bmin, bmax = liquid(8, seed=11)
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_MIXED, cluster_size=C,
                           traversal=traversal)
    e.set_particles(pos, vel)
    g = e.compute_forces()[0]
    F = e.forces()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    R = R[: len(pos)]
    err = rel_rms(F, R)
    assert err <= 1e-6, err
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-6)
    # the interacting set of the mixed kernel equals the FP64 one (near-cutoff pairs are re-tested in FP64)
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    n = len(pos)
    assert g["num_pairs"] == int(np.sum(ib < n)) + int(np.sum(ib >= n)) // 2


def test_multi_type_mixing_and_shift(eng_mod, orc):
    rng = np.random.default_rng(21)
    from autopas_gb300 import workloads
    bmin, bmax = np.zeros(3), np.full(3, 14.0)
    pos = workloads.rsa(1800, bmin, bmax, bmin, bmax, 0.85, seed=5)
    types = rng.choice(4, size=len(pos), p=[0.4, 0.3, 0.2, 0.1]).astype(np.int32)
    eps, sig = [1.0, 0.8, 1.2, 0.6], [1.0, 1.1, 0.9, 1.2]
    rc, skin = 3.0, 0.3
    lj = orc.LJ(rc, epsilon=eps, sigma=sig, shift=True)
    allpos, own, allt, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin, types=types)
    R, glob, _ = orc.lj_forces(allpos, lj, own=own, types=allt)
    R = R[: len(pos)]
    for prec, tol in ((eng_mod.PRECISION_FP64, 1e-12), (eng_mod.PRECISION_MIXED, 1e-6)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1, 1, 1, 1],
                               shift=True, precision=prec)
        e.set_particles(pos, types=types)
        g = e.compute_forces()[0]
        F = e.forces()
        if prec == eng_mod.PRECISION_FP64:
            np.testing.assert_allclose(F, R, rtol=0, atol=tol * np.abs(R).max())
        else:
            assert rel_rms(F, R) <= tol
        assert g["upot"] == pytest.approx(glob[0], rel=tol)


@pytest.mark.parametrize("ntypes", [1, 3])
def test_shifted_energy_keeps_fp64_accuracy_in_mixed_precision(eng_mod, orc, ntypes):
    """With the shifted potential, each pair's energy is eps24 lj12m6 + shift6, the two terms nearly cancelling
    near rc; the mixed kernels form the pair energy before summing it.  On a dense 3,000-particle system the FP32
    rounding of the pair terms alone gives ~8e-8 relative (a float emulation of the sums agrees), so the bound
    is 2e-7; a lost or doubled shift would be off by 0.2 (single type)."""
    from autopas_gb300 import workloads
    rng = np.random.default_rng(33)
    bmin, bmax = np.zeros(3), np.full(3, 16.0)
    pos = workloads.rsa(3000, bmin, bmax, bmin, bmax, 0.85, seed=8)
    types = rng.integers(0, ntypes, size=len(pos)).astype(np.int32)
    eps, sig = [1.0, 0.8, 1.2][:ntypes], [1.0, 1.1, 0.9][:ntypes]
    rc, skin = 3.0, 0.3
    lj = orc.LJ(rc, epsilon=eps, sigma=sig, shift=True)
    allpos, own, allt, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin, types=types)
    _, glob, _ = orc.lj_forces(allpos, lj, own=own, types=allt)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1.0] * ntypes,
                           shift=True, precision=eng_mod.PRECISION_MIXED)
    e.set_particles(pos, types=types)
    g = e.compute_forces()[0]
    e.close()
    assert abs(g["upot"] - glob[0]) <= 2e-7 * abs(glob[0])
    assert abs(g["virial"] - glob[1]) <= 2e-7 * abs(glob[1])


def test_md_trajectory_fp64_matches_oracle(eng_mod, orc):
    pos, vel, bmin, bmax = liquid(5, seed=13, jitter=0.02)
    rc, skin, dt, nsteps = 2.5, 0.3, 0.002, 40
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_FP64,
                           rebuild_frequency=10)
    e.set_particles(pos, vel)
    e.compute_forces()
    g = e.step(dt, nsteps)[0]
    P, V = e.state()
    lj = orc.LJ(rc)
    rp, rv, rf, en = orc.md_run(pos, vel, None, [1.0], bmin, bmax, skin, lj, dt, nsteps)
    d = P - rp
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    assert np.abs(d).max() < 1e-9
    assert np.abs(V - rv).max() < 1e-8
    assert g["upot"] == pytest.approx(en[-1, 0], rel=1e-9)


@pytest.mark.parametrize("traversal", [0, 1])
def test_ensemble_systems_are_independent(eng_mod, orc, traversal):
    from autopas_gb300 import workloads
    systems = workloads.ensemble(3, nmin=600, nmax=3000, seed=4)
    rc, skin = 2.5, 0.3
    boxes = [(s["bmin"], s["bmax"]) for s in systems]
    pos = np.concatenate([s["pos"] for s in systems])
    sysid = np.concatenate([np.full(len(s["pos"]), k, np.int32) for k, s in enumerate(systems)])
    for prec in (eng_mod.PRECISION_FP64, eng_mod.PRECISION_MIXED):
        e = eng_mod.PairEngine(rc, skin, boxes, periodic=True, precision=prec, traversal=traversal)
        e.set_particles(pos, system=sysid)
        gs = e.compute_forces()
        F = e.forces()
        for k, s in enumerate(systems):
            allpos, own, _, _, _ = orc.periodic_system(s["pos"], s["bmin"], s["bmax"], rc, skin)
            R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
            R = R[: len(s["pos"])]
            Fk = F[sysid == k]
            if prec == eng_mod.PRECISION_FP64:
                np.testing.assert_allclose(Fk, R, rtol=0, atol=1e-12 * np.abs(R).max())
                assert gs[k]["upot"] == pytest.approx(glob[0], rel=1e-12)
            else:
                assert rel_rms(Fk, R) <= 1e-6
                assert gs[k]["upot"] == pytest.approx(glob[0], rel=1e-6)


def test_ensemble_with_an_empty_system(eng_mod, orc):
    """Three systems, the middle one without particles: it gets no reduction chunk (the chunks' systems are found
    through the table of first chunks, which the empty system shares with the next), its globals are zero, and its
    neighbours' forces and globals are their own oracle's (FP64 form, 1e-12)."""
    from autopas_gb300 import workloads
    systems = workloads.ensemble(2, nmin=600, nmax=3000, seed=8)
    rc, skin = 2.5, 0.3
    boxes = [(systems[0]["bmin"], systems[0]["bmax"]), (np.zeros(3), np.full(3, 9.0)),
             (systems[1]["bmin"], systems[1]["bmax"])]
    pos = np.concatenate([systems[0]["pos"], systems[1]["pos"]])
    sysid = np.concatenate([np.zeros(len(systems[0]["pos"]), np.int32), np.full(len(systems[1]["pos"]), 2, np.int32)])
    for traversal in (1, 2):
        e = eng_mod.PairEngine(rc, skin, boxes, periodic=True, precision=eng_mod.PRECISION_FP64, traversal=1,
                               cluster_size=8) if traversal == 1 else \
            eng_mod.PairEngine(rc, skin, boxes, periodic=True, traversal=2, newton3=1, cluster_size=8)
        e.set_particles(pos, system=sysid)
        gs = e.compute_forces()
        F = e.forces()
        e.close()
        assert gs[1]["upot"] == 0.0 and gs[1]["virial"] == 0.0 and gs[1]["num_pairs"] == 0
        tol = 1e-12 if traversal == 1 else 1e-6
        for k, s in ((0, systems[0]), (2, systems[1])):
            allpos, own, _, _, _ = orc.periodic_system(s["pos"], s["bmin"], s["bmax"], rc, skin)
            R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
            R = R[: len(s["pos"])]
            Fk = F[sysid == k]
            if traversal == 1:
                np.testing.assert_allclose(Fk, R, rtol=0, atol=tol * np.abs(R).max())
            else:
                assert rel_rms(Fk, R) <= tol
            assert gs[k]["upot"] == pytest.approx(glob[0], rel=tol)


def test_more_systems_than_one_block_of_the_chunk_table(eng_mod, orc):
    """1,100 small systems in one engine: the globals reduction's chunk table is built on the device by one
    block of 1,024 threads, a thread per system, so these systems span two tiles of it.  Each system's Upot and
    virial (FP64 form) must be its own oracle's within 1e-12 of the sum of the magnitudes of their terms (in
    some of these systems attraction and repulsion cancel to 1e-4 of that sum).  With a = sum of
    eps24 (sigma^2/r^2)^6 and b = sum of eps24 (sigma^2/r^2)^3, Upot = (a - b)/6 and virial = 2a - b; a second
    oracle run with sigma^2 scaled by 2^(1/3) gives Upot' = (4a - 2b)/6, hence a and b."""
    from autopas_gb300 import workloads
    systems = workloads.ensemble(1100, nmin=300, nmax=700, seed=5)
    rc, skin = 2.5, 0.3
    boxes = [(s["bmin"], s["bmax"]) for s in systems]
    pos = np.concatenate([s["pos"] for s in systems])
    sysid = np.concatenate([np.full(len(s["pos"]), k, np.int32) for k, s in enumerate(systems)])
    e = eng_mod.PairEngine(rc, skin, boxes, periodic=True, precision=eng_mod.PRECISION_FP64, cluster_size=8,
                           traversal=1)
    e.set_particles(pos, system=sysid)
    gs = e.compute_forces()
    e.close()
    assert len(gs) == len(systems)
    lj, lj2 = orc.LJ(rc), orc.LJ.single(rc, 24.0, 2.0 ** (1.0 / 3.0))
    for k, s in enumerate(systems):
        allpos, own, allt, _, _ = orc.periodic_system(s["pos"], s["bmin"], s["bmax"], rc, skin)
        _, glob, _ = orc.cpu_lc_c08(allpos, lj, skin, own=own, types=allt)
        _, glob2, _ = orc.cpu_lc_c08(allpos, lj2, skin, own=own, types=allt)
        a = 3.0 * glob2[0] - 6.0 * glob[0]
        b = a - 6.0 * glob[0]
        assert abs(gs[k]["upot"] - glob[0]) <= 1e-12 * max(abs(glob[0]), (a + b) / 6.0), k
        assert abs(gs[k]["virial"] - glob[1]) <= 1e-12 * max(abs(glob[1]), 2.0 * a + b), k


def test_long_cutoff_grows_the_list_buffer(eng_mod, orc):
    """rc 6, skin 1, C = 4 at density 0.9: a cluster has more candidate cluster pairs than the list build's
    first on-chip buffer holds; the build grows the buffer and the forces stay the oracle's."""
    from autopas_gb300 import workloads
    bmin, bmax = np.zeros(3), np.full(3, 16.0)
    pos = workloads.rsa(3600, bmin, bmax, bmin, bmax, 0.85, seed=9)
    rc, skin = 6.0, 1.0
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    R = R[: len(pos)]
    for prec, tol in ((eng_mod.PRECISION_FP64, 1e-12), (eng_mod.PRECISION_MIXED, 1e-6)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=prec, cluster_size=4, traversal=1)
        e.set_particles(pos)
        g = e.compute_forces()[0]
        assert rel_rms(e.forces(), R) <= tol
        assert g["upot"] == pytest.approx(glob[0], rel=tol)
        info = e.info()
        assert info["num_cluster_pairs"] > 512 * info["num_clusters"]  # more than the first buffer, on average


def test_errors_are_reported_not_hidden(eng_mod):
    with pytest.raises(eng_mod.EngineError) as ei:
        eng_mod.PairEngine(2.5, 0.3, ([0, 0, 0], [4.0, 20, 20]), periodic=True).set_particles(
            np.random.default_rng(0).uniform(0, 4, (100, 3)))
    assert ei.value.code == -8  # periodic box shorter than 2(rc+skin)
    e = eng_mod.PairEngine(2.5, 0.3, ([0, 0, 0], [10, 10, 10]))
    with pytest.raises(eng_mod.EngineError) as ei:
        e.compute_forces()
    assert ei.value.code == -6


@pytest.mark.parametrize("C", [4, 8])
def test_tower_grid_matches_reference_formula(eng_mod, orc, C):
    """Reference tower sizing (ClusterTowerBlock2D::estimateOptimalGridSideLength) in container mode."""
    pos, vel, bmin, bmax = liquid(5, seed=2)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, cluster_size=C, tower_sizing=0, traversal=0)
    e.set_particles(allpos, ownership=own)
    side, num, halo, origin = e.tower_grid(0)
    rside, rnum, rhalo = orc.tower_grid(bmin, bmax, len(allpos), C, rc + skin)
    assert np.array_equal(side, rside)
    assert np.array_equal(num, rnum)
    assert halo == rhalo
    np.testing.assert_array_equal(origin, bmin[:2] - side * halo)


def test_local_density_towers_keep_pair_set(eng_mod, orc):
    """Tower sizing changes only the cluster shapes: the pair set of a slab is the same either way."""
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.slab(n_total=20000, seed=3)
    rc, skin = 3.0, 0.4
    sets = []
    for ts in (0, 1):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, tower_sizing=ts)
        e.set_particles(pos, vel)
        e.rebuild()
        a, b, c = e.pair_set(0)
        sets.append(np.unique(np.stack([a, b, c], 1), axis=0))
    assert np.array_equal(sets[0], sets[1])
    ref = canonical_oracle_pairs(orc, pos, bmin, bmax, rc, skin, 0)
    assert np.array_equal(sets[1], ref)


def test_tuner_full_search_keeps_results(eng_mod, orc):
    """The engine tuner times every (cluster size, traversal, variant) candidate -- force evaluation and the
    rebuild amortised over the rebuild frequency -- and keeps the cheapest per step; whatever it picks, the
    forces stay those of the oracle."""
    pos, vel, bmin, bmax = liquid(7, seed=17)
    rc, skin = 2.5, 0.3
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_MIXED, cluster_size=0,
                           traversal=-1)
    e.set_particles(pos, vel)
    g = e.compute_forces()[0]
    tun = e.tuning()
    cands = tun["candidates"]
    # cluster sizes 4 and 8, each with the cluster-pair traversal and every particle-list kernel variant
    assert {c["cluster_size"] for c in cands} == {4, 8}
    assert {c["traversal"] for c in cands} == {0, 1}
    assert len(cands) == 2 * (1 + len({c["variant"] for c in cands if c["traversal"] == 1}))
    assert 0 <= tun["chosen"] < len(cands)
    best = tun["candidates"][tun["chosen"]]
    for c in cands:
        assert c["rebuild_ms"] > 0
        assert c["score"] == pytest.approx(c["ms"] + c["rebuild_ms"] / 10)  # rebuild_frequency 10
    assert best["score"] == min(c["score"] for c in cands)
    info = e.info()
    assert (info["cluster_size"], info["traversal"]) == (best["cluster_size"], best["traversal"])
    F = e.forces()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    assert rel_rms(F, R[: len(pos)]) <= 1e-6
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
    e.step(0.002, 5)


# ------------------------------------------------------------------------------------------- three-body (ATM)
# The triplet arithmetic is FP32 (on displacements rounded once from FP64), so the ATM checks use a relative
# tolerance of 1e-5 on forces and energies instead of the reference's FP64 absolute 1e-7.
def test_atm_known_answer_through_engine(eng_mod):
    """ATMFunctorTestNoGlobals.h:19-32 (cutoff 1, nu 1) with the pair term switched off (epsilon 0)."""
    pos = np.array([[0.0, 0.0, 0.0], [0.1, 0.2, 0.3], [0.3, 0.2, 0.1]])
    e = eng_mod.PairEngine(1.0, 0.3, ([-1, -1, -1], [2, 2, 2]), periodic=False, epsilon=[0.0], sigma=[1.0],
                           precision=eng_mod.PRECISION_MIXED)
    e.set_particles(pos)
    e.compute_forces()
    g = e.compute_atm(1.0, 1.0)[0]
    F = e.forces()
    exp = np.array([[-188761.250385809] * 3, [-95789.2912405596, 94380.6251929043, 284550.541626368],
                    [284550.541626368, 94380.6251929043, -95789.2912405596]])
    np.testing.assert_allclose(F, exp, rtol=1e-5, atol=1e-5 * np.abs(exp).max())
    assert g["num_pairs"] == 1


def test_atm_globals_known_answer(eng_mod):
    """ATMFunctorTestGlobals.cpp:12-78 (cutoff 5, nu 0.7), all three particles owned."""
    import math
    p = np.array([[0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, 0.2, 0.3]])
    e = eng_mod.PairEngine(5.0, 0.3, ([-1, -1, -1], [2, 2, 2]), periodic=False, epsilon=[0.0], sigma=[1.0])
    e.set_particles(p)
    e.compute_forces()
    g = e.compute_atm(0.7, 5.0)[0]
    ij, ik, jk = p[0] - p[1], p[0] - p[2], p[1] - p[2]
    dij, dik, djk = (math.sqrt(float(v @ v)) for v in (ij, ik, jk))
    ci = float(ik @ ij) / (dik * dij)
    cj = -float(jk @ ij) / (djk * dij)
    ck = float(ik @ jk) / (dik * djk)
    expected = 0.7 * (3 * ci * cj * ck + 1.0) / (dij * djk * dik) ** 3
    assert g["upot"] == pytest.approx(expected, rel=1e-5)


def test_atm_periodic_liquid_matches_oracle(eng_mod, orc):
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(4, 0.8, 1.0, seed=2)
    rng = np.random.default_rng(2)
    pos = np.mod(pos + rng.normal(0, 0.07, pos.shape), bmax)
    rc, skin, nu = 2.5, 0.3, 0.073
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=[0.0], sigma=[1.0])
    e.set_particles(pos, vel)
    e.compute_forces()
    g = e.compute_atm(nu, rc)[0]
    F = e.forces()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, hits = orc.atm_forces(allpos, nu, rc, own=own)
    R = R[: len(pos)]
    assert rel_rms(F, R) <= 1e-5
    assert g["upot"] == pytest.approx(glob[0], rel=1e-5)


def test_atm_fp64_form_matches_oracle(eng_mod, orc):
    """The plain FP64 triplet kernel against the oracle's FP64 AxilrodTellerMuto restatement (cell-list form,
    checked against the quadratic one in the oracle tests): forces within 1e-12 of the largest, Upot and virial
    within 1e-12 relative."""
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(6, 0.8, 1.0, seed=3)
    pos = np.mod(pos + np.random.default_rng(3).normal(0, 0.05, pos.shape), bmax)
    rc, skin, nu = 2.5, 0.3, 0.073
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=[0.0], sigma=[1.0],
                           precision=eng_mod.PRECISION_FP64)
    e.set_particles(pos, vel)
    e.compute_forces()
    g = e.compute_atm(nu, rc)[0]
    F = e.forces()
    e.close()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.atm_forces_cells(allpos, nu, rc, own=own)
    R = R[: len(pos)]
    np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * np.abs(R).max())
    assert g["upot"] == pytest.approx(glob[0], rel=1e-12)
    assert g["virial"] == pytest.approx(glob[1], rel=1e-12)


def test_atm_mixed_form_error_on_32k_particles(eng_mod, orc):
    """The FP32 triplet kernel on a 32,000-particle melted FCC liquid (density 0.8, nu 0.073, triplet cutoff
    2.5): three-body force RMS error relative to the RMS three-body force <= 1e-6, three-body energy within 1e-6."""
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(20, 0.8, 1.0, seed=29)
    pos = np.mod(pos + np.random.default_rng(29).normal(0, 0.02, pos.shape), bmax)
    rc, skin, nu = 2.5, 0.3, 0.073
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=[0.0], sigma=[1.0])
    e.set_particles(pos, vel)
    e.compute_forces()
    g = e.compute_atm(nu, rc)[0]
    F = e.forces()
    e.close()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    R, glob, _ = orc.atm_forces_cells(allpos, nu, rc, own=own)
    R = R[: len(pos)]
    err = rel_rms(F, R)
    print(f"ATM mixed form on {len(pos)} particles: force RMS error {err:.3g}, "
          f"energy {abs(g['upot'] - glob[0]) / abs(glob[0]):.3g}")
    assert err <= 1e-6
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)


def test_graph_replay_matches_eager_steps(eng_mod):
    """Steps replayed from the captured CUDA graph give the same bits as steps launched one kernel at a time."""
    pos, vel, bmin, bmax = liquid(5, seed=21)
    out = []
    for graphs in (False, True):
        e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, rebuild_frequency=7, use_graphs=graphs)
        e.set_particles(pos, vel)
        e.compute_forces()
        g = e.step(0.002, 23)[0]
        P, V = e.state()
        out.append((P, V, e.forces(), g["upot"]))
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(a, b)
    assert out[0][3] == out[1][3]


def test_fused_position_update_gives_the_same_bits(eng_mod):
    """pe_step over many steps lets the force kernel advance the next step's positions (double-buffered);
    stepping one step per call takes the plain path.  Both give the same bits, with graphs and without."""
    pos, vel, bmin, bmax = liquid(5, seed=33)
    out = []
    for graphs in (False, True):
        for chunk in (1, 17):
            e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_MIXED,
                                   rebuild_frequency=6, use_graphs=graphs)
            e.set_particles(pos, vel)
            e.compute_forces()
            for _ in range(34 // chunk):
                g = e.step(0.002, chunk)[0]
            P, V = e.state()
            out.append((P, V, e.forces(), g["upot"], g["ekin"]))
    for o in out[1:]:
        for a, b in zip(out[0][:3], o[:3]):
            assert np.array_equal(a, b)
        assert out[0][3] == o[3] and out[0][4] == o[4]


def test_fused_position_update_keeps_explicit_halos(eng_mod, orc):
    """Container mode (owned + static halo particles, no periodic images): many steps per call, with the force
    kernel advancing the positions, give the bits of one step per call, and the halos do not move."""
    pos, vel, bmin, bmax = liquid(5, seed=37)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    allvel = np.zeros_like(allpos)
    allvel[: len(pos)] = vel * 0.1
    out = []
    for chunk in (1, 9):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=eng_mod.PRECISION_MIXED,
                               rebuild_frequency=5)
        e.set_particles(allpos, allvel, ownership=own)
        e.compute_forces()
        for _ in range(18 // chunk):
            g = e.step(0.002, chunk)[0]
        P, V = e.state()
        out.append((P, V, g["upot"]))
        assert np.array_equal(P[len(pos):], allpos[len(pos):])
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_graph_replay_with_three_body_forces(eng_mod):
    """Steps with pair and three-body forces replayed from the CUDA graph give the same bits as eager steps
    (the three-body buffers are allocated before the capture)."""
    pos, vel, bmin, bmax = liquid(5, rho=0.8, seed=27)
    out = []
    for graphs in (False, True):
        e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, rebuild_frequency=5, use_graphs=graphs,
                               atm_nu=0.073, atm_cutoff=2.5)
        e.set_particles(pos, vel)
        e.compute_forces()
        g = e.step(0.002, 12)[0]
        P, V = e.state()
        out.append((P, V, g["upot"]))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


def test_fcc_32000_trajectory_matches_oracle(eng_mod, orc):
    """Full-size FCC case: 20^3 unit cells (32,000 particles) at density 0.8442, T* 0.72, rc 2.5, skin 0.3,
    velocity Verlet dt 0.002 for 100 steps with a rebuild every 10.  The FP64 form follows the oracle's
    md-flexible trajectory to 1e-9 (positions) and the mixed form conserves energy as well as FP64 does."""
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(20, 0.8442, 0.72, seed=1)
    rc, skin, dt, nsteps = 2.5, 0.3, 0.002, 100
    rp, rv, rf, en = orc.md_run(pos, vel, None, [1.0], bmin, bmax, skin, orc.LJ(rc), dt, nsteps)
    res = {}
    for prec in (eng_mod.PRECISION_FP64, eng_mod.PRECISION_MIXED):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=prec, rebuild_frequency=10)
        e.set_particles(pos, vel)
        g0 = e.compute_forces()[0]
        g = e.step(dt, nsteps)[0]
        P, V = e.state()
        res[prec] = (P, V, g0, g)
    P, V, g0, g = res[eng_mod.PRECISION_FP64]
    d = P - rp
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    assert np.abs(d).max() < 1e-9
    assert np.abs(V - rv).max() < 1e-8
    assert g["upot"] == pytest.approx(en[-1, 0], rel=1e-10)
    assert g["ekin"] == pytest.approx(en[-1, 1], rel=1e-10)
    e0_ref = res[eng_mod.PRECISION_FP64][2]["upot"] + 0.5 * float((vel ** 2).sum())
    drift64 = abs(g["upot"] + g["ekin"] - e0_ref)
    gm = res[eng_mod.PRECISION_MIXED][3]
    driftm = abs(gm["upot"] + gm["ekin"] - e0_ref)
    assert driftm <= max(2 * drift64, 1e-6 * abs(e0_ref))


@pytest.mark.parametrize("prec", [0, 1])
def test_pruned_lists_keep_the_interacting_set(eng_mod, orc, prec):
    """With rolling pruning the force kernels read lists at rc + buffer, refreshed on the device; the interacting
    set of every step stays the FP64 one and the trajectory stays that of the unpruned engine."""
    pos, vel, bmin, bmax = liquid(7, seed=31, jitter=0.05)
    vel = vel * 2.0  # fast particles: several prunes between rebuilds
    runs = []
    for buf in (0.0, 0.08):
        e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=prec, rebuild_frequency=10,
                               prune_buffer=buf)
        e.set_particles(pos, vel)
        g0 = e.compute_forces()[0]
        pairs = [g0["num_pairs"]]
        for _ in range(6):
            g = e.step(0.002, 5)[0]
            pairs.append(g["num_pairs"])
        P, V = e.state()
        runs.append((pairs, P, e.forces(), g, e.stats()["prunes"]))
    assert runs[0][4] == 0
    assert runs[1][4] >= 3  # at least one after each rebuild
    assert runs[0][0] == runs[1][0]
    tol = 1e-9 if prec == 0 else 1e-5
    np.testing.assert_allclose(runs[1][1], runs[0][1], rtol=0, atol=tol)
    assert runs[1][3]["upot"] == pytest.approx(runs[0][3]["upot"], rel=1e-7)
    # and the pruned forces of the final state are the oracle's
    P = np.mod(runs[1][1], bmax)
    allpos, own, _, _, _ = orc.periodic_system(P, bmin, bmax, 2.5, 0.3)
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(2.5), own=own)
    assert rel_rms(runs[1][2], R[: len(P)]) <= (1e-12 if prec == 0 else 1e-6)


def test_checkpoint_restart_continues_the_trajectory(eng_mod, tmp_path):
    """A run checkpointed at a rebuild step and restarted in a new engine continues bit for bit."""
    from autopas_gb300 import checkpoint
    pos, vel, bmin, bmax = liquid(5, seed=41)
    kw = dict(periodic=True, rebuild_frequency=10, precision=eng_mod.PRECISION_MIXED)
    e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), **kw)
    e.set_particles(pos, vel)
    e.compute_forces()
    e.step(0.002, 20)
    P1, V1 = e.state()
    e.step(0.002, 20)
    Pref, Vref = e.state()
    p = tmp_path / "lj_0_20.vtu"
    checkpoint.write_rank_record(p, P1, V1, np.zeros_like(P1), np.zeros(len(P1)), np.arange(len(P1)))
    r = checkpoint.read_rank_record(p)
    e2 = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), **kw)
    e2.set_particles(np.mod(r["pos"], bmax), r["vel"])
    e2.compute_forces()
    e2.step(0.002, 20)
    P2, V2 = e2.state()
    d = P2 - Pref
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    assert np.abs(d).max() < 1e-12
    assert np.abs(V2 - Vref).max() < 1e-12


def test_page_locked_host_buffers_are_read_and_written_directly(eng_mod):
    """Positions from page-locked host memory and forces into it (the kernels use the buffers' device mapping)
    give bit for bit what the staged copies give."""
    torch = pytest.importorskip("torch")
    pos, vel, bmin, bmax = liquid(5, seed=43)
    e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_MIXED)
    e.set_particles(pos, vel)
    e.compute_forces()
    moved = pos + np.random.default_rng(5).normal(0.0, 0.01, pos.shape)
    e.update_positions(moved)
    e.compute_forces()
    f_ref = e.forces()

    def pinned():
        return torch.empty(len(pos), dtype=torch.float64, pin_memory=True).numpy()

    hx, hy, hz = pinned(), pinned(), pinned()
    hx[:], hy[:], hz[:] = moved[:, 0], moved[:, 1], moved[:, 2]
    e.update_positions(pos)
    e.update_positions_soa(hx, hy, hz)
    e.compute_forces()
    fx, fy, fz = pinned(), pinned(), pinned()
    e.forces_into(fx, fy, fz)
    np.testing.assert_array_equal(np.stack([fx, fy, fz], 1), f_ref)
    P, _ = e.state()
    np.testing.assert_array_equal(P, moved)


@pytest.mark.parametrize("traversal,n3", [(0, 0), (1, 0), (2, 1)])
def test_dummies_at_the_top_of_towers(eng_mod, orc, traversal, n3):
    """Particles the caller marks as dummies keep their slots and are z-sorted with the others; where they are the
    highest particles of their towers, whole clusters hold dummies only.  The tower search still sees every
    cluster below them: the pair sets (rc+skin and rc) are the oracle's bit for bit and the forces match."""
    pos, vel, bmin, bmax = liquid(5, seed=43)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    o = own.copy()
    o[allpos[:, 2] > bmax[2] + 0.5] = 0
    assert (o == 0).sum() > 100
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, traversal=traversal, newton3=n3)
    e.set_particles(allpos, ownership=o)
    g = e.compute_forces()[0]
    F = e.forces()
    for which in (0, 1):
        a, b, _ = e.pair_set(which)
        dev = np.unique(np.stack([np.minimum(a, b), np.maximum(a, b)], 1), axis=0)
        if which == 0:
            ra, rb = orc.pair_set(allpos, rc + skin, own=o)
        else:
            ra, rb = orc.interacting_set(allpos, rc, own=o)
        ref = np.unique(np.stack([np.minimum(ra, rb), np.maximum(ra, rb)], 1), axis=0)
        assert np.array_equal(dev, ref)
    e.close()
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=o)
    real = o == 1
    assert rel_rms(F[real], R[real]) <= 1e-6
    assert g["upot"] == pytest.approx(glob[0], rel=1e-6)
