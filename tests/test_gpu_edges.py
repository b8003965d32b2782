"""Edge cases of the engine on the GPU: empty and single-particle systems, a pair exactly at the cutoff, and a
large sparse box (coarse position encoding) whose pair sets must still equal the oracle's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng_mod():
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine
    return engine


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_empty_and_single_particle(eng_mod, prec):
    p = eng_mod.PRECISION_MIXED if prec == "mixed" else eng_mod.PRECISION_FP64
    bmin, bmax = np.zeros(3), np.full(3, 10.0)
    for n in (0, 1):
        e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=p)
        pos = np.full((n, 3), 5.0)
        e.set_particles(pos, np.zeros((n, 3)))
        g = e.compute_forces()[0]
        F = e.forces()
        assert F.shape == (n, 3) and not np.any(F)
        assert g["num_pairs"] == 0 and g["upot"] == 0.0 and g["virial"] == 0.0
        if n:
            e.step(0.002, 3)
            P, V = e.state()
            assert np.array_equal(P, pos)
        e.close()


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_pair_exactly_at_the_cutoff(eng_mod, orc, prec):
    """dr2 == rc^2 interacts (LJFunctor.h mask dr2 <= cutoffSquared); one ulp further apart does not."""
    p = eng_mod.PRECISION_MIXED if prec == "mixed" else eng_mod.PRECISION_FP64
    rc, skin = 2.5, 0.3
    bmin, bmax = np.zeros(3), np.full(3, 20.0)
    lj = orc.LJ(rc)
    x0 = 5.0
    for x1, interacts in ((x0 + rc, True), (np.nextafter(x0 + rc, 10.0), False)):
        pos = np.array([[x0, 6.0, 7.0], [x1, 6.0, 7.0]])
        assert ((pos[1, 0] - pos[0, 0]) ** 2 <= rc * rc) == interacts
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=p)
        e.set_particles(pos, np.zeros((2, 3)))
        g = e.compute_forces()[0]
        F = e.forces()
        e.close()
        R, glob, _ = orc.lj_forces(pos, lj)
        assert g["num_pairs"] == (1 if interacts else 0)
        if interacts:
            np.testing.assert_allclose(F, R, rtol=1e-6 if prec == "mixed" else 1e-13)
            assert g["upot"] == pytest.approx(glob[0], rel=1e-6 if prec == "mixed" else 1e-13)
        else:
            assert not np.any(F) and g["upot"] == 0.0


@pytest.mark.parametrize("traversal", [0, 1])
def test_large_sparse_box_pair_sets(eng_mod, orc, traversal):
    """A 600-wide periodic box puts the encoding base B at 2048 (ulp(B) = 2.4e-4): the particle lists, built
    from the hi parts of the records alone, must still hold every pair within rc+skin, and the interacting
    set must be the FP64 one."""
    from autopas_gb300 import workloads
    rc, skin = 3.0, 0.4
    bmin, bmax = np.zeros(3), np.array([600.0, 40.0, 40.0])
    pos = workloads.rsa(12000, bmin, bmax, bmin, bmax, 0.9, seed=23)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, traversal=traversal)
    e.set_particles(pos, np.zeros_like(pos))
    e.rebuild()
    for which in (0, 1):
        a, b, c = e.pair_set(which)
        dev = np.unique(np.stack([a, b, c], 1), axis=0)
        allpos, own, allt, owner, code = orc.periodic_system(pos, bmin, bmax, rc, skin)
        n = len(pos)
        if which == 0:
            ra, rb = orc.pair_set(allpos, rc + skin, own=own)
        else:
            ra, rb = orc.interacting_set(allpos, rc, own=own)
        halo_b = rb >= n
        bb = np.where(halo_b, owner[np.where(halo_b, rb - n, 0)], rb)
        cc = np.where(halo_b, code[np.where(halo_b, rb - n, 0)], 13)
        ref = np.unique(np.stack([ra, bb, cc], 1), axis=0)
        assert np.array_equal(dev, ref)
    g = e.compute_forces()[0]
    e.close()
    ia, ib = orc.interacting_set(allpos, rc, own=own)
    assert g["num_pairs"] == int(np.sum(ib < n)) + int(np.sum(ib >= n)) // 2


@pytest.mark.parametrize("traversal", [0, 1])
def test_default_distance_form_is_the_references_contraction(eng_mod, orc, straddling_pairs, traversal):
    """Pairs straddling (rc+skin)^2 and rc^2 by an ulp, where the uncontracted expression and the reference's
    contracted one (fma(dz,dz, fma(dx,dx, dy*dy)), what GCC makes of LJFunctor.h:287-293 with the reference's
    flags) disagree: an engine with the default options reproduces the contracted pair sets and interacting
    count, bit for bit, in both precision forms."""
    rc, skin = 2.5, 0.3
    spacing = 3 * (rc + skin)
    pos_l, _ = straddling_pairs(orc, rc + skin, 27, seed=3, spacing=spacing)
    pos_c, _ = straddling_pairs(orc, rc, 27, seed=4, spacing=spacing)
    pos_c = pos_c + np.array([3 * spacing + spacing, 0.0, 0.0])  # a second block of sites beside the first
    pos = np.concatenate([pos_l, pos_c])
    bmin, bmax = np.zeros(3), np.array([8 * spacing, 4 * spacing, 4 * spacing])
    own = np.ones(len(pos), np.int8)
    for which, rule, radius in ((0, orc.pair_set, rc + skin), (1, orc.interacting_set, rc)):
        ra, rb = rule(pos, radius)  # the oracle's default form
        sa, sb = rule(pos, radius, dist_mode=orc.DIST_STRICT)
        assert len(ra) != len(sa) or not np.array_equal(ra, sa), "the case no longer separates the forms"
        ref = np.unique(np.stack([ra, rb], 1), axis=0)
        for prec in (eng_mod.PRECISION_FP64, eng_mod.PRECISION_MIXED):
            e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=prec, traversal=traversal)
            e.set_particles(pos, ownership=own)
            e.rebuild()
            a, b, c = e.pair_set(which)
            dev = np.unique(np.stack([np.minimum(a, b), np.maximum(a, b)], 1), axis=0)
            assert np.array_equal(dev, ref), (which, prec)
            g = e.compute_forces()[0]
            ia, _ = orc.interacting_set(pos, rc)
            assert g["num_pairs"] == len(ia), (which, prec)
            e.close()


def test_capped_force_soft_start_separates_overlaps(eng_mod):
    """Uniform random positions (overlapping pairs) at density 0.7: forces reported under the cap never exceed it,
    and 200 capped-force steps with the velocity scaling (FP64 form) leave no pair closer than 0.7 sigma and a
    finite, uncapped force field at the thermostat's temperature."""
    rng = np.random.default_rng(5)
    n, rho = 3000, 0.7
    side = (n / rho) ** (1.0 / 3.0)
    bmin, bmax = np.zeros(3), np.full(3, side)
    pos = rng.uniform(0, side, (n, 3))
    vel = rng.normal(0, 1.0, (n, 3))
    e = eng_mod.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_FP64,
                           rebuild_frequency=10, traversal=1)
    e.set_particles(pos, vel)
    e.set_force_cap(100.0)
    e.compute_forces()
    F = e.forces()
    assert np.sqrt((F ** 2).sum(1)).max() <= 100.0 * (1 + 1e-12)
    e.soft_start(0.002, 200, 100.0, 1.0)
    P, V = e.state()
    F = e.forces()
    e.close()
    assert np.all(np.isfinite(F))
    d = P[:, None, :] - P[None, :, :]
    d -= side * np.round(d / side)
    r2 = (d ** 2).sum(-1)
    np.fill_diagonal(r2, np.inf)
    assert np.sqrt(r2.min()) > 0.7
    t = (V ** 2).sum() / (3 * n)
    assert 0.5 < t < 2.0


def test_rebuild_on_previous_sizes_and_its_redo(eng_mod, orc):
    """After a first rebuild, a rebuild runs on the previous rebuild's sizes (one host synchronisation); when a
    tower outgrows the size it assumed (here: 160 particles moved into one tower's column), it is redone with the
    read-back sizes.  After each rebuild the FP64 forces equal the oracle's to 1e-12 of the largest force."""
    from autopas_gb300 import workloads
    bmin, bmax = np.zeros(3), np.full(3, 20.0)
    rc, skin = 2.5, 0.3
    pos1 = workloads.rsa(2000, bmin, bmax, bmin, bmax, 0.85, seed=17)
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_FP64, cluster_size=8,
                           traversal=1)
    e.set_particles(pos1)

    def check(pos):
        e.rebuild()
        e.compute_forces()
        F = e.forces()
        allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
        R, _, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
        R = R[: len(pos)]
        np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * np.abs(R).max())
        return e.stats(reset=True)["rebuilds_redone"]

    e.compute_forces()                     # the first rebuild reads its sizes back
    assert check(pos1) == 0                # the same configuration: the previous sizes hold
    maxt1 = e.info()["max_tower_size"]
    assumed = 2
    while assumed < maxt1 + maxt1 // 4 + 1:  # the size the next rebuild assumes (the engine's rule)
        assumed *= 2
    assert assumed < 160, "the scenario needs a dense column larger than the assumed tower size"
    side, num, _, origin = e.tower_grid()
    lo = np.array([origin[0] + 0.05, origin[1] + 0.05, bmin[2]])
    hi = np.array([origin[0] + side[0] - 0.05, origin[1] + side[1] - 0.05, bmax[2]])
    col = workloads.rsa(160, bmin, bmax, lo, hi, 0.7, seed=18)
    pos2 = workloads.rsa(1840, bmin, bmax, bmin, bmax, 0.85, seed=19, existing=col)
    e.update_positions(pos2)
    assert check(pos2) == 1                # one tower outgrew the assumed size: redone
    assert e.info()["max_tower_size"] >= 160
    assert check(pos2) == 0                # the new sizes are assumed next time
    e.close()


def test_integer_pipe_conversions_match_the_converter(eng_mod):
    """The per-slot epilogues widen forces and narrow velocities with integer-pipe conversions; every float bit
    pattern widened and the rounding ties of every float narrowed give the hardware converter's bits."""
    assert eng_mod.check_conversions() == 0
