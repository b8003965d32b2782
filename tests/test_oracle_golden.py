"""Pins the CPU oracle against the reference's own known-answer tests (read as text from the reference):

* applicationLibrary/molecularDynamics/tests/singleSiteTests/LJFunctorTestNoGlobals.h:27-31 (force triples)
* .../LJFunctorTestGlobals.cpp:12-73 with tests/testAutopas/testingHelpers/LJPotential.h (Upot, virial, where-factor)
* .../ForceCalculationTest.cpp:45-95 (2x2x1 grid, +-24 and zero forces, 1e-13)
* .../ATMFunctorTestNoGlobals.h:19-32 (ATM forces, with and without mixing)
* .../ATMFunctorTestGlobals.cpp:12-78 with testingHelpers/ATMPotential.h (ATM Upot and virial)
plus self-consistency checks of the restated traversals.
"""
import math

import numpy as np
import pytest


# ---------------------------------------------------------------------------------------- LJ known answers
def test_lj_aos_no_globals_known_answer(orc):
    lj = orc.LJ.single(1.0, 24.0, 1.0)
    expected = np.array([-4547248.8989645941, -9094497.7979291882, -13641746.696893783])
    for newton3 in (True, False):
        fi, fj, _, hit = orc.lj_aos([0, 0, 0], [0.1, 0.2, 0.3], lj, newton3=newton3)
        assert hit == 1
        np.testing.assert_allclose(fi, expected, rtol=0, atol=1e-7)
        if newton3:
            np.testing.assert_allclose(fj, -expected, rtol=0, atol=1e-7)
        else:
            assert np.all(fj == 0)


def test_lj_aos_no_globals_mixing_known_answer(orc):
    lj = orc.LJ(1.0, epsilon=[1.0, 2.0], sigma=[1.0, 2.0])
    expected = np.array([-835415983.7676939964294, -1670831967.5353879928588, -2506247951.3030819892883])
    fi, fj, _, _ = orc.lj_aos([0, 0, 0], [0.1, 0.2, 0.3], lj, ti=0, tj=1)
    np.testing.assert_allclose(fi, expected, rtol=0, atol=1e-7)
    np.testing.assert_allclose(fj, -expected, rtol=0, atol=1e-7)


def lj_potential_ref(pi, pj, cutoff, sigma, epsilon):
    """testingHelpers/LJPotential.h:21-47 restated."""
    d = np.subtract(pi, pj)
    dist = math.sqrt(float(d @ d))
    if dist > cutoff:
        return 0.0
    sdr = sigma / dist
    lj6 = sdr ** 6
    return 4.0 * epsilon * (lj6 * lj6 - lj6)


def lj_virial_ref(pi, pj, cutoff, sigma, epsilon):
    """testingHelpers/LJPotential.h:56-136 restated: analytic force, virial = sum_k dr_k * F_k."""
    d = np.subtract(pi, pj)
    dist = math.sqrt(float(d @ d))
    if dist > cutoff:
        return 0.0
    r6 = dist ** 6
    s6 = sigma ** 6
    dlj6 = s6 / (r6 * dist)
    dlj12 = (s6 * s6) / (r6 * r6 * dist)
    dUr = 48.0 * epsilon * (dlj12 - 0.5 * dlj6)
    f = d / dist * dUr
    return float((d * f).sum())


@pytest.mark.parametrize("where,factor,own", [("inside", 1.0, (1, 1)), ("boundary", 0.5, (1, 2)),
                                              ("outside", 0.0, (2, 2))])
@pytest.mark.parametrize("newton3", [True, False])
def test_lj_globals_where_factor(orc, where, factor, own, newton3):
    """LJFunctorTestGlobals.cpp:12-73: owned/halo ownership scales Upot and virial by the where-factor."""
    xoff = {"inside": 0.0, "boundary": 4.9, "outside": 5.0}[where]
    p1 = np.array([0.0 + xoff, 0.0, 0.0])
    p2 = np.array([0.1 + xoff, 0.2, 0.3])
    lj = orc.LJ.single(1.0, 24.0, 1.0)
    glob = np.zeros(4)
    fi, fj = np.zeros(3), np.zeros(3)
    orc.lj_aos(p1, p2, lj, own_i=own[0], own_j=own[1], newton3=newton3, fi=fi, fj=fj, glob=glob)
    if not newton3:
        orc.lj_aos(p2, p1, lj, own_i=own[1], own_j=own[0], newton3=newton3, fi=fj, fj=fi, glob=glob)
    upot = glob[0] * 0.5 / 6.0
    vir = glob[1:].sum() * 0.5
    e_ref = lj_potential_ref(p1, p2, 1.0, 1.0, 1.0)
    v_ref = lj_virial_ref(p1, p2, 1.0, 1.0, 1.0)
    assert upot == pytest.approx(factor * e_ref, abs=1e-7)
    assert vir == pytest.approx(factor * v_ref, abs=1e-7, rel=1e-12)


def grid_2x2x1(spacing):
    """GridGenerator::fillWithParticles with offset 0.5 (tools/autopasTools/generators/GridGenerator.h:61-75)."""
    pts = []
    for z in range(1):
        for y in range(2):
            for x in range(2):
                pts.append([x * spacing + 0.5, y * spacing + 0.5, z * spacing + 0.5])
    return np.array(pts)


@pytest.mark.parametrize("spacing,cutoff,expected", [
    (1.0, 1.1, [[-24, -24, 0], [24, -24, 0], [-24, 24, 0], [24, 24, 0]]),
    (2 ** (1 / 6), 1.3, [[0, 0, 0]] * 4),
])
def test_force_calculation_grid(orc, spacing, cutoff, expected):
    """ForceCalculationTest.cpp:45-95 (lc_c08, setParticleProperties(24, 1)), tolerance 1e-13."""
    lj = orc.LJ.single(cutoff, 24.0, 1.0)
    F, _, _ = orc.lj_forces(grid_2x2x1(spacing), lj)
    np.testing.assert_allclose(F, np.array(expected, float), rtol=0, atol=1e-13)
    F2, _, _ = orc.cpu_lc_c08(grid_2x2x1(spacing), lj, skin=0.0, nthreads=2)
    np.testing.assert_allclose(F2, np.array(expected, float), rtol=0, atol=1e-13)


# ---------------------------------------------------------------------------------------- ATM known answers
def test_atm_no_globals_known_answer(orc):
    p1, p2, p3 = [0.0, 0.0, 0.0], [0.1, 0.2, 0.3], [0.3, 0.2, 0.1]
    fi, fj, fk, _, hit = orc.atm_aos(p1, p2, p3, 1.0, 1.0)
    assert hit == 1
    np.testing.assert_allclose(fi, [-188761.250385809] * 3, rtol=0, atol=1e-7)
    np.testing.assert_allclose(fj, [-95789.2912405596, 94380.6251929043, 284550.541626368], rtol=0, atol=1e-7)
    np.testing.assert_allclose(fk, [284550.541626368, 94380.6251929043, -95789.2912405596], rtol=0, atol=1e-7)
    # mixing: nu = cbrt(1 * 1.25 * 0.1) = 0.5 (ParticlePropertiesLibrary ATM mixing)
    nu = (1.0 * 1.25 * 0.1) ** (1 / 3)
    fi, fj, fk, _, _ = orc.atm_aos(p1, p2, p3, nu, 1.0)
    np.testing.assert_allclose(fi, [-94380.6251929043] * 3, rtol=0, atol=1e-7)
    np.testing.assert_allclose(fj, [-47894.6456202798, 47190.3125964521, 142275.270813184], rtol=0, atol=1e-7)


def atm_potential_ref(pi, pj, pk, nu):
    """testingHelpers/ATMPotential.h:25-61 restated."""
    pi, pj, pk = map(np.asarray, (pi, pj, pk))
    ij, ik, jk = pi - pj, pi - pk, pj - pk
    dij, dik, djk = (math.sqrt(float(v @ v)) for v in (ij, ik, jk))
    cos_i = float(ik @ ij) / (dik * dij)
    cos_j = -float(jk @ ij) / (djk * dij)
    cos_k = float(ik @ jk) / (dik * djk)
    rrr = dij * djk * dik
    return nu * (3 * cos_i * cos_j * cos_k + 1.0) / rrr ** 3


@pytest.mark.parametrize("own,factor", [((1, 1, 1), 1.0), ((1, 1, 2), 2 / 3), ((1, 2, 2), 1 / 3), ((2, 2, 2), 0.0)])
def test_atm_globals(orc, own, factor):
    """ATMFunctorTestGlobals.cpp:12-78: Upot x where-factor (cutoff 5, nu 0.7, abs 1e-8)."""
    p1, p2, p3 = [0.0, 0.0, 0.0], [0.1, 0.0, 0.0], [0.0, 0.2, 0.3]
    _, _, _, g, _ = orc.atm_aos(p1, p2, p3, 0.7, 5.0, own=own)
    upot = g[0] / 3.0 / 3.0
    assert upot == pytest.approx(factor * atm_potential_ref(p1, p2, p3, 0.7), abs=1e-8)


def test_atm_forces_sum_to_zero_and_match_aos(orc):
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 3.0, size=(60, 3))
    F, glob, hits = orc.atm_forces(pos, 0.073, 1.5)
    assert hits > 0
    np.testing.assert_allclose(F.sum(0), 0, atol=1e-9 * np.abs(F).max())


# ---------------------------------------------------------------------------------------- restated traversals
def test_c08_baseline_matches_oracle_forces(orc):
    rng = np.random.default_rng(1)
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(6, 0.8442, 0.72, seed=1)
    pos = pos + rng.normal(0, 0.05, pos.shape)
    pos = np.mod(pos, bmax)
    lj = orc.LJ(2.5)
    allpos, own, allt, owner, code = orc.periodic_system(pos, bmin, bmax, 2.5, 0.3)
    F1, g1, h1 = orc.lj_forces(allpos, lj, own=own)
    F2, g2, h2 = orc.cpu_lc_c08(allpos, lj, 0.3, own=own, nthreads=4)
    n = len(pos)
    scale = np.abs(F1[:n]).max()
    np.testing.assert_allclose(F2[:n], F1[:n], rtol=0, atol=1e-12 * scale)
    assert g2[0] == pytest.approx(g1[0], rel=1e-12)
    assert g2[1] == pytest.approx(g1[1], rel=1e-12)


def test_periodic_halos_md_flexible_rule(orc):
    """Every owned particle within rc+skin of a face gets an image; image positions are x +- len."""
    rng = np.random.default_rng(2)
    bmin, bmax = np.zeros(3), np.array([10.0, 11.0, 12.0])
    pos = rng.uniform(0, 1, size=(500, 3)) * bmax
    hpos, owner, code = orc.make_halos(pos, bmin, bmax, 2.5, 0.3)
    L = 2.8
    for k in range(len(hpos)):
        s = np.array([code[k] % 3 - 1, (code[k] // 3) % 3 - 1, code[k] // 9 - 1])
        p = pos[owner[k]]
        for d in range(3):
            if s[d] == 1:
                assert p[d] < bmin[d] + L and hpos[k, d] == p[d] + (bmax[d] - bmin[d])
            elif s[d] == -1:
                assert p[d] >= bmax[d] - L and hpos[k, d] == p[d] - (bmax[d] - bmin[d])
            else:
                assert hpos[k, d] == p[d]
    # expected count: product over dims of (1 + near-low + near-high) - 1 per particle
    exp = 0
    for p in pos:
        m = 1
        for d in range(3):
            m *= 1 + (p[d] < L) + (p[d] >= bmax[d] - L)
        exp += m - 1
    assert len(hpos) == exp


def test_pair_set_rules(orc):
    """Verlet rule dr2 < L^2 vs LJ mask dr2 <= rc^2; halo-halo pairs never appear."""
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 6, size=(400, 3))
    own = np.where(pos[:, 0] < 1.0, 2, 1).astype(np.int8)
    a, b = orc.pair_set(pos, 1.5, own=own)
    assert not np.any((own[a] == 2) & (own[b] == 2))
    d2 = ((pos[a] - pos[b]) ** 2).sum(1)
    assert np.all(d2 < 1.5 ** 2 * (1 + 1e-15))
    # brute force count
    dd = ((pos[:, None] - pos[None]) ** 2).sum(-1)
    iu = np.triu_indices(len(pos), 1)
    m = (dd[iu] < 2.25) & ~((own[iu[0]] == 2) & (own[iu[1]] == 2))
    assert m.sum() == len(a)


def test_dist_modes_differ_only_by_contraction(orc):
    L = orc.lib()
    rng = np.random.default_rng(4)
    diff = 0
    for _ in range(2000):
        dx, dy, dz = rng.uniform(-3, 3, 3)
        s = L.orc_dist2(dx, dy, dz, orc.DIST_STRICT)
        f = L.orc_dist2(dx, dy, dz, orc.DIST_FMA_SOA)
        assert s == pytest.approx(f, rel=1e-15)
        diff += s != f
        assert s == (dx * dx + dy * dy) + dz * dz
    assert diff > 0


def test_reference_flags_contract_dr2_to_the_default_form(orc):
    """The reference's SoA distance expression (LJFunctor.h:287-293), compiled by this host's C compiler with the
    reference's flags, gives exactly fma(dz,dz, fma(dx,dx, dy*dy)): the engine's default distance form
    (PE_DIST_FMA_SOA) is the one the reference binary computes on this host."""
    probe = orc.contraction_probe()
    L = orc.lib()
    rng = np.random.default_rng(12)
    n = 20000
    pi = rng.uniform(0, 50, (n, 3))
    # displacements of every scale, many near the cutoff radii the engine tests against
    pj = pi + rng.normal(0, 1, (n, 3)) * rng.choice([1e-3, 0.5, 1.0, 3.4], (n, 1))
    got = probe(pi[:, 0], pi[:, 1], pi[:, 2], pj[:, 0], pj[:, 1], pj[:, 2])
    d = pi - pj
    forms = {m: np.array([L.orc_dist2(*d[k], m) for k in range(n)])
             for m in (orc.DIST_FMA_SOA, orc.DIST_STRICT, orc.DIST_FMA_DOT)}
    assert np.array_equal(got, forms[orc.DIST_FMA_SOA])
    # the test can tell the forms apart: the uncontracted and the dot forms differ on many of these inputs
    assert (got != forms[orc.DIST_STRICT]).sum() > n // 20
    assert (got != forms[orc.DIST_FMA_DOT]).sum() > n // 20


def test_contraction_changes_the_pair_sets_of_straddling_pairs(orc, straddling_pairs):
    """Pairs built to straddle (rc+skin)^2 and rc^2: the oracle's Verlet and interacting sets differ between the
    uncontracted expression and the reference's contracted one, so a parity test on them can tell a wrong
    default distance form."""
    rc, skin = 2.5, 0.3
    for radius, rule in ((rc + skin, orc.pair_set), (rc, orc.interacting_set)):
        pos, flags = straddling_pairs(orc, radius, 27, seed=3, spacing=3 * (rc + skin))
        arg = rc + skin if rule is orc.pair_set else rc
        a_s, b_s = rule(pos, arg, dist_mode=orc.DIST_STRICT)
        a_f, b_f = rule(pos, arg, dist_mode=orc.DIST_FMA_SOA)
        col = (0, 2) if rule is orc.pair_set else (1, 3)
        assert len(a_s) == flags[:, col[0]].sum() and len(a_f) == flags[:, col[1]].sum()
        assert len(a_s) != len(a_f) or not np.array_equal(a_s, a_f)


def test_atm_cell_list_oracle_matches_the_quadratic_one(orc):
    """The cell-list ATM restatement (full-size checks, CPU baseline) against the quadratic enumeration."""
    from autopas_gb300 import workloads
    p, v, b0, b1 = workloads.fcc_lj(6, 0.8, 1.0, seed=31)
    p = np.mod(p + np.random.default_rng(31).normal(0, 0.03, p.shape), b1)
    allpos, own, _, _, _ = orc.periodic_system(p, b0, b1, 2.5, 0.3)
    R, g, _ = orc.atm_forces(allpos, 0.073, 2.5, own=own)
    R2, g2, _ = orc.atm_forces_cells(allpos, 0.073, 2.5, own=own)
    n = len(p)
    np.testing.assert_allclose(R2[:n], R[:n], rtol=0, atol=1e-13 * np.abs(R[:n]).max())
    assert g2[0] == pytest.approx(g[0], rel=1e-13)
    assert g2[1] == pytest.approx(g[1], rel=1e-11)  # the virial sum cancels: 11.5 from terms of ~1e3


def test_tower_grid_geometry(orc):
    """ClusterTowerBlock2D::estimateOptimalGridSideLength restated (side, towers incl. halo)."""
    side, num, halo = orc.tower_grid([0, 0, 0], [33.0, 34.0, 35.0], 32000, 4, 2.8)
    opt = float(np.cbrt(4 / (32000 / (33.0 * 34.0 * 35.0))))
    owned = math.ceil(33.0 / opt)
    assert side[0] == pytest.approx(33.0 / owned, rel=1e-15)
    assert num[0] == owned + 2 * math.ceil(2.8 / side[0])
    assert halo == max(math.ceil(2.8 / side[0]), math.ceil(2.8 / side[1]))
    idx = orc.tower_index([0.0, 33.0, 5.0], [0, 0, 0], [33.0, 34.0, 35.0], side, num, halo, 2.8)
    assert idx[0] == halo and idx[1] == int(33.0 / side[1]) + halo


def test_wrap_rule(orc):
    L = orc.lib()
    assert L.orc_wrap(-0.5, 0.0, 10.0) == 9.5
    assert L.orc_wrap(10.0, 0.0, 10.0) == 0.0
    assert L.orc_wrap(-1e-20, 0.0, 10.0) == np.nextafter(10.0, 0.0)


def test_checkpoint_roundtrip_is_exact(tmp_path):
    from autopas_gb300 import checkpoint
    rng = np.random.default_rng(8)
    pos, vel, f = rng.normal(size=(50, 3)) * 7, rng.normal(size=(50, 3)), rng.normal(size=(50, 3)) * 1e3
    t, ids = rng.integers(0, 4, 50), np.arange(50) * 3 + 1
    p = tmp_path / "run_0_100.vtu"
    checkpoint.write_rank_record(p, pos, vel, f, t, ids)
    r = checkpoint.read_rank_record(p)
    for k, ref in (("pos", pos), ("vel", vel), ("forces", f), ("type_ids", t), ("ids", ids)):
        assert np.array_equal(r[k], ref), k
