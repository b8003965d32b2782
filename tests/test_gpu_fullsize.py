"""Parity at the full sizes of the benchmark workloads, through checks that hold at any size.

The pair-by-pair comparisons with the oracle (test_gpu_parity.py) run on systems of a few thousand particles.
Here the engine runs the full workloads -- the 2,000,000-particle vapour-liquid slab (rc 3.0, skin 0.4), the
4,000,000-particle four-type mixture (Lorentz-Berthelot mixing, shifted potential, rc 3.0, skin 0.3) and the
512-system ensemble (5.7 M particles, rc 2.5, skin 0.3) -- and is compared with the oracle's LinkedCells c08
restatement (FP64, OpenMP on all host cores), which finishes these sizes in seconds.  Tolerances:

* FP64 form: forces within 1e-12 of the largest force, Upot and virial within 1e-12 relative.  One missing or
  extra pair would show: a pair at rc = 3 carries a force of 0.011, about 1e-5 of the largest force here.
* mixed form: force RMS error relative to the RMS force <= 1e-6 (the stated accuracy target), Upot and virial
  within 1e-6 relative.  In the ensemble some small systems have a net Upot or virial far below the size of its
  terms (attraction and repulsion cancel), and there the bound is 1e-6 of the sum of the terms' magnitudes,
  the scale of FP32 rounding in a sum: with a = sum of eps24 (sigma^2/r^2)^6 and b = sum of eps24
  (sigma^2/r^2)^3 over the interacting pairs, Upot = (a - b)/6 and virial = 2a - b, so the magnitudes are
  (a + b)/6 and 2a + b.  a and b come from a second oracle run with sigma^2 scaled by 2^(1/3), which doubles
  every (sigma^2/r^2)^3 and quadruples every (sigma^2/r^2)^6: Upot' = (4a - 2b)/6.
* mixed form, ensemble forces: the RMS error relative to the RMS force <= 1e-6 in every one of the 512 systems
  and over all 5.7 M particles.  Systems near density 0.43 start from a jittered lattice whose pair forces
  nearly cancel; the mixed kernels carry the rounding error of each FP32 displacement into r^2 (r2_resid2), which
  a CPU emulation of the arithmetic puts at 6.3-6.9e-7 for the worst of them (9-10e-7 without it).
* the newton3 path (pair-group half lists, reactions added by float reductions) is held to the same bounds.
* both forms: the number of interacting pairs (dr2 <= rc^2, each unordered periodic pair once) equals the
  oracle's, counted as owned-owned pairs plus half the owned-halo pairs (the oracle counts pairs over the owned
  particles alone, the halo images alone and both together).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng_mod():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine
    return engine


def rel_rms(F, R):
    return float(np.sqrt(((F - R) ** 2).sum(1).mean()) / np.sqrt((R ** 2).sum(1).mean()))


def oracle_reference(orc, pos, bmin, bmax, rc, skin, lj, types=None, magnitudes=False):
    """Oracle forces on the owned particles, globals and the unique interacting-pair count of a periodic
    system given as owned particles plus md-flexible halo images.  With magnitudes (one type, eps 1, sigma 1,
    unshifted), also the sums of the magnitudes of the Upot and virial terms."""
    allpos, own, allt, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin, types=types)
    n = len(pos)
    R, glob, h_all = orc.cpu_lc_c08(allpos, lj, skin, own=own, types=allt)
    _, _, h_oo = orc.cpu_lc_c08(allpos[:n], lj, skin, types=allt[:n])
    _, _, h_hh = orc.cpu_lc_c08(allpos[n:], lj, skin, types=allt[n:]) if len(allpos) > n else (None, None, 0)
    h_oh = h_all - h_oo - h_hh
    assert h_oh % 2 == 0  # every periodic owned-halo pair appears once from each side of the boundary
    if not magnitudes:
        return R[:n], glob, h_oo + h_oh // 2
    _, glob2, _ = orc.cpu_lc_c08(allpos, orc.LJ.single(rc, 24.0, 2.0 ** (1.0 / 3.0)), skin, own=own, types=allt)
    a = 3.0 * glob2[0] - 6.0 * glob[0]
    b = a - 6.0 * glob[0]
    return R[:n], glob, h_oo + h_oh // 2, ((a + b) / 6.0, 2.0 * a + b)


@pytest.fixture(scope="module")
def slab():
    from autopas_gb300 import workloads
    return workloads.slab(n_total=2_000_000, seed=7)


def test_slab_2m_matches_oracle(eng_mod, orc, slab):
    pos, vel, bmin, bmax = slab
    rc, skin = 3.0, 0.4
    R, glob, pairs = oracle_reference(orc, pos, bmin, bmax, rc, skin, orc.LJ(rc))
    scale = np.abs(R).max()
    for prec, C, traversal in ((eng_mod.PRECISION_FP64, 8, 1), (eng_mod.PRECISION_MIXED, 8, 1),
                               (eng_mod.PRECISION_MIXED, 4, 0), (eng_mod.PRECISION_MIXED, 8, 2)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=prec, cluster_size=C,
                               traversal=traversal, newton3=1 if traversal == 2 else 0, rebuild_frequency=20)
        e.set_particles(pos, vel)
        g = e.compute_forces()[0]
        F = e.forces()
        e.close()
        what = f"precision {prec}, C = {C}, traversal {traversal}"
        assert g["num_pairs"] == pairs, what
        if prec == eng_mod.PRECISION_FP64:
            np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * scale, err_msg=what)
            tol = 1e-12
        else:
            assert rel_rms(F, R) <= 1e-6, what
            tol = 1e-6
        assert g["upot"] == pytest.approx(glob[0], rel=tol), what
        assert g["virial"] == pytest.approx(glob[1], rel=tol), what


def test_slab_2m_newton3_steps_in_pieces(eng_mod, slab):
    """At 2M particles the newton3 evaluation runs in pieces (force kernels on two streams, each piece's finish
    on a third as soon as the pieces up to it are complete), replayed from CUDA graphs with the velocity and
    position halves fused.  After thirty velocity-Verlet steps with a rebuild at step 20, the forces of the last
    evaluation match the FP64 form's at the same positions (force RMS error <= 1e-6, Upot 1e-6, the same
    interacting pairs), and the trajectory stays near the particle-list one: the slab starts from random
    sequential addition with forces up to ~10^3, so FP32 differences of ~1e-3 in them move positions by ~1e-6
    over these steps; a lost or doubled reaction would move them by orders of magnitude more."""
    pos, vel, bmin, bmax = slab
    rc, skin, dt = 3.0, 0.4, 0.002
    out = {}
    for traversal in (1, 2):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, cluster_size=8, traversal=traversal,
                               newton3=1 if traversal == 2 else 0, rebuild_frequency=20, use_graphs=True)
        e.set_particles(pos, vel)
        e.compute_forces()
        g = e.step(dt, 30)[0]
        P, V = e.state()
        out[traversal] = (P, V, g, e.forces())
        e.close()
    P2, V2, g2, F2 = out[2]
    e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=eng_mod.PRECISION_FP64,
                           cluster_size=8, traversal=1)
    e.set_particles(P2, V2)
    g64 = e.compute_forces()[0]
    F64 = e.forces()
    e.close()
    assert rel_rms(F2, F64) <= 1e-6
    assert g2["num_pairs"] == g64["num_pairs"]
    assert g2["upot"] == pytest.approx(g64["upot"], rel=1e-6)
    P1 = out[1][0]
    d = P1 - P2
    d -= (bmax - bmin) * np.round(d / (bmax - bmin))
    print(f"newton3 in pieces against particle lists after 30 steps: max position difference {np.abs(d).max():.3g}")
    assert np.abs(d).max() < 1e-4


def test_mixture_4m_matches_oracle(eng_mod, orc):
    from autopas_gb300 import workloads
    n, rho, rc, skin = 4_000_000, 0.7, 3.0, 0.3
    side = (n / rho) ** (1.0 / 3.0)
    bmin, bmax = np.zeros(3), np.full(3, side)
    pos = workloads.rsa(n, bmin, bmax, bmin, bmax, 0.8, seed=23)
    rng = np.random.default_rng(23)
    types = rng.choice(4, size=len(pos), p=[0.4, 0.3, 0.2, 0.1]).astype(np.int32)
    eps, sig = [1.0, 0.8, 1.2, 0.6], [1.0, 1.1, 0.9, 1.2]
    lj = orc.LJ(rc, epsilon=eps, sigma=sig, shift=True)
    R, glob, pairs = oracle_reference(orc, pos, bmin, bmax, rc, skin, lj, types=types)
    scale = np.abs(R).max()
    for prec, traversal in ((eng_mod.PRECISION_FP64, 1), (eng_mod.PRECISION_MIXED, 1), (eng_mod.PRECISION_MIXED, 2)):
        e = eng_mod.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1, 1, 1, 1],
                               shift=True, precision=prec, cluster_size=8, traversal=traversal,
                               newton3=1 if traversal == 2 else 0)
        e.set_particles(pos, types=types)
        g = e.compute_forces()[0]
        F = e.forces()
        e.close()
        assert g["num_pairs"] == pairs, prec
        if prec == eng_mod.PRECISION_FP64:
            np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * scale)
            tol = 1e-12
        else:
            assert rel_rms(F, R) <= 1e-6
            tol = 1e-6
        assert g["upot"] == pytest.approx(glob[0], rel=tol), prec
        assert g["virial"] == pytest.approx(glob[1], rel=tol), prec


def test_ensemble_512_systems_match_oracle(eng_mod, orc):
    """Every one of the 512 systems against its own oracle run: forces, globals and pair count per system."""
    from autopas_gb300 import workloads
    rc, skin = 2.5, 0.3
    systems = workloads.ensemble(512, seed=11)
    boxes = [(s["bmin"], s["bmax"]) for s in systems]
    pos = np.concatenate([s["pos"] for s in systems])
    sysid = np.concatenate([np.full(len(s["pos"]), k, np.int32) for k, s in enumerate(systems)])
    lj = orc.LJ(rc)
    ref = [oracle_reference(orc, s["pos"], s["bmin"], s["bmax"], rc, skin, lj, magnitudes=True) for s in systems]
    Rall = np.zeros((len(pos), 3))
    for k, r in enumerate(ref):
        Rall[sysid == k] = r[0]
    for prec, traversal in ((eng_mod.PRECISION_FP64, 1), (eng_mod.PRECISION_MIXED, 1), (eng_mod.PRECISION_MIXED, 2)):
        e = eng_mod.PairEngine(rc, skin, boxes, periodic=True, precision=prec, cluster_size=8, traversal=traversal,
                               newton3=1 if traversal == 2 else 0)
        e.set_particles(pos, system=sysid)
        gs = e.compute_forces()
        F = e.forces()
        e.close()
        assert len(gs) == len(systems)
        if prec == eng_mod.PRECISION_MIXED:
            per_system = [rel_rms(F[sysid == k], r[0]) for k, r in enumerate(ref)]
            print(f"ensemble mixed force RMS error (traversal {traversal}): all particles {rel_rms(F, Rall):.3g}, worst system "
                  f"{max(per_system):.3g}, median {np.median(per_system):.3g}, "
                  f"{sum(x > 1e-6 for x in per_system)} systems above 1e-6")
            assert rel_rms(F, Rall) <= 1e-6
        for k, (R, glob, pairs, (u_abs, w_abs)) in enumerate(ref):
            Fk = F[sysid == k]
            what = f"precision {prec}, traversal {traversal}, system {k} ({len(R)} particles)"
            assert gs[k]["num_pairs"] == pairs, what
            if prec == eng_mod.PRECISION_FP64:
                np.testing.assert_allclose(Fk, R, rtol=0, atol=1e-12 * np.abs(R).max(), err_msg=what)
                assert gs[k]["upot"] == pytest.approx(glob[0], rel=1e-12), what
                assert gs[k]["virial"] == pytest.approx(glob[1], rel=1e-12), what
            else:
                assert rel_rms(Fk, R) <= 1e-6, what
                assert abs(gs[k]["upot"] - glob[0]) <= 1e-6 * max(abs(glob[0]), u_abs), what
                assert abs(gs[k]["virial"] - glob[1]) <= 1e-6 * max(abs(glob[1]), w_abs), what
