"""A slab rank's force evaluation on the GPU: the engine with an explicit-halo system over the rank's owned
particles and the halos the decomposition exchanged (here one rank, exchanging with itself) gives the periodic
engine's forces: FP64 form within 1e-12 of the largest force, the same Upot and virial; the pair counts follow
each container's convention."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_engine_as_slab_rank_force_function(orc):
    from autopas_gb300 import decomposition as D
    from autopas_gb300 import engine
    from autopas_gb300.build import build
    build()
    rc, skin = 2.5, 0.3
    ell = 12.0
    bmin, bmax = np.zeros(3), np.array([3 * ell, ell, ell])
    pos = orc.gen_rsa(int(0.7 * 3 * ell ** 3), bmin, bmax, bmin, bmax, 0.8, seed=31)
    dec = D.SlabDecomposition(0, 1, bmin, bmax, rc, skin)
    halos = dec.exchange_halos(D.Comm(None), np.concatenate([pos, np.arange(len(pos))[:, None]], 1))
    F, glob = D.engine_forces(engine, rc, skin, dec.lmin, dec.lmax, precision=engine.PRECISION_FP64)(pos, halos[:, :3])
    e = engine.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=engine.PRECISION_FP64)
    e.set_particles(pos)
    g = e.compute_forces()[0]
    R = e.forces()
    e.close()
    np.testing.assert_allclose(F, R, rtol=0, atol=1e-12 * np.abs(R).max())
    assert glob[0] == pytest.approx(g["upot"], rel=1e-12)
    assert glob[1] == pytest.approx(g["virial"], rel=1e-12)
    # the container counts every owned-halo pair once (the periodic engine counts each physical pair once)
    allpos = np.concatenate([pos, halos[:, :3]])
    own = np.concatenate([np.ones(len(pos), np.int8), np.full(len(halos), 2, np.int8)])
    oo, oh, _ = orc.count_interacting(allpos, rc, own=own)
    assert glob[2] == oo + oh
    assert g["num_pairs"] == oo + oh // 2


def test_engine_as_slab_rank_force_function_newton3(orc):
    """The same rank's force evaluation on the newton3 path (mixed form, explicit halos): forces within the mixed
    form's 1e-6 RMS bound of the FP64 periodic engine's, Upot and virial within 1e-6, the container's pair count."""
    from autopas_gb300 import decomposition as D
    from autopas_gb300 import engine
    from autopas_gb300.build import build
    build()
    rc, skin = 2.5, 0.3
    ell = 12.0
    bmin, bmax = np.zeros(3), np.array([3 * ell, ell, ell])
    pos = orc.gen_rsa(int(0.7 * 3 * ell ** 3), bmin, bmax, bmin, bmax, 0.8, seed=33)
    dec = D.SlabDecomposition(0, 1, bmin, bmax, rc, skin)
    halos = dec.exchange_halos(D.Comm(None), np.concatenate([pos, np.arange(len(pos))[:, None]], 1))
    F, glob = D.engine_forces(engine, rc, skin, dec.lmin, dec.lmax, precision=engine.PRECISION_MIXED, traversal=2,
                              newton3=1)(pos, halos[:, :3])
    e = engine.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=engine.PRECISION_FP64)
    e.set_particles(pos)
    g = e.compute_forces()[0]
    R = e.forces()
    e.close()
    rel = np.sqrt(((F - R) ** 2).sum(1).mean()) / np.sqrt((R ** 2).sum(1).mean())
    assert rel <= 1e-6
    assert glob[0] == pytest.approx(g["upot"], rel=1e-6)
    assert glob[1] == pytest.approx(g["virial"], rel=1e-6)
    allpos = np.concatenate([pos, halos[:, :3]])
    own = np.concatenate([np.ones(len(pos), np.int8), np.full(len(halos), 2, np.int8)])
    oo, oh, _ = orc.count_interacting(allpos, rc, own=own)
    assert glob[2] == oo + oh
