"""pe_lj_forces_noalloc: forces for callers that cannot allocate device memory.

Such callers (hosts whose device memory is all handed out by a framework's pool, plug-in hosts that forbid
plug-ins to allocate, loops that must not block in cudaMalloc) own their particle buffers and call this entry
point, which itself allocates nothing.  The tests call it through the C ABI and compare it with the engine's
regular entry point (pe_compute_forces in the FP64 form) and with the CPU oracle on the same owned + halo
particles, on two calls in a row, with the FP64 tolerance of the other parity tests: forces within 1e-12 of the
largest force, Upot and virial within 1e-12 relative, the interacting-pair count exactly.  The second call must
leave the device's free memory unchanged.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine
    return torch, engine


def owned_and_halo(orc, seed, ncells=5):
    from autopas_gb300 import workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(ncells, 0.8442, 0.72, seed=seed)
    rng = np.random.default_rng(seed)
    pos = np.mod(pos + rng.normal(0, 0.06, pos.shape), bmax)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    return allpos, own, bmin, bmax, rc, skin


def run_noalloc(torch, engine, cfg, allpos, own, types=None, calls=2):
    """Calls the entry point `calls` times on the same device buffers; returns the forces and globals of each
    call and the device's free memory before and after the last call."""
    n = len(allpos)
    dev = torch.device("cuda", torch.cuda.current_device())
    x, y, z = (torch.tensor(np.ascontiguousarray(allpos[:, d]), dtype=torch.float64, device=dev) for d in range(3))
    o = torch.tensor(own, dtype=torch.int8, device=dev)
    t = None if types is None else torch.tensor(types, dtype=torch.int32, device=dev)
    fx, fy, fz = (torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3))
    glob = torch.empty(6, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    out, free = [], []
    for call in range(calls):
        for buf in (fx, fy, fz, glob):
            buf.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        if call == calls - 1:
            free.append(torch.cuda.mem_get_info(dev)[0])
        engine.lj_forces_noalloc(cfg, n, x.data_ptr(), y.data_ptr(), z.data_ptr(),
                                 None if t is None else t.data_ptr(), o.data_ptr(), fx.data_ptr(), fy.data_ptr(),
                                 fz.data_ptr(), glob.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        if call == calls - 1:
            free.append(torch.cuda.mem_get_info(dev)[0])
        out.append((torch.stack([fx, fy, fz], 1).cpu().numpy(), glob.cpu().numpy()))
    return out, free


def check_against(F, gl, ref_F, ref_upot, ref_virial, ref_pairs, label):
    scale = np.abs(ref_F).max()
    np.testing.assert_allclose(F, ref_F, rtol=0, atol=1e-12 * scale, err_msg=label)
    assert gl[0] == pytest.approx(ref_upot, rel=1e-12), label
    assert gl[1] == pytest.approx(ref_virial, rel=1e-12), label
    assert int(round(gl[5])) == ref_pairs, label


def test_noalloc_entry_point_matches_engine_and_oracle_on_two_calls(env, orc):
    torch, engine = env
    allpos, own, bmin, bmax, rc, skin = owned_and_halo(orc, seed=4)
    n = len(allpos)
    assert n <= engine.NOALLOC_MAX_PARTICLES

    e = engine.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=engine.PRECISION_FP64)
    e.set_particles(allpos, ownership=own)
    g = e.compute_forces()[0]
    ref = e.forces()
    e.close()
    R, glob, _ = orc.lj_forces(allpos, orc.LJ(rc), own=own)
    R[own != orc.ORC_OWNED] = 0.0
    ia, _ = orc.interacting_set(allpos, rc, own=own)

    cfg, keep = engine.make_config(rc)
    out, free = run_noalloc(torch, engine, cfg, allpos, own)
    for call, (F, gl) in enumerate(out):
        check_against(F, gl, ref, g["upot"], g["virial"], g["num_pairs"], f"engine, call {call}")
        check_against(F, gl, R, glob[0], glob[1], len(ia), f"oracle, call {call}")
    assert free[0] == free[1], "the call changed the device's free memory"
    del keep


def test_noalloc_entry_point_with_mixing_and_shift(env, orc):
    """Three types with unequal epsilon and sigma, shifted potential: the Lorentz-Berthelot table the entry
    point builds on the host and its per-type indexing, against the FP64 engine and the oracle."""
    torch, engine = env
    allpos, own, bmin, bmax, rc, skin = owned_and_halo(orc, seed=6)
    n = len(allpos)
    eps, sig = (1.0, 0.8, 1.2), (1.0, 1.1, 0.9)
    types = np.random.default_rng(6).integers(0, 3, n).astype(np.int32)
    e = engine.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=engine.PRECISION_FP64,
                          epsilon=eps, sigma=sig, mass=(1.0, 1.0, 1.0), shift=True)
    e.set_particles(allpos, types=types, ownership=own)
    g = e.compute_forces()[0]
    ref = e.forces()
    e.close()
    lj = orc.LJ(rc, epsilon=eps, sigma=sig, shift=True)
    R, glob, _ = orc.lj_forces(allpos, lj, types=types, own=own)
    R[own != orc.ORC_OWNED] = 0.0
    ia, _ = orc.interacting_set(allpos, rc, own=own)
    cfg, keep = engine.make_config(rc, epsilon=eps, sigma=sig, mass=(1.0, 1.0, 1.0), shift=True)
    out, _ = run_noalloc(torch, engine, cfg, allpos, own, types=types)
    for call, (F, gl) in enumerate(out):
        check_against(F, gl, ref, g["upot"], g["virial"], g["num_pairs"], f"engine, call {call}")
        check_against(F, gl, R, glob[0], glob[1], len(ia), f"oracle, call {call}")
    del keep


def test_noalloc_entry_point_flags_bad_types_and_ignores_unknown_ownership(env, orc):
    torch, engine = env
    allpos, own, bmin, bmax, rc, skin = owned_and_halo(orc, seed=8, ncells=4)
    cfg, keep = engine.make_config(rc)
    # ownership values outside {owned, halo}: the particles are ignored, as if they were not there
    odd = own.copy()
    odd[::7] = 3
    odd[3::11] = -1
    out, _ = run_noalloc(torch, engine, cfg, allpos, odd, calls=1)
    keepm = (odd == orc.ORC_OWNED) | (odd == orc.ORC_HALO)
    R, glob, _ = orc.lj_forces(allpos[keepm], orc.LJ(rc), own=odd[keepm])
    R[odd[keepm] != orc.ORC_OWNED] = 0.0
    F, gl = out[0]
    assert not np.any(F[~keepm])
    scale = np.abs(R).max()
    np.testing.assert_allclose(F[keepm], R, rtol=0, atol=1e-12 * scale)
    assert gl[0] == pytest.approx(glob[0], rel=1e-12)
    # one type beyond the table: every global of the call is NaN; the next valid call is clean again
    types = np.zeros(len(allpos), np.int32)
    types[5] = 7
    out, _ = run_noalloc(torch, engine, cfg, allpos, own, types=types, calls=1)
    assert np.all(np.isnan(out[0][1]))
    out, _ = run_noalloc(torch, engine, cfg, allpos, own, types=np.zeros(len(allpos), np.int32), calls=1)
    assert np.all(np.isfinite(out[0][1]))
    del keep


def test_noalloc_entry_point_rejects_sizes_beyond_its_limit(env):
    torch, engine = env
    dev = torch.device("cuda", torch.cuda.current_device())
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    cfg, keep = engine.make_config(2.5)
    p = buf.data_ptr()
    with pytest.raises(engine.EngineError) as ei:
        engine.lj_forces_noalloc(cfg, engine.NOALLOC_MAX_PARTICLES + 1, p, p, p, None, None, p, p, p, p, None)
    assert ei.value.code == -9
    del keep
