"""pe_lj_forces_noalloc: forces for callers that cannot allocate device memory.

Such callers (hosts whose device memory is all handed out by a framework's pool, plug-in hosts that forbid
plug-ins to allocate, loops that must not block in cudaMalloc) own their particle buffers and call this entry
point, which itself allocates nothing.  The test checks it through the C ABI against the engine's regular
entry point (pe_compute_forces in the FP64 form) on the same owned + halo particles, on two calls in a row,
with the FP64 tolerance of the other parity tests: forces within 1e-12 of the largest force, Upot and virial
within 1e-12 relative, the interacting-pair count exactly.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_entry_point_matches_engine_on_two_calls(orc):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine, workloads

    pos, vel, bmin, bmax = workloads.fcc_lj(5, 0.8442, 0.72, seed=4)
    rng = np.random.default_rng(4)
    pos = np.mod(pos + rng.normal(0, 0.06, pos.shape), bmax)
    rc, skin = 2.5, 0.3
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    n = len(allpos)
    assert n <= engine.NOALLOC_MAX_PARTICLES

    e = engine.PairEngine(rc, skin, (bmin, bmax), periodic=False, precision=engine.PRECISION_FP64)
    e.set_particles(allpos, ownership=own)
    g = e.compute_forces()[0]
    ref = e.forces()
    e.close()

    dev = torch.device("cuda", torch.cuda.current_device())
    x, y, z = (torch.tensor(np.ascontiguousarray(allpos[:, d]), dtype=torch.float64, device=dev) for d in range(3))
    o = torch.tensor(own, dtype=torch.int8, device=dev)
    fx, fy, fz = (torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3))
    glob = torch.empty(6, dtype=torch.float64, device=dev)
    cfg, keep = engine.make_config(rc)
    stream = torch.cuda.current_stream(dev).cuda_stream
    scale = np.abs(ref).max()
    for call in range(2):
        for t in (fx, fy, fz, glob):
            t.fill_(float("nan"))
        engine.lj_forces_noalloc(cfg, n, x.data_ptr(), y.data_ptr(), z.data_ptr(), None, o.data_ptr(),
                                 fx.data_ptr(), fy.data_ptr(), fz.data_ptr(), glob.data_ptr(), stream)
        torch.cuda.synchronize(dev)
        F = torch.stack([fx, fy, fz], 1).cpu().numpy()
        gl = glob.cpu().numpy()
        np.testing.assert_allclose(F, ref, rtol=0, atol=1e-12 * scale, err_msg=f"call {call}")
        assert gl[0] == pytest.approx(g["upot"], rel=1e-12), call
        assert gl[1] == pytest.approx(g["virial"], rel=1e-12), call
        assert int(round(gl[5])) == g["num_pairs"], call
    del keep


def test_noalloc_entry_point_rejects_sizes_beyond_its_limit():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from autopas_gb300.build import build
    build()
    from autopas_gb300 import engine
    dev = torch.device("cuda", torch.cuda.current_device())
    buf = torch.zeros(8, dtype=torch.float64, device=dev)
    cfg, keep = engine.make_config(2.5)
    p = buf.data_ptr()
    with pytest.raises(engine.EngineError) as ei:
        engine.lj_forces_noalloc(cfg, engine.NOALLOC_MAX_PARTICLES + 1, p, p, p, None, None, p, p, p, p, None)
    assert ei.value.code == -9
    del keep
