"""The C-ABI library builds, loads and exports every entry point include/*.h declares (no GPU needed)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(pe_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from autopas_gb300.build import build
    path = build()
    return ctypes.CDLL(path)


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "pe_create" in names and "pe_compute_forces" in names and "pe_gen_rsa" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_lists_engine_exports():
    from autopas_gb300 import engine
    decl = set(declared_symbols())
    assert set(engine.EXPORTS) <= decl
    assert {n for n in decl if not n.startswith("pe_gen_")} <= set(engine.EXPORTS)


def test_create_without_gpu_reports_no_device(lib):
    """Without a GPU pe_create must fail with PE_ERR_NO_DEVICE, never fall back to anything."""
    from autopas_gb300 import engine
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    with pytest.raises(engine.EngineError) as ei:
        engine.PairEngine(2.5, 0.3, ([0, 0, 0], [10, 10, 10]))
    assert ei.value.code in (-7, -3)


def test_rsa_generator_min_distance(lib):
    import numpy as np
    from autopas_gb300 import workloads
    pos = workloads.rsa(2000, [0, 0, 0], [12, 12, 12], [0, 0, 0], [12, 12, 12], 0.8, seed=3)
    d = pos[:, None, :] - pos[None, :, :]
    d -= 12 * np.round(d / 12)
    r2 = (d ** 2).sum(-1)
    np.fill_diagonal(r2, 1e9)
    assert r2.min() >= 0.64 - 1e-12
    assert pos.min() >= 0 and pos.max() < 12


def test_reference_arm_generates_the_same_slab_without_the_engine_library(lib, orc):
    """The benchmark's reference arm builds its slab with the oracle library's copy of the generator (the same
    source file, compiled the same way), so both arms time identical positions and the reference arm never
    loads the engine library."""
    import numpy as np
    from autopas_gb300 import workloads
    a = workloads.slab(n_total=6000, seed=7)
    b = workloads.slab(n_total=6000, seed=7, rsa_fn=orc.gen_rsa)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
