import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine library")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    from oracle import oracle as o
    o.build()
    return o


def contraction_pairs(orc, radius, count, seed, spacing):
    """Isolated particle pairs whose FP64 squared distance lies within a few ulps of radius^2 and on opposite
    sides of it under the uncontracted expression and under the reference's contracted one (PE_DIST_FMA_SOA).
    Pairs sit on a cubic grid `spacing` apart (no other particle within radius).  Returns (pos, flags) with
    flags[k] = (strict < r^2, strict <= r^2, fma < r^2, fma <= r^2) of pair k."""
    import numpy as np
    L = orc.lib()
    rng = np.random.default_rng(seed)
    r2 = radius * radius
    m = int(np.ceil(count ** (1.0 / 3.0)))
    sites = (np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)[:count] + 0.5) * spacing
    pos, flags = [], []
    for site in sites:
        for _ in range(100000):
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            pi = site + rng.uniform(-0.1, 0.1, 3)
            pj = pi + u * radius
            for _ in range(64):
                d = pi - pj
                s = L.orc_dist2(*d, orc.DIST_STRICT)
                f = L.orc_dist2(*d, orc.DIST_FMA_SOA)
                if (s < r2) != (f < r2) or (s <= r2) != (f <= r2):
                    break
                # walk pj one ulp per coordinate towards or away from pi, following the sign of the error
                toward = s > r2
                pj = np.array([np.nextafter(pj[q], pi[q] if toward else 2 * pj[q] - pi[q]) for q in range(3)])
            else:
                continue
            pos += [pi, pj]
            flags.append((s < r2, s <= r2, f < r2, f <= r2))
            break
    return np.array(pos), np.array(flags)


@pytest.fixture(scope="session")
def straddling_pairs():
    return contraction_pairs
