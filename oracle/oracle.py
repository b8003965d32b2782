"""ctypes binding of the CPU oracle (oracle/build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
cpu_baseline leg of ``bench.py``.  The engine never imports this module.
Each function states the reference code it restates (see oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib = None

ORC_DUMMY, ORC_OWNED, ORC_HALO = 0, 1, 2
DIST_FMA_SOA, DIST_STRICT, DIST_FMA_DOT = 0, 1, 2

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")


class LJParams(C.Structure):
    _fields_ = [
        ("cutoff", C.c_double),
        ("ntypes", C.c_int),
        ("eps24", C.POINTER(C.c_double)),
        ("sig2", C.POINTER(C.c_double)),
        ("shift6", C.POINTER(C.c_double)),
        ("dist_mode", C.c_int),
    ]


def build() -> str:
    """Compile the oracle with its Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def contraction_probe():
    """The reference's dr2 expression compiled with the reference's flags (contraction_probe.c):
    f(xi, yi, zi, xj, yj, zj) -> dr2 over arrays."""
    path = os.path.join(_HERE, "build", "libcontraction.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    L.probe_dist2.restype = None
    L.probe_dist2.argtypes = [C.c_int64] + [_dp] * 7

    def dist2(xi, yi, zi, xj, yj, zj):
        a = [np.ascontiguousarray(v, np.float64) for v in (xi, yi, zi, xj, yj, zj)]
        out = np.empty(len(a[0]))
        L.probe_dist2(len(out), *a, out)
        return out
    return dist2


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_dist2.restype = C.c_double
        L.orc_dist2.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_mixing.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_int, _dp, _dp, _dp]
        L.orc_lj_aos.restype = C.c_int
        L.orc_lj_aos.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(LJParams),
                                 _dp, _dp, _dp]
        L.orc_lj_forces.restype = C.c_int64
        L.orc_lj_forces.argtypes = [C.c_int64, _dp, _dp, _dp, _i32p, _i8p, C.POINTER(LJParams), _dp, _dp, _dp,
                                    _dp]
        for name in ("orc_pair_set", "orc_interacting_set"):
            f = getattr(L, name)
            f.restype = C.c_int64
            f.argtypes = [C.c_int64, _dp, _dp, _dp, _i8p, C.c_double, C.c_int, C.c_int64, _i64p, _i64p]
        L.orc_make_halos.restype = C.c_int64
        L.orc_make_halos.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int64, _dp,
                                     _dp, _dp, _i64p, _i32p]
        L.orc_wrap.restype = C.c_double
        L.orc_wrap.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_md_run.restype = C.c_int
        L.orc_md_run.argtypes = [C.c_int64, _dp, _dp, _dp, _i32p, _dp, _dp, _dp, C.c_double, C.POINTER(LJParams),
                                 C.c_double, C.c_int, C.c_void_p]
        L.orc_tower_grid.argtypes = [_dp, _dp, C.c_int64, C.c_int, C.c_double, _dp, _i64p, _i64p]
        L.orc_tower_index.argtypes = [_dp, _dp, _dp, _dp, _i64p, C.c_int64, C.c_double, _i64p]
        L.orc_atm_aos.restype = C.c_int
        L.orc_atm_aos.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp,
                                  _dp, _dp, _dp]
        L.orc_atm_forces.restype = C.c_int64
        L.orc_atm_forces.argtypes = [C.c_int64, _dp, _dp, _dp, _i8p, C.c_double, C.c_double, _dp, _dp, _dp, _dp]
        L.orc_count_interacting.restype = C.c_int
        L.orc_count_interacting.argtypes = [C.c_int64, _dp, _dp, _dp, _i8p, C.c_double, C.c_int, _i64p]
        L.pe_gen_rsa.restype = C.c_int64
        L.pe_gen_rsa.argtypes = [C.c_int64, C.c_int64, _dp, _dp, _dp, _dp, C.c_double, C.c_uint64, C.c_int64, _dp]
        L.orc_atm_forces_cells.restype = C.c_int64
        L.orc_atm_forces_cells.argtypes = [C.c_int64, _dp, _dp, _dp, _i8p, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                           _dp, _dp]
        L.orc_cpu_lc_c08.restype = C.c_int64
        L.orc_cpu_lc_c08.argtypes = [C.c_int64, _dp, _dp, _dp, _i32p, _i8p, C.POINTER(LJParams), C.c_double,
                                     C.c_int, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


class LJ:
    """Mixing table + parameters (ParticlePropertiesLibrary.h:444-473, LJFunctor constructor)."""

    def __init__(self, cutoff, epsilon=(1.0,), sigma=(1.0,), shift=False, dist_mode=DIST_FMA_SOA, table=None):
        self.cutoff = float(cutoff)
        eps = np.ascontiguousarray(epsilon, dtype=np.float64)
        sig = np.ascontiguousarray(sigma, dtype=np.float64)
        T = len(eps)
        self.ntypes = T
        if table is not None:  # explicit (eps24, sig2, shift6) as the functor's setParticleProperties does
            self.eps24, self.sig2, self.shift6 = (np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
                                                  for a in table)
            self.ntypes = int(round(len(self.eps24) ** 0.5))
        else:
            self.eps24 = np.zeros(T * T)
            self.sig2 = np.zeros(T * T)
            self.shift6 = np.zeros(T * T)
            lib().orc_mixing(T, eps, sig, self.cutoff, int(shift), self.eps24, self.sig2, self.shift6)
        self.p = LJParams(self.cutoff, self.ntypes, self.eps24.ctypes.data_as(C.POINTER(C.c_double)),
                          self.sig2.ctypes.data_as(C.POINTER(C.c_double)),
                          self.shift6.ctypes.data_as(C.POINTER(C.c_double)), int(dist_mode))

    @classmethod
    def single(cls, cutoff, epsilon24, sigma_squared, shift=False, dist_mode=DIST_FMA_SOA):
        """LJFunctor::setParticleProperties(epsilon24, sigmaSquared) (LJFunctor.h:583-590)."""
        c2 = cutoff * cutoff
        sh = 0.0
        if shift:
            s2 = sigma_squared / c2
            s6 = s2 * s2 * s2
            sh = epsilon24 * (s6 - s6 * s6)
        return cls(cutoff, table=([epsilon24], [sigma_squared], [sh]), dist_mode=dist_mode)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def lj_aos(ri, rj, lj: LJ, ti=0, tj=0, own_i=ORC_OWNED, own_j=ORC_OWNED, newton3=True, fi=None, fj=None, glob=None):
    fi = np.zeros(3) if fi is None else fi
    fj = np.zeros(3) if fj is None else fj
    glob = np.zeros(4) if glob is None else glob
    hit = lib().orc_lj_aos(_c(ri, np.float64), _c(rj, np.float64), ti, tj, own_i, own_j, int(newton3),
                           C.byref(lj.p), fi, fj, glob)
    return fi, fj, glob, hit


def lj_forces(pos, lj: LJ, own=None, types=None):
    """Forces on owned+halo particles (non-periodic).  Returns (F[n,3], glob[5], hits)."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    types = np.zeros(n, np.int32) if types is None else _c(types, np.int32)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    glob = np.zeros(5)
    hits = lib().orc_lj_forces(n, x, y, z, types, own, C.byref(lj.p), fx, fy, fz, glob)
    return np.stack([fx, fy, fz], 1), glob, hits


def _set(fn, pos, own, radius, dist_mode):
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    cap = 1 << 16
    while True:
        pa = np.zeros(cap, np.int64)
        pb = np.zeros(cap, np.int64)
        cnt = fn(n, x, y, z, own, float(radius), int(dist_mode), cap, pa, pb)
        if cnt <= cap:
            return pa[:cnt], pb[:cnt]
        cap = int(cnt)


def pair_set(pos, L, own=None, dist_mode=DIST_FMA_SOA):
    """VerletListHelpers.h:64-123 rule: dr2 < L^2.  Returns (a, b) index arrays, a < b."""
    return _set(lib().orc_pair_set, pos, own, L, dist_mode)


def interacting_set(pos, rc, own=None, dist_mode=DIST_FMA_SOA):
    """LJFunctor mask dr2 <= rc^2."""
    return _set(lib().orc_interacting_set, pos, own, rc, dist_mode)


def count_interacting(pos, rc, own=None, dist_mode=DIST_FMA_SOA):
    """Interacting pairs per ownership class: (owned-owned, owned-halo, halo-halo)."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    out = np.zeros(3, np.int64)
    if lib().orc_count_interacting(n, x, y, z, own, float(rc), int(dist_mode), out) != 0:
        raise MemoryError("cell list")
    return tuple(int(v) for v in out)


def gen_rsa(n, bmin, bmax, rmin, rmax, dmin, seed, existing=None):
    """The benchmark's random sequential addition (same source as the engine library's pe_gen_rsa)."""
    m = 0 if existing is None else len(existing)
    pos = np.zeros((m + n, 3))
    if m:
        pos[:m] = existing
    arrs = [_c(v, np.float64) for v in (bmin, bmax, rmin, rmax)]
    flat = pos.reshape(-1)
    placed = lib().pe_gen_rsa(m, n, *arrs, float(dmin), int(seed), int(200 * n + 10000), flat)
    if placed != n:
        raise RuntimeError(f"random sequential addition placed {placed} of {n} particles")
    return pos


def make_halos(pos, bmin, bmax, cutoff, skin):
    """md-flexible halo images.  Returns (hpos[m,3], owner[m], code[m])."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    cap = 4 * n + 1024
    while True:
        hx, hy, hz = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        owner = np.zeros(cap, np.int64)
        code = np.zeros(cap, np.int32)
        m = lib().orc_make_halos(n, x, y, z, _c(bmin, np.float64), _c(bmax, np.float64), cutoff, skin, cap, hx,
                                 hy, hz, owner, code)
        if m <= cap:
            return np.stack([hx[:m], hy[:m], hz[:m]], 1), owner[:m], code[:m]
        cap = int(m)


def periodic_system(pos, bmin, bmax, cutoff, skin, types=None):
    """owned + halo arrays for a periodic system, as md-flexible hands them to the container."""
    pos = np.asarray(pos, dtype=np.float64)
    hpos, owner, code = make_halos(pos, bmin, bmax, cutoff, skin)
    allpos = np.concatenate([pos, hpos])
    own = np.concatenate([np.full(len(pos), ORC_OWNED, np.int8), np.full(len(hpos), ORC_HALO, np.int8)])
    t = np.zeros(len(pos), np.int32) if types is None else np.asarray(types, np.int32)
    allt = np.concatenate([t, t[owner]]).astype(np.int32)
    return allpos, own, allt, owner, code


def md_run(pos, vel, types, mass, bmin, bmax, skin, lj: LJ, dt, nsteps, forces=None):
    """md-flexible semantics (see oracle.h).  Returns (pos, vel, f, energy[nsteps,3])."""
    x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1).copy()
    v = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1).copy()
    n = len(x) // 3
    t = np.zeros(n, np.int32) if types is None else _c(types, np.int32)
    m = _c(mass, np.float64)
    bmin, bmax = _c(bmin, np.float64), _c(bmax, np.float64)
    if forces is None:
        f = np.zeros(3 * n)
        lib().orc_md_run(n, x, v, f, t, m, bmin, bmax, skin, C.byref(lj.p), dt, 0, None)
    else:
        f = np.ascontiguousarray(forces, dtype=np.float64).reshape(-1).copy()
    e = np.zeros(3 * max(nsteps, 1))
    if nsteps > 0:
        lib().orc_md_run(n, x, v, f, t, m, bmin, bmax, skin, C.byref(lj.p), dt, nsteps, e.ctypes.data)
    return x.reshape(n, 3), v.reshape(n, 3), f.reshape(n, 3), e.reshape(-1, 3)[:nsteps]


def tower_grid(bmin, bmax, num_particles, cluster_size, interaction_length):
    side = np.zeros(2)
    num = np.zeros(2, np.int64)
    halo = np.zeros(1, np.int64)
    lib().orc_tower_grid(_c(bmin, np.float64), _c(bmax, np.float64), int(num_particles), int(cluster_size),
                         float(interaction_length), side, num, halo)
    return side, num, int(halo[0])


def tower_index(pos, bmin, bmax, side, num, halo, interaction_length):
    out = np.zeros(2, np.int64)
    lib().orc_tower_index(_c(pos, np.float64), _c(bmin, np.float64), _c(bmax, np.float64), _c(side, np.float64),
                          _c(num, np.int64), int(halo), float(interaction_length), out)
    return out


def atm_aos(ri, rj, rk, nu, cutoff, own=(1, 1, 1), newton3=True):
    fi, fj, fk, g = np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(4)
    hit = lib().orc_atm_aos(_c(ri, np.float64), _c(rj, np.float64), _c(rk, np.float64), own[0], own[1], own[2],
                            int(newton3), nu, cutoff, fi, fj, fk, g)
    return fi, fj, fk, g, hit


def atm_forces(pos, nu, cutoff, own=None):
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    glob = np.zeros(2)
    hits = lib().orc_atm_forces(n, x, y, z, own, nu, cutoff, fx, fy, fz, glob)
    return np.stack([fx, fy, fz], 1), glob, hits


def atm_forces_cells(pos, nu, cutoff, own=None, nthreads=0):
    """ATM forces on the owned particles via a cell list (OpenMP).  Returns (F, glob[2], triplet evaluations
    summed over owned vertices)."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    glob = np.zeros(2)
    hits = lib().orc_atm_forces_cells(n, x, y, z, own, nu, cutoff, int(nthreads), fx, fy, fz, glob)
    return np.stack([fx, fy, fz], 1), glob, hits


def cpu_lc_c08(pos, lj: LJ, skin, own=None, types=None, nthreads=0):
    """Timed CPU baseline (LinkedCells + c08 + SoA LJ, OpenMP).  Returns (F, glob, hits)."""
    pos = np.asarray(pos, dtype=np.float64)
    n = len(pos)
    own = np.full(n, ORC_OWNED, np.int8) if own is None else _c(own, np.int8)
    types = np.zeros(n, np.int32) if types is None else _c(types, np.int32)
    x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    glob = np.zeros(5)
    hits = lib().orc_cpu_lc_c08(n, x, y, z, types, own, C.byref(lj.p), float(skin), int(nthreads), fx, fy, fz,
                                glob)
    return np.stack([fx, fy, fz], 1), glob, hits
