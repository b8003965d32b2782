"""Seeded synthetic inputs with the shapes, sizes and value distributions of the benchmark configurations.

* fcc_lj:   FCC lattice, n^3 unit cells at reduced density rho in a periodic cube, Maxwell-Boltzmann velocities
            at T with zero net momentum (md-flexible's cube-closest-packed object + Thermostat::addBrownianMotion
            role, examples/md-flexible/src/Thermostat.h:175-215).
* slab:     inhomogeneous vapour-liquid system in a 3:1:1 periodic box: the middle third along x is liquid at
            density 0.75, the rest vapour at 0.02, positions uniform within each region with a minimum pair
            distance (random sequential addition, seeded).  The liquid volume fraction (1/3) is a choice of this
            generator.
* ensemble: many independent periodic systems with log-uniform sizes, uniform densities and temperatures.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import engine as _engine


def mb_velocities(n, T, mass=1.0, seed=0):
    """Gaussian velocities at temperature T (k_B = 1), zero net momentum, rescaled to exactly T."""
    rng = np.random.default_rng(seed)
    v = rng.normal(0.0, math.sqrt(T / mass), size=(n, 3))
    v -= v.mean(axis=0)
    ek = 0.5 * mass * (v ** 2).sum()
    target = 1.5 * n * T
    if ek > 0:
        v *= math.sqrt(target / ek)
    return v


def fcc_lattice(ncells, rho):
    """FCC positions for ncells^3 unit cells (4 sites each) at density rho.  Returns (pos, bmin, bmax)."""
    if np.ndim(ncells) == 0:
        ncells = (ncells, ncells, ncells)
    a = (4.0 / rho) ** (1.0 / 3.0)
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(k) for k in ncells], indexing="ij"), -1).reshape(-1, 3)
    pos = ((g[:, None, :] + base[None]) * a).reshape(-1, 3) + a / 4.0
    bmax = np.array(ncells, float) * a
    return pos, np.zeros(3), bmax


def fcc_lj(ncells=20, rho=0.8442, T=0.72, seed=1):
    pos, bmin, bmax = fcc_lattice(ncells, rho)
    vel = mb_velocities(len(pos), T, seed=seed)
    return pos, vel, bmin, bmax


def rsa(n, bmin, bmax, rmin, rmax, dmin, seed, existing=None):
    """Random sequential addition through the engine library's host generator."""
    L = _engine.load()
    L.pe_gen_rsa.restype = C.c_int64
    L.pe_gen_rsa.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                             C.c_uint64, C.c_int64, C.c_void_p]
    m = 0 if existing is None else len(existing)
    pos = np.zeros((m + n, 3))
    if m:
        pos[:m] = existing
    arrs = [np.ascontiguousarray(v, np.float64) for v in (bmin, bmax, rmin, rmax)]
    placed = L.pe_gen_rsa(m, n, *[a.ctypes.data for a in arrs], float(dmin), int(seed), int(200 * n + 10000),
                          pos.ctypes.data)
    if placed != n:
        raise RuntimeError(f"random sequential addition placed {placed} of {n} particles")
    return pos


def slab(n_total=2_000_000, rho_liq=0.75, rho_vap=0.02, dmin=0.8, T=0.8, seed=7, rsa_fn=None):
    """Vapour-liquid slab in a 3:1:1 box (x long), liquid in the middle third.  Returns (pos, vel, bmin, bmax).
    rsa_fn: the random-sequential-addition routine (signature of `rsa`); the engine library's by default."""
    rsa_fn = rsa if rsa_fn is None else rsa_fn
    # n_total = rho_liq * V/3 + rho_vap * 2V/3 with V = 3 l^3
    V = n_total / (rho_liq / 3.0 + 2.0 * rho_vap / 3.0)
    ell = (V / 3.0) ** (1.0 / 3.0)
    bmin = np.zeros(3)
    bmax = np.array([3 * ell, ell, ell])
    n_liq = int(round(rho_liq * V / 3.0))
    n_vap = n_total - n_liq
    liq = rsa_fn(n_liq, bmin, bmax, [ell, 0, 0], [2 * ell, ell, ell], dmin, seed)
    both = rsa_fn(n_vap, bmin, bmax, bmin, bmax, dmin, seed + 1, existing=liq)
    # vapour candidates may land in the slab region too; keep the count per region as drawn
    vel = mb_velocities(n_total, T, seed=seed + 2)
    return both, vel, bmin, bmax


def ensemble(num_systems=512, nmin=500, nmax=50_000, rho=(0.3, 0.9), T=(0.7, 1.5), seed=11, max_total=None):
    """Independent periodic systems on jittered cubic lattices.  Returns a list of dicts."""
    rng = np.random.default_rng(seed)
    out = []
    total = 0
    for k in range(num_systems):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        if max_total is not None and total + n > max_total:
            break
        r = rng.uniform(*rho)
        t = rng.uniform(*T)
        side = (n / r) ** (1.0 / 3.0)
        m = int(math.ceil(n ** (1.0 / 3.0)))
        h = side / m
        g = np.stack(np.meshgrid(*[np.arange(m)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
        pos = (g + 0.5) * h + rng.uniform(-0.1, 0.1, size=(n, 3)) * h
        pos = np.mod(pos, side)
        vel = mb_velocities(n, t, seed=seed * 1000 + k)
        out.append({"pos": pos, "vel": vel, "bmin": np.zeros(3), "bmax": np.full(3, side), "rho": r, "T": t})
        total += n
    return out
