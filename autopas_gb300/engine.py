"""Python binding of the engine's C ABI (include/pairengine.h) over ctypes.

This is a thin host wrapper for tests, benchmarks and scripting; the C++ mirror of the AutoPas container /
traversal / functor interface lives in autopas_gb300/include/.  The library must have been built
(``autopas_gb300.build.build()``); there is no fallback of any kind when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

PE_OK = 0
ERRORS = {
    -1: "PE_ERR_ARG", -2: "PE_ERR_OOM", -3: "PE_ERR_CUDA", -4: "PE_ERR_LIST_OVERFLOW", -5: "PE_ERR_TOWER_OVERFLOW",
    -6: "PE_ERR_STATE", -7: "PE_ERR_NO_DEVICE", -8: "PE_ERR_DOMAIN", -9: "PE_ERR_TOO_LARGE",
}
NOALLOC_MAX_PARTICLES = 16384
PRECISION_FP64, PRECISION_MIXED = 0, 1
DIST_FMA_SOA, DIST_STRICT, DIST_FMA_DOT = 0, 1, 2
DUMMY, OWNED, HALO = 0, 1, 2

# every symbol include/pairengine.h declares
EXPORTS = [
    "pe_create", "pe_destroy", "pe_last_error", "pe_set_particles", "pe_update_positions", "pe_rebuild",
    "pe_compute_forces", "pe_get_forces", "pe_get_state", "pe_step", "pe_get_info", "pe_get_tower_grid",
    "pe_pair_set", "pe_get_stats", "pe_device_timer", "pe_tune", "pe_get_tuning", "pe_lj_forces_noalloc",
    "pe_compute_atm", "pe_update_ownership", "pe_set_force_cap", "pe_scale_velocities", "pe_measure_fp32_peak",
    "pe_measure_fp64_peak", "pe_check_conversions",
]


class PeConfig(C.Structure):
    _fields_ = [
        ("cutoff", C.c_double), ("skin", C.c_double), ("num_types", C.c_int),
        ("epsilon", C.POINTER(C.c_double)), ("sigma", C.POINTER(C.c_double)), ("mass", C.POINTER(C.c_double)),
        ("apply_shift", C.c_int), ("precision", C.c_int), ("cluster_size", C.c_int), ("newton3", C.c_int),
        ("dist_mode", C.c_int), ("rebuild_frequency", C.c_int), ("calc_globals", C.c_int),
        ("tower_sizing", C.c_int), ("traversal", C.c_int), ("atm_nu", C.c_double), ("atm_cutoff", C.c_double),
        ("use_graphs", C.c_int), ("prune_buffer", C.c_double), ("kernel_variant", C.c_int), ("n3_pieces", C.c_int),
    ]


class PeSystem(C.Structure):
    _fields_ = [("box_min", C.c_double * 3), ("box_max", C.c_double * 3), ("periodic", C.c_int)]


class PeGlobals(C.Structure):
    _fields_ = [("upot", C.c_double), ("virial", C.c_double), ("virial_xyz", C.c_double * 3),
                ("num_pairs", C.c_int64), ("ekin", C.c_double)]


class PeStats(C.Structure):
    _fields_ = [("force_ms", C.c_double), ("force_launches", C.c_int64), ("kernel_launches", C.c_int64),
                ("pairs_total", C.c_int64), ("rebuilds", C.c_int64), ("prunes", C.c_int64),
                ("rebuilds_redone", C.c_int64)]


class PeTuningEntry(C.Structure):
    _fields_ = [("cluster_size", C.c_int), ("traversal", C.c_int), ("variant", C.c_int), ("ms", C.c_double),
                ("rebuild_ms", C.c_double), ("score", C.c_double)]


class PeInfo(C.Structure):
    _fields_ = [("cluster_size", C.c_int), ("newton3", C.c_int), ("precision", C.c_int), ("traversal", C.c_int),
                ("num_particles", C.c_int64), ("num_slots", C.c_int64), ("num_clusters", C.c_int64),
                ("num_towers", C.c_int64), ("num_cluster_pairs", C.c_int64), ("max_tower_size", C.c_int64),
                ("num_list_entries", C.c_int64), ("list_capacity", C.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(path: str | None = None):
    """Load libpairengine.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise RuntimeError(f"engine library {p} is missing; build it with autopas_gb300.build.build()")
    L = C.CDLL(p)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.pe_create.argtypes = [C.POINTER(PeConfig), C.c_int, C.POINTER(PeSystem), C.POINTER(vp)]
    L.pe_destroy.argtypes = [vp]
    L.pe_last_error.argtypes = [vp]
    L.pe_last_error.restype = C.c_char_p
    L.pe_set_particles.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.pe_update_positions.argtypes = [vp, vp, vp, vp]
    L.pe_rebuild.argtypes = [vp]
    L.pe_update_ownership.argtypes = [vp, vp, C.POINTER(C.c_int)]
    L.pe_set_force_cap.argtypes = [vp, C.c_double]
    L.pe_measure_fp32_peak.argtypes = [C.POINTER(C.c_double)]
    L.pe_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    L.pe_check_conversions.argtypes = [C.POINTER(C.c_int64)]
    L.pe_scale_velocities.argtypes = [vp, vp]
    L.pe_compute_forces.argtypes = [vp, vp]
    L.pe_get_forces.argtypes = [vp, vp, vp, vp]
    L.pe_get_state.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.pe_step.argtypes = [vp, C.c_double, C.c_int, vp]
    L.pe_get_info.argtypes = [vp, C.POINTER(PeInfo)]
    L.pe_get_tower_grid.argtypes = [vp, C.c_int, dp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), dp]
    L.pe_pair_set.argtypes = [vp, C.c_int, C.c_int64, vp, vp, vp, C.POINTER(C.c_int64)]
    L.pe_get_stats.argtypes = [vp, C.c_int, C.POINTER(PeStats)]
    L.pe_device_timer.argtypes = [vp, C.c_int, dp]
    L.pe_tune.argtypes = [vp, C.c_int]
    L.pe_compute_atm.argtypes = [vp, C.c_double, C.c_double, vp]
    L.pe_lj_forces_noalloc.argtypes = [C.POINTER(PeConfig), C.c_int64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.pe_get_tuning.argtypes = [vp, C.c_int, C.POINTER(PeTuningEntry), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    for name in EXPORTS:
        if name != "pe_last_error":
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


class EngineError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class PairEngine:
    """One engine instance (one CUDA stream) holding one or more particle systems."""

    def __init__(self, cutoff, skin, boxes, periodic=True, epsilon=(1.0,), sigma=(1.0,), mass=(1.0,),
                 shift=False, precision=PRECISION_MIXED, cluster_size=8, newton3=0, dist_mode=DIST_FMA_SOA,
                 rebuild_frequency=10, calc_globals=True, tower_sizing=1, traversal=1, atm_nu=0.0, atm_cutoff=0.0,
                 use_graphs=True, prune_buffer=0.0, kernel_variant=0, n3_pieces=0):
        L = load()
        self._L = L
        self._eps = np.ascontiguousarray(epsilon, np.float64)
        self._sig = np.ascontiguousarray(sigma, np.float64)
        self._mass = np.ascontiguousarray(mass, np.float64)
        T = len(self._eps)
        dp = C.POINTER(C.c_double)
        cfg = PeConfig(cutoff, skin, T, self._eps.ctypes.data_as(dp), self._sig.ctypes.data_as(dp),
                       self._mass.ctypes.data_as(dp), int(shift), int(precision), int(cluster_size), int(newton3),
                       int(dist_mode), int(rebuild_frequency), int(calc_globals), int(tower_sizing),
                       int(traversal), float(atm_nu), float(atm_cutoff), int(use_graphs), float(prune_buffer),
                       int(kernel_variant), int(n3_pieces))
        boxes = list(boxes)
        if np.ndim(boxes[0]) == 1:  # single (bmin, bmax)
            boxes = [boxes]
        per = periodic if isinstance(periodic, (list, tuple)) else [periodic] * len(boxes)
        arr = (PeSystem * len(boxes))()
        for k, (bmin, bmax) in enumerate(boxes):
            arr[k].box_min[:] = [float(v) for v in bmin]
            arr[k].box_max[:] = [float(v) for v in bmax]
            arr[k].periodic = int(per[k])
        self.num_systems = len(boxes)
        h = C.c_void_p()
        rc = L.pe_create(C.byref(cfg), len(boxes), arr, C.byref(h))
        if rc != PE_OK:
            raise EngineError(rc, "pe_create failed")
        self._h = h
        self.n = 0

    def _check(self, rc):
        if rc != PE_OK:
            raise EngineError(rc, self._L.pe_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.pe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, pos, vel=None, types=None, ownership=None, ids=None, system=None):
        pos = np.asarray(pos, np.float64)
        n = len(pos)
        self._x, self._y, self._z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
        if vel is not None:
            vel = np.asarray(vel, np.float64)
            self._vx, self._vy, self._vz = (np.ascontiguousarray(vel[:, d]) for d in range(3))
        else:
            self._vx = self._vy = self._vz = None
        t = None if types is None else np.ascontiguousarray(types, np.int32)
        o = None if ownership is None else np.ascontiguousarray(ownership, np.int8)
        i = None if ids is None else np.ascontiguousarray(ids, np.int64)
        s = None if system is None else np.ascontiguousarray(system, np.int32)
        self._check(self._L.pe_set_particles(self._h, n, _ptr(self._x), _ptr(self._y), _ptr(self._z),
                                             _ptr(self._vx), _ptr(self._vy), _ptr(self._vz), _ptr(t), _ptr(o),
                                             _ptr(i), _ptr(s)))
        self.n = n

    def set_particles_soa(self, x, y, z, vx=None, vy=None, vz=None, types=None, ownership=None, system=None):
        """Zero-copy variant: the arrays (contiguous, possibly pinned) are passed as they are."""
        self._check(self._L.pe_set_particles(self._h, len(x), _ptr(x), _ptr(y), _ptr(z), _ptr(vx), _ptr(vy),
                                             _ptr(vz), _ptr(types), _ptr(ownership), None, _ptr(system)))
        self.n = len(x)

    def update_positions(self, pos):
        pos = np.asarray(pos, np.float64)
        x, y, z = (np.ascontiguousarray(pos[:, d]) for d in range(3))
        self._check(self._L.pe_update_positions(self._h, _ptr(x), _ptr(y), _ptr(z)))

    def update_positions_soa(self, x, y, z):
        """Zero-copy variant: contiguous float64 arrays; page-locked ones are read by the GPU directly."""
        self._check(self._L.pe_update_positions(self._h, _ptr(x), _ptr(y), _ptr(z)))

    def rebuild(self):
        self._check(self._L.pe_rebuild(self._h))

    def set_force_cap(self, max_force):
        """Caps each particle's force at max_force before integration (0: off)."""
        self._check(self._L.pe_set_force_cap(self._h, float(max_force)))

    def scale_velocities(self, factors):
        """Velocities times factors[type] (a scalar applies to every type)."""
        f = np.ascontiguousarray(np.broadcast_to(np.asarray(factors, np.float64), (len(self._eps),)))
        self._check(self._L.pe_scale_velocities(self._h, _ptr(f)))

    def soft_start(self, dt, nsteps, max_force, temperature, mass=1.0):
        """Capped-force steps from overlapping positions, each followed by a velocity scaling to the target
        temperature (the thermostat), then the cap is switched off.  Returns the globals of the last step."""
        n_owned = None
        self.set_force_cap(max_force)
        self.compute_forces()
        g = None
        for _ in range(nsteps):
            g = self.step(dt, 1)
            ekin = sum(x["ekin"] for x in g)
            if n_owned is None:
                n_owned = self.n
            t_now = 2.0 * ekin / (3.0 * n_owned)
            if t_now > 0:
                self.scale_velocities((temperature / t_now) ** 0.5)
        self.set_force_cap(0.0)
        self.compute_forces()
        return g

    def update_ownership(self, ownership):
        """New OwnershipState values (user order); returns whether the lists stayed valid."""
        o = np.ascontiguousarray(ownership, np.int8)
        v = C.c_int()
        self._check(self._L.pe_update_ownership(self._h, _ptr(o), C.byref(v)))
        return bool(v.value)

    def compute_forces(self, want_globals=True):
        """Forces of the current positions; with want_globals the per-system globals are read back (a host
        wait for the device), without it the call returns at once (None) and the forces are read later."""
        g = (PeGlobals * self.num_systems)() if want_globals else None
        self._check(self._L.pe_compute_forces(self._h, g))
        return _globals(g) if want_globals else None

    def compute_atm(self, nu, cutoff3):
        """Adds Axilrod-Teller-Muto forces to the current forces; returns per-system ATM globals."""
        g = (PeGlobals * self.num_systems)()
        self._check(self._L.pe_compute_atm(self._h, float(nu), float(cutoff3), g))
        return _globals(g)

    def forces(self, out=None):
        n = self.n
        if out is None:
            out = [np.empty(n), np.empty(n), np.empty(n)]
        self._check(self._L.pe_get_forces(self._h, _ptr(out[0]), _ptr(out[1]), _ptr(out[2])))
        return np.stack(out, 1)

    def forces_into(self, fx, fy, fz):
        self._check(self._L.pe_get_forces(self._h, _ptr(fx), _ptr(fy), _ptr(fz)))

    def state(self):
        n = self.n
        a = [np.empty(n) for _ in range(6)]
        self._check(self._L.pe_get_state(self._h, *[_ptr(v) for v in a]))
        return np.stack(a[:3], 1), np.stack(a[3:], 1)

    def step(self, dt, nsteps, want_globals=True):
        g = (PeGlobals * self.num_systems)() if want_globals else None
        self._check(self._L.pe_step(self._h, float(dt), int(nsteps), g))
        return _globals(g) if want_globals else None

    def info(self):
        i = PeInfo()
        self._check(self._L.pe_get_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in PeInfo._fields_}

    def tower_grid(self, system=0):
        side = (C.c_double * 2)()
        num = (C.c_int64 * 2)()
        halo = C.c_int64()
        origin = (C.c_double * 2)()
        self._check(self._L.pe_get_tower_grid(self._h, system, side, num, C.byref(halo), origin))
        return np.array(side[:]), np.array(num[:]), int(halo.value), np.array(origin[:])

    def pair_set(self, which=0):
        """(a, b, code) of the covered pairs within rc+skin (which=0) or rc (which=1)."""
        cnt = C.c_int64()
        self._check(self._L.pe_pair_set(self._h, int(which), 0, None, None, None, C.byref(cnt)))
        cap = int(cnt.value)
        a = np.empty(max(cap, 1), np.int64)
        b = np.empty(max(cap, 1), np.int64)
        c = np.empty(max(cap, 1), np.int32)
        self._check(self._L.pe_pair_set(self._h, int(which), cap, _ptr(a), _ptr(b), _ptr(c), C.byref(cnt)))
        return a[:cap], b[:cap], c[:cap]

    def stats(self, reset=True):
        st = PeStats()
        self._check(self._L.pe_get_stats(self._h, int(reset), C.byref(st)))
        return {k: getattr(st, k) for k, _ in PeStats._fields_}

    def tune(self, samples=3):
        self._check(self._L.pe_tune(self._h, int(samples)))
        return self.tuning()

    def tuning(self):
        arr = (PeTuningEntry * 64)()
        cnt = C.c_int()
        chosen = C.c_int()
        self._check(self._L.pe_get_tuning(self._h, 64, arr, C.byref(cnt), C.byref(chosen)))
        return {"candidates": [{"cluster_size": a.cluster_size, "traversal": a.traversal, "variant": a.variant,
                                "ms": a.ms, "rebuild_ms": a.rebuild_ms, "score": a.score}
                               for a in arr[:cnt.value]], "chosen": chosen.value}

    def timer_start(self):
        self._check(self._L.pe_device_timer(self._h, 0, None))

    def timer_stop(self):
        ms = C.c_double()
        self._check(self._L.pe_device_timer(self._h, 1, C.byref(ms)))
        return ms.value


def make_config(cutoff, skin=0.0, epsilon=(1.0,), sigma=(1.0,), mass=(1.0,), shift=False, dist_mode=DIST_FMA_SOA):
    """A PeConfig for calls that take one without an engine (pe_lj_forces_noalloc).  Returns (cfg, keepalive)."""
    eps = np.ascontiguousarray(epsilon, np.float64)
    sig = np.ascontiguousarray(sigma, np.float64)
    ms = np.ascontiguousarray(mass, np.float64)
    dp = C.POINTER(C.c_double)
    cfg = PeConfig(cutoff, skin, len(eps), eps.ctypes.data_as(dp), sig.ctypes.data_as(dp), ms.ctypes.data_as(dp),
                   int(shift), PRECISION_FP64, 8, 0, int(dist_mode), 1, 1, 1, 1, 0.0, 0.0, 0, 0.0, 0)
    return cfg, (eps, sig, ms)


def measure_fp32_peak():
    """FP32 CUDA-core FMA throughput of the current device, TFLOP/s (pe_measure_fp32_peak)."""
    v = C.c_double()
    rc = load().pe_measure_fp32_peak(C.byref(v))
    if rc != PE_OK:
        raise EngineError(rc, "pe_measure_fp32_peak failed")
    return v.value


def measure_fp64_peak():
    """FP64 FMA throughput of the current device, TFLOP/s (pe_measure_fp64_peak)."""
    v = C.c_double()
    rc = load().pe_measure_fp64_peak(C.byref(v))
    if rc != PE_OK:
        raise EngineError(rc, "pe_measure_fp64_peak failed")
    return v.value


def check_conversions():
    """Mismatches of the engine's integer-pipe float<->double conversions against the hardware converter
    (pe_check_conversions); 0 expected."""
    v = C.c_int64()
    rc = load().pe_check_conversions(C.byref(v))
    if rc != PE_OK:
        raise EngineError(rc, "pe_check_conversions failed")
    return v.value


def lj_forces_noalloc(cfg, n, x, y, z, type_ptr, own_ptr, fx, fy, fz, globals_ptr, stream=None):
    """Direct call of pe_lj_forces_noalloc with device addresses (ints); raises on a non-zero status."""
    L = load()
    rc = L.pe_lj_forces_noalloc(C.byref(cfg), int(n), x, y, z, type_ptr, own_ptr, fx, fy, fz, globals_ptr, stream)
    if rc != PE_OK:
        raise EngineError(rc, "pe_lj_forces_noalloc failed")


def _globals(g):
    return [{"upot": x.upot, "virial": x.virial, "virial_xyz": tuple(x.virial_xyz), "num_pairs": x.num_pairs,
             "ekin": x.ekin} for x in g]
