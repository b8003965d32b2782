#!/usr/bin/env python
"""Benchmark of the GB300 LJ pair-force engine: pair interactions/s and MD steps/s, FP32-mixed vs FP64.

Workload (one GPU): a vapour-liquid slab of 2,000,000 LJ particles in a 3:1:1 periodic box, liquid (density
0.75) in the middle third, vapour (0.02) elsewhere, positions uniform within each region with minimum pair
distance 0.8, T* = 0.8, cutoff 3.0, skin 0.4, lists rebuilt every 20 steps, velocity Verlet dt = 0.002,
truncated (unshifted) potential, single type (eps = sigma = m = 1).  Seeded synthetic data.

A step is one full MD step on the device (position update, list rebuild when due, forces + globals, velocity
update).  value = interacting pairs (dr2 <= rc^2, each unordered pair once) summed over the timed steps /
device time of those steps (CUDA events on the engine's stream).  The working set (~0.5 GB) exceeds the 129 MB
L2, so no flush is needed between steps.

--impl reference times the reference's CPU path restated in the oracle (LinkedCells + c08 colouring + SoA LJ
functor with newton3, OpenMP on all host cores) on the same 2,000,000-particle slab: one step is one force
evaluation of the whole slab.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RC, SKIN, DT, REBUILD = 3.0, 0.4, 0.002, 20
REFERENCE_BUDGET_S = 150.0  # timed CPU work of the reference arm, at most
FLOP_PER_PAIR = 38  # 8 distance + 18 newton3 kernel + 12 globals (unshifted), LJFunctor.h:722-789


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=2_000_000, help="particles of the slab workload")
    p.add_argument("--fp64-steps", type=int, default=10)
    p.add_argument("--cluster-size", type=int, default=0, help="0: the engine's tuner picks 4 or 8")
    p.add_argument("--traversal", type=int, default=-1,
                   help="-1: tuner; 0 cluster pairs; 1 particle lists; 2 pair-group half lists (newton3)")
    p.add_argument("--newton3", type=int, default=-1, help="-1: the tuner may pick newton3; 0 off; 1 required")
    p.add_argument("--prune", type=float, default=0.0, help="rolling-prune buffer of the particle lists (0: off)")
    p.add_argument("--variant", type=int, default=0, help="particle-list kernel variant when the tuner is off")
    p.add_argument("--n3-pieces", type=int, default=0, help="newton3 evaluation pieces (0: by size)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--profile", action="store_true", help="small run for ncu: no fp64 leg, no baselines")
    p.add_argument("--workload", default="slab", choices=["slab", "ensemble", "drift", "mixture", "atm"],
                   help="slab: the headline 2M-particle system; ensemble: 512 independent systems in one engine")
    p.add_argument("--systems", type=int, default=512)
    return p.parse_args()


# ---------------------------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def host_link_rates(nbytes):
    """Copy-engine bandwidth between page-locked host memory and the device for one step's position (or
    force) bytes: the floor under the end-to-end step, whose transfers cross the same link."""
    try:
        import torch
        h = torch.empty(nbytes // 8, dtype=torch.float64, pin_memory=True)
        d = torch.empty(nbytes // 8, dtype=torch.float64, device="cuda")
        st = torch.cuda.Stream()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        with torch.cuda.stream(st):
            for _ in range(2):
                d.copy_(h, non_blocking=True)
                h.copy_(d, non_blocking=True)
            ev[0].record(st)
            for _ in range(5):
                d.copy_(h, non_blocking=True)
            ev[1].record(st)
            for _ in range(5):
                h.copy_(d, non_blocking=True)
            ev[2].record(st)
        st.synchronize()
        t_h2d, t_d2h = ev[0].elapsed_time(ev[1]) / 5, ev[1].elapsed_time(ev[2]) / 5
        return {"h2d_gbs": nbytes / (t_h2d * 1e6), "d2h_gbs": nbytes / (t_d2h * 1e6),
                "transfer_floor_ms": t_h2d + t_d2h,
                "what": f"cudaMemcpyAsync of {nbytes} bytes each way between page-locked host and device memory"}
    except Exception as ex:  # a host without torch or CUDA: no figure
        return {"unavailable": str(ex)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


# ---------------------------------------------------------------------------------------------- distributed
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        # replicas only: each rank drives its own GPU; gloo carries the barrier and the max-over-ranks time
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


from autopas_gb300.sharding import barrier, max_over_ranks, sum_over_ranks  # noqa: E402


# ---------------------------------------------------------------------------------------------- workload
def make_slab(n, seed=7, rsa_fn=None):
    from autopas_gb300 import workloads
    return workloads.slab(n_total=n, seed=seed, rsa_fn=rsa_fn)


def cpu_reference_rate(pos, bmin, bmax, pairs, nthreads, budget_s=None, warmup=1, steps=None):
    """Pair interactions/s of the reference's CPU path (the oracle's restatement: LinkedCells, c08 colouring, SoA
    LJ functor with newton3, FP64, OpenMP) on the whole workload: each evaluation bins the owned particles and
    their periodic halo copies into cells and computes all forces and globals.  `pairs` is the workload's
    interacting-pair count (each unordered physical pair once).  Times `steps` evaluations, or as many as fit in
    budget_s, whichever is fewer (at least three when both are given).  Returns (rate, evaluations, seconds)."""
    from oracle import oracle as orc
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, RC, SKIN)
    lj = orc.LJ(RC)
    for _ in range(max(warmup, 0)):
        orc.cpu_lc_c08(allpos, lj, SKIN, own=own, nthreads=nthreads)
    evals, t_total = 0, 0.0
    while True:
        t0 = time.perf_counter()
        orc.cpu_lc_c08(allpos, lj, SKIN, own=own, nthreads=nthreads)
        t_total += time.perf_counter() - t0
        evals += 1
        if steps is not None and evals >= steps:
            break
        if budget_s is not None and t_total >= budget_s and (steps is None or evals >= 3):
            break
    return pairs * evals / t_total, evals, t_total


def run_reference(args):
    """The reference arm: the reference's CPU path (oracle restatement) on the same workload and configuration
    as our arm, all host threads.  The slab comes from the oracle library's copy of the generator (same source
    and seed as our arm), so this process never loads the engine library."""
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.build()
    nthreads = os.cpu_count() or 1
    pos, vel, bmin, bmax = make_slab(args.n, seed=7, rsa_fn=orc.gen_rsa)
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, RC, SKIN)
    oo, oh, _ = orc.count_interacting(allpos, RC, own=own)
    pairs = oo + oh // 2
    del allpos, own
    # one evaluation of the whole 2M slab takes ~0.6 s on 16 cores: the timed evaluations are bounded by the
    # requested steps and by a time budget, so that the arm ends within a few minutes for any --steps
    rate, evals, t = cpu_reference_rate(pos, bmin, bmax, pairs, nthreads, budget_s=REFERENCE_BUDGET_S,
                                        warmup=min(args.warmup, 2), steps=args.steps)
    sample = (f"the whole workload: one step = one force evaluation (LinkedCells cell binning, c08 colouring, SoA LJ "
              f"with newton3, FP64, OpenMP on {nthreads} threads) of all {args.n} particles of the slab plus their "
              f"periodic halo copies; {pairs} interacting pairs per step; {evals} of the {args.steps} requested "
              f"steps timed ({t:.1f} s, budget {REFERENCE_BUDGET_S:.0f} s), after {min(args.warmup, 2)} untimed")
    line = {
        "impl": "reference", "metric": metric_name(), "value": rate, "unit": "pair interactions/s",
        "n_gpus": args.gpus, "steps": evals, "warmup": min(args.warmup, 2), "ms_per_step": 1e3 * t / evals,
        "steps_requested": args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args),
        "cpu_baseline": {"value": rate, "unit": "pair interactions/s", "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": "pair interactions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def metric_name():
    return "pair interactions/s & MD steps/s on 1 GB300: FP32-mixed vs FP64 GPU at stated error"


def config_dict(args):
    return {"workload": f"LJ vapour-liquid slab: {args.n} particles, 3:1:1 periodic box, liquid 0.75 in the middle "
                        f"third / vapour 0.02, dmin 0.8, T* 0.8, rc {RC}, skin {SKIN}, rebuild every {REBUILD} "
                        f"steps, dt {DT}, truncated LJ, eps=sigma=m=1",
            "particles": args.n, "cutoff": RC, "skin": SKIN, "rebuild_frequency": REBUILD,
            "cluster_size": args.cluster_size or "tuned", "traversal": "tuned" if args.traversal < 0 else args.traversal,
            "prune_buffer": args.prune,
            "newton3": {-1: "tuned", 0: False, 1: True}.get(args.newton3, args.newton3),
            "l2_policy": "inputs larger than L2 (no flush)"}


# ---------------------------------------------------------------------------------------------- our arm
def run_ours(args):
    world, rank, local, pg = dist_setup(args)
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    from autopas_gb300 import engine as E

    pos, vel, bmin, bmax = make_slab(args.n, seed=7 + rank)
    n = len(pos)

    def new_engine(prec, use_graphs=True):
        e = E.PairEngine(RC, SKIN, (bmin, bmax), periodic=True, precision=prec, cluster_size=args.cluster_size,
                         newton3=args.newton3 if prec == E.PRECISION_MIXED else 0, rebuild_frequency=REBUILD,
                         calc_globals=True,
                         traversal=args.traversal if prec == E.PRECISION_MIXED or args.traversal < 2 else -1,
                         prune_buffer=args.prune, use_graphs=use_graphs, kernel_variant=args.variant,
                         n3_pieces=args.n3_pieces)
        e.set_particles(pos, vel)
        return e

    # ---- force error of the mixed form against the FP64 form on the initial configuration
    err = None
    if not args.profile:
        e64 = new_engine(E.PRECISION_FP64)
        g64 = e64.compute_forces()[0]
        F64 = e64.forces()
        e64.close()
        em = new_engine(E.PRECISION_MIXED)
        gm = em.compute_forces()[0]
        Fm = em.forces()
        em.close()
        d = Fm - F64
        fr = np.sqrt((F64 ** 2).sum(1))
        frms = float(np.sqrt((fr ** 2).mean()))
        err = {"rms_rel": float(np.sqrt((d ** 2).sum(1).mean()) / frms),
               "max_rel": float((np.sqrt((d ** 2).sum(1)) / np.maximum(fr, frms)).max()),
               "upot_rel": abs(gm["upot"] - g64["upot"]) / abs(g64["upot"]),
               "virial_rel": abs(gm["virial"] - g64["virial"]) / abs(g64["virial"]),
               "pairs_equal": gm["num_pairs"] == g64["num_pairs"], "num_pairs": g64["num_pairs"],
               "against": "this engine's FP64 form (checked against the CPU oracle to 1e-12 in tests)",
               "definition": "rms_rel = sqrt(mean|dF|^2)/sqrt(mean|F|^2); max_rel = max |dF|/max(|F|, F_rms)"}
        del F64, Fm

    # ---- mixed MD steps (the headline)
    e = new_engine(E.PRECISION_MIXED)
    e.compute_forces()
    tuning = e.tuning()
    e.step(DT, args.warmup, want_globals=False)
    e.stats(reset=True)
    info = e.info()
    barrier(pg)
    clk = ClockSampler(local) if rank == 0 else None
    if clk:
        clk.start()
    e.timer_start()
    g_last = e.step(DT, args.steps, want_globals=True)[0]
    ms = e.timer_stop()
    clocks = clk.stop() if clk else None
    st = e.stats(reset=True)
    ms_max = max_over_ranks(pg, ms)
    pairs_total = st["pairs_total"]
    pairs_all = sum_over_ranks(pg, pairs_total)
    value = pairs_all / (ms_max * 1e-3)
    steps_per_s = args.steps / (ms_max * 1e-3)
    e.close()
    # the force kernel alone: the same steps without graph replay, every force launch timed with CUDA events on
    # the engine's stream (rebuild steps, prune steps and plain steps in their natural proportion)
    ek = new_engine(E.PRECISION_MIXED, use_graphs=False)
    ek.compute_forces()
    ek.step(DT, args.warmup, want_globals=False)
    ek.stats(reset=True)
    nk = min(args.steps, 2 * REBUILD * 5)
    ek.step(DT, nk, want_globals=True)
    st_k = ek.stats(reset=True)
    ek.close()
    force_ms_per_launch = st_k["force_ms"] / max(st_k["force_launches"], 1)
    pairs_per_launch = st_k["pairs_total"] / max(st_k["force_launches"], 1)

    # ---- FP64 form on the same workload
    fp64 = None
    if not args.profile and args.fp64_steps > 0:
        e2 = new_engine(E.PRECISION_FP64)
        e2.compute_forces()
        e2.step(DT, 1, want_globals=False)
        e2.stats(reset=True)
        e2.timer_start()
        e2.step(DT, args.fp64_steps, want_globals=True)
        ms2 = e2.timer_stop()
        st2 = e2.stats(reset=True)
        # the FP64 force kernel alone: eager evaluations, each timed with CUDA events on the engine's stream
        for _ in range(3):
            gk = e2.compute_forces()[0]
        stk = e2.stats(reset=True)
        e2.close()
        k_ms = stk["force_ms"] / max(stk["force_launches"], 1)
        fp64_peak = max(E.measure_fp64_peak() for _ in range(2))
        fp64 = {"value": st2["pairs_total"] / (ms2 * 1e-3), "unit": "pair interactions/s",
                "md_steps_per_s": args.fp64_steps / (ms2 * 1e-3), "ms_per_step": ms2 / args.fp64_steps,
                "steps": args.fp64_steps, "force_kernel_ms": k_ms,
                "roofline": {"bound": "fp64", "achieved": FLOP_PER_PAIR * gk["num_pairs"] / (k_ms * 1e-3) / 1e12,
                             "peak": fp64_peak, "unit": "TFLOP/s",
                             "frac": FLOP_PER_PAIR * gk["num_pairs"] / (k_ms * 1e-3) / 1e12 / fp64_peak,
                             "peak_source": "measured in this run: FP64 FMA throughput (pe_measure_fp64_peak)"}}

    # ---- end to end through the C ABI with host buffers (pinned when torch is present)
    e2e = None
    if not args.no_e2e and not args.profile:
        try:
            import torch
            pin = lambda k: torch.empty(k, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
        except Exception:
            pin = lambda k: np.empty(k)  # noqa: E731
        hx, hy, hz = pin(n), pin(n), pin(n)
        hx[:], hy[:], hz[:] = pos[:, 0], pos[:, 1], pos[:, 2]
        fx, fy, fz = pin(n), pin(n), pin(n)
        ee = new_engine(E.PRECISION_MIXED)
        ee.compute_forces()
        nst = max(min(args.steps, 40), 5)
        for k in range(3):
            ee.update_positions(pos)
            ee.compute_forces()
            ee.forces_into(fx, fy, fz)
        ee.stats(reset=True)
        barrier(pg)
        t0 = time.perf_counter()
        for k in range(nst):
            if k % REBUILD == 0:
                ee.rebuild()
            ee._check(ee._L.pe_update_positions(ee._h, hx.ctypes.data, hy.ctypes.data, hz.ctypes.data))
            ee.compute_forces(want_globals=False)
            ee.forces_into(fx, fy, fz)
        t_e2e = time.perf_counter() - t0
        st3 = ee.stats(reset=True)
        ee.close()
        t_e2e = max_over_ranks(pg, t_e2e)
        e2e = {"value": sum_over_ranks(pg, st3["pairs_total"]) / t_e2e, "unit": "pair interactions/s",
               "h2d_bytes_per_step": 3 * 8 * n, "d2h_bytes_per_step": 3 * 8 * n + 48,
               "steps": nst, "ms_per_step": 1e3 * t_e2e / nst,
               "what": "per step: pe_update_positions from pinned host x,y,z + pe_compute_forces (forces and "
                       f"globals on the device, pe_rebuild every {REBUILD} steps) + pe_get_forces into pinned host "
                       "fx,fy,fz; host wall clock",
               "host_link": host_link_rates(3 * 8 * n)}

    # ---- CPU baseline (rank 0, N = 1): the reference's CPU path on the same 2M-particle slab, ~10 s of evaluations
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.profile and err is not None:
        nthreads = os.cpu_count() or 1
        rate, evals, tt = cpu_reference_rate(pos, bmin, bmax, err["num_pairs"], nthreads, budget_s=10.0)
        cpu = {"value": rate, "unit": "pair interactions/s", "cores": nthreads, "kind": "port",
               "sample": f"{evals} force evaluations (LinkedCells + c08 + SoA LJ with newton3, FP64, OpenMP) of the "
                         f"whole {n}-particle slab with its periodic halo copies ({err['num_pairs']} interacting "
                         f"pairs each), {tt:.1f} s"}

    if rank != 0:
        return 0
    peaks = measured_peaks()
    traffic = None
    tr_source = None
    try:
        # DRAM bytes per particle of the force evaluation (per traversal) from an ncu capture of the same kernels
        # on a 400,000-particle slab, scaled by the particle count
        with open(os.path.join(ROOT, "profiles", "force_kernel_traffic.json")) as f:
            tr = json.load(f)["traversals"].get(str(info["traversal"]))
        if tr:
            traffic = tr["dram_bytes_per_particle"] * n
            tr_source = tr["kernels"]
    except Exception:
        traffic = None
    # the FP32 CUDA-core peak of this GPU, measured now (the best of three ~10 ms runs)
    fp32_peak = max(E.measure_fp32_peak() for _ in range(3))
    achieved = FLOP_PER_PAIR * pairs_per_launch / (force_ms_per_launch * 1e-3) / 1e12
    kernel = {0: "k_lj_mixed_full", 1: "k_lj_mixed_plist", 2: "k_lj_mixed_n3 + k_n3_finish"}[info["traversal"]]
    chosen = tuning["chosen"]
    variant = tuning["candidates"][chosen]["variant"] if chosen >= 0 else args.variant
    if info["traversal"] == 2 and variant == 3:
        kernel = "k_lj_mixed_n3_sorted + k_n3_finish"  # each block's pair groups in decreasing order of list length
    line = {
        "metric": metric_name(), "value": value, "unit": "pair interactions/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 LJ arithmetic on f64 state", "data": "synthetic",
        "config": config_dict(args),
        "md_steps_per_s": steps_per_s,
        "force_kernel": {"ms_per_launch": force_ms_per_launch, "pairs_per_launch": pairs_per_launch,
                         "pair_interactions_per_s": pairs_per_launch / (force_ms_per_launch * 1e-3),
                         "launches_timed": st_k["force_launches"], "prunes": st_k["prunes"]},
        "fp64_gpu": fp64,
        "speedup_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "force_error": err,
        "upot_last_step": g_last["upot"], "rebuilds_in_timed_region": st["rebuilds"],
        "prunes_in_timed_region": st["prunes"],
        "engine": {k: info[k] for k in ("cluster_size", "traversal", "newton3", "num_clusters", "num_cluster_pairs",
                                        "max_tower_size", "num_towers", "list_capacity", "num_list_entries")},
        "tuning": tuning,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "traffic_note": (f"dram__bytes_read.sum + dram__bytes_write.sum per force evaluation ({tr_source})"
                                      ", scaled by particle count from profiles/force_kernel_traffic.json (the same "
                                      "kernels on a 400,000-particle slab)") if traffic else None,
                     "hbm_view": ({"achieved_gbs": traffic / (force_ms_per_launch * 1e-3) / 1e9,
                                   "peak_gbs": peaks.get("hbm_gbs"),
                                   "frac": traffic / (force_ms_per_launch * 1e-3) / 1e9 / peaks["hbm_gbs"],
                                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy)"}
                                  if traffic and peaks.get("hbm_gbs") else None),
                     "kernel": f"{kernel} (C = {info['cluster_size']})",
                     "algorithmic": f"{FLOP_PER_PAIR} FLOP per interacting pair (reference convention), "
                                    f"{pairs_per_launch:.0f} pairs per force evaluation",
                     "peak_source": "measured in this run: FP32 CUDA-core FMA throughput (pe_measure_fp32_peak, "
                                    "packed FP32x2 FMA chains on every SM, CUDA events) -- the force kernels' work "
                                    "is CUDA-core FP32 arithmetic; MEASURED_PEAKS.json holds HBM and tensor figures"},
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": st["kernel_launches"], "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------- ensemble
def run_ensemble(args):
    """512 independent periodic LJ systems (sizes log-uniform in 500-50,000, densities 0.3-0.9, T* 0.7-1.5,
    rc 2.5, skin 0.3, rebuild every 10) stepped together by one engine with CUDA-graph replay, against the same
    systems run one engine at a time in the FP64 form (all of them)."""
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    from autopas_gb300 import engine as E, workloads
    rc, skin, reb = 2.5, 0.3, 10
    world, rank, local, pg = dist_setup(args)
    systems = workloads.ensemble(args.systems, seed=11)
    if world > 1:
        # strong scaling: the same ensemble split over the ranks by LPT on the estimated pair work
        from autopas_gb300 import sharding
        costs = [sharding.pair_work(len(s_["pos"]), s_["rho"], rc + skin) for s_ in systems]
        mine, _ = sharding.lpt_assign(costs, world)
        systems = [systems[k] for k in mine[rank]]
    boxes = [(s_["bmin"], s_["bmax"]) for s_ in systems]
    pos = np.concatenate([s_["pos"] for s_ in systems])
    vel = np.concatenate([s_["vel"] for s_ in systems])
    sysid = np.concatenate([np.full(len(s_["pos"]), k, np.int32) for k, s_ in enumerate(systems)])
    e = E.PairEngine(rc, skin, boxes, periodic=True, precision=E.PRECISION_MIXED, cluster_size=0, traversal=-1,
                     newton3=args.newton3,
                     rebuild_frequency=reb, use_graphs=True)
    e.set_particles(pos, vel, system=sysid)
    e.compute_forces()
    tuning = e.tuning()
    e.step(0.002, args.warmup, want_globals=False)
    e.stats(reset=True)
    barrier(pg)
    e.timer_start()
    e.step(0.002, args.steps, want_globals=True)
    ms = max_over_ranks(pg, e.timer_stop())
    st = e.stats(reset=True)
    value = sum_over_ranks(pg, st["pairs_total"]) / (ms * 1e-3)
    if rank != 0:
        return 0
    # one at a time, FP64 form: every system in its own engine (the whole ensemble, not a sample)
    pairs1 = 0
    ms1 = 0.0
    for k in range(len(systems)):
        s_ = systems[k]
        e1 = E.PairEngine(rc, skin, (s_["bmin"], s_["bmax"]), periodic=True, precision=E.PRECISION_FP64,
                          cluster_size=8, traversal=1, rebuild_frequency=reb, use_graphs=False)
        e1.set_particles(s_["pos"], s_["vel"])
        e1.compute_forces()
        e1.stats(reset=True)
        e1.timer_start()
        e1.step(0.002, 10, want_globals=True)
        ms1 += e1.timer_stop()
        pairs1 += e1.stats(reset=True)["pairs_total"]
        e1.close()
    one = pairs1 / (ms1 * 1e-3)
    line = {"metric": "pair interactions/s, batched ensemble (FP32-mixed, one engine, CUDA graph) vs one-at-a-time FP64",
            "value": value, "unit": "pair interactions/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32 LJ arithmetic on f64 state", "data": "synthetic",
            "config": {"workload": f"{len(systems)} periodic LJ systems, sizes log-uniform 500-50,000 "
                                   f"({len(pos)} particles), densities U(0.3,0.9), T* U(0.7,1.5), rc {rc}, skin {skin}, "
                                   f"rebuild every {reb}", "particles": int(len(pos)), "systems": len(systems)},
            "one_at_a_time_fp64": {"value": one, "unit": "pair interactions/s",
                                   "sample": f"all {len(systems)} systems, each in its own engine, 10 steps"},
            "speedup_vs_one_at_a_time_fp64": value / one, "tuning": tuning, "gpu_launches": st["kernel_launches"]}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------- mixture
def run_mixture(args):
    """4,000,000 particles of 4 types (fractions 0.4/0.3/0.2/0.1, sigma 1.0/1.1/0.9/1.2, epsilon
    1.0/0.8/1.2/0.6), Lorentz-Berthelot mixing, shifted potential, rc = 2.5 x max sigma = 3.0, skin 0.3, density
    0.7 in a periodic cube, rebuild every 10; cluster size, traversal and kernel variant tuned.  Positions are
    uniform random (seeded), then 200 soft-start steps with every force capped at |F| <= 100 and the velocities
    scaled to T* 1.0 after each step (the thermostat's scaling), run in the FP64 form (overlapping starts put pair
    terms beyond FP32's range before the cap applies); the timed FP32-mixed run starts from the result and is
    compared with the engine's FP64 form on the same configuration."""
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    from autopas_gb300 import engine as E, workloads
    world, rank, local, pg = dist_setup(args)
    n = args.n if args.n != 2_000_000 else 4_000_000
    rho, rc, skin, reb = 0.7, 3.0, 0.3, 10
    side = (n / rho) ** (1.0 / 3.0)
    bmin, bmax = np.zeros(3), np.full(3, side)
    rng = np.random.default_rng(23)
    pos = bmin + rng.uniform(0.0, 1.0, (n, 3)) * (bmax - bmin)
    types = rng.choice(4, size=len(pos), p=[0.4, 0.3, 0.2, 0.1]).astype(np.int32)
    vel = workloads.mb_velocities(len(pos), 1.0, seed=23)
    eps, sig = [1.0, 0.8, 1.2, 0.6], [1.0, 1.1, 0.9, 1.2]
    # the capped-force soft start (FP64 form)
    es = E.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1, 1, 1, 1], shift=True,
                      precision=E.PRECISION_FP64, rebuild_frequency=reb, cluster_size=8, traversal=1)
    es.set_particles(pos, vel, types=types)
    t0 = time.perf_counter()
    es.soft_start(DT, 200, 100.0, 1.0)
    t_soft = time.perf_counter() - t0
    pos, vel = es.state()
    pos = np.mod(pos, bmax)
    es.close()

    def engine(prec, **kw):
        e = E.PairEngine(rc, skin, (bmin, bmax), periodic=True, epsilon=eps, sigma=sig, mass=[1, 1, 1, 1],
                         shift=True, precision=prec, rebuild_frequency=reb, **kw)
        e.set_particles(pos, vel, types=types)
        return e

    e = engine(E.PRECISION_MIXED, cluster_size=0, traversal=-1, newton3=args.newton3)
    g0 = e.compute_forces()[0]
    F = e.forces()
    tuning = e.tuning()
    e.step(DT, args.warmup, want_globals=False)
    e.stats(reset=True)
    barrier(pg)
    e.timer_start()
    e.step(DT, args.steps, want_globals=True)
    ms = max_over_ranks(pg, e.timer_stop())
    st = e.stats(reset=True)
    info = e.info()
    e.close()
    value = sum_over_ranks(pg, st["pairs_total"]) / (ms * 1e-3)
    if rank != 0:
        return 0
    e2 = engine(E.PRECISION_FP64, cluster_size=8, traversal=1)
    g2 = e2.compute_forces()[0]
    F64 = e2.forces()
    e2.stats(reset=True)
    e2.timer_start()
    e2.step(DT, 5, want_globals=True)
    ms2 = e2.timer_stop()
    st2 = e2.stats(reset=True)
    e2.close()
    dF = F - F64
    err = {"rms_rel": float(np.sqrt((dF ** 2).sum(1).mean() / (F64 ** 2).sum(1).mean())),
           "upot_rel": abs(g0["upot"] - g2["upot"]) / abs(g2["upot"]),
           "virial_rel": abs(g0["virial"] - g2["virial"]) / abs(g2["virial"]),
           "pairs_equal": g0["num_pairs"] == g2["num_pairs"]}
    line = {"metric": "pair interactions/s, 4-type LJ mixture (FP32-mixed vs FP64 GPU)", "value": value,
            "unit": "pair interactions/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 LJ arithmetic on f64 state", "data": "synthetic",
            "config": {"workload": f"4-type LJ mixture: {len(pos)} particles, density {rho}, Lorentz-Berthelot, "
                                   f"shifted, rc {rc}, skin {skin}, rebuild every {reb}, uniform random start + 200 "
                                   "capped-force (|F| <= 100) soft-start steps at T* 1.0",
                       "particles": int(len(pos)), "soft_start_s": t_soft},
            "fp64_gpu": {"value": st2["pairs_total"] / (ms2 * 1e-3), "unit": "pair interactions/s",
                         "ms_per_step": ms2 / 5},
            "force_error": err, "engine": {k: info[k] for k in ("cluster_size", "traversal", "num_list_entries")},
            "tuning": tuning, "gpu_launches": st["kernel_launches"]}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------- three-body
def run_atm(args):
    """LJ plus Axilrod-Teller-Muto: 200,000 particles (an FCC lattice jittered by 0.02 with MB velocities at a
    liquid state point, where it melts; a jitter of 0.1 already puts some of the 2.4 million nearest-neighbour
    pairs at overlapping distances) at density 0.8, T* 1.0, nu 0.073, pair rc 2.5 with skin 0.3, triplet cutoff
    2.5.  value: whole MD steps per second with both force kernels (FP32 triplet arithmetic, FP64 sums).  Beside
    it, for the three-body evaluation alone on the same configuration: the FP32 kernel, the plain FP64 kernel and
    the oracle's FP64 restatement on the host cores (cell list, OpenMP, each triplet evaluated from every owned
    vertex), all as interacting triplets per second; and the FP32 kernel's error against that FP64 oracle on the
    whole 200,000-particle system."""
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    from autopas_gb300 import engine as E, workloads
    world, rank, local, pg = dist_setup(args)
    nu, rc, skin, rho = 0.073, 2.5, 0.3, 0.8
    nc = 37  # 4 * 37^3 = 202,612 particles
    pos, vel, bmin, bmax = workloads.fcc_lj(nc, rho, 1.0, seed=29)
    pos = np.mod(pos + np.random.default_rng(29).normal(0, 0.02, pos.shape), bmax)
    e = E.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=E.PRECISION_MIXED, rebuild_frequency=10,
                     atm_nu=nu, atm_cutoff=rc)
    e.set_particles(pos, vel)
    e.compute_forces()
    e.step(DT, args.warmup, want_globals=False)
    e.stats(reset=True)
    barrier(pg)
    e.timer_start()
    nst = min(args.steps, 100)
    e.step(DT, nst, want_globals=True)
    ms = max_over_ranks(pg, e.timer_stop())
    st = e.stats(reset=True)
    e.close()
    if rank != 0:
        return 0
    # the three-body evaluation alone (pair term off: epsilon 0), FP32 and FP64 kernels, same positions
    three = {}
    for name, prec in (("fp32", E.PRECISION_MIXED), ("fp64", E.PRECISION_FP64)):
        e3 = E.PairEngine(rc, skin, (bmin, bmax), periodic=True, precision=prec, epsilon=[0.0], sigma=[1.0])
        e3.set_particles(pos, vel)
        e3.compute_forces()
        f0 = e3.forces()
        g = e3.compute_atm(nu, rc)[0]
        F3 = e3.forces() - f0
        reps = 3 if prec == E.PRECISION_MIXED else 1
        e3.compute_forces()
        e3.timer_start()
        for _ in range(reps):
            e3.compute_atm(nu, rc)
        t3 = e3.timer_stop() / reps
        e3.close()
        three[name] = {"F": F3, "upot": g["upot"], "triplets": g["num_pairs"], "ms": t3}
    from oracle import oracle as orc
    orc.build()
    allpos, own, _, _, _ = orc.periodic_system(pos, bmin, bmax, rc, skin)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    R3, glob3, vertex_evals = orc.atm_forces_cells(allpos, nu, rc, own=own, nthreads=nthreads)
    t_cpu = time.perf_counter() - t0
    R3 = R3[: len(pos)]
    triplets = vertex_evals / 3.0  # each triplet was evaluated from each of its three owned vertices

    def err(F, upot):
        return {"force_rms_rel": float(np.sqrt(((F - R3) ** 2).sum(1).mean() / (R3 ** 2).sum(1).mean())),
                "upot3_rel": abs(upot - glob3[0]) / abs(glob3[0])}
    rate = lambda ms: triplets / (ms * 1e-3)  # noqa: E731
    line = {"metric": "MD steps/s, LJ + Axilrod-Teller-Muto (FP32 triplets, FP64 accumulation)",
            "value": nst / (ms * 1e-3), "unit": "steps/s", "n_gpus": world, "steps": nst, "warmup": args.warmup,
            "ms_per_step": ms / nst, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 triplet arithmetic, f64 sums", "data": "synthetic",
            "config": {"workload": f"{len(pos)} particles, FCC start (jitter 0.02), density {rho}, T* 1.0, nu {nu}, "
                                   f"pair rc {rc} skin {skin}, triplet cutoff {rc}", "particles": int(len(pos))},
            "pair_interactions_per_s": st["pairs_total"] / (ms * 1e-3),
            "three_body": {"triplets": triplets,
                           "fp32_gpu": {"ms": three["fp32"]["ms"], "triplets_per_s": rate(three["fp32"]["ms"]),
                                        "error": err(three["fp32"]["F"], three["fp32"]["upot"])},
                           "fp64_gpu": {"ms": three["fp64"]["ms"], "triplets_per_s": rate(three["fp64"]["ms"]),
                                        "error": err(three["fp64"]["F"], three["fp64"]["upot"])},
                           "speedup_fp32_vs_fp64": three["fp64"]["ms"] / three["fp32"]["ms"],
                           "error_against": f"the oracle's FP64 AxilrodTellerMuto restatement on all {len(pos)} "
                                            "particles"},
            "cpu_baseline": {"value": triplets / t_cpu, "unit": "triplet interactions/s", "cores": nthreads,
                             "kind": "port", "sample": f"one three-body evaluation of all {len(pos)} particles "
                             f"(cell list, OpenMP, each triplet from every owned vertex), {t_cpu:.1f} s"},
            "gpu_launches": st["kernel_launches"]}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------- energy drift
def run_drift(args):
    """Energy drift of the FP32-mixed (full lists, and newton3 pair-group lists) and FP64 forms over --steps steps
    (default 10^4) on the FCC case:
    20^3 unit cells (32,000 particles), density 0.8442, T* 0.72, rc 2.5, skin 0.3, dt 0.002, rebuild every 10.
    Each form also runs from three more starts whose velocities differ by a relative 1e-10: MD is chaotic, so two
    trajectories part within a few thousand steps whatever their precision, and the spread of the drift over these
    starts is the scale on which the two forms' drifts can be told apart."""
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    from autopas_gb300 import engine as E, workloads
    pos, vel, bmin, bmax = workloads.fcc_lj(20, 0.8442, 0.72, seed=1)
    nsteps = max(args.steps, 10000)
    rng = np.random.default_rng(5)
    starts = [vel] + [vel * (1.0 + 1e-10 * rng.standard_normal(vel.shape)) for _ in range(3)]

    def run(prec, v0, **kw):
        e = E.PairEngine(2.5, 0.3, (bmin, bmax), periodic=True, precision=prec, rebuild_frequency=10, **kw)
        e.set_particles(pos, v0)
        g = e.compute_forces()[0]
        E0 = g["upot"] + g["ekin"]
        series = []
        t0 = time.perf_counter()
        for _ in range(nsteps // 100):
            g = e.step(0.002, 100)[0]
            series.append(g["upot"] + g["ekin"])
        wall = time.perf_counter() - t0
        e.close()
        s_ = np.array(series)
        slope = np.polyfit(np.arange(1, len(s_) + 1) * 100 * 0.002, s_ / len(pos), 1)[0]
        return {"E0_per_particle": E0 / len(pos), "drift_rel": float((s_[-1] - E0) / abs(E0)),
                "max_dev_rel": float(np.abs(s_ - E0).max() / abs(E0)),
                "slope_per_particle_per_time": float(slope), "steps": nsteps, "steps_per_s": nsteps / wall}

    out, spread = {}, {}
    forms = (("fp64", E.PRECISION_FP64, {}), ("mixed", E.PRECISION_MIXED, {}),
             ("mixed_newton3", E.PRECISION_MIXED, {"traversal": 2, "newton3": 1, "cluster_size": 8}))
    for name, prec, kw in forms:
        runs = [run(prec, v0, **kw) for v0 in starts]
        out[name] = runs[0]
        d = np.array([r["drift_rel"] for r in runs])
        spread[name] = {"drift_rel": d.tolist(), "mean": float(d.mean()), "std": float(d.std(ddof=1)),
                        "min": float(d.min()), "max": float(d.max())}
    gap = abs(spread["mixed"]["mean"] - spread["fp64"]["mean"])
    gap_n3 = abs(spread["mixed_newton3"]["mean"] - spread["fp64"]["mean"])
    scale = spread["fp64"]["max"] - spread["fp64"]["min"]
    line = {"metric": "energy drift over MD steps, FP32-mixed vs FP64 (32,000-particle FCC LJ)",
            "value": out["mixed"]["drift_rel"], "unit": "relative total-energy change", "n_gpus": 1,
            "steps": nsteps, "warmup": 0, "higher_is_better": False, "data": "synthetic",
            "config": {"workload": "FCC 20^3 unit cells, density 0.8442, T* 0.72, rc 2.5, skin 0.3, dt 0.002, "
                                   "rebuild every 10, truncated LJ"},
            "mixed": out["mixed"], "fp64": out["fp64"], "mixed_newton3": out["mixed_newton3"],
            "starts": {"what": "drift_rel of each form from the same start and from three starts whose velocities "
                               "differ by a relative 1e-10 (seeded)", "fp64": spread["fp64"], "mixed": spread["mixed"],
                       "mixed_newton3": spread["mixed_newton3"],
                       "mean_gap": gap, "mean_gap_newton3": gap_n3, "fp64_range": scale,
                       "mixed_within_fp64_range": bool(gap <= scale),
                       "mixed_newton3_within_fp64_range": bool(gap_n3 <= scale)}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.workload == "drift" and args.impl != "reference":
        return run_drift(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "mixture":
        return run_mixture(args)
    if args.workload == "atm":
        return run_atm(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
