"""Benchmark of the GB300 time step (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: the 2-D bubble swarm at scale -- lx = 4 (walls) x ly = 2
(periodic), 2048 x 1024 cells, 64 non-overlapping bubbles with radii
U[0.05, 0.10] (seed 0), density ratio 1e-3, viscosity ratio 1e-2, Re = 100,
Bo = We = 5, Fr = 1, CFL 0.4.  A step is one full integrate(): decide_dt plus
the three RK substages.  Metric: Mcell-steps/s = nx * ny * steps / s / 1e6.

value : device-resident steps (state already in HBM), CUDA events on the
        library's stream around K graph-launched steps; the ~0.5 GB working
        set is larger than L2, so no flush is needed between steps.
e2e   : the same metric through the drop-in C ABI, integrate() with host
        (page-locked) buffers: every step uploads the state and writes it
        back, as a reference caller sees it.
roofline : the dominant kernel (largest share of a profiled step), its
        algorithmic bytes per launch over its average duration, measured live
        with CUDA events around each launch on the library's stream.
cpu_baseline : the CPU port of the reference time step (oracle/, OpenMP over
        all host cores) on a bounded sample of the same workload.

--impl reference times that CPU implementation alone (rank 0; other ranks
exit without work).  Multi-GPU (--gpus N under torchrun): independent
replicas of the workload, one per GPU (the path has no exchange step on one
GPU per case); value = all ranks' cell-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "kernel_traffic.txt")
HBM_FALLBACK_GBS = 6800.0

# algorithmic bytes per cell and launch: every field a kernel reads or
# writes counted once per cell (8 bytes per double); see the design doc
ALG_DOUBLES_PER_CELL = {
    "k_props": 1 + 4,          # vof -> visux, visuy, dvof(2)
    "k_curv_list": 3 + 1,      # vof, dvof(2) -> curv (+ list of interface cells)
    "k_interface_cells": 0,    # listed cells only (a few percent of the domain)
    "k_flux_force": 5 + 4,     # ux, uy, vof, den, curv -> fluxx, fluxy, ifrcx, ifrcy
    "k_vof_advance": 6 + 5,    # fluxx, fluxy, vof, src_b, ux, uy -> src_a, vof, den1, mflux(2)
    "k_momflux": 6 + 4,        # ux, uy, visux, visuy, mflux(2) -> momentum fluxes (4)
    "k_predict_mf": 14 + 6,    # ux, uy, fluxes(4), p, ifrc(2), den(2), psi_old, src_b(2) -> u*(2), src_a(2), e grad psi(2)
    "k_poisson_fwd": 4 + 1,    # u*(2), e grad psi(2) -> spectrum
    "k_poisson_tdm": 2 + 1,    # spectrum, pivots -> spectrum
    "k_poisson_inv": 1 + 1,    # spectrum -> psi
    "k_correct": 6 + 3,        # u*(2), psi, e grad psi(2), p -> u(2), p
    "k_decide_dt": 2,          # ux, uy
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=1024)
    ap.add_argument("--bubbles", type=int, default=64)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--profile-steps", type=int, default=10)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0, help="target seconds of CPU-baseline work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=("swarm", "single_bubble", "static_drop", "ensemble"), default="swarm",
                    help="swarm: the 2048x1024 bubble swarm (default); single_bubble: 256x128, one bubble; "
                         "static_drop: n x n (--n); ensemble: 256 independent cases in batches")
    ap.add_argument("--n", type=int, default=256, help="static drop grid")
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--curvature", choices=("plain", "learned"), default="plain",
                    help="learned: train the closure on the GPU first, then time the step with it")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch.distributed as tdist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "gloo"
            tdist.init_process_group(backend=backend)
            self.tdist = tdist

    def barrier(self):
        if self.ws > 1:
            self.tdist.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.tdist.all_reduce(t, op=self.tdist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.tdist.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs"""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for _, _, p in rows:
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def workload(args):
    from simplebubblyflowsolver_gb300 import ic
    if args.workload == "single_bubble":
        return ic.single_bubble(256, 128)
    if args.workload == "static_drop":
        return ic.static_drop(args.n)
    return ic.bubble_swarm(args.nx, args.ny, nbubbles=args.bubbles, seed=0)


def config_of(wl, args, ws):
    big = wl.cells * 8 * 35 > 129e6
    cfg = {"workload": f"{wl.name}_{wl.nx}x{wl.ny}", "nx": wl.nx, "ny": wl.ny, "bubbles": len(wl.discs),
           "lx": wl.lx, "ly": wl.ly, "Re": wl.Re, "Bo": wl.We, "Fr": wl.Fr, "denr": wl.denr, "visr": wl.visr,
           "cfl": wl.coef_dt_adv, "parallelism": f"replicas{ws}",
           "l2": ("working set larger than L2, no flush" if big else
                  "working set fits in L2: an L2-resident, launch-latency-bound case (no flush)")}
    if wl.name == "bubble_swarm":
        cfg.update(radii="U[0.05,0.10]", seed=0)
    return cfg


def make_state(wl, backend):
    from simplebubblyflowsolver_gb300 import state_from_fields
    for k, v in wl.env().items():
        os.environ[k] = v
    st = state_from_fields(wl.fields(), Re=wl.Re, We=wl.We, Fr=wl.Fr, denr=wl.denr, visr=wl.visr)
    backend.apply_initial_boundaries(st)
    return st


def cpu_run(wl, steps, seconds_cap, warmup=1):
    """the CPU port of the reference (oracle/) with all host cores: `warmup`
    untimed steps (first touch, caches), then up to `steps` timed ones within
    seconds_cap; returns (Mcell-steps/s, threads, steps done, seconds)"""
    import oracle
    orc = oracle.Oracle()
    orc.set_threads(os.cpu_count() or 1)
    orc.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = make_state(wl, orc)
    t0 = time.perf_counter()
    for _ in range(max(1, warmup)):
        orc.integrate(st)
        if time.perf_counter() - t0 > seconds_cap / 4:
            break
    done, t0 = 0, time.perf_counter()
    while done < steps:
        orc.integrate(st)
        done += 1
        if time.perf_counter() - t0 > seconds_cap:
            break
    el = time.perf_counter() - t0
    return wl.cells * done / el / 1e6, orc.threads(), done, el


def load_traffic():
    out = {}
    if os.path.exists(TRAFFIC_FILE):
        for line in open(TRAFFIC_FILE):
            p = line.split()
            if len(p) >= 4 and not line.startswith("#"):
                out[(p[0], p[1])] = {"traffic": float(p[2]), "fp64_flop": float(p[3])}
    return out


def ensemble_config(wls, ws):
    from collections import Counter
    grids = Counter(f"{w.ny}x{w.nx}" for w in wls)
    return {"workload": f"ensemble_{len(wls)}", "cases": len(wls), "grids_ny_x_nx": dict(grids), "seed": 0,
            "We": "log-U[1,100]", "Re": "log-U[10,100]", "denr": "log-U[1e-3,1e-1]", "visr": 0.1, "Fr": 1.0,
            "cfl": wls[0].coef_dt_adv, "parallelism": f"replicas{ws}",
            "l2": "working set (~4 GB) larger than L2, no flush"}


def cpu_ensemble(wls, seconds_cap):
    """the CPU port on every 8th case (one warm step, then timed steps until
    the cap); returns (Mcell-steps/s, threads, case-steps, seconds)"""
    import oracle
    orc = oracle.Oracle()
    orc.set_threads(os.cpu_count() or 1)
    orc.set_dt_coefs(wls[0].coef_dt_adv, wls[0].coef_dt_dif, wls[0].coef_dt_int)
    sample = wls[::8]
    sts = [make_state(w, orc) for w in sample]
    for st in sts:
        orc.integrate(st)
    cells, done, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds_cap:
        for w, st in zip(sample, sts):
            orc.integrate(st)
            cells += w.cells
            done += 1
    el = time.perf_counter() - t0
    return cells / el / 1e6, orc.threads(), done, el


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    if args.workload == "ensemble":
        from simplebubblyflowsolver_gb300 import ic
        wls = ic.ensemble(args.cases, seed=0)
        val, threads, done, el = cpu_ensemble(wls, seconds_cap=60.0)
        line = {"metric": METRIC, "value": round(val, 4), "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
                "steps": done, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": ensemble_config(wls, 1),
                "cpu_baseline": {"value": round(val, 4), "unit": METRIC, "cores": threads, "kind": "port",
                                 "sample": f"{done} case-steps over every 8th case, {el:.1f} s"},
                "e2e": {"value": round(val, 4), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    wl = workload(args)
    # W untimed steps, then K timed steps, capped so the run stays within minutes
    val, threads, done, el = cpu_run(wl, args.steps, seconds_cap=180.0, warmup=args.warmup)
    line = {"metric": METRIC, "value": round(val, 4), "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": done, "warmup": args.warmup, "ms_per_step": round(1e3 * el / done, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(wl, args, 1),
            "cpu_baseline": {"value": round(val, 4), "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{done} timed full steps of the workload after {args.warmup} untimed "
                                       f"(timed part capped at 180 s)"},
            "e2e": {"value": round(val, 4), "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    ws, rank, local = dist_info()
    dist = Dist(ws)
    if args.impl == "reference":
        reference_arm(args, ws, rank)
        dist.close()
        return
    from simplebubblyflowsolver_gb300 import SYNC_NONE, SYNC_STATE, build_library, load_library
    build_library()
    lib = load_library()
    lib.set_device(local)
    lib.set_autotune(not args.no_autotune)
    learned = None
    if args.curvature == "learned":
        from simplebubblyflowsolver_gb300 import learned_curvature as L
        t0 = time.perf_counter()
        _, params, hist = L.train_default(lib, seed=0)
        learned = {"train_s": round(time.perf_counter() - t0, 1), "final_loss": hist[-1]}
        lib.mlp_set_params(params)
        lib.set_curvature_model(1)
    if args.workload == "ensemble":
        run_ensemble(args, lib, dist, ws, rank, local, learned)
        dist.close()
        return
    wl = workload(args)
    lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = make_state(wl, lib)
    cells = wl.cells

    # ---- device-resident throughput
    lib.set_sync_mode(SYNC_NONE)
    lib.invalidate_device()
    lib.run_steps_timed(st, args.warmup)
    dist.barrier()
    with ClockSampler(local) as clk:
        ms, dt_last = lib.run_steps_timed(st, args.steps)
    dist.barrier()
    t_max = dist.max(ms / 1e3)
    value = ws * cells * args.steps / t_max / 1e6
    clocks = clk.summary()

    # ---- per-kernel shares and the dominant kernel (eager launches, events)
    prof = lib.profile_steps(st, args.profile_steps)
    total = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    dom_avg_s = dom_ms / dom_n / 1e3
    alg_bytes = ALG_DOUBLES_PER_CELL[dom] * 8 * cells
    achieved = alg_bytes / dom_avg_s / 1e9
    peaks = json.load(open(PEAKS_FILE)) if os.path.exists(PEAKS_FILE) else {}
    hbm_peak = peaks.get("hbm_gbs", HBM_FALLBACK_GBS)
    tr = load_traffic().get((dom, f"{wl.nx}x{wl.ny}"))
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "traffic": tr["traffic"] if tr else None,
                "peak_source": "measured" if peaks else "fallback",
                "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": round(dom_avg_s * 1e3, 4),
                "share": round(dom_ms / total, 4),
                "shares": {k: round(v[0] / total, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}}
    fp64_peak = lib.measure_fp64_peak()
    roofline["fp64_peak_gflops"] = round(fp64_peak, 1)
    if tr and tr.get("fp64_flop"):
        ach = tr["fp64_flop"] / dom_avg_s / 1e9
        roofline["fp64"] = {"achieved": round(ach, 1), "peak": round(fp64_peak, 1), "unit": "GFLOP/s",
                            "frac": round(ach / fp64_peak, 4),
                            "peak_source": "measured live: FMA loop (sbfs_measure_fp64_peak)",
                            "flop_source": "ncu sass FP64 instruction counts (profiles/kernel_traffic.txt)"}

    # ---- end to end through integrate() with page-locked host buffers
    lib.set_sync_mode(SYNC_STATE)
    lib.pin_host_state(st)
    for _ in range(2):
        lib.integrate(st)
    ne = min(args.e2e_steps, args.steps)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ne):
        lib.integrate(st)
    t_e2e = dist.max(time.perf_counter() - t0)
    lib.unpin_host_state(st)
    state_bytes = sum(st.interior_rows(s).nbytes for s in ("ux", "uy", "p", "psi0", "vof"))
    h2d = state_bytes
    d2h = state_bytes + st.interior_rows("psi1").nbytes + 8 * 33
    e2e = {"value": round(ws * cells * ne / t_e2e / 1e6, 4), "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ne}

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        per_step = cells / 15e6  # rough seconds per step to size the sample
        n = max(2, int(args.cpu_sample_s / per_step))
        val, threads, done, el = cpu_run(wl, n, seconds_cap=2 * args.cpu_sample_s)
        cpu = {"value": round(val, 4), "unit": METRIC, "cores": threads, "kind": "port",
               "sample": f"{done} full steps of the same workload, {el:.1f} s"}

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(config_of(wl, args, ws), curvature=args.curvature), "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu, "learned_curvature": learned, "tiles": lib.tiles(),
                "clocks": clocks, "gpu_launches": lib.kernels_per_step() * args.steps,
                "dt_last": dt_last}
        print(json.dumps(line), flush=True)
    dist.close()


def run_ensemble(args, lib, dist, ws, rank, local, learned=None):
    """256 independent cases (three grids, random physics) advanced together:
    every kernel of the step runs all cases of one grid in one launch"""
    from simplebubblyflowsolver_gb300 import SYNC_NONE, SYNC_STATE, ic
    wls = ic.ensemble(args.cases, seed=0)
    lib.set_dt_coefs(wls[0].coef_dt_adv, wls[0].coef_dt_dif, wls[0].coef_dt_int)
    sts = [make_state(w, lib) for w in wls]
    cells = sum(w.cells for w in wls)
    lib.set_sync_mode(SYNC_NONE)
    lib.integrate_batch(sts)
    lib.run_batch_steps_timed(args.warmup)
    dist.barrier()
    with ClockSampler(local) as clk:
        ms = lib.run_batch_steps_timed(args.steps)
    dist.barrier()
    t_max = dist.max(ms / 1e3)
    value = ws * cells * args.steps / t_max / 1e6
    clocks = clk.summary()
    groups = lib.batch_groups()

    # per-kernel shares (eager, events on each group's stream; groups overlap,
    # so the per-class sums are upper bounds of the class's wall time)
    prof = lib.profile_batch_steps(args.profile_steps)
    total = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    # a launch covers all cases of one group: over the profiled steps the
    # class moved ALG * 8 B * (all cells) once per launch round of the groups
    alg_total = ALG_DOUBLES_PER_CELL[dom] * 8 * cells * dom_n / len(groups)
    achieved = alg_total / (dom_ms / 1e3) / 1e9
    peaks = json.load(open(PEAKS_FILE)) if os.path.exists(PEAKS_FILE) else {}
    hbm_peak = peaks.get("hbm_gbs", HBM_FALLBACK_GBS)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "traffic": None,
                "peak_source": "measured" if peaks else "fallback",
                "alg_bytes_per_launch": round(alg_total / dom_n),
                "avg_launch_ms": round(dom_ms / dom_n, 4), "share": round(dom_ms / total, 4),
                "shares": {k: round(v[0] / total, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
                "note": "all cases of the dominant kernel class per step / summed event time of its launches"}
    roofline["fp64_peak_gflops"] = round(lib.measure_fp64_peak(), 1)

    # end to end: sbfs_integrate_batch with page-locked host state of every case
    lib.set_sync_mode(SYNC_STATE)
    for st in sts:
        lib.pin_host_state(st)
    lib.integrate_batch(sts)
    ne = max(2, min(args.e2e_steps, args.steps) // 10)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ne):
        lib.integrate_batch(sts)
    t_e2e = dist.max(time.perf_counter() - t0)
    for st in sts:
        lib.unpin_host_state(st)
    h2d = sum(sum(st.interior_rows(s).nbytes for s in ("ux", "uy", "p", "psi0", "vof")) for st in sts)
    d2h = h2d + sum(st.interior_rows("psi1").nbytes for st in sts) + len(sts) * 8 * 65
    e2e = {"value": round(ws * cells * ne / t_e2e / 1e6, 4), "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ne}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        val, threads, done, el = cpu_ensemble(wls, seconds_cap=args.cpu_sample_s)
        cpu = {"value": round(val, 4), "unit": METRIC, "cores": threads, "kind": "port",
               "sample": f"{done} case-steps over every 8th case, {el:.1f} s"}
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(ensemble_config(wls, ws), groups=groups, curvature=args.curvature),
                "e2e": e2e, "roofline": roofline, "learned_curvature": learned,
                "tiles": [lib.tiles(q) for q in range(len(groups))],
                "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": lib.kernels_per_step() * len(groups) * args.steps}
        print(json.dumps(line), flush=True)
    lib.batch_release()


if __name__ == "__main__":
    main()
