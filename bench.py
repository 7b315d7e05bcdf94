"""Benchmark of the GB300 time step (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: the 2-D bubble swarm at scale -- lx = 4 (walls) x ly = 2
(periodic), 2048 x 1024 cells, 64 non-overlapping bubbles with radii
U[0.05, 0.10] (seed 0), density ratio 1e-3, viscosity ratio 1e-2, Re = 100,
Bo = We = 5, Fr = 1, CFL 0.4.  A step is one full integrate(): decide_dt plus
the three RK substages.  Metric: Mcell-steps/s = nx * ny * steps / s / 1e6.

value : device-resident steps (state already in HBM), CUDA events on the
        library's stream around K graph-launched steps; the ~0.6 GB working
        set is larger than L2, so no flush is needed between steps.
e2e   : the same metric through the drop-in C ABI, integrate() on
        page-locked host buffers: every step reads the state from the host and
        writes it back.  The same on the caller's own pageable buffers (as the
        reference's calloc leaves them) is reported beside it.
roofline : the dominant kernel (largest share of a profiled step) against
        the FP64 pipe, which bounds this solver on GB300: its FP64 operations
        per launch (ncu counts on this workload, profiles/kernel_traffic.txt)
        over its average duration (CUDA events around each launch on the
        library's stream), against the FP64 FMA rate measured live; its HBM
        fraction (algorithmic bytes) beside it; step-wide figures too.
cpu_baseline : the reference's own time-step sources (oracle/_ref, built on
        this machine) as one single-thread process per host core, each
        stepping the workload (the reference parallelises with MPI ranks
        only, and there is no MPI here), on a bounded sample; the oracle's
        OpenMP port and a single reference process are reported beside it.
metric_arms : the metric's second form, FP64 plain against learned curvature
        + batching, on the ensemble of 256 independent cases (three grids):
        plain batched, learned + batched (the closure trained on the GPU
        first) and plain one case at a time, with the static-drop curvature
        error and parasitic velocity of plain and learned curvature.

--impl reference times the reference's own sources alone, as above (rank 0;
other ranks exit without work).  Multi-GPU (--gpus N under torchrun):
independent replicas of the workload, one per GPU (the path has no exchange
step on one GPU per case); value = all ranks' cell-steps / the slowest
rank's time.
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
# writes counted once per cell (8 bytes per double)
ALG_DOUBLES_PER_CELL = {
    "k_props": 1 + 4,          # vof -> visux, visuy, dvof(2)
    "k_curv_list": 3 + 1,      # vof, dvof(2) -> curv (+ list of interface cells)
    "k_interface_cells": 0,    # listed cells only (a few percent of the domain)
    "k_flux_force": 5 + 4,     # ux, uy, vof, den, curv -> fluxx, fluxy, ifrcx, ifrcy
    "k_vof_advance": 6 + 5,    # fluxx, fluxy, vof, src_b, ux, uy -> src_a, vof, den1, mflux(2)
    "k_momflux": 6 + 4,        # ux, uy, visux, visuy, mflux(2) -> momentum fluxes (4)
    "k_predict_mf": 16 + 10,   # ux, uy, fluxes(4), p, ifrc(2), den1, 2rho(2), dpsi(2), src_b(2) -> u*(2), src_a(2), e grad psi(2), q(2), 2rho(2)
    "k_poisson_fwd": 2 + 1,    # q(2) -> spectrum
    "k_poisson_tdm": 2 + 1,    # spectrum, pivots -> spectrum
    "k_poisson_inv": 1 + 1,    # spectrum -> psi
    "k_correct": 6 + 5,        # u*(2), psi, e grad psi(2), p -> u(2), p, dpsi(2)
    "k_decide_dt": 2,          # ux, uy
    "k_csf_force": 3 + 2,      # vof, den, curv -> ifrcx, ifrcy
    "k_face_flux": 0,          # listed cells only
    "k_bulk_flux": 3 + 2,      # ux, uy, vof -> fluxx, fluxy
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
    ap.add_argument("--no-arms", action="store_true", help="skip the metric's learned + batched arm")
    ap.add_argument("--ref-seconds", type=float, default=30.0,
                    help="timed seconds per process of the reference arm")
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


def time_cpu(backend, workload, procs, seconds, steps, warmup, threads=1, nx=2048, ny=1024, nbubbles=64,
             cases=256):
    """one run of oracle.time_ref in its own process tree (the reference keeps
    per-grid static state, so it never runs in this process); returns its
    JSON result"""
    cmd = [sys.executable, "-m", "oracle.time_ref", "--backend", backend, "--workload", workload,
           "--nx", str(nx), "--ny", str(ny), "--nbubbles", str(nbubbles), "--cases", str(cases),
           "--steps", str(steps), "--warmup", str(warmup), "--seconds", str(seconds),
           "--threads", str(threads), "--procs", str(procs)]
    r = subprocess.run(cmd, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle.time_ref failed ({r.returncode}): {' '.join(cmd)}")
    for line in reversed(r.stdout.splitlines()):
        if line.startswith("{"):
            return json.loads(line)
    raise RuntimeError("oracle.time_ref printed no result")


def cpu_baseline(args, seconds, steps, warmup):
    """the reference's own sources on every host core (one single-thread
    process per core), beside one reference process and the OpenMP port;
    the port alone when the reference could not be built here"""
    import oracle
    wname = args.workload if args.workload != "swarm" else "swarm"
    kw = dict(nx=args.nx if args.workload != "static_drop" else args.n, ny=args.ny, nbubbles=args.bubbles,
              cases=args.cases)
    cores = os.cpu_count() or 1
    port = time_cpu("oracle", wname, 1, seconds / 2, steps, warmup, threads=cores, **kw)
    side = {"port_openmp": {"value": round(port["value"], 4), "threads": port["threads"],
                            "sample": f"{port['steps']} steps, {port['seconds']:.1f} s"}}
    if not oracle.ref_available():
        return {"value": round(port["value"], 4), "unit": METRIC, "cores": port["threads"], "kind": "port",
                "sample": f"{port['steps']} steps of the workload, {port['seconds']:.1f} s (OpenMP over every "
                          f"core; the reference's own sources were not built on this machine)"}, side
    many = time_cpu("ref", wname, cores, seconds, steps, warmup, **kw)
    one = time_cpu("ref", wname, 1, seconds, steps, warmup, **kw)
    side["reference_one_process"] = {"value": round(one["value"], 4), "cores": 1,
                                     "sample": f"{one['steps']} steps, {one['seconds']:.1f} s"}
    what = ("one case each (cases spread over the ensemble)" if wname == "ensemble" else
            "each stepping the whole workload")
    base = {"value": round(many["value"], 4), "unit": METRIC, "cores": cores, "kind": "reference",
            "sample": f"{cores} independent single-thread processes of the reference's own time-step sources "
                      f"(oracle/_ref built here; no MPI on this machine), {what}: at least {many['steps']} "
                      f"timed steps each after {warmup} untimed, {many['seconds']:.1f} s; aggregate cell-steps "
                      f"over the slowest process's time"}
    return base, side


def load_traffic():
    out = {}
    if os.path.exists(TRAFFIC_FILE):
        for line in open(TRAFFIC_FILE):
            p = line.split()
            if len(p) >= 4 and not line.startswith("#"):
                out[(p[0], p[1])] = {"traffic": float(p[2]), "fp64_flop": float(p[3]),
                                     "fp64_inst": float(p[4]) if len(p) >= 5 else None}
    return out


def ensemble_config(wls, ws):
    from collections import Counter
    grids = Counter(f"{w.ny}x{w.nx}" for w in wls)
    return {"workload": f"ensemble_{len(wls)}", "cases": len(wls), "grids_ny_x_nx": dict(grids), "seed": 0,
            "We": "log-U[1,100]", "Re": "log-U[10,100]", "denr": "log-U[1e-3,1e-1]", "visr": 0.1, "Fr": 1.0,
            "cfl": wls[0].coef_dt_adv, "parallelism": f"replicas{ws}",
            "l2": "working set (~4 GB) larger than L2, no flush"}


def reference_arm(args, ws, rank):
    """--impl reference: the reference's own sources on every host core"""
    if rank != 0:
        return
    # W untimed steps (at most two: the reference takes about a second a step
    # on the swarm), then up to K timed steps within --ref-seconds per process
    base, side = cpu_baseline(args, args.ref_seconds, args.steps, min(args.warmup, 2))
    if args.workload == "ensemble":
        from simplebubblyflowsolver_gb300 import ic
        cfg = ensemble_config(ic.ensemble(args.cases, seed=0), 1)
    else:
        cfg = config_of(workload(args), args, 1)
    line = {"metric": METRIC, "value": base["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(cfg, curvature=args.curvature), "cpu_baseline": base, "cpu_other": side,
            "e2e": {"value": base["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    roofline = roofline_of(prof, lib, cells, f"{wl.nx}x{wl.ny}", t_max * 1e3 / args.steps)

    # ---- end to end through integrate(): page-locked host buffers, then the
    # caller's own pageable ones (as the reference's calloc leaves them)
    lib.set_sync_mode(SYNC_STATE)
    ne = min(args.e2e_steps, args.steps)
    lib.pin_host_state(st)
    t_pinned = e2e_time(lib, st, ne, dist)
    lib.unpin_host_state(st)
    t_pageable = e2e_time(lib, st, ne, dist)
    state_bytes = sum(st.interior_rows(s).nbytes for s in ("ux", "uy", "p", "psi0", "vof"))
    h2d = state_bytes
    d2h = state_bytes + st.interior_rows("psi1").nbytes + 8 * 33
    e2e = {"value": round(ws * cells * ne / t_pinned / 1e6, 4), "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ne, "host_buffers": "page-locked (sbfs_pin_host_state)",
           "pageable": round(ws * cells * ne / t_pageable / 1e6, 4)}

    # ---- CPU baseline (rank 0, N = 1 only), the GPU idle meanwhile
    cpu, cpu_other = None, None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu, cpu_other = cpu_baseline(args, args.cpu_sample_s, max(args.steps, 2), 1)

    # ---- the metric's second form (rank 0, N = 1 only)
    arms = None
    if rank == 0 and ws == 1 and not args.no_arms and args.workload == "swarm":
        arms = metric_arms(args, lib)

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(config_of(wl, args, ws), curvature=args.curvature), "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu, "cpu_other": cpu_other, "metric_arms": arms, "learned_curvature": learned,
                "tiles": lib.tiles(), "clocks": clocks, "gpu_launches": lib.kernels_per_step() * args.steps,
                "dt_last": dt_last}
        print(json.dumps(line), flush=True)
    dist.close()


def e2e_time(lib, st, n, dist):
    """seconds of n integrate() calls on the host state, after two untimed"""
    for _ in range(2):
        lib.integrate(st)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(n):
        lib.integrate(st)
    return dist.max(time.perf_counter() - t0)


def roofline_of(prof, lib, cells, grid, step_ms):
    """roofline of the dominant kernel against the FP64 pipe (what bounds this
    solver on GB300) with its HBM fraction beside it, and step-wide figures.
    prof: {kernel: (ms, launches)} of profiled eager steps.  FP64 operations
    and DRAM bytes per launch are ncu counts on this grid
    (profiles/kernel_traffic.txt); the FP64 rate is measured live."""
    total = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dom]
    dom_avg_s = dom_ms / dom_n / 1e3
    peaks = json.load(open(PEAKS_FILE)) if os.path.exists(PEAKS_FILE) else {}
    hbm_peak = peaks.get("hbm_gbs", HBM_FALLBACK_GBS)
    fp64_peak = lib.measure_fp64_peak()
    traffic = {k: v for (k, g), v in load_traffic().items() if g == grid}
    tr = traffic.get(dom)
    alg_bytes = ALG_DOUBLES_PER_CELL[dom] * 8 * cells
    hbm = {"achieved": round(alg_bytes / dom_avg_s / 1e9, 1), "peak": hbm_peak, "unit": "GB/s",
           "frac": round(alg_bytes / dom_avg_s / 1e9 / hbm_peak, 4), "alg_bytes_per_launch": alg_bytes,
           "peak_source": "measured" if peaks else "fallback"}
    out = {"bound": "fp64", "kernel": dom, "achieved": None, "peak": round(fp64_peak, 1), "unit": "GFLOP/s",
           "frac": None, "traffic": tr["traffic"] if tr else None, "fp64_flop_per_launch": None,
           "peak_source": "measured live: FP64 FMA loop on this GPU (sbfs_measure_fp64_peak), of measured",
           "flop_source": "ncu DADD + DMUL + 2 DFMA thread instructions on this grid (profiles/kernel_traffic.txt)",
           "avg_launch_ms": round(dom_avg_s * 1e3, 4), "share": round(dom_ms / total, 4), "hbm": hbm,
           "shares": {k: round(v[0] / total, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}}
    if tr:
        ach = tr["fp64_flop"] / dom_avg_s / 1e9
        out.update(achieved=round(ach, 1), frac=round(ach / fp64_peak, 4), fp64_flop_per_launch=tr["fp64_flop"])
        if tr.get("fp64_inst"):
            # DADD and DMUL take an FP64 issue slot like an FMA: the fraction of
            # the pipe's instruction rate (peak / 2 FMA per second) the kernel issues
            out["issue_frac"] = round(tr["fp64_inst"] / dom_avg_s / 1e9 / (fp64_peak / 2.0), 4)
    # step-wide: every launch class of a step (decide_dt once, the rest three times)
    if traffic and all(k in traffic for k, v in prof.items() if v[1] > 0):
        per = {k: v[1] / max(1, prof["k_decide_dt"][1]) for k, v in prof.items() if v[1] > 0}
        flop = sum(traffic[k]["fp64_flop"] * n for k, n in per.items())
        inst = sum((traffic[k]["fp64_inst"] or 0.0) * n for k, n in per.items())
        out["step"] = {"fp64_flop_per_cell_step": round(flop / cells, 1),
                       "fp64_frac": round(flop / (step_ms / 1e3) / 1e9 / fp64_peak, 4),
                       "fp64_inst_per_cell_step": round(inst / cells, 1),
                       "fp64_issue_frac": round(inst / (step_ms / 1e3) / 1e9 / (fp64_peak / 2.0), 4),
                       "fused_hbm_frac": round(720.0 * cells / (step_ms / 1e3) / 1e9 / hbm_peak, 4),
                       "dram_bytes_per_cell_step": round(sum(traffic[k]["traffic"] * n for k, n in per.items())
                                                         / cells, 1),
                       "note": "fp64_frac: the step's FP64 flops (ncu, FMA = 2) over its device time and the live "
                               "FMA rate; fp64_issue_frac: its FP64 instructions (an FMA, DADD or DMUL each takes "
                               "one issue slot) over the FMA instruction rate; fused_hbm_frac: 720 B per cell-step "
                               "(the fused-minimum dataflow) over the measured HBM bandwidth"}
    return out


def metric_arms(args, lib):
    """FP64 plain against learned curvature + batching on the ensemble of 256
    independent cases (three grids, random physics), and what the closure
    does to the static drop's curvature error and parasitic currents"""
    from simplebubblyflowsolver_gb300 import SYNC_NONE, ic
    from simplebubblyflowsolver_gb300 import learned_curvature as L
    wls = ic.ensemble(args.cases, seed=0)
    cells = sum(w.cells for w in wls)
    lib.set_dt_coefs(wls[0].coef_dt_adv, wls[0].coef_dt_dif, wls[0].coef_dt_int)
    lib.set_sync_mode(SYNC_NONE)
    steps, warm = max(args.steps, 10), max(args.warmup, 3)

    def batched(model):
        # (training and the static drops set their own dt factors and modes)
        lib.set_dt_coefs(wls[0].coef_dt_adv, wls[0].coef_dt_dif, wls[0].coef_dt_int)
        lib.set_sync_mode(SYNC_NONE)
        lib.set_curvature_model(model)
        sts = [make_state(w, lib) for w in wls]
        lib.integrate_batch(sts)
        lib.run_batch_steps_timed(warm)
        ms = lib.run_batch_steps_timed(steps)
        lib.batch_release()
        return cells * steps / (ms / 1e3) / 1e6

    plain = batched(0)
    # one case at a time: the step time of four cases of each grid alone,
    # scaled to the ensemble's case count per grid
    per_grid = {}
    for w in wls:
        key = (w.nx, w.ny)
        if len(per_grid.setdefault(key, [])) < 4:
            st = make_state(w, lib)
            lib.invalidate_device()
            lib.run_steps_timed(st, warm)
            ms, _ = lib.run_steps_timed(st, steps)
            per_grid[key].append(ms / steps)
    one_ms = sum(sum(per_grid[(w.nx, w.ny)]) / len(per_grid[(w.nx, w.ny)]) for w in wls)
    t0 = time.perf_counter()
    tstats = {}
    _, params, hist = L.train_default(lib, seed=0, stats=tstats)
    train_s = time.perf_counter() - t0
    lib.mlp_set_params(params)
    learned = batched(1)
    lib.set_curvature_model(0)
    drop = {}
    nsteps = L.matched_steps(64)
    for name, model in (("plain", 0), ("learned", 1)):
        r = L.evaluate_static_drop(lib, n=64, steps=nsteps, model=model, params=params if model else None,
                                   record_every=nsteps // 20)
        drop[name] = {"kappa_rms_rel_err": round(r["kappa_rms_rel_err"], 4),
                      "umax_mean": float(np.mean([h[2] for h in r["umax_history"]])),
                      "laplace_dp_rel_err": round(r["dp_rel_err"], 4),
                      "laplace_dp_late_rel_err": round(r["dp_late_rel_err"], 4)}
    lib.set_sync_mode(SYNC_NONE)
    return {"workload": f"ensemble_{len(wls)} (grids ny x nx 64x128, 128x256, 256x512; seed 0)",
            "plain_batched": round(plain, 3), "learned_batched": round(learned, 3),
            "plain_one_at_a_time": round(cells / one_ms * 1e3 / 1e6, 3),
            "learned_batched_over_plain_one_at_a_time": round(learned / (cells / one_ms * 1e3 / 1e6), 3),
            "learned_batched_over_plain_batched": round(learned / plain, 4),
            "steps": steps, "train_s": round(train_s, 1), "train_final_loss": hist[-1],
            "training": dict(tstats, note="the closure's training on the GPU: data generation (exact-area and "
                             "solver-advected circles, relaxed drops) and the Adam epochs (1024-row batches, "
                             "one gradient and one update launch each); rows_per_s = epochs x rows / training s"),
            "static_drop_64": dict(drop, steps=nsteps, note="kappa: rms relative error of the curvature the "
                                   "last substage used in the interface cells (exact 1/r = 4); umax_mean: "
                                   "max |u| sampled 20 times over the run, averaged (parasitic currents); "
                                   "laplace_dp_rel_err: the pressure jump at the end (exact 4); "
                                   "laplace_dp_late_rel_err: its mean over the run's second half"),
            "one_at_a_time_note": "device-resident steps of four cases of each grid alone (CUDA events), "
                                  "their mean step time times the ensemble's cases on that grid"}


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
    # the FP64 pipe bounds the step; ncu FP64 counts exist for the swarm
    # grid only, so this line carries the dominant class's HBM fraction
    roofline = {"bound": "fp64", "kernel": dom, "achieved": None, "peak": round(lib.measure_fp64_peak(), 1),
                "unit": "GFLOP/s", "frac": None, "traffic": None,
                "peak_source": "measured live: FP64 FMA loop on this GPU, of measured",
                "avg_launch_ms": round(dom_ms / dom_n, 4), "share": round(dom_ms / total, 4),
                "hbm": {"achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                        "frac": round(achieved / hbm_peak, 4), "alg_bytes_per_launch": round(alg_total / dom_n),
                        "peak_source": "measured" if peaks else "fallback",
                        "note": "all cases of the dominant kernel class per step / summed event time of its "
                                "launches"},
                "shares": {k: round(v[0] / total, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}}

    # end to end: sbfs_integrate_batch on page-locked host state of every
    # case, then on the cases' own pageable arrays
    lib.set_sync_mode(SYNC_STATE)
    ne = max(2, min(args.e2e_steps, args.steps) // 10)

    def batch_e2e():
        lib.integrate_batch(sts)
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(ne):
            lib.integrate_batch(sts)
        return dist.max(time.perf_counter() - t0)

    for st in sts:
        lib.pin_host_state(st)
    t_pinned = batch_e2e()
    for st in sts:
        lib.unpin_host_state(st)
    t_pageable = batch_e2e()
    h2d = sum(sum(st.interior_rows(s).nbytes for s in ("ux", "uy", "p", "psi0", "vof")) for st in sts)
    d2h = h2d + sum(st.interior_rows("psi1").nbytes for st in sts) + len(sts) * 8 * 65
    e2e = {"value": round(ws * cells * ne / t_pinned / 1e6, 4), "unit": METRIC, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ne, "host_buffers": "page-locked (sbfs_pin_host_state)",
           "pageable": round(ws * cells * ne / t_pageable / 1e6, 4)}

    cpu, cpu_other = None, None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu, cpu_other = cpu_baseline(args, args.cpu_sample_s, max(args.steps, 2), 1)
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": METRIC, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(t_max * 1e3 / args.steps, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(ensemble_config(wls, ws), groups=groups, curvature=args.curvature),
                "e2e": e2e, "roofline": roofline, "learned_curvature": learned,
                "tiles": [lib.tiles(q) for q in range(len(groups))],
                "cpu_baseline": cpu, "cpu_other": cpu_other, "clocks": clocks,
                "gpu_launches": lib.kernels_per_step() * len(groups) * args.steps}
        print(json.dumps(line), flush=True)
    lib.batch_release()


if __name__ == "__main__":
    main()
