"""Time a CPU checker on a workload -- TEST AND BASELINE INFRASTRUCTURE ONLY.

    python -m oracle.time_ref --backend ref --workload swarm --steps 5 --seconds 20
    python -m oracle.time_ref --backend ref --workload swarm --procs 16 ...

backend "ref" is the reference's own time-step sources (oracle/_ref, one
thread: the reference parallelises with MPI ranks only); "oracle" is the
C restatement with OpenMP over --threads.  With --procs N the workload runs
as N independent processes at once, one per core (the reference keeps
function-static per-grid state, so each process owns one case): the
aggregate throughput of the reference's own code on N cores without MPI.
Prints one JSON line: Mcell-steps/s, steps, seconds, processes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def workload(name, nx, ny, nbubbles, case, cases):
    from simplebubblyflowsolver_gb300 import ic
    if name == "swarm":
        return ic.bubble_swarm(nx, ny, nbubbles=nbubbles, seed=0)
    if name == "single_bubble":
        return ic.single_bubble(256, 128)
    if name == "static_drop":
        return ic.static_drop(nx)
    if name == "ensemble":
        return ic.ensemble(cases, seed=0)[case]
    raise ValueError(name)


def json_line(text):
    """the JSON line of a run's output (the reference also prints to stdout)"""
    for line in reversed(text.splitlines()):
        if line.startswith("{"):
            return json.loads(line)
    raise ValueError("no result line in: " + text[-500:])


def run_one(a):
    """this process: warm-up steps, then timed steps until a.steps or a.seconds"""
    import oracle
    from simplebubblyflowsolver_gb300.binding import state_from_fields
    wl = workload(a.workload, a.nx, a.ny, a.nbubbles, a.case, a.cases)
    for k, v in wl.env().items():
        os.environ[k] = v
    if a.backend == "ref":
        be = oracle.RefShim()
        info = be.info()
    else:
        be = oracle.Oracle()
        be.set_threads(a.threads)
        be.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
        info = None
    st = state_from_fields(wl.fields(), Re=wl.Re, We=wl.We, Fr=wl.Fr, denr=wl.denr, visr=wl.visr, info=info)
    be.apply_initial_boundaries(st)
    for _ in range(a.warmup):
        be.integrate(st)
    done, t0 = 0, time.perf_counter()
    while done < a.steps:
        be.integrate(st)
        done += 1
        if time.perf_counter() - t0 > a.seconds:
            break
    el = time.perf_counter() - t0
    threads = be.threads() if a.backend == "oracle" else 1
    return {"cells": wl.cells, "steps": done, "seconds": el, "value": wl.cells * done / el / 1e6,
            "threads": threads, "procs": 1}


def run_many(a):
    """a.procs copies of this script at once; case i of an ensemble goes to
    process i (cases spread over the ensemble), the swarm runs in every one"""
    cmd = [sys.executable, "-m", "oracle.time_ref", "--backend", a.backend, "--workload", a.workload,
           "--nx", str(a.nx), "--ny", str(a.ny), "--nbubbles", str(a.nbubbles), "--steps", str(a.steps),
           "--warmup", str(a.warmup), "--seconds", str(a.seconds), "--threads", "1", "--cases", str(a.cases)]
    stride = max(1, a.cases // a.procs)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    ps = [subprocess.Popen(cmd + ["--case", str((i * stride) % a.cases)], cwd=ROOT, env=env,
                           stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True) for i in range(a.procs)]
    outs = []
    for p in ps:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise SystemExit(f"time_ref process failed ({p.returncode})")
        outs.append(json_line(out))
    # every process ran at once: aggregate cell-steps over the slowest process's time
    el = max(o["seconds"] for o in outs)
    cs = sum(o["cells"] * o["steps"] for o in outs)
    return {"cells": sum(o["cells"] for o in outs), "steps": min(o["steps"] for o in outs), "seconds": el,
            "value": cs / el / 1e6, "threads": 1, "procs": a.procs,
            "per_process": [round(o["value"], 3) for o in outs]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--backend", choices=("ref", "oracle"), default="ref")
    ap.add_argument("--workload", choices=("swarm", "single_bubble", "static_drop", "ensemble"), default="swarm")
    ap.add_argument("--nx", type=int, default=2048)
    ap.add_argument("--ny", type=int, default=1024)
    ap.add_argument("--nbubbles", type=int, default=64)
    ap.add_argument("--case", type=int, default=0)
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--seconds", type=float, default=20.0)
    ap.add_argument("--threads", type=int, default=1)
    ap.add_argument("--procs", type=int, default=1)
    a = ap.parse_args()
    out = run_many(a) if a.procs > 1 else run_one(a)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
