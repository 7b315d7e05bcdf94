"""Run a workload for N steps on a CPU checker and save the state.

    python -m oracle.run_case --backend ref --workload single_bubble \
        --nx 64 --ny 32 --steps 10 --out out.npz

The reference build keeps function-static solver state (one grid per
process), so each case runs in its own process.  TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from simplebubblyflowsolver_gb300 import ic  # noqa: E402
from simplebubblyflowsolver_gb300.binding import state_from_fields  # noqa: E402

STATE_SLOTS = ("ux", "uy", "p", "psi0", "vof")


def make_workload(name, nx, ny, seed=0, nbubbles=64):
    if name == "single_bubble":
        return ic.single_bubble(nx, ny)
    if name == "bubble_swarm":
        return ic.bubble_swarm(nx, ny, nbubbles=nbubbles, seed=seed)
    if name == "static_drop":
        return ic.static_drop(nx)
    raise ValueError(name)


LOG_FILES = ("progress.dat", "divergence.dat", "momentum.dat", "extrema.dat", "energy.dat", "stress.dat", "vof.dat")


def run(backend_name, wl, steps, monitor=None):
    """monitor (reference backend only): a directory in which the reference's
    own logging writes its seven monitor files after every step and its
    statistics collect every step's state and are written after the last"""
    for k, v in wl.env().items():
        os.environ[k] = v
    import oracle
    if backend_name == "ref":
        be = oracle.RefShim()
        info = be.info()
    else:
        be = oracle.Oracle()
        be.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
        info = None
    st = state_from_fields(wl.fields(), Re=wl.Re, We=wl.We, Fr=wl.Fr, denr=wl.denr,
                           visr=wl.visr, info=info)
    be.apply_initial_boundaries(st)
    dts = []
    here = os.getcwd()
    if monitor:
        os.makedirs(os.path.join(monitor, "output", "log"), exist_ok=True)
        os.makedirs(os.path.join(monitor, "output", "stat"), exist_ok=True)
        os.environ.setdefault("stat_rate", "1.0")
        os.environ.setdefault("stat_after", "0.0")
        os.chdir(monitor)
        be.stats_init(st, 0.0)
    try:
        t = 0.0
        for step in range(1, steps + 1):
            dts.append(be.integrate(st))
            t += dts[-1]
            if monitor:
                be.log(st, step, t, dts[-1], 0.0)
                be.stats_collect(st)
        if monitor:
            be.stats_output(st, steps)
    finally:
        os.chdir(here)
    out = {s: st.interior_rows(s).copy() for s in STATE_SLOTS}
    out["dt"] = np.array(dts)
    if monitor:
        # the stress the last predictor left (the wall-stress log reads it)
        out["txy"] = st.interior_rows("txy").copy()
        for name in LOG_FILES:
            with open(os.path.join(monitor, "output", "log", name)) as fh:
                out["log_" + name.split(".")[0]] = np.array(fh.read())
        sdir = os.path.join(monitor, "output", "stat", f"step{steps:010d}")
        for name in ("num", "ux1", "uy1", "vof1"):
            out["stat_" + name] = np.load(os.path.join(sdir, name + ".npy"))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--backend", choices=("ref", "oracle"), required=True)
    ap.add_argument("--workload", default="single_bubble")
    ap.add_argument("--nx", type=int, default=256)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nbubbles", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--out", required=True)
    ap.add_argument("--monitor", default=None, help="directory for the reference's logging and statistics output")
    a = ap.parse_args()
    wl = make_workload(a.workload, a.nx, a.ny, a.seed, a.nbubbles)
    out = run(a.backend, wl, a.steps, a.monitor)
    np.savez(a.out, **out)


if __name__ == "__main__":
    main()
