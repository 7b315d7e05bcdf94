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


def run(backend_name, wl, steps):
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
    for _ in range(steps):
        dts.append(be.integrate(st))
    out = {s: st.interior_rows(s).copy() for s in STATE_SLOTS}
    out["dt"] = np.array(dts)
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
    a = ap.parse_args()
    wl = make_workload(a.workload, a.nx, a.ny, a.seed, a.nbubbles)
    out = run(a.backend, wl, a.steps)
    np.savez(a.out, **out)


if __name__ == "__main__":
    main()
