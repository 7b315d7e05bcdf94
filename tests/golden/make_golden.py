"""Generate the golden fixtures of this directory from the reference's own
sources (oracle/_ref/libsbfs_ref.so, built by `make -C oracle ref` from the
reference checkout).  Each case runs in its own process because the
reference keeps function-static solver state.

    python tests/golden/make_golden.py

Fixture content: the state after N steps of integrate() (ux, uy, p, psi, vof
interior rows with x ghosts, i.e. the reference's .npy layout), the dt of
every step, and what the reference's own monitoring wrote over the run: its
seven log files after every step (log_*, the text of src/logging/*.c) with
the txy the last predictor left (the wall-stress log reads it), and its
statistics sums over the N steps (stat_num, stat_ux1, stat_uy1, stat_vof1,
the arrays src/statistics.c writes).  Inputs are regenerated by
simplebubblyflowsolver_gb300.ic with the case parameters stored alongside.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

CASES = [
    # name, workload, nx, ny, extra, steps
    ("single_bubble_256x128", "single_bubble", 256, 128, {}, 10),
    ("swarm_128x64", "bubble_swarm", 128, 64, {"nbubbles": 6, "seed": 0}, 10),
    ("static_drop_64", "static_drop", 64, 64, {}, 10),
]


def main():
    sys.path.insert(0, ROOT)
    import oracle
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libsbfs_ref.so missing: run `make -C oracle ref` first")
    manifest = {}
    for name, wl, nx, ny, extra, steps in CASES:
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "out.npz")
            cmd = [sys.executable, "-m", "oracle.run_case", "--backend", "ref", "--workload", wl,
                   "--nx", str(nx), "--ny", str(ny), "--steps", str(steps), "--out", out, "--monitor", td]
            for k, v in extra.items():
                cmd += [f"--{k}", str(v)]
            subprocess.run(cmd, check=True, cwd=ROOT, stdout=subprocess.DEVNULL)
            data = dict(np.load(out))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **data)
        manifest[name] = {"workload": wl, "nx": nx, "ny": ny, "steps": steps, **extra,
                          "source": "reference time-step, logging, statistics and file-layer sources + "
                                    "single-rank stand-ins (oracle/_ref)"}
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
