"""Initial conditions in the reference's .npy schema, with exact-area VOF.

The reference's generator (initial_condition/main.py:6-83) writes
step, time, xf, xc, glsizes, lengths, vof, ux, uy, p, psi; its VOF is a
tanh-smoothed circle.  The workloads of this package instead need the exact
area fraction of each cell covered by one or more discs, computed here in
closed form: over x, the covered height of a cell is a piecewise function
(0, the cell height, or a chord clipped to the cell) whose pieces are
separated by the points where the circle crosses the cell's edges; on each
piece the integral is analytic through
    S(u) = integral sqrt(r^2 - u^2) du = (u sqrt(r^2 - u^2) + r^2 asin(u/r)) / 2.
vof = 1 marks the inside of a bubble (density ratio denr), as in the
reference, where den = 1 + (denr - 1) vof.  y is periodic, so discs are
wrapped across it.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


def _chord_integral(u0, u1, r):
    def S(u):
        u = np.clip(u, -r, r)
        return 0.5 * (u * np.sqrt(np.maximum(r * r - u * u, 0.0)) + r * r * np.arcsin(u / r))
    return S(u1) - S(u0)


def disc_cell_fraction(x0, x1, y0, y1, xc, yc, r):
    """Exact area of disc((xc, yc), r) inside [x0,x1]x[y0,y1], divided by the
    cell area.  All arguments broadcast elementwise (numpy arrays)."""
    x0, x1, y0, y1, xc, yc, r = np.broadcast_arrays(
        *(np.asarray(a, dtype=np.float64) for a in (x0, x1, y0, y1, xc, yc, r)))
    shape = x0.shape
    x0, x1, y0, y1, xc, yc, r = (a.ravel() for a in (x0, x1, y0, y1, xc, yc, r))
    # candidate breakpoints in x, relative to the centre
    bps = [x0 - xc, x1 - xc, -r, r]
    for yy in (y0, y1):
        dy = yy - yc
        inside = np.abs(dy) < r
        w = np.sqrt(np.where(inside, r * r - dy * dy, 0.0))
        bps.append(np.where(inside, -w, x0 - xc))
        bps.append(np.where(inside, +w, x0 - xc))
    B = np.stack(bps, axis=1)
    lo = (x0 - xc)[:, None]
    hi = (x1 - xc)[:, None]
    B = np.clip(B, lo, hi)
    B.sort(axis=1)
    ylo = (y0 - yc)[:, None]
    yhi = (y1 - yc)[:, None]
    rr = r[:, None]
    a, b = B[:, :-1], B[:, 1:]
    m = 0.5 * (a + b)
    s = np.sqrt(np.maximum(rr * rr - m * m, 0.0))
    top_is_chord = s < yhi          # top boundary is the circle on this piece
    bot_is_chord = -s > ylo
    width = b - a
    chord = _chord_integral(a, b, rr)
    top = np.where(top_is_chord, chord, yhi * width)
    bot = np.where(bot_is_chord, -chord, ylo * width)
    piece = top - bot
    valid = (np.abs(m) < rr) & (np.minimum(yhi, s) > np.maximum(ylo, -s)) & (width > 0)
    area = np.where(valid, piece, 0.0).sum(axis=1)
    cell = (x1 - x0) * (y1 - y0)
    return np.clip(area / cell, 0.0, 1.0).reshape(shape)


def vof_from_discs(xf, ly, ny, discs):
    """VOF on the reference's vof layout (ny, nx+2): interior columns 1..nx,
    wall ghost columns 0 and nx+1 left at 0 (they are overwritten by the
    boundary condition vof = 0 anyway).  `discs` is a list of (xc, yc, r)."""
    nx = len(xf) - 1
    dy = ly / ny
    yf = np.arange(ny + 1) * dy
    X0, Y0 = np.meshgrid(xf[:-1], yf[:-1])
    X1, Y1 = np.meshgrid(xf[1:], yf[1:])
    vof = np.zeros((ny, nx))
    for (cx, cy, r) in discs:
        for shift in (-ly, 0.0, ly):
            yy = cy + shift
            if yy + r < 0.0 or yy - r > ly:
                continue
            jlo = max(0, int(math.floor((yy - r) / dy)) - 1)
            jhi = min(ny, int(math.ceil((yy + r) / dy)) + 1)
            ilo = max(0, int(np.searchsorted(xf, cx - r)) - 2)
            ihi = min(nx, int(np.searchsorted(xf, cx + r)) + 2)
            if jlo >= jhi or ilo >= ihi:
                continue
            sl = (slice(jlo, jhi), slice(ilo, ihi))
            vof[sl] += disc_cell_fraction(X0[sl], X1[sl], Y0[sl], Y1[sl], cx, yy, r)
    out = np.zeros((ny, nx + 2))
    out[:, 1:-1] = np.clip(vof, 0.0, 1.0)
    return out


@dataclass
class Workload:
    """A rising-bubble case: grid, discs and physics (env keys of the
    reference: Re, We, Fr, denr, visr, coef_dt_adv/dif/int)."""
    name: str
    nx: int
    ny: int
    lx: float
    ly: float
    discs: list
    Re: float
    We: float
    Fr: float
    denr: float
    visr: float
    coef_dt_adv: float = 0.4
    coef_dt_dif: float = 0.5
    coef_dt_int: float = 0.95
    steps: int = 10
    meta: dict = field(default_factory=dict)

    @property
    def cells(self):
        return self.nx * self.ny

    def env(self) -> dict:
        return {k: repr(float(getattr(self, k))) for k in
                ("Re", "We", "Fr", "denr", "visr", "coef_dt_adv", "coef_dt_dif", "coef_dt_int")}

    def grid(self):
        xf = np.linspace(0.0, self.lx, self.nx + 1, endpoint=True)
        xc = np.concatenate(([0.0], 0.5 * xf[:-1] + 0.5 * xf[1:], [self.lx]))
        return xf, xc

    def fields(self) -> dict:
        """initial fields in the reference .npy schema"""
        xf, xc = self.grid()
        ny, nx = self.ny, self.nx
        return {
            "step": np.array(0, dtype=np.uint64),
            "time": np.array(0.0, dtype=np.float64),
            "xf": xf, "xc": xc,
            "glsizes": np.array([nx, ny], dtype=np.uint64),
            "lengths": np.array([self.lx, self.ly], dtype=np.float64),
            "vof": vof_from_discs(xf, self.ly, ny, self.discs),
            "ux": np.zeros((ny, nx + 1)),
            "uy": np.zeros((ny, nx + 2)),
            "p": np.zeros((ny, nx + 2)),
            "psi": np.zeros((ny, nx + 2)),
        }


def single_bubble(nx=256, ny=128, steps=10) -> Workload:
    """One bubble r = 0.25 at (0.5, 0.5) in lx = 2 (walls) x ly = 1 (periodic),
    Re = 35, Bo (= We with Fr = 1) = 10, density and viscosity ratio 0.1."""
    return Workload("single_bubble", nx, ny, 2.0, 1.0, [(0.5, 0.5, 0.25)],
                    Re=35.0, We=10.0, Fr=1.0, denr=0.1, visr=0.1, steps=steps)


def bubble_swarm(nx=2048, ny=1024, nbubbles=64, seed=0, steps=2000) -> Workload:
    """64 non-overlapping bubbles, radii U[0.05, 0.10], in lx = 4 x ly = 2;
    density ratio 1e-3, viscosity ratio 1e-2, Re = 100, Bo = 5.  Centres are
    drawn by rejection sampling (seeded), kept one radius plus two cells off
    the walls and separated by at least two cells between interfaces
    (distance measured periodically in y)."""
    lx, ly = 4.0, 2.0
    rng = np.random.default_rng(seed)
    dx = lx / nx
    discs = []
    tries = 0
    while len(discs) < nbubbles:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place bubbles")
        r = rng.uniform(0.05, 0.10)
        cx = rng.uniform(r + 2 * dx, lx - r - 2 * dx)
        cy = rng.uniform(0.0, ly)
        ok = True
        for (ox, oy, orr) in discs:
            ddy = abs(cy - oy)
            ddy = min(ddy, ly - ddy)
            if math.hypot(cx - ox, ddy) < r + orr + 2 * dx:
                ok = False
                break
        if ok:
            discs.append((cx, cy, r))
    return Workload("bubble_swarm", nx, ny, lx, ly, discs, Re=100.0, We=5.0, Fr=1.0,
                    denr=1e-3, visr=1e-2, steps=steps, meta={"seed": seed})


ENSEMBLE_GRIDS = ((128, 64), (256, 128), (512, 256))  # (nx, ny): ny x nx = 64x128, 128x256, 256x512


def ensemble(ncases=256, seed=0, steps=500, grids=ENSEMBLE_GRIDS) -> list:
    """Independent rising-bubble cases for batched runs, each with the single
    bubble's geometry (lx = 2 x ly = 1, one bubble r = 0.25 at (0.5, 0.5)):
    grid uniform-random over `grids` (square cells), log-uniform We in
    [1, 100], Re in [10, 100] and density ratio in [1e-3, 1e-1], viscosity
    ratio 0.1, Fr = 1.  (With the viscosity ratio equal to the density ratio,
    135 of the 256 cases blow up in the reference's own step within a few
    steps of the start from rest: its diffusive dt bound then allows steps
    at which the pressure splitting, started with zero pressure, diverges.
    With 0.1 all 256 start cleanly.)"""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(ncases):
        nx, ny = grids[int(rng.integers(len(grids)))]
        We = float(np.exp(rng.uniform(np.log(1.0), np.log(100.0))))
        Re = float(np.exp(rng.uniform(np.log(10.0), np.log(100.0))))
        denr = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1))))
        out.append(Workload("ensemble_case", nx, ny, 2.0, 1.0, [(0.5, 0.5, 0.25)], Re=Re, We=We, Fr=1.0, denr=denr,
                            visr=0.1, steps=steps, meta={"seed": seed, "case": k}))
    return out


def static_drop(n=64, steps=1000) -> Workload:
    """Static drop r = 0.25 in a 1 x 1 box, density ratio 1e-3, no gravity
    (Fr = inf), Laplace number La = Re^2 / We = 12000 with We = 1."""
    return Workload("static_drop", n, n, 1.0, 1.0, [(0.5, 0.5, 0.25)], Re=math.sqrt(12000.0),
                    We=1.0, Fr=math.inf, denr=1e-3, visr=1e-3, steps=steps)


def save_ic(dirname: str, fields: dict):
    """write the reference's IC schema ('<f8' / '<u8' C-order .npy files)"""
    os.makedirs(dirname, exist_ok=True)
    for k, v in fields.items():
        np.save(os.path.join(dirname, f"{k}.npy"), v)


def load_ic(dirname: str) -> dict:
    names = ("step", "time", "xf", "xc", "glsizes", "lengths", "vof", "ux", "uy", "p", "psi")
    return {k: np.load(os.path.join(dirname, f"{k}.npy")) for k in names}


def reference_bubble(nx, ny, lx=4.0, ly=2.0) -> Workload:
    """The reference generator's case (initial_condition/main.py:27-45): one
    bubble of diameter 1 centred at (1, 1), here as exact cell area fractions
    instead of the reference's tanh profile; physics of exec/main.sh
    (Re 35, We 10, Fr 1, density ratio 0.0013, viscosity ratio 0.018, CFL
    0.2)."""
    return Workload("reference_bubble", nx, ny, lx, ly, [(1.0, 1.0, 0.5)], Re=35.0, We=10.0, Fr=1.0,
                    denr=0.0013, visr=0.018, coef_dt_adv=0.2)


def main(argv=None):
    """Command-line generator, the counterpart of the reference's
    initial_condition/main.sh + main.py: writes step, time, xf, xc, glsizes,
    lengths, vof, ux, uy, p and psi into DIR (the reference's schema, which
    its domain_init / fluid_init / interface_init and this library's read)
    and prints the environment the solver reads for the case's physics
    (Re, We, Fr, denr, visr and the dt safety factors), as export lines.

        python -m simplebubblyflowsolver_gb300.ic DIR
            the reference's case on the grid of the environment variables
            lx, ly, glisize, gljsize (those initial_condition/main.sh sets)
        python -m simplebubblyflowsolver_gb300.ic DIR --workload swarm --nx 2048 --ny 1024 --bubbles 64 --seed 0
        python -m simplebubblyflowsolver_gb300.ic DIR --workload single_bubble --nx 256 --ny 128
        python -m simplebubblyflowsolver_gb300.ic DIR --workload static_drop --nx 64
        python -m simplebubblyflowsolver_gb300.ic DIR --workload ensemble_case --case 17 --seed 0
    """
    import argparse
    ap = argparse.ArgumentParser(prog="python -m simplebubblyflowsolver_gb300.ic",
                                 description="initial condition in the reference's .npy schema")
    ap.add_argument("dirname")
    ap.add_argument("--workload", default="reference",
                    choices=("reference", "single_bubble", "swarm", "static_drop", "ensemble_case"))
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--ny", type=int, default=None)
    ap.add_argument("--bubbles", type=int, default=64)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--case", type=int, default=0, help="ensemble_case: which of the ensemble's cases")
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--env-file", default=None, help="also write the export lines to this file")
    a = ap.parse_args(argv)
    if a.workload == "reference":
        try:
            lx, ly = float(os.environ["lx"]), float(os.environ["ly"])
            nx = int(os.environ["glisize"]) if a.nx is None else a.nx
            ny = int(os.environ["gljsize"]) if a.ny is None else a.ny
        except KeyError as e:
            ap.error(f"environment variable {e.args[0]} not set (initial_condition/main.sh sets lx, ly, "
                     "glisize, gljsize)")
        wl = reference_bubble(nx, ny, lx, ly)
    elif a.workload == "single_bubble":
        wl = single_bubble(a.nx or 256, a.ny or 128)
    elif a.workload == "swarm":
        wl = bubble_swarm(a.nx or 2048, a.ny or 1024, nbubbles=a.bubbles, seed=a.seed)
    elif a.workload == "static_drop":
        wl = static_drop(a.nx or 64)
    else:
        cases = ensemble(a.cases, seed=a.seed)
        if not 0 <= a.case < len(cases):
            ap.error(f"--case must be in 0..{len(cases) - 1}")
        wl = cases[a.case]
    save_ic(a.dirname, wl.fields())
    lines = [f"export {k}={v}" for k, v in wl.env().items()]
    if a.env_file:
        with open(a.env_file, "w") as fh:
            fh.write("\n".join(lines) + "\n")
    print("\n".join(lines))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
