"""The benchmarked configuration itself, the 64-bubble swarm on 2048 x 1024
cells, for ten steps against the oracle (run on every host core) and against
the oracle's own rounding floor, plus its size-independent invariants: VOF
mass and the discrete divergence after the projection.

Why a floor: in the second step corner normals of the THINC tails
(rounding-noise gradients normalised to unit length, reference
src/interface/curvature_tensor.c:37-45) turn different ways in different
roundings, and the oracle built as is and the oracle built with fused
multiply-add contraction (two faithful builds of the same arithmetic) part by
1e-4 there.  No second implementation can be held closer to one of them than
they are to each other, so each step is held to the larger of 1e-10 and ten
times that spread, field by field."""
import os

import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE, ic

from ._helpers import clone, compare_state, new_state, set_env

pytestmark = pytest.mark.gpu

STEPS = 10


@pytest.fixture(scope="module")
def swarm_runs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    gpu, orc, fma = load_library(), oracle.Oracle(), oracle.Oracle(variant="fma")
    for lib in (orc, fma):
        lib.set_threads(os.cpu_count() or 1)
    wl = ic.bubble_swarm()  # 2048 x 1024, 64 bubbles, seed 0
    set_env(wl)
    for lib in (gpu, orc, fma):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b, c = clone(st0), clone(st0), clone(st0)
    m0 = orc.vof_stats(st0)[2]
    rows = []
    for step in range(1, STEPS + 1):
        dts = (gpu.integrate(a), orc.integrate(b), fma.integrate(c))
        rows.append({"step": step, "dt": dts, "gpu_vs_oracle": compare_state(a, b),
                     "gpu_vs_fma": compare_state(a, c), "oracle_vs_fma": compare_state(b, c)})
    for r in rows:
        print(r["step"], "gpu-oracle %.1e" % max(r["gpu_vs_oracle"].values()),
              "gpu-fma %.1e" % max(r["gpu_vs_fma"].values()),
              "oracle-fma %.1e" % max(r["oracle_vs_fma"].values()))
    return a, b, rows, m0, orc


def test_full_size_swarm_ten_steps_within_the_rounding_floor(swarm_runs):
    """every field after every step within max(1e-10, 10 x the oracle-vs-FMA
    spread of that field); the first step within 1e-10 outright; dt within
    max(1e-10, 10 x the spread of the two oracle builds' dt)"""
    _, _, rows, _, _ = swarm_runs
    first = rows[0]["gpu_vs_oracle"]
    assert max(first.values()) <= 1e-10, first
    for r in rows:
        for f, e in r["gpu_vs_oracle"].items():
            bar = max(1e-10, 10.0 * r["oracle_vs_fma"][f])
            assert e <= bar, (r["step"], f, e, bar)
        dg, do, df = r["dt"]
        bar = max(1e-10, 10.0 * abs(do - df) / do)
        assert abs(dg - do) <= bar * do, (r["step"], dg, do, df)


def test_full_size_swarm_invariants(swarm_runs):
    """after ten steps: VOF mass to 1e-12 relative, and the discrete
    divergence no larger than the oracle's own (it grows with 1 / dx: the
    oracle leaves 3.5e-11 here against 1e-12 on the 256 x 128 bubble)"""
    a, b, _, m0, orc = swarm_runs
    m1 = orc.vof_stats(a)[2]
    dg, do = orc.max_divergence(a), orc.max_divergence(b)
    print("mass", m0, m1, "max |div u| gpu", dg, "oracle", do)
    assert abs(m1 - m0) <= 1e-12 * abs(m0), (m0, m1)
    assert dg <= max(1e-12, 2 * do), (dg, do)
