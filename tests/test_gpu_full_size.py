"""The benchmarked configuration itself, the 64-bubble swarm on 2048 x 1024
cells, against the oracle (run on every host core) and through its
size-independent invariants: VOF mass and the discrete divergence after the
projection."""
import os

import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE, ic

from ._helpers import clone, compare_state, new_state, set_env

pytestmark = pytest.mark.gpu

STEPS = 5


@pytest.fixture(scope="module")
def swarm_runs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    gpu, orc = load_library(), oracle.Oracle()
    orc.set_threads(os.cpu_count() or 1)
    wl = ic.bubble_swarm()  # 2048 x 1024, 64 bubbles, seed 0
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    m0 = orc.vof_stats(st0)[2]
    dts, errs = [], []
    for _ in range(STEPS):
        dts.append((gpu.integrate(a), orc.integrate(b)))
        errs.append(compare_state(a, b))
    return a, b, dts, errs, m0, orc


def test_full_size_swarm_matches_oracle(swarm_runs):
    """one full step (three substages) within 1e-10 of the oracle.  Later
    steps are no parity case at this size: in the second step corner normals
    of the THINC tails (rounding-noise gradients normalised to unit length)
    turn different ways in different roundings; the oracle and the oracle
    built with FMA contraction part by 1.4e-4 there, this build and the
    oracle by 8.9e-7 (5.6e-6 after five steps)."""
    _, _, dts, errs, _, _ = swarm_runs
    dg, do = dts[0]
    assert abs(dg - do) <= 1e-14 * do, (dg, do)
    print("step 1", {k: f"{v:.1e}" for k, v in errs[0].items()})
    assert max(errs[0].values()) <= 1e-10, errs[0]
    for dg, do in dts:
        assert abs(dg - do) <= 1e-10 * do, (dg, do)


def test_full_size_swarm_invariants(swarm_runs):
    """after five steps: VOF mass to 1e-12 relative, and the discrete
    divergence no larger than the oracle's own (it grows with 1 / dx: the
    oracle leaves 3.5e-11 here against 1e-12 on the 256 x 128 bubble)"""
    a, b, _, _, m0, orc = swarm_runs
    m1 = orc.vof_stats(a)[2]
    dg, do = orc.max_divergence(a), orc.max_divergence(b)
    print("mass", m0, m1, "max |div u| gpu", dg, "oracle", do)
    assert abs(m1 - m0) <= 1e-12 * abs(m0), (m0, m1)
    assert dg <= max(1e-12, 2 * do), (dg, do)
