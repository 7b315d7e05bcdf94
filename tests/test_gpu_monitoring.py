"""Device-side logging reductions and statistics against the oracle's
restatement of src/logging/*.c and src/statistics.c."""
import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import SYNC_NONE, SYNC_STATE, ic

from ._helpers import clone, new_state, set_env

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    return load_library(), oracle.Oracle()


def test_diagnostics_match_oracle(libs):
    gpu, orc = libs
    wl = ic.bubble_swarm(256, 128, nbubbles=6)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st = new_state(wl, orc)
    for _ in range(5):
        orc.integrate(st)
    a = gpu.diagnostics(clone(st))
    b = orc.diagnostics(st)
    for k in a:
        scale = max(abs(b[k]), 1e-300)
        tol = 0.0 if k in ("vof_min", "vof_max", "umax", "vmax", "volume") else 1e-11
        if k == "divmax":
            assert a[k] <= 1e-12 and b[k] <= 1e-12
            continue
        # sums of signed terms (momentum, wall stress) may cancel: absolute floor
        assert abs(a[k] - b[k]) <= tol * scale + (1e-16 if tol else 0.0), (k, a[k], b[k])


def test_resident_diagnostics_and_statistics(libs):
    gpu, orc = libs
    wl = ic.single_bubble(128, 64)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = new_state(wl, orc)
    ref = clone(st)
    gpu.set_sync_mode(SYNC_NONE)
    gpu.invalidate_device()
    gpu.statistics_reset()
    sums = [np.zeros_like(ref.interior_rows(s)) for s in ("ux", "uy", "vof")]
    for _ in range(4):
        gpu.integrate(st)
        orc.integrate(ref)
        gpu.statistics_collect(st)
        for acc, s in zip(sums, ("ux", "uy", "vof")):
            acc += ref.interior_rows(s)
    d = gpu.diagnostics(st)
    gpu.sync_to_host(st)
    gpu.set_sync_mode(SYNC_STATE)
    o = orc.diagnostics(ref)
    assert abs(d["vof_integral"] - o["vof_integral"]) <= 1e-12 * o["vof_integral"]
    assert abs(d["energy_x"] - o["energy_x"]) <= 1e-8 * abs(o["energy_x"])
    ux1, uy1, vof1, num = gpu.statistics_fetch(st.nx, st.ny)
    assert num == 4
    for got, want in zip((ux1, uy1, vof1), sums):
        assert np.abs(got - want).max() <= 1e-9 * max(np.abs(want).max(), 1e-300)
