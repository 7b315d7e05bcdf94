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


def test_logging_files_in_the_reference_format(libs, tmp_path):
    """sbfs_logging_output writes the seven monitor files with the
    reference's line formats (src/logging/*.c), values from the oracle"""
    gpu, orc = libs
    wl = ic.single_bubble(128, 64)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st = new_state(wl, orc)
    t = 0.0
    for step in range(1, 4):
        dt = orc.integrate(st)
        t += dt
        gpu.logging_output(str(tmp_path), clone(st), step, t, dt, 0.5)
    b = orc.diagnostics(st)
    files = {p.name: p.read_text().splitlines() for p in tmp_path.iterdir()}
    assert sorted(files) == sorted(["progress.dat", "divergence.dat", "momentum.dat", "extrema.dat", "energy.dat",
                                    "stress.dat", "vof.dat"])
    assert all(len(v) == 3 for v in files.values())
    assert files["progress.dat"][-1] == f"step {3:10d}, time {t:.3f}, dt {dt:.3e}, elapsed {0.5:.1f} [sec]"
    assert files["divergence.dat"][-1].startswith(f"{t:8.2f} ")
    expect = {
        "momentum.dat": (b["momentum_x"], b["momentum_y"]),
        "extrema.dat": (b["umax"], b["vmax"]),
        "energy.dat": (b["energy_x"], b["energy_y"]),
        "stress.dat": (b["wall_stress_xm"], b["wall_stress_xp"]),
        "vof.dat": (b["vof_min"], b["vof_max"], b["vof_integral"] / b["volume"], b["interface_area"]),
    }
    for name, vals in expect.items():
        line = files[name][-1]
        ref = f"{t:8.2f} " + " ".join(f"{v: 18.15e}" for v in vals)
        assert len(line) == len(ref) and line[:9] == ref[:9], (name, line, ref)
        got = [float(x) for x in line.split()[1:]]
        for g, v in zip(got, vals):
            assert abs(g - v) <= 1e-11 * abs(v) + 1e-16, (name, g, v)
