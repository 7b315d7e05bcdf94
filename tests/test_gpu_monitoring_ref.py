"""The device-side logging and statistics against the reference's own
monitoring code (src/logging/*.c, src/statistics.c built into oracle/_ref;
their output stored in tests/golden/ by make_golden.py).

* Logging: the reference's state after ten steps of each fixture case (with
  the txy its last predictor left) is handed to sbfs_logging_output, whose
  lines must match the reference's last log line of each of the seven files:
  the same text where the reference prints text (step, time, dt), the same
  numbers to 1e-11 relative where it prints reductions (sums in another
  order), and both divergence maxima at rounding level.
* Statistics: the GPU steps the same case ten times, collecting after every
  step; the sums sbfs_statistics_output writes must match the reference's
  sums, within the parity bar of the ten states they add up."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE

from ._helpers import fma_noise_floor, new_state, set_env

pytestmark = pytest.mark.gpu

GDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MANIFEST = json.load(open(os.path.join(GDIR, "manifest.json")))
FILES = ("progress", "divergence", "momentum", "extrema", "energy", "stress", "vof")


@pytest.fixture(scope="module")
def gpu():
    from simplebubblyflowsolver_gb300 import load_library
    lib = load_library()
    lib.set_sync_mode(SYNC_STATE)
    return lib


def case(name):
    from oracle.run_case import make_workload
    spec = MANIFEST[name]
    wl = make_workload(spec["workload"], spec["nx"], spec["ny"], spec.get("seed", 0), spec.get("nbubbles", 64))
    return wl, spec, np.load(os.path.join(GDIR, f"{name}.npz"))


def numbers(line):
    return [float(x) for x in line.split()[1:]]


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_logging_matches_the_reference_logs(gpu, name, tmp_path):
    import oracle
    wl, spec, gold = case(name)
    set_env(wl)
    gpu.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = new_state(wl, oracle.Oracle())
    for s in ("ux", "uy", "p", "psi0", "vof", "txy"):
        st.interior_rows(s)[...] = gold[s]
    t = 0.0
    for dt in gold["dt"]:
        t += float(dt)  # the order run_case sums them in
    steps = spec["steps"]
    gpu.logging_output(str(tmp_path), st, steps, t, float(gold["dt"][-1]), 0.0)
    for f in FILES:
        ref = str(gold["log_" + f]).splitlines()
        assert len(ref) == steps, (name, f, len(ref))
        got = (tmp_path / f"{f}.dat").read_text().splitlines()
        assert len(got) == 1, (name, f, got)
        g, r = got[0], ref[-1]
        if f == "progress":
            assert g == r, (name, g, r)
            continue
        assert g[:9] == r[:9] and len(g) == len(r), (name, f, g, r)
        gv, rv = numbers(g), numbers(r)
        if f == "divergence":
            # printed to two digits; both maxima are rounding noise
            assert gv[0] <= 1e-12 and rv[0] <= 1e-12, (name, gv, rv)
            continue
        for a, b in zip(gv, rv):
            # signed sums (momentum, wall stress) may cancel: an absolute floor
            assert abs(a - b) <= 1e-11 * abs(b) + 1e-16, (name, f, a, b)


@pytest.mark.parametrize("name", sorted(MANIFEST))
def test_statistics_match_the_reference_sums(gpu, name, tmp_path):
    import oracle
    wl, spec, gold = case(name)
    set_env(wl)
    gpu.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = new_state(wl, oracle.Oracle())
    gpu.statistics_reset()
    for _ in range(spec["steps"]):
        gpu.integrate(st)
        gpu.statistics_collect(st)
    out = tmp_path / "stat"
    out.mkdir()
    gpu.lib.sbfs_statistics_output.argtypes = [C.c_char_p, C.c_void_p]
    assert gpu.lib.sbfs_statistics_output(str(out).encode(), C.addressof(st.domain)) == 0
    assert int(np.load(out / "num.npy")) == int(gold["stat_num"]) == spec["steps"]
    # the states the sums add up are held to 1e-10 (ten times the oracle's
    # FMA spread for the static drop, whose flow amplifies rounding)
    bar = 1e-10
    if spec["workload"] == "static_drop":
        bar = max(bar, 10 * max(fma_noise_floor(wl, spec["steps"]).values()))
    for s in ("ux1", "uy1", "vof1"):
        a, b = np.load(out / f"{s}.npy"), gold["stat_" + s]
        assert a.shape == b.shape and a.dtype == b.dtype == np.float64, (name, s, a.shape, b.shape)
        err = np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)
        print(name, s, f"{err:.2e}", "bar", bar)
        assert err <= bar, (name, s, err, bar)
    gpu.statistics_reset()

