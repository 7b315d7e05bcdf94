"""Host code against the reference's own file layer and monitoring (no GPU).

oracle/_ref holds the reference's src/fileio.c, src/array.c, src/domain.c,
src/fluid/{init,save}.c, src/interface/{init,save}.c and src/logging/*.c,
compiled unmodified against single-rank MPI and NPY-header stand-ins.  So:

* the library's .npy entry points (domain_init, fluid_init, interface_init
  and the *_save functions, csrc/sbfs_npyio.cpp) must load exactly what the
  reference loads from the same initial-condition directory, write the same
  files as the reference's save, and read back what the reference writes;
* the oracle's restatement of the logging reductions (used by the GPU tests)
  must reproduce the numbers the reference's own logging printed for the
  fixture states.

Skipped where oracle/_ref was not built (it needs the reference sources).
The reference keeps per-grid function-static state (its halo exchange's
datatypes), so every reference call in this process uses one grid, 64 x 32."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import LIBRARY_PATH, build_library, ic
from simplebubblyflowsolver_gb300._abi import NADDS, DomainT, FluidT, InterfaceT

import oracle

pytestmark = pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built (no reference sources)")

GDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def libs():
    build_library()
    ours = C.CDLL(LIBRARY_PATH)
    for fn in ("domain_init", "domain_save"):
        getattr(ours, fn).argtypes = [C.c_char_p, C.c_void_p]
    for fn in ("fluid_init", "fluid_save", "interface_init", "interface_save"):
        getattr(ours, fn).argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    return ours, oracle.RefShim().lib


def load(lib, d):
    dom, fl, itf = DomainT(), FluidT(), InterfaceT()
    assert lib.domain_init(d.encode(), C.byref(dom)) == 0
    assert lib.fluid_init(d.encode(), C.byref(dom), C.byref(fl)) == 0
    assert lib.interface_init(d.encode(), C.byref(dom), C.byref(itf)) == 0
    return dom, fl, itf


def save(lib, d, st):
    dom, fl, itf = st
    os.makedirs(d, exist_ok=True)
    assert lib.domain_save(d.encode(), C.byref(dom)) == 0
    assert lib.fluid_save(d.encode(), C.byref(dom), C.byref(fl)) == 0
    assert lib.interface_save(d.encode(), C.byref(dom), C.byref(itf)) == 0


def buf(a, name, nx, ny):
    """whole buffer of an array_t, y and x ghosts included"""
    (ax0, ax1), (ay0, ay1) = NADDS[name]
    shape = (ny + ay0 + ay1, nx + ax0 + ax1)
    return np.ctypeslib.as_array(C.cast(a.data, C.POINTER(C.c_double)), shape=shape).copy()


def arrays(st):
    dom, fl, itf = st
    nx, ny = dom.glsizes[0], dom.glsizes[1]
    out = {"hy": np.array(dom.hy), "lengths": np.array(list(dom.lengths)),
           "glsizes": np.array(list(dom.glsizes)), "mysizes": np.array(list(dom.mysizes))}
    for name, n in (("xf", nx + 1), ("xc", nx + 2), ("hxxf", nx + 1), ("hxxc", nx), ("jdxf", nx + 1),
                    ("jdxc", nx)):
        out[name] = np.ctypeslib.as_array(getattr(dom, name), shape=(n,)).copy()
    for name, a in (("ux", fl.ux), ("uy", fl.uy), ("p", fl.p), ("psi", fl.psi[0]), ("vof", itf.vof)):
        out[name] = buf(a, name, nx, ny)
    for k in ("Re", "Fr", "denr", "visr", "refden"):
        out[k] = np.array(getattr(fl, k))
    out["We"] = np.array(itf.We)
    return out


def ic_dir(tmp_path, wl):
    fields = wl.fields()
    rng = np.random.default_rng(3)
    for k in ("ux", "uy", "p", "psi"):  # something non-trivial to carry through
        fields[k] = fields[k] + rng.standard_normal(fields[k].shape) * 1e-2
    d = str(tmp_path / "ic")
    ic.save_ic(d, fields)
    for k, v in wl.env().items():
        os.environ[k] = v
    return d


@pytest.mark.parametrize("wl", [ic.bubble_swarm(64, 32, nbubbles=3, seed=1), ic.single_bubble(64, 32)],
                         ids=["swarm_64x32", "bubble_64x32"])
def test_init_loads_what_the_reference_loads(libs, tmp_path, wl):
    """every loaded array, ghosts and boundary values included, bit for bit"""
    ours, ref = libs
    d = ic_dir(tmp_path, wl)
    a, b = arrays(load(ours, d)), arrays(load(ref, d))
    assert sorted(a) == sorted(b)
    for k in a:
        assert a[k].shape == b[k].shape and np.array_equal(a[k], b[k]), k


def test_save_writes_what_the_reference_writes(libs, tmp_path):
    """the same file names, dtypes, shapes and values as the reference's
    domain_save / fluid_save / interface_save of the same state, and each
    side reads the other's files back to the same arrays"""
    ours, ref = libs
    wl = ic.bubble_swarm(64, 32, nbubbles=3, seed=2)
    d = ic_dir(tmp_path, wl)
    so, sr = load(ours, d), load(ref, d)
    save(ours, str(tmp_path / "ours"), so)
    save(ref, str(tmp_path / "ref"), sr)
    names = sorted(os.listdir(tmp_path / "ref"))
    assert sorted(os.listdir(tmp_path / "ours")) == names
    for n in names:
        x, y = np.load(tmp_path / "ours" / n), np.load(tmp_path / "ref" / n)
        assert x.dtype == y.dtype and x.shape == y.shape and np.array_equal(x, y), n
    # cross reads: the reference loads our files, the library loads the reference's
    base = arrays(so)
    for lib, src in ((ref, "ours"), (ours, "ref")):
        got = arrays(load(lib, str(tmp_path / src)))
        for k in base:
            assert np.array_equal(got[k], base[k]), (src, k)


def test_oracle_logging_reductions_match_the_reference_logs():
    """the oracle's restatement of src/logging/*.c (the GPU monitoring tests'
    checker) against the numbers the reference's own logging printed for the
    fixtures' final states (printed to 16 digits)"""
    from oracle.run_case import make_workload
    from ._helpers import new_state, set_env
    manifest = json.load(open(os.path.join(GDIR, "manifest.json")))
    orc = oracle.Oracle()
    names = {"momentum": ("momentum_x", "momentum_y"), "extrema": ("umax", "vmax"),
             "energy": ("energy_x", "energy_y"), "stress": ("wall_stress_xm", "wall_stress_xp")}
    for name, spec in sorted(manifest.items()):
        wl = make_workload(spec["workload"], spec["nx"], spec["ny"], spec.get("seed", 0), spec.get("nbubbles", 64))
        set_env(wl)
        gold = np.load(os.path.join(GDIR, f"{name}.npz"))
        st = new_state(wl, orc)
        for s in ("ux", "uy", "p", "psi0", "vof", "txy"):
            st.interior_rows(s)[...] = gold[s]
        orc.apply_initial_boundaries(st)  # y ghost rows of the loaded state
        orc.compute_density(st, 1)        # den[1]: the density of the final vof, as after a step
        got = orc.diagnostics(st)
        last = {f: [float(x) for x in str(gold["log_" + f]).splitlines()[-1].split()[1:]]
                for f in ("momentum", "extrema", "energy", "stress", "vof", "divergence")}
        for f, keys in names.items():
            for k, v in zip(keys, last[f]):
                assert abs(got[k] - v) <= 1e-14 * abs(v) + 1e-300, (name, k, got[k], v)
        vmin, vmax, vmean, area = last["vof"]
        assert abs(got["vof_min"] - vmin) <= 1e-14 * abs(vmin) + 1e-300
        assert abs(got["vof_max"] - vmax) <= 1e-14 * abs(vmax)
        assert abs(got["vof_integral"] / got["volume"] - vmean) <= 1e-14 * abs(vmean)
        assert abs(got["interface_area"] - area) <= 1e-14 * abs(area)
        assert float(f"{got['divmax']:.1e}") == last["divergence"][0], (name, got["divmax"], last["divergence"])


def test_command_line_generator_writes_what_the_reference_reads(libs, tmp_path):
    """python -m simplebubblyflowsolver_gb300.ic, driven like the reference's
    initial_condition/main.sh (lx, ly, glisize, gljsize in the environment):
    the directory holds the reference's schema, step and time included, and
    the reference's init and the library's load it to the same arrays"""
    import subprocess
    import sys
    ours, ref = libs
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    d = tmp_path / "ic"
    env = dict(os.environ, lx="4.0", ly="2.0", glisize="64", gljsize="32", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-m", "simplebubblyflowsolver_gb300.ic", str(d)], env=env, cwd=str(tmp_path),
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exports = dict(line[len("export "):].split("=", 1) for line in r.stdout.splitlines())
    assert sorted(exports) == sorted(["Re", "We", "Fr", "denr", "visr", "coef_dt_adv", "coef_dt_dif", "coef_dt_int"])
    assert np.load(d / "step.npy").dtype == np.uint64 and int(np.load(d / "step.npy")) == 0
    assert np.load(d / "time.npy").dtype == np.float64 and float(np.load(d / "time.npy")) == 0.0
    vof = np.load(d / "vof.npy")
    assert vof.shape == (32, 66) and abs(vof.sum() * (4.0 / 64) * (2.0 / 32) - np.pi / 4) < 1e-12
    for k, v in exports.items():
        os.environ[k] = v
    a, b = arrays(load(ours, str(d))), arrays(load(ref, str(d)))
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # a missing environment key is reported, as the reference's script needs them
    env.pop("glisize")
    r = subprocess.run([sys.executable, "-m", "simplebubblyflowsolver_gb300.ic", str(tmp_path / "x")], env=env,
                       cwd=str(tmp_path), capture_output=True, text=True)
    assert r.returncode != 0 and "glisize" in r.stderr
