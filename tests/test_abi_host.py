"""Host-side tests of the C-ABI library that need no GPU: it loads, exports
every symbol its header declares, and its .npy initialisation / save entry
points follow the reference's schema and error behaviour."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import LIBRARY_PATH, build_library, ic
from simplebubblyflowsolver_gb300._abi import DomainT, FluidT, InterfaceT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build_library()
    return C.CDLL(LIBRARY_PATH)


def declared_functions():
    names = []
    for h in ("sbfs_gb300.h",):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _init(lib, d, env):
    for k, v in env.items():
        os.environ[k] = v
    dom, fl, itf = DomainT(), FluidT(), InterfaceT()
    args = [C.c_char_p, C.c_void_p]
    lib.domain_init.argtypes = args
    lib.fluid_init.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    lib.interface_init.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    rc = lib.domain_init(d.encode(), C.byref(dom))
    if rc:
        return rc, None
    rc = lib.fluid_init(d.encode(), C.byref(dom), C.byref(fl))
    if rc:
        return rc, None
    rc = lib.interface_init(d.encode(), C.byref(dom), C.byref(itf))
    return rc, (dom, fl, itf)


def test_npy_init_and_save_round_trip(lib, tmp_path):
    wl = ic.bubble_swarm(64, 32, nbubbles=3, seed=1)
    fields = wl.fields()
    fields["ux"][:, 3] = 0.25  # something non-trivial to carry through
    src = tmp_path / "ic"
    ic.save_ic(str(src), fields)
    rc, st = _init(lib, str(src), wl.env())
    assert rc == 0
    dom, fl, itf = st
    assert (dom.glsizes[0], dom.glsizes[1]) == (64, 32)
    assert dom.hy == 2.0 / 32
    # vof: the wall ghost columns are set to 0 and the two ghost rows wrap
    vof = np.ctypeslib.as_array(C.cast(itf.vof.data, C.POINTER(C.c_double)), shape=(32 + 4, 66))
    assert np.array_equal(vof[2:-2, 1:-1], fields["vof"][:, 1:-1])
    assert np.array_equal(vof[0], vof[32]) and np.array_equal(vof[-1], vof[3])
    assert fl.Re == wl.Re and fl.refden == min(1.0, wl.denr) and itf.We == wl.We
    out = tmp_path / "save"
    out.mkdir()
    for fn in ("domain_save", "fluid_save", "interface_save"):
        getattr(lib, fn).argtypes = [C.c_char_p, C.c_void_p] + ([C.c_void_p] if fn != "domain_save" else [])
    assert lib.domain_save(str(out).encode(), C.byref(dom)) == 0
    assert lib.fluid_save(str(out).encode(), C.byref(dom), C.byref(fl)) == 0
    assert lib.interface_save(str(out).encode(), C.byref(dom), C.byref(itf)) == 0
    ux = np.load(out / "ux.npy")
    assert ux.dtype == np.float64 and ux.shape == (32, 65)
    want = fields["ux"].copy()
    want[:, 0] = 0.0
    want[:, -1] = 0.0
    assert np.array_equal(ux, want)
    assert np.load(out / "glsizes.npy").dtype == np.uint64
    assert float(np.load(out / "Re.npy")) == wl.Re
    assert np.array_equal(np.load(out / "xc.npy"), fields["xc"])
    lib.sbfs_free_state.argtypes = [C.c_void_p] * 3
    assert lib.sbfs_free_state(C.byref(dom), C.byref(fl), C.byref(itf)) == 0


def test_init_errors(lib, tmp_path):
    wl = ic.single_bubble(32, 16)
    fields = wl.fields()
    d = tmp_path / "ic"
    ic.save_ic(str(d), fields)
    env = wl.env()
    # missing environment key
    lib.sbfs_last_error.restype = C.c_char_p
    os.environ.pop("We", None)
    rc, _ = _init(lib, str(d), {k: v for k, v in env.items() if k != "We"})
    assert rc != 0
    assert "We" in lib.sbfs_last_error().decode()
    # wrong shape
    np.save(d / "uy.npy", np.zeros((16, 33)))
    rc, _ = _init(lib, str(d), env)
    assert rc != 0
    assert "shape" in lib.sbfs_last_error().decode()
    # wrong dtype
    np.save(d / "uy.npy", np.zeros((16, 34), dtype=np.float32))
    rc, _ = _init(lib, str(d), env)
    assert rc != 0
    assert "dtype" in lib.sbfs_last_error().decode()
    # non-uniform x grid
    np.save(d / "uy.npy", np.zeros((16, 34)))
    xf = fields["xf"].copy()
    xf[5] += 1e-3
    np.save(d / "xf.npy", xf)
    rc, _ = _init(lib, str(d), env)
    assert rc != 0
    # missing file
    os.remove(d / "xf.npy")
    rc, _ = _init(lib, str(d), env)
    assert rc != 0


def test_switches_reject_bad_modes(lib):
    """the run-mode switches check their argument on the host, before any
    CUDA call, and report through sbfs_last_error"""
    lib.sbfs_last_error.restype = C.c_char_p
    for bad in (-2, 2):
        assert lib.sbfs_set_compaction(bad) != 0
        assert "compaction" in lib.sbfs_last_error().decode()
    for mode in (0, 1, -1):  # ends on the default
        assert lib.sbfs_set_compaction(mode) == 0
    for bad in (-1, 3):
        assert lib.sbfs_set_host_link(bad) != 0
        assert "host-link" in lib.sbfs_last_error().decode()
    assert lib.sbfs_set_host_link(1) == 0  # the default
