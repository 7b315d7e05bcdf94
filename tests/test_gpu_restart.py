"""Restart through the library's own .npy entry points: N steps, save (what
the reference's save_entrypoint writes, src/main.c:16-36: step, time,
domain_save, fluid_save, interface_save), a fresh initialisation from that
directory (domain_init, fluid_init, interface_init, as exec/main.sh restarts
from output/save/...), M more steps -- bit for bit the state of N + M steps
without the break.  The state a step starts from is ux, uy, p, psi and vof
(the sources and densities are recomputed), and the files hold them exactly."""
import ctypes as C
import os

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE, ic
from simplebubblyflowsolver_gb300._abi import NADDS, DomainT, FluidT, InterfaceT

from ._helpers import set_env

pytestmark = pytest.mark.gpu


def bind(lib):
    for fn in ("domain_init", "domain_save"):
        getattr(lib, fn).argtypes = [C.c_char_p, C.c_void_p]
    for fn in ("fluid_init", "fluid_save", "interface_init", "interface_save"):
        getattr(lib, fn).argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
    lib.integrate.argtypes = [C.c_void_p] * 3 + [C.POINTER(C.c_double)]
    lib.sbfs_free_state.argtypes = [C.c_void_p] * 3


def load(lib, d):
    st = DomainT(), FluidT(), InterfaceT()
    assert lib.domain_init(d.encode(), C.byref(st[0])) == 0
    assert lib.fluid_init(d.encode(), C.byref(st[0]), C.byref(st[1])) == 0
    assert lib.interface_init(d.encode(), C.byref(st[0]), C.byref(st[2])) == 0
    return st


def step(lib, st, n):
    dts = []
    for _ in range(n):
        dt = C.c_double(0.0)
        assert lib.integrate(C.byref(st[0]), C.byref(st[1]), C.byref(st[2]), C.byref(dt)) == 0
        dts.append(dt.value)
    return dts


def state(st):
    dom, fl, itf = st
    nx, ny = dom.glsizes[0], dom.glsizes[1]
    out = {}
    for name, a in (("ux", fl.ux), ("uy", fl.uy), ("p", fl.p), ("psi", fl.psi[0]), ("vof", itf.vof)):
        (ax0, ax1), (ay0, ay1) = NADDS[name]
        shape = (ny + ay0 + ay1, nx + ax0 + ax1)
        out[name] = np.ctypeslib.as_array(C.cast(a.data, C.POINTER(C.c_double)), shape=shape).copy()
    return out


@pytest.mark.parametrize("wl", [ic.bubble_swarm(128, 64, nbubbles=6, seed=0), ic.single_bubble(128, 64)],
                         ids=["swarm_128x64", "bubble_128x64"])
def test_restart_continues_bit_for_bit(wl, tmp_path):
    from simplebubblyflowsolver_gb300 import load_library
    gpu = load_library()
    lib = gpu.lib
    bind(lib)
    set_env(wl)
    gpu.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    d0 = str(tmp_path / "ic")
    ic.save_ic(d0, wl.fields())
    N, M = 4, 3
    whole = load(lib, d0)
    dts_whole = step(lib, whole, N + M)
    first = load(lib, d0)
    dts_first = step(lib, first, N)
    saved = str(tmp_path / "save" / f"step{N:010d}")
    os.makedirs(saved)
    np.save(os.path.join(saved, "step.npy"), np.array(N, dtype=np.uint64))
    np.save(os.path.join(saved, "time.npy"), np.array(sum(dts_first), dtype=np.float64))
    assert lib.domain_save(saved.encode(), C.byref(first[0])) == 0
    assert lib.fluid_save(saved.encode(), C.byref(first[0]), C.byref(first[1])) == 0
    assert lib.interface_save(saved.encode(), C.byref(first[0]), C.byref(first[2])) == 0
    assert lib.sbfs_free_state(*(C.byref(x) for x in first)) == 0
    second = load(lib, saved)
    dts_second = step(lib, second, M)
    assert dts_first + dts_second == dts_whole
    a, b = state(whole), state(second)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert int(np.load(os.path.join(saved, "step.npy"))) == N
    for st in (whole, second):
        assert lib.sbfs_free_state(*(C.byref(x) for x in st)) == 0
