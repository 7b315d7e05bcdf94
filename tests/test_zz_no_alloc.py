"""decide_dt without allocation, for callers that may not allocate GPU memory
(programs that own all device memory through their own pool, or must not
call cudaMalloc / cudaFree while running): the variant reads velocities the
caller already holds on the GPU and keeps its scratch in a fixed array inside
the library.  Its time step must equal the one the regular decide_dt entry
point computes from the same fields, on calls in a row (each call finds the
previous call's words in the shared scratch array): two where the advective
limit sets dt, then one with slow velocities where the diffusive / capillary
bound does (the one part of the computation this variant does differently,
from lx / nx instead of the minimum of HXXF).  After the first call on the GPU
(its set-up), a call allocates no device memory.

This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import ic

from ._helpers import new_state, set_env

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


def test_decide_dt_noalloc_matches_decide_dt():
    import torch

    from simplebubblyflowsolver_gb300 import load_library
    lib = load_library()
    wl = ic.bubble_swarm(256, 128, nbubbles=6)
    set_env(wl)
    lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = new_state(wl, lib)
    fn = lib.lib.sbfs_decide_dt_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p] + \
        [C.c_double] * 7 + [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.lib.sbfs_noalloc_last_error.restype = C.c_char_p
    nx, ny = st.nx, st.ny
    pitch = nx + 8
    rng = np.random.default_rng(0)
    hxxf = torch.from_numpy(st.hxxf.copy()).cuda()
    dt_fixed_bound = wl.coef_dt_dif * 0.1 * wl.Re * 0.25 * (st.lx / nx) ** 2
    for call, scale in enumerate((50.0, 20.0, 1e-6)):
        # calls 0, 1: velocities large enough that the advective limit sets
        # dt; call 2: so slow that the fixed bound does
        st.interior_rows("ux")[...] = scale * rng.standard_normal(st.interior_rows("ux").shape)
        st.interior_rows("uy")[...] = scale * rng.standard_normal(st.interior_rows("uy").shape)
        lib.update_boundaries(st, "ux")
        lib.update_boundaries(st, "uy")
        dt_ref = lib.decide_dt(st)
        ux = torch.zeros((ny, pitch), dtype=torch.float64, device="cuda")
        uy = torch.zeros((ny, pitch), dtype=torch.float64, device="cuda")
        ux[:, :nx + 1] = torch.from_numpy(st.interior_rows("ux").copy())
        uy[:, :nx + 2] = torch.from_numpy(st.interior_rows("uy").copy())
        scalars = torch.full((64,), -1.0, dtype=torch.float64, device="cuda")
        status = torch.zeros((1,), dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = fn(nx, ny, st.lx, st.ly, _dev_ptr(ux), _dev_ptr(uy), pitch, _dev_ptr(hxxf), wl.Re, wl.denr, wl.visr,
                wl.We, wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int, _dev_ptr(scalars), _dev_ptr(status), None)
        assert rc == 0, lib.lib.sbfs_noalloc_last_error().decode()
        torch.cuda.synchronize()
        if call >= 1:
            # past the set-up call, nothing is allocated on the device
            assert torch.cuda.mem_get_info()[0] == free_before, (call, free_before, torch.cuda.mem_get_info()[0])
        dt = float(scalars[0].item())
        assert int(status[0].item()) == 0
        if call < 2:
            assert dt < 0.9 * dt_fixed_bound, "advective limit not active"
            # the same kernel and the same expressions: within an ulp or so
            assert abs(dt - dt_ref) <= 1e-14 * dt_ref, (call, dt, dt_ref)
        else:
            # the fixed bound: lx / nx against the minimum of HXXF, equal up
            # to the rounding of the grid's face positions
            assert abs(dt - dt_fixed_bound) <= 1e-12 * dt_fixed_bound, "the fixed bound does not set dt"
            assert abs(dt - dt_ref) <= 1e-13 * dt_ref, (call, dt, dt_ref)
    # sizes beyond the fixed scratch array are refused
    rc = fn(8193, ny, st.lx, st.ly, _dev_ptr(ux), _dev_ptr(uy), 8200, _dev_ptr(hxxf), wl.Re, wl.denr, wl.visr,
            wl.We, wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int, _dev_ptr(scalars), _dev_ptr(status), None)
    assert rc != 0 and b"SBFS_NOALLOC_MAX_NX" in lib.lib.sbfs_noalloc_last_error()
