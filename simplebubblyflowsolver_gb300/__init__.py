"""GB300 implementation of SimpleBubblyFlowSolver's 2-D two-phase time step.

The product is ``libsbfs_gb300.so``: the reference solver's C entry points
(integrate, decide_dt, fluid_*, interface_*, *_init, *_save) implemented with
hand-written sm_103a CUDA kernels.  This package builds it in-tree, binds it
with ctypes and provides the host-side pieces a Python user needs
(initial conditions in the reference's .npy schema, a state container).
There is no CPU fallback: :func:`load_library` raises if the library is
missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes as C
import os

from ._abi import SolverState
from .binding import RK_ALPHA, RK_BETA, RK_GAMMA, ReferenceAPI, SolverError, state_from_fields
from .build import LIB as LIBRARY_PATH
from .build import build as build_library

SYNC_STATE, SYNC_ALL, SYNC_NONE = 0, 1, 2

__all__ = [
    "SolverState", "SolverError", "ReferenceAPI", "GpuLibrary", "load_library", "build_library",
    "state_from_fields", "LIBRARY_PATH", "RK_ALPHA", "RK_BETA", "RK_GAMMA",
    "SYNC_STATE", "SYNC_ALL", "SYNC_NONE",
]

_LIB = None


class GpuLibrary(ReferenceAPI):
    """The reference entry points of libsbfs_gb300.so plus its additions."""

    def __init__(self, lib: C.CDLL):
        super().__init__(lib, prefix="", name="libsbfs_gb300")
        lib.sbfs_last_error.restype = C.c_char_p
        lib.sbfs_set_sync_mode.argtypes = [C.c_int]
        lib.sbfs_set_use_graphs.argtypes = [C.c_int]
        lib.sbfs_set_host_link.argtypes = [C.c_int]
        lib.sbfs_set_pdl.argtypes = [C.c_int]
        lib.sbfs_set_dt_coefs.argtypes = [C.c_double] * 3
        lib.sbfs_sync_to_host.argtypes = [C.c_void_p] * 3
        lib.sbfs_run_steps_timed.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                             C.POINTER(C.c_float), C.POINTER(C.c_double)]
        lib.sbfs_device_status.argtypes = [C.POINTER(C.c_int)]
        lib.sbfs_set_device.argtypes = [C.c_int]
        lib.sbfs_measure_fp64_peak.argtypes = [C.POINTER(C.c_double)]
        lib.sbfs_diagnostics.argtypes = [C.c_void_p] * 4
        lib.sbfs_statistics_collect.argtypes = [C.c_void_p] * 3
        lib.sbfs_statistics_fetch.argtypes = [C.POINTER(C.c_double)] * 3 + [C.POINTER(C.c_size_t)]
        lib.sbfs_check_newton_raphson.argtypes = [C.POINTER(C.c_double)] * 3 + [C.c_int]
        lib.sbfs_pin_host_state.argtypes = [C.c_void_p, C.c_void_p]
        lib.sbfs_unpin_host_state.argtypes = [C.c_void_p, C.c_void_p]
        lib.sbfs_kernel_name.restype = C.c_char_p
        lib.sbfs_kernel_name.argtypes = [C.c_int]
        lib.sbfs_profile_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                           C.POINTER(C.c_float), C.POINTER(C.c_int)]

    def _call(self, fn, *args):
        rc = self._fns[fn](*args)
        if rc != 0:
            raise SolverError(f"{fn} failed: {self.last_error()}")
        return rc

    def _ext(self, fn, *args):
        rc = getattr(self.lib, fn)(*args)
        if rc != 0:
            raise SolverError(f"{fn} failed: {self.last_error()}")

    def last_error(self) -> str:
        return self.lib.sbfs_last_error().decode()

    def set_sync_mode(self, mode: int):
        self._ext("sbfs_set_sync_mode", mode)

    def set_use_graphs(self, on: bool):
        self._ext("sbfs_set_use_graphs", 1 if on else 0)

    def set_pdl(self, on: bool):
        """launch the step's kernels with programmatic dependent launch"""
        self._ext("sbfs_set_pdl", 1 if on else 0)

    def set_compaction(self, mode: int):
        """interface-branch compaction: -1 as tuned (default), 0 off, 1 on"""
        self._ext("sbfs_set_compaction", int(mode))

    def set_stream_priorities(self, on: bool):
        """launch the step's kernels at their streams' priorities (main high,
        side low; default True)"""
        self._ext("sbfs_set_stream_priorities", 1 if on else 0)

    def set_tdm_cluster(self, on: bool):
        """solve a wavenumber pair's four tridiagonal systems as a cluster of
        four CTAs where the grid takes four warps a system (default True)"""
        self._ext("sbfs_set_tdm_cluster", 1 if on else 0)

    def set_geometry_ahead(self, on: bool):
        """form each substage's interface geometry and CSF force ahead of its
        velocity, beside the previous substage's predictor (default True)"""
        self._ext("sbfs_set_geometry_ahead", 1 if on else 0)

    def set_host_link(self, on):
        """strict-mode steps copy the state in and out themselves, overlapped
        with their kernels, when the GPU can address the host arrays (True or
        1); 2 links registered arrays only; False or 0 never"""
        self._ext("sbfs_set_host_link", int(on))

    def host_link_used(self) -> bool:
        """whether the last integrate() was host-linked"""
        return bool(self.lib.sbfs_host_link_used())

    def set_dt_coefs(self, adv, dif, itf):
        self._ext("sbfs_set_dt_coefs", adv, dif, itf)

    def invalidate_device(self):
        self._ext("sbfs_invalidate_device")

    def sync_to_host(self, st: SolverState):
        self._ext("sbfs_sync_to_host", *self._ptrs(st))

    def run_steps_timed(self, st: SolverState, nsteps: int):
        ms = C.c_float(0.0)
        dt = C.c_double(0.0)
        self._ext("sbfs_run_steps_timed", *self._ptrs(st), nsteps, C.byref(ms), C.byref(dt))
        return ms.value, dt.value

    def check_newton_raphson(self, x):
        """(1/x, 1/sqrt(x)) from the device helpers, for accuracy tests"""
        import numpy as np
        x = np.ascontiguousarray(x, dtype=np.float64)
        r = np.empty_like(x)
        q = np.empty_like(x)
        dp = C.POINTER(C.c_double)
        self._ext("sbfs_check_newton_raphson", x.ctypes.data_as(dp), r.ctypes.data_as(dp), q.ctypes.data_as(dp),
                  x.size)
        return r, q

    def diagnostics(self, st: SolverState) -> dict:
        """the reference's logging quantities reduced on the GPU"""
        out = (C.c_double * 14)()
        self._ext("sbfs_diagnostics", *self._ptrs(st), C.byref(out))
        names = ["divmax", "vof_min", "vof_max", "vof_integral", "volume", "interface_area", "momentum_x",
                 "momentum_y", "energy_x", "energy_y", "umax", "vmax", "wall_stress_xm", "wall_stress_xp"]
        return dict(zip(names, list(out)))

    def logging_output(self, dirname: str, st: SolverState, step: int, time: float, dt: float, wtime: float = 0.0):
        """append the reference's monitor lines to dirname/*.dat"""
        self.lib.sbfs_logging_output.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                                 C.c_double, C.c_double, C.c_double]
        self._ext("sbfs_logging_output", dirname.encode(), *self._ptrs(st), step, time, dt, wtime)

    def statistics_collect(self, st: SolverState):
        self._ext("sbfs_statistics_collect", *self._ptrs(st))

    def statistics_reset(self):
        self._ext("sbfs_statistics_reset")

    def statistics_fetch(self, nx: int, ny: int):
        import numpy as np
        ux1 = np.zeros((ny, nx + 1))
        uy1 = np.zeros((ny, nx + 2))
        vof1 = np.zeros((ny, nx + 2))
        num = C.c_size_t(0)
        dp = C.POINTER(C.c_double)
        self._ext("sbfs_statistics_fetch", ux1.ctypes.data_as(dp), uy1.ctypes.data_as(dp),
                  vof1.ctypes.data_as(dp), C.byref(num))
        return ux1, uy1, vof1, num.value

    def measure_fp64_peak(self) -> float:
        out = C.c_double(0.0)
        self._ext("sbfs_measure_fp64_peak", C.byref(out))
        return out.value

    def set_device(self, device: int):
        self._ext("sbfs_set_device", device)

    def pin_host_state(self, st: SolverState):
        self._ext("sbfs_pin_host_state", C.addressof(st.fluid), C.addressof(st.interface))

    def unpin_host_state(self, st: SolverState):
        self._ext("sbfs_unpin_host_state", C.addressof(st.fluid), C.addressof(st.interface))

    def profile_steps(self, st: SolverState, nsteps: int) -> dict:
        """{kernel name: (total ms, launches)} of nsteps eager device-resident steps"""
        n = self.lib.sbfs_kernel_classes()
        ms = (C.c_float * n)()
        cnt = (C.c_int * n)()
        self._ext("sbfs_profile_steps", *self._ptrs(st), nsteps, ms, cnt)
        return {self.lib.sbfs_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n)}

    def kernels_per_step(self) -> int:
        return self.lib.sbfs_kernels_per_step()

    def device_status(self) -> int:
        s = C.c_int(0)
        self._ext("sbfs_device_status", C.byref(s))
        return s.value

    def release(self):
        self._ext("sbfs_release")

    # ---- batches of independent cases
    def _batch_args(self, states):
        n = len(states)
        vp = C.c_void_p * n
        d = vp(*[C.addressof(st.domain) for st in states])
        f = vp(*[C.addressof(st.fluid) for st in states])
        i = vp(*[C.addressof(st.interface) for st in states])
        return n, d, f, i

    def integrate_batch(self, states):
        """one step of every case (each with its own dt); returns the dts"""
        import numpy as np
        n, d, f, i = self._batch_args(states)
        dts = np.zeros(n)
        self.lib.sbfs_integrate_batch.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                                  C.POINTER(C.c_double)]
        self._ext("sbfs_integrate_batch", n, d, f, i, dts.ctypes.data_as(C.POINTER(C.c_double)))
        # the library swapped psi pointers inside the structs (SYNC_STATE/ALL)
        return dts

    def run_batch_steps_timed(self, nsteps: int) -> float:
        ms = C.c_float(0.0)
        self.lib.sbfs_run_batch_steps_timed.argtypes = [C.c_int, C.POINTER(C.c_float)]
        self._ext("sbfs_run_batch_steps_timed", nsteps, C.byref(ms))
        return ms.value

    def batch_sync_to_host(self, states):
        n, d, f, i = self._batch_args(states)
        self.lib.sbfs_batch_sync_to_host.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        self._ext("sbfs_batch_sync_to_host", n, d, f, i)

    def profile_batch_steps(self, nsteps: int) -> dict:
        """{kernel name: (total ms, launches)} of nsteps eager steps of the resident batch"""
        n = self.lib.sbfs_kernel_classes()
        ms = (C.c_float * n)()
        cnt = (C.c_int * n)()
        self.lib.sbfs_profile_batch_steps.argtypes = [C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int)]
        self._ext("sbfs_profile_batch_steps", nsteps, ms, cnt)
        return {self.lib.sbfs_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(n)}

    def set_autotune(self, on: bool):
        self._ext("sbfs_set_autotune", 1 if on else 0)

    def tiles(self, group: int = -1) -> dict:
        """launch shapes in use (group -1: the single-case context)"""
        bx = (C.c_int * 16)()
        by = (C.c_int * 16)()
        fw = C.c_int(0)
        mb = C.c_int(0)
        gw = C.c_int(0)
        cm = C.c_int(0)
        self.lib.sbfs_tiles.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self._ext("sbfs_tiles", group, bx, by, C.byref(fw), C.byref(mb), C.byref(gw), C.byref(cm))
        names = ["k_props", "k_curv_list", "k_flux_force", "k_vof_advance", "k_momflux", "k_predict_mf",
                 "k_correct", "k_csf_force"]
        out = {n: f"{bx[k]}x{by[k]}" for k, n in enumerate(names)}
        out["fft_cols"] = fw.value
        out["tdm_modes"] = mb.value  # 0: a cluster of four CTAs per pair
        out["tdm_warps"] = gw.value
        out["compact"] = cm.value
        return out

    def batch_groups(self):
        ng = C.c_int(0)
        cases = (C.c_int * 64)()
        self.lib.sbfs_batch_groups.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self._ext("sbfs_batch_groups", C.byref(ng), cases)
        return list(cases[:ng.value])

    def batch_release(self):
        self._ext("sbfs_batch_release")

    # ---- learned curvature closure (device pointers are plain ints)
    def _mlp(self, fn, *args):
        rc = getattr(self.lib, fn)(*args)
        if rc != 0:
            raise SolverError(f"{fn} failed: {self.lib.sbfs_mlp_last_error().decode()}")

    def _mlp_types(self):
        L = self.lib
        if getattr(L, "_mlp_typed", False):
            return
        vp, fp, dp = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_double)
        L.sbfs_mlp_last_error.restype = C.c_char_p
        L.sbfs_mlp_set_params.argtypes = [fp, C.c_int]
        L.sbfs_mlp_get_params.argtypes = [fp, C.c_int]
        L.sbfs_mlp_gradient.argtypes = [vp, vp, vp, C.c_int, fp, dp]
        L.sbfs_mlp_train_epoch.argtypes = [vp, vp, vp, C.c_int, C.c_int, C.c_float, dp]
        L.sbfs_mlp_predict.argtypes = [vp, C.c_int, vp]
        L.sbfs_mlp_take_usage.argtypes = [C.POINTER(C.c_longlong)]
        L.sbfs_set_curvature_model.argtypes = [C.c_int]
        L.sbfs_mlp_set_range.argtypes = [C.c_double, C.c_double]
        L._mlp_typed = True

    def mlp_set_params(self, params):
        import numpy as np
        self._mlp_types()
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._mlp("sbfs_mlp_set_params", p.ctypes.data_as(C.POINTER(C.c_float)), p.size)

    def mlp_get_params(self):
        import numpy as np
        self._mlp_types()
        p = np.empty(self.lib.sbfs_mlp_nparams(), dtype=np.float32)
        self._mlp("sbfs_mlp_get_params", p.ctypes.data_as(C.POINTER(C.c_float)), p.size)
        return p

    def mlp_gradient(self, X_ptr: int, Y_ptr: int, idx_ptr: int, n: int):
        """(gradient (float32, host), loss) of the mean-square error over n rows"""
        import numpy as np
        self._mlp_types()
        g = np.empty(self.lib.sbfs_mlp_nparams(), dtype=np.float32)
        loss = C.c_double(0.0)
        self._mlp("sbfs_mlp_gradient", X_ptr, Y_ptr, idx_ptr, n, g.ctypes.data_as(C.POINTER(C.c_float)),
                  C.byref(loss))
        return g, loss.value

    def mlp_train_epoch(self, X_ptr: int, Y_ptr: int, idx_ptr: int, n: int, batch: int, lr: float) -> float:
        self._mlp_types()
        loss = C.c_double(0.0)
        self._mlp("sbfs_mlp_train_epoch", X_ptr, Y_ptr, idx_ptr, n, batch, lr, C.byref(loss))
        return loss.value

    def mlp_predict(self, X_ptr: int, n: int, out_ptr: int):
        self._mlp_types()
        self._mlp("sbfs_mlp_predict", X_ptr, n, out_ptr)

    def mlp_take_usage(self) -> int:
        self._mlp_types()
        u = C.c_longlong(0)
        self._mlp("sbfs_mlp_take_usage", C.byref(u))
        return u.value

    def mlp_set_range(self, lo: float, hi: float):
        """the closure's range in |kappa dx| (default 1/128 .. 0.5)"""
        self._mlp_types()
        self._mlp("sbfs_mlp_set_range", lo, hi)

    def set_curvature_model(self, model: int):
        """0: the reference's kappa = -div n; 1: the learned closure"""
        self._mlp_types()
        self._ext("sbfs_set_curvature_model", model)


def load_library(path: str | None = None, build_if_missing: bool = False) -> GpuLibrary:
    """Load libsbfs_gb300.so (built in-tree by :func:`build_library`)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIBRARY_PATH
    if not os.path.exists(p):
        if build_if_missing:
            build_library()
        else:
            raise RuntimeError(f"{p} is missing: build it with `python -m simplebubblyflowsolver_gb300.build`")
    lib = GpuLibrary(C.CDLL(p))
    if path is None:
        _LIB = lib
    return lib
