"""CPU checkers for the CUDA library -- TEST INFRASTRUCTURE ONLY.

* ``liboracle.so``: the project's C restatement of the reference time step
  (exported with an ``orc_`` prefix).
* ``_ref/libsbfs_ref.so``: the reference's own time-step sources built against
  single-rank stand-ins for MPI, SimpleDecomp and FFTW (only where the
  reference sources were available at build time).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package, and only to check or to time the CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

from simplebubblyflowsolver_gb300.binding import ReferenceAPI

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
ORACLE_FMA_SO = os.path.join(HERE, "liboracle_fma.so")
REF_SO = os.path.join(HERE, "_ref", "libsbfs_ref.so")


STAGED = os.path.join(HERE, "_ref", "src")


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """compile liboracle.so, and _ref/libsbfs_ref.so: from ref_dir when it
    holds the reference checkout (whose sources are then also staged into
    _ref/src, git-ignored, so that a machine without the checkout can build
    the same library), else from a staged copy when there is one"""
    out = subprocess.DEVNULL if quiet else None
    err = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "liboracle.so", "liboracle_fma.so"], check=True, stdout=out)
    if ref_dir and os.path.isdir(os.path.join(ref_dir, "src")):
        ref_dir = os.path.abspath(ref_dir)
        subprocess.run(["make", "-C", HERE, "ref", f"REF={ref_dir}"], check=True, stdout=out, stderr=err)
        subprocess.run(["make", "-C", HERE, "stage", f"REF={ref_dir}"], check=True, stdout=out, stderr=err)
    elif os.path.isdir(os.path.join(STAGED, "src")):
        subprocess.run(["make", "-C", HERE, "ref", f"REF={STAGED}"], check=True, stdout=out, stderr=err)


class Oracle(ReferenceAPI):
    """variant "fma": the same sources built with fused multiply-add
    contraction (a second build that differs only in rounding)"""

    def __init__(self, variant: str = ""):
        path = ORACLE_FMA_SO if variant == "fma" else ORACLE_SO
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        super().__init__(lib, prefix="orc_", name="oracle")
        lib.orc_set_dt_coefs.argtypes = [C.c_double] * 3
        lib.orc_set_threads.argtypes = [C.c_int]
        lib.orc_get_threads.restype = C.c_int
        lib.orc_max_divergence.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
        lib.orc_vof_stats.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double * 4)]
        lib.orc_diagnostics.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double * 16)]

    def set_dt_coefs(self, adv, dif, itf):
        self.lib.orc_set_dt_coefs(adv, dif, itf)

    def set_threads(self, n):
        self.lib.orc_set_threads(int(n))

    def threads(self):
        return self.lib.orc_get_threads()

    def max_divergence(self, st):
        out = C.c_double(0.0)
        self.lib.orc_max_divergence(C.addressof(st.domain), C.addressof(st.fluid), C.byref(out))
        return out.value

    def diagnostics(self, st) -> dict:
        out = (C.c_double * 16)()
        self.lib.orc_diagnostics(*self._ptrs(st), C.byref(out))
        return diag_dict(list(out))

    def vof_stats(self, st):
        out = (C.c_double * 4)()
        self.lib.orc_vof_stats(C.addressof(st.domain), C.addressof(st.interface), C.byref(out))
        return tuple(out)


DIAG_NAMES = ["divmax", "vof_min", "vof_max", "vof_integral", "volume", "interface_area", "momentum_x",
              "momentum_y", "energy_x", "energy_y", "umax", "vmax", "wall_stress_xm", "wall_stress_xp"]


def diag_dict(vals) -> dict:
    return dict(zip(DIAG_NAMES, vals))


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class RefShim(ReferenceAPI):
    """The reference's own sources (one grid per process: they keep
    function-static solver state; its statistics accumulate across cases)."""

    def __init__(self):
        lib = C.CDLL(REF_SO)
        super().__init__(lib, prefix="", name="reference")
        lib.sbfs_refshim_info.restype = C.c_void_p
        P = C.c_void_p
        lib.sbfs_refshim_log.argtypes = [P, C.c_size_t, C.c_double, C.c_double, C.c_double, P, P]
        lib.sbfs_refshim_stats_init.argtypes = [P, C.c_double]
        lib.sbfs_refshim_stats_collect.argtypes = [P, P, P]
        lib.sbfs_refshim_stats_output.argtypes = [P, C.c_size_t]
        for fn in ("domain_init", "domain_save"):
            getattr(lib, fn).argtypes = [C.c_char_p, P]
        for fn in ("fluid_init", "fluid_save", "interface_init", "interface_save"):
            getattr(lib, fn).argtypes = [C.c_char_p, P, P]

    def info(self):
        return self.lib.sbfs_refshim_info()

    # the reference's logging and statistics (src/logging/, src/statistics.c);
    # they write under output/ of the current directory, as the reference does
    def log(self, st, step, time, dt, wtime):
        d, f, i = self._ptrs(st)
        self.lib.sbfs_refshim_log(d, step, time, dt, wtime, f, i)

    def stats_init(self, st, time):
        if self.lib.sbfs_refshim_stats_init(C.addressof(st.domain), time):
            raise RuntimeError("reference statistics.init failed (stat_rate / stat_after unset?)")

    def stats_collect(self, st):
        d, f, i = self._ptrs(st)
        self.lib.sbfs_refshim_stats_collect(d, f, i)

    def stats_output(self, st, step):
        if self.lib.sbfs_refshim_stats_output(C.addressof(st.domain), step):
            raise RuntimeError("reference statistics.output failed")
