"""ctypes binding of the SimpleBubblyFlowSolver C entry points.

The signatures are those of the reference headers include/integrate.h:5-10,
include/decide_dt.h:5-10, include/fluid_solver.h:10-89 and
include/interface_solver.h:8-48; every entry point returns 0 on success and
non-zero on failure.  :class:`ReferenceAPI` binds them from any shared library
that exports them under an optional name prefix, so the CUDA library and the
CPU checkers are driven by the same code.
"""
from __future__ import annotations

import ctypes as C

from ._abi import ArrayT, SolverState

P = C.c_void_p
SZ = C.c_size_t
D = C.c_double

SIGNATURES = {
    "integrate": [P, P, P, C.POINTER(D)],
    "decide_dt": [P, P, P, C.POINTER(D)],
    "fluid_compute_density": [P, P, P, SZ],
    "fluid_compute_viscosity": [P, P, P],
    "fluid_predict_field": [P, SZ, D, P, P],
    "fluid_compute_potential": [P, D, D, P],
    "fluid_correct_velocity": [P, D, D, P],
    "fluid_update_pressure": [P, P],
    "fluid_update_boundaries_ux": [P, P],
    "fluid_update_boundaries_uy": [P, P],
    "fluid_update_boundaries_p": [P, P],
    "fluid_update_boundaries_psi": [P, P],
    "interface_compute_curvature_tensor": [P, P],
    "interface_compute_force": [P, P, P],
    "interface_compute_mass_flux": [P, P, P],
    "interface_update_vof": [P, SZ, D, P, P],
    "interface_update_boundaries_vof": [P, P],
}

# RK3 coefficients (reference src/runge_kutta.c:8-15)
RK_ALPHA = (32.0 / 60.0, 25.0 / 60.0, 45.0 / 60.0)
RK_BETA = (0.0 / 60.0, -17.0 / 60.0, -25.0 / 60.0)
RK_GAMMA = tuple(a + b for a, b in zip(RK_ALPHA, RK_BETA))


class SolverError(RuntimeError):
    pass


class ReferenceAPI:
    """The reference's C entry points bound from `lib` (a ctypes.CDLL)."""

    def __init__(self, lib: C.CDLL, prefix: str = "", name: str = "library"):
        self.lib = lib
        self.prefix = prefix
        self.name = name
        self._fns = {}
        for fn, argtypes in SIGNATURES.items():
            f = getattr(lib, prefix + fn)
            f.argtypes = argtypes
            f.restype = C.c_int
            self._fns[fn] = f

    def _call(self, fn, *args):
        rc = self._fns[fn](*args)
        if rc != 0:
            raise SolverError(f"{self.name}: {fn} returned {rc}")
        return rc

    @staticmethod
    def _ptrs(st: SolverState):
        return (C.addressof(st.domain), C.addressof(st.fluid), C.addressof(st.interface))

    @staticmethod
    def _arr(a: ArrayT):
        return C.addressof(a)

    # ---- the reference's operators, one call each
    def integrate(self, st: SolverState) -> float:
        d, f, i = self._ptrs(st)
        dt = D(0.0)
        self._call("integrate", d, f, i, C.byref(dt))
        return dt.value

    def decide_dt(self, st: SolverState) -> float:
        d, f, i = self._ptrs(st)
        dt = D(0.0)
        self._call("decide_dt", d, f, i, C.byref(dt))
        return dt.value

    def compute_density(self, st, index):
        d, f, i = self._ptrs(st)
        self._call("fluid_compute_density", d, f, i, index)

    def compute_viscosity(self, st):
        d, f, i = self._ptrs(st)
        self._call("fluid_compute_viscosity", d, f, i)

    def compute_curvature_tensor(self, st):
        d, _, i = self._ptrs(st)
        self._call("interface_compute_curvature_tensor", d, i)

    def compute_force(self, st):
        d, f, i = self._ptrs(st)
        self._call("interface_compute_force", d, f, i)

    def update_vof(self, st, rkstep, dt):
        d, f, i = self._ptrs(st)
        self._call("interface_update_vof", d, rkstep, dt, f, i)

    def compute_mass_flux(self, st):
        d, f, i = self._ptrs(st)
        self._call("interface_compute_mass_flux", d, f, i)

    def predict_field(self, st, rkstep, dt):
        d, f, i = self._ptrs(st)
        self._call("fluid_predict_field", d, rkstep, dt, f, i)

    def compute_potential(self, st, dt_old, dt_new):
        d, f, _ = self._ptrs(st)
        self._call("fluid_compute_potential", d, dt_old, dt_new, f)

    def correct_velocity(self, st, dt_old, dt_new):
        d, f, _ = self._ptrs(st)
        self._call("fluid_correct_velocity", d, dt_old, dt_new, f)

    def update_pressure(self, st):
        d, f, _ = self._ptrs(st)
        self._call("fluid_update_pressure", d, f)

    def update_boundaries(self, st, slot):
        d = C.addressof(st.domain)
        fn = {"ux": "fluid_update_boundaries_ux", "uy": "fluid_update_boundaries_uy",
              "p": "fluid_update_boundaries_p", "psi0": "fluid_update_boundaries_psi",
              "psi1": "fluid_update_boundaries_psi", "vof": "interface_update_boundaries_vof"}[slot]
        self._call(fn, d, self._arr(st._array_t(slot)))

    def apply_initial_boundaries(self, st):
        """what fluid_init / interface_init do after loading the fields
        (reference src/fluid/init.c:97-100, src/interface/init.c:64)"""
        for s in ("ux", "uy", "p", "psi0", "vof"):
            self.update_boundaries(st, s)

    def substage(self, st, rkstep, dt):
        """one RK substage, operator by operator (reference src/integrate.c:23-66)"""
        self.compute_density(st, 0)
        self.compute_viscosity(st)
        self.compute_curvature_tensor(st)
        self.compute_force(st)
        self.update_vof(st, rkstep, dt)
        self.compute_density(st, 1)
        self.compute_mass_flux(st)
        self.predict_field(st, rkstep, dt)
        dt_old = RK_GAMMA[(rkstep + 2) % 3] * dt
        dt_new = RK_GAMMA[rkstep] * dt
        self.compute_potential(st, dt_old, dt_new)
        self.correct_velocity(st, dt_old, dt_new)
        self.update_pressure(st)


def state_from_fields(fields: dict, *, Re, We, Fr, denr, visr, info=None) -> SolverState:
    """SolverState holding an initial condition in the reference .npy schema
    (boundaries not yet applied)."""
    nx, ny = (int(v) for v in fields["glsizes"])
    lx, ly = (float(v) for v in fields["lengths"])
    st = SolverState(nx, ny, lx, ly, xf=fields["xf"], xc=fields["xc"], Re=Re, Fr=Fr,
                     denr=denr, visr=visr, We=We, info=info)
    for k in ("ux", "uy", "p", "vof"):
        st.set_rows(k, fields[k])
    st.set_rows("psi0", fields["psi"])
    return st
