"""ctypes mirror of the SimpleBubblyFlowSolver C data structures.

The layouts follow the reference headers (include/array.h:10-23,
include/domain.h:20-30, include/fluid.h:27-45, include/interface.h:13-24) and
this package's include/sbfs_types.h.  :class:`SolverState` owns numpy buffers
for every field with the reference's ghost widths
(include/array_macros/**), so the same state can be handed to the CUDA
library, the CPU oracle or the reference build, all through one C ABI.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

NDIMS = 2

# extra cells [dim][lower, upper] of every field (reference include/array_macros)
NADDS = {
    "ux": ((0, 1), (1, 1)),
    "uy": ((1, 1), (1, 1)),
    "p": ((1, 1), (1, 1)),
    "psi": ((1, 1), (1, 1)),
    "den": ((1, 1), (1, 1)),
    "visux": ((0, 1), (1, 1)),
    "visuy": ((1, 1), (1, 1)),
    "txx": ((0, 0), (1, 1)),
    "txy": ((0, 1), (1, 1)),
    "tyy": ((0, 0), (1, 1)),
    "srcux": ((-1, 0), (0, 0)),
    "srcuy": ((0, 0), (0, 0)),
    "vof": ((1, 1), (2, 2)),
    "ifrcx": ((-1, 0), (0, 0)),
    "ifrcy": ((0, 0), (0, 0)),
    "dvof": ((0, 1), (1, 2)),
    "normal": ((0, 0), (1, 1)),
    "curv": ((1, 1), (1, 1)),
    "fluxx": ((0, 1), (1, 1)),
    "fluxy": ((1, 1), (1, 1)),
    "src": ((0, 0), (0, 0)),
}
# components per element
NCOMP = {"dvof": 2, "normal": 3}


class ArrayT(C.Structure):
    _fields_ = [
        ("size", C.c_size_t),
        ("nadds", C.POINTER(C.c_int * 2)),
        ("datasize", C.c_size_t),
        ("data", C.c_void_p),
    ]


class DomainT(C.Structure):
    _fields_ = [
        ("info", C.c_void_p),
        ("glsizes", C.c_size_t * NDIMS),
        ("mysizes", C.c_size_t * NDIMS),
        ("offsets", C.c_size_t * NDIMS),
        ("lengths", C.c_double * NDIMS),
        ("xf", C.POINTER(C.c_double)),
        ("xc", C.POINTER(C.c_double)),
        ("jdxf", C.POINTER(C.c_double)),
        ("jdxc", C.POINTER(C.c_double)),
        ("hxxf", C.POINTER(C.c_double)),
        ("hxxc", C.POINTER(C.c_double)),
        ("hy", C.c_double),
    ]


class FluidT(C.Structure):
    _fields_ = [
        ("ux", ArrayT),
        ("uy", ArrayT),
        ("p", ArrayT),
        ("psi", ArrayT * 2),
        ("den", ArrayT * 2),
        ("visux", ArrayT),
        ("visuy", ArrayT),
        ("txx", ArrayT),
        ("txy", ArrayT),
        ("tyy", ArrayT),
        ("srcux", ArrayT * 3),
        ("srcuy", ArrayT * 3),
        ("Re", C.c_double),
        ("Fr", C.c_double),
        ("denr", C.c_double),
        ("visr", C.c_double),
        ("refden", C.c_double),
    ]


class InterfaceT(C.Structure):
    _fields_ = [
        ("vof", ArrayT),
        ("ifrcx", ArrayT),
        ("ifrcy", ArrayT),
        ("dvof", ArrayT),
        ("normal", ArrayT),
        ("curv", ArrayT),
        ("fluxx", ArrayT),
        ("fluxy", ArrayT),
        ("src", ArrayT * 2),
        ("We", C.c_double),
    ]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def field_shape(name: str, nx: int, ny: int) -> tuple:
    """numpy shape (rows incl. y ghosts, cols incl. x ghosts[, comps])."""
    (ax0, ax1), (ay0, ay1) = NADDS[name]
    shape = (ny + ay0 + ay1, nx + ax0 + ax1)
    nc = NCOMP.get(name, 1)
    return shape + ((nc,) if nc > 1 else ())


# (struct attribute, slot index or None, NADDS key) for every array_t
FLUID_SLOTS = [
    ("ux", None, "ux"), ("uy", None, "uy"), ("p", None, "p"),
    ("psi", 0, "psi"), ("psi", 1, "psi"), ("den", 0, "den"), ("den", 1, "den"),
    ("visux", None, "visux"), ("visuy", None, "visuy"),
    ("txx", None, "txx"), ("txy", None, "txy"), ("tyy", None, "tyy"),
    ("srcux", 0, "srcux"), ("srcux", 1, "srcux"), ("srcux", 2, "srcux"),
    ("srcuy", 0, "srcuy"), ("srcuy", 1, "srcuy"), ("srcuy", 2, "srcuy"),
]
INTERFACE_SLOTS = [
    ("vof", None, "vof"), ("ifrcx", None, "ifrcx"), ("ifrcy", None, "ifrcy"),
    ("dvof", None, "dvof"), ("normal", None, "normal"), ("curv", None, "curv"),
    ("fluxx", None, "fluxx"), ("fluxy", None, "fluxy"),
    ("src", 0, "src"), ("src", 1, "src"),
]


def slot_name(attr: str, idx) -> str:
    return attr if idx is None else f"{attr}{idx}"


class SolverState:
    """Host-side state of one case: domain_t, fluid_t and interface_t whose
    array_t buffers are numpy arrays owned by this object.

    Fields are addressed by slot name ("ux", "psi0", "srcux2", "vof", ...).
    Libraries may swap array_t.data pointers (as the reference does for the
    RK sources and the potentials); :meth:`field` always returns the buffer
    a slot currently points at.
    """

    def __init__(self, nx: int, ny: int, lx: float, ly: float, *, xf=None, xc=None,
                 Re=35.0, Fr=1.0, denr=0.1, visr=0.1, We=10.0, info=None):
        self.nx, self.ny = int(nx), int(ny)
        self.lx, self.ly = float(lx), float(ly)
        if xf is None:
            xf = np.linspace(0.0, lx, nx + 1, endpoint=True)
        if xc is None:
            xc = np.concatenate(([0.0], 0.5 * xf[:-1] + 0.5 * xf[1:], [lx]))
        self.xf = np.ascontiguousarray(xf, dtype=np.float64)
        self.xc = np.ascontiguousarray(xc, dtype=np.float64)
        # scale factors and Jacobians (reference src/domain.c:90-144)
        self.hy = ly / ny
        self.hxxf = np.array([self.xc[i] - self.xc[i - 1] for i in range(1, nx + 2)])
        self.hxxc = np.array([self.xf[i] - self.xf[i - 1] for i in range(1, nx + 1)])
        self.jdxf = self.hxxf * self.hy
        self.jdxc = self.hxxc * self.hy
        d = DomainT()
        d.info = info
        d.glsizes[:] = (nx, ny)
        d.mysizes[:] = (nx, ny)
        d.offsets[:] = (0, 0)
        d.lengths[:] = (lx, ly)
        d.xf, d.xc = _dp(self.xf), _dp(self.xc)
        d.jdxf, d.jdxc = _dp(self.jdxf), _dp(self.jdxc)
        d.hxxf, d.hxxc = _dp(self.hxxf), _dp(self.hxxc)
        d.hy = self.hy
        self.domain = d
        self.fluid = FluidT()
        self.interface = InterfaceT()
        self._buffers = {}      # id(buffer) -> ndarray
        self._nadds = []        # keep nadds arrays alive
        for attr, idx, key in FLUID_SLOTS:
            self._alloc(self.fluid, attr, idx, key)
        for attr, idx, key in INTERFACE_SLOTS:
            self._alloc(self.interface, attr, idx, key)
        self.fluid.Re, self.fluid.Fr = Re, Fr
        self.fluid.denr, self.fluid.visr = denr, visr
        self.fluid.refden = min(1.0, denr)
        self.interface.We = We

    def _alloc(self, struct, attr, idx, key):
        shape = field_shape(key, self.nx, self.ny)
        buf = np.zeros(shape, dtype=np.float64)
        na = (C.c_int * 2 * 2)()
        (ax0, ax1), (ay0, ay1) = NADDS[key]
        na[0][0], na[0][1], na[1][0], na[1][1] = ax0, ax1, ay0, ay1
        self._nadds.append(na)
        arr = getattr(struct, attr) if idx is None else getattr(struct, attr)[idx]
        arr.size = 8 * NCOMP.get(key, 1)
        arr.nadds = C.cast(na, C.POINTER(C.c_int * 2))
        arr.datasize = buf.nbytes
        arr.data = buf.ctypes.data
        self._buffers[buf.ctypes.data] = buf

    def _array_t(self, slot: str):
        for struct, slots in ((self.fluid, FLUID_SLOTS), (self.interface, INTERFACE_SLOTS)):
            for attr, idx, _ in slots:
                if slot_name(attr, idx) == slot:
                    return getattr(struct, attr) if idx is None else getattr(struct, attr)[idx]
        raise KeyError(slot)

    def field(self, slot: str) -> np.ndarray:
        """numpy view of the buffer slot `slot` currently points at."""
        return self._buffers[self._array_t(slot).data]

    def slots(self):
        return [slot_name(a, i) for a, i, _ in FLUID_SLOTS + INTERFACE_SLOTS]

    # ---- state in the reference's .npy schema (x-ghost-inclusive, no y ghosts)
    def interior_rows(self, slot: str) -> np.ndarray:
        key = slot.rstrip("012") if slot[-1].isdigit() else slot
        ay0 = NADDS[key][1][0]
        return self.field(slot)[ay0:ay0 + self.ny]

    def set_rows(self, slot: str, values: np.ndarray):
        self.interior_rows(slot)[...] = values

    def copy_fields_from(self, other: "SolverState", slots=None):
        for s in slots or self.slots():
            self.field(s)[...] = other.field(s)

    def snapshot(self, slots=None) -> dict:
        return {s: self.field(s).copy() for s in (slots or self.slots())}

    def pointers(self):
        return C.byref(self.domain), C.byref(self.fluid), C.byref(self.interface)
