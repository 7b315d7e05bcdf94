"""Shared test helpers: building states, running the checkers, comparing."""
from __future__ import annotations

import copy
import os

import numpy as np

from simplebubblyflowsolver_gb300 import ic
from simplebubblyflowsolver_gb300.binding import state_from_fields

STATE = ("ux", "uy", "p", "psi0", "vof")


def set_env(wl):
    for k, v in wl.env().items():
        os.environ[k] = v


def new_state(wl, backend, fields=None):
    fields = fields if fields is not None else wl.fields()
    st = state_from_fields(fields, Re=wl.Re, We=wl.We, Fr=wl.Fr, denr=wl.denr, visr=wl.visr)
    backend.apply_initial_boundaries(st)
    return st


def clone(st):
    """deep copy of a SolverState (fresh buffers, same values and swaps)"""
    from simplebubblyflowsolver_gb300._abi import SolverState
    new = SolverState(st.nx, st.ny, st.lx, st.ly, xf=st.xf, xc=st.xc, Re=st.fluid.Re, Fr=st.fluid.Fr,
                      denr=st.fluid.denr, visr=st.fluid.visr, We=st.interface.We)
    for s in st.slots():
        new.field(s)[...] = st.field(s)
    return new


def rel_err(a, b):
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(a - b).max()) / scale


def demean(a):
    return a - a.mean()


def compare_state(sa, sb, slots=STATE):
    """relative max errors per field; p and psi compared without their mean
    (the potential is defined up to a constant, the reference leaves one)"""
    out = {}
    for s in slots:
        a, b = sa.interior_rows(s), sb.interior_rows(s)
        if s in ("p", "psi0", "psi1"):
            a, b = demean(a[:, 1:-1]), demean(b[:, 1:-1])
        out[s] = rel_err(a, b)
    return out


def fma_noise_floor(wl, steps, slots=STATE):
    """spread between the oracle built as is and the oracle built with fused
    multiply-add contraction (liboracle_fma.so): two faithful builds of the
    same algorithm that differ only in rounding.  A second implementation is
    held to a small multiple of this floor where the flow amplifies rounding
    beyond the 1e-10 bar."""
    import oracle
    a_lib, b_lib = oracle.Oracle(), oracle.Oracle(variant="fma")
    for lib in (a_lib, b_lib):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    set_env(wl)
    a, b = new_state(wl, a_lib), new_state(wl, b_lib)
    for _ in range(steps):
        a_lib.integrate(a)
        b_lib.integrate(b)
    return compare_state(a, b, slots)


def rounding_sensitivity(wl, steps, eps=1e-15, seed=0, slots=STATE):
    """spread of the oracle's own solution after `steps` steps when the
    initial vof of the interface cells is perturbed by a relative eps (a few
    ulps): how far rounding-level differences in the input carry.  Cases
    with strong surface tension amplify them through the THINC tails, where
    the normalised corner normals are rounding noise."""
    import oracle
    lib = oracle.Oracle()
    lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    set_env(wl)
    a = new_state(wl, lib)
    fields = wl.fields()
    vof = fields["vof"]
    rng = np.random.default_rng(seed)
    itf = (vof > 0) & (vof < 1)
    vof[itf] = np.clip(vof[itf] * (1 + eps * rng.uniform(-1, 1, int(itf.sum()))), 0.0, 1.0)
    b = new_state(wl, lib, fields)
    for _ in range(steps):
        lib.integrate(a)
        lib.integrate(b)
    return compare_state(a, b, slots)
