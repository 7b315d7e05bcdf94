"""Grid sizes at the edges of what the library accepts, against the oracle:
ny at its minimum (8) and maximum (8192, one transform column per block),
nx at its maximum (8192: the tridiagonal systems of a wavenumber pair exceed
shared memory and are staged in global memory; 4 warps per system), nx that no
block shape divides, and chunked systems padded past nx (200 x 16)."""
import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE, ic

from ._helpers import clone, compare_state, fma_noise_floor, new_state, rounding_sensitivity, set_env

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    return load_library(), oracle.Oracle()


def square_cells(nx, ny, We):
    """one disc in a domain of square cells, the shorter side at least 0.5"""
    h = max(2.0 / nx, 0.5 / ny)
    lx, ly = nx * h, ny * h
    r = min(0.25, 0.3 * ly, 0.3 * lx)
    return ic.Workload("edge", nx, ny, lx, ly, [(min(0.5, lx / 2), ly / 2, r)],
                       Re=35.0, We=We, Fr=1.0, denr=0.1, visr=0.1)


def bubble(nx, ny, We):
    wl = ic.single_bubble(nx, ny)
    wl.We = We
    return wl


# (nx, ny, domain, We, steps).  Each case is one where both rounding floors
# below stay small (at most 1.4e-7).  Near some states the reference's
# algorithm turns rounding into O(1) changes: corner normals in the THINC
# tails are a rounding-noise gradient normalised by max(|grad|, DBL_EPSILON),
# and the curvature takes them without a vof cut-off.  A 1e-15 change of the
# initial vof then moves the velocity by tens of percent (nx = 100 here), or
# two roundings part by 1e-9 in one step once a noisy tail cell borders the
# interface (a bubble of radius 0.25 at dx = 1/64, in the third step: the
# oracle built with FMA contraction parts from itself there as well).  Such a
# state is no parity case.  At nx = 8192 the floors grow by orders of
# magnitude a step after the second, so that case runs two steps.
CASES = [
    (64, 8, bubble, 10.0, 5),            # min ny
    (8192, 8, bubble, 10.0, 2),          # max nx: global staging, 4 warps, 64 rows a lane
    (37, 64, bubble, 10.0, 5),           # odd nx, ragged blocks of every shape
    (200, 16, bubble, 10.0, 5),          # 2 warps, 4 rows a lane, 56 padding rows
    (256, 512, square_cells, 10.0, 5),   # a tall domain, 129 wavenumber pairs
    (32, 4096, square_cells, 100.0, 5),  # two transform columns per block
    (32, 8192, square_cells, 100.0, 5),  # max ny: one transform column per block
]


@pytest.mark.parametrize("nx,ny,domain,We,steps", CASES, ids=[f"{c[0]}x{c[1]}" for c in CASES])
def test_edge_size_matches_oracle(libs, nx, ny, domain, We, steps):
    gpu, orc = libs
    wl = domain(nx, ny, We)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    for _ in range(steps):
        da = gpu.integrate(a)
        db = orc.integrate(b)
        assert abs(da - db) <= 1e-10 * db
    errs = compare_state(a, b)
    # 1e-10, or where the flow amplifies rounding beyond it ten times the
    # larger of the spread between two faithful CPU builds and the oracle's
    # own response to a few-ulp perturbation of the initial interface
    tol = 1e-10
    if max(errs.values()) > tol:
        floor = max(max(fma_noise_floor(wl, steps).values()), max(rounding_sensitivity(wl, steps).values()))
        tol = max(tol, 10 * floor)
    print((nx, ny), {k: f"{v:.1e}" for k, v in errs.items()}, "tol", tol)
    assert max(errs.values()) <= tol, (errs, tol)
