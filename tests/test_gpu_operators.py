"""Per-operator parity of the CUDA library with the CPU oracle, through the
reference's C entry points (fine-grained path: host arrays in, host arrays
out).  Tolerances are relative to the largest magnitude of each field."""
import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import RK_GAMMA, ic

from ._helpers import clone, demean, new_state, rel_err, set_env

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def libs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    return load_library(), oracle.Oracle()


@pytest.fixture(scope="module", params=[(64, 32), (48, 16)], ids=["64x32", "48x16"])
def mid(libs, request):
    """a state 6 steps into a rising-bubble run, with every array of the
    first substage's operators filled (by the oracle)"""
    gpu, orc = libs
    nx, ny = request.param
    wl = ic.single_bubble(nx, ny)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st = new_state(wl, orc)
    for _ in range(6):
        orc.integrate(st)
    dt = orc.decide_dt(st)
    orc.compute_density(st, 0)
    orc.compute_viscosity(st)
    orc.compute_curvature_tensor(st)
    orc.compute_force(st)
    orc.update_vof(st, 0, dt)
    orc.compute_density(st, 1)
    orc.compute_mass_flux(st)
    orc.predict_field(st, 0, dt)
    return st, dt


def run_both(libs, st, fn):
    gpu, orc = libs
    a, b = clone(st), clone(st)
    ra = fn(gpu, a)
    rb = fn(orc, b)
    return a, b, ra, rb


def check(a, b, slots, tol=TOL):
    errs = {s: rel_err(a.field(s), b.field(s)) for s in slots}
    bad = {s: e for s, e in errs.items() if not e <= tol}
    assert not bad, f"fields over tolerance {tol}: {bad}"


def test_decide_dt(libs, mid):
    st, _ = mid
    a, b, da, db = run_both(libs, st, lambda L, s: L.decide_dt(s))
    assert abs(da - db) <= 2e-16 * db


@pytest.mark.parametrize("index", [0, 1])
def test_density(libs, mid, index):
    st, _ = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_density(s, index))
    check(a, b, [f"den{index}"])


def test_viscosity(libs, mid):
    st, _ = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_viscosity(s))
    check(a, b, ["visux", "visuy"])


def test_curvature_tensor(libs, mid):
    st, _ = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_curvature_tensor(s))
    check(a, b, ["dvof", "normal", "curv"])


def test_force(libs, mid):
    st, _ = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_force(s))
    check(a, b, ["ifrcx", "ifrcy"])


@pytest.mark.parametrize("rk", [0, 1, 2])
def test_update_vof(libs, mid, rk):
    st, dt = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.update_vof(s, rk, dt))
    check(a, b, ["fluxx", "fluxy", "src0", "src1", "vof"])


def test_mass_flux(libs, mid):
    st, _ = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_mass_flux(s))
    check(a, b, ["fluxx", "fluxy"])


@pytest.mark.parametrize("rk", [0, 1, 2])
def test_predict(libs, mid, rk):
    st, dt = mid
    a, b, _, _ = run_both(libs, st, lambda L, s: L.predict_field(s, rk, dt))
    check(a, b, ["ux", "uy", "txx", "txy", "tyy", "srcux0", "srcux1", "srcux2", "srcuy0", "srcuy1", "srcuy2"])


@pytest.mark.parametrize("rk", [0, 1, 2])
def test_potential(libs, mid, rk):
    st, dt = mid
    dt_old, dt_new = RK_GAMMA[(rk + 2) % 3] * dt, RK_GAMMA[rk] * dt
    a, b, _, _ = run_both(libs, st, lambda L, s: L.compute_potential(s, dt_old, dt_new))
    pa, pb = a.interior_rows("psi1")[:, 1:-1], b.interior_rows("psi1")[:, 1:-1]
    assert rel_err(demean(pa), demean(pb)) < 1e-11
    # Neumann ghost columns
    for s in (a,):
        f = s.interior_rows("psi1")
        assert np.array_equal(f[:, 0], f[:, 1]) and np.array_equal(f[:, -1], f[:, -2])


def test_correct_velocity(libs, mid):
    st, dt = mid
    dt_old, dt_new = RK_GAMMA[2] * dt, RK_GAMMA[0] * dt
    st = clone(st)
    libs[1].compute_potential(st, dt_old, dt_new)
    a, b, _, _ = run_both(libs, st, lambda L, s: L.correct_velocity(s, dt_old, dt_new))
    check(a, b, ["ux", "uy"])


def test_update_pressure(libs, mid):
    st, dt = mid
    st = clone(st)
    libs[1].compute_potential(st, RK_GAMMA[2] * dt, RK_GAMMA[0] * dt)
    a, b, _, _ = run_both(libs, st, lambda L, s: L.update_pressure(s))
    check(a, b, ["p", "psi0", "psi1"], tol=0.0)


@pytest.mark.parametrize("slot", ["ux", "uy", "p", "psi0", "vof"])
def test_boundaries(libs, mid, slot):
    st, _ = mid
    st = clone(st)
    rng = np.random.default_rng(3)
    st.field(slot)[...] = rng.standard_normal(st.field(slot).shape)
    a, b, _, _ = run_both(libs, st, lambda L, s: L.update_boundaries(s, slot))
    check(a, b, [slot], tol=0.0)


def test_substage_sequence(libs, mid):
    """one full RK3 step operator by operator through the fine-grained ABI"""
    st, _ = mid
    gpu, orc = libs

    def step(L, s):
        dt = L.decide_dt(s)
        for k in range(3):
            L.substage(s, k, dt)
        return dt

    a, b, da, db = run_both(libs, st, step)
    for s in ("ux", "uy", "vof"):
        assert rel_err(a.interior_rows(s), b.interior_rows(s)) < 1e-11, s
