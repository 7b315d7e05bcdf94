"""Host-linked steps (strict sync mode): the step's own kernels read the
caller's host arrays and write the results back, overlapped with the step.
Every host array must end exactly as after the cudaMemcpy path, ghost rows
included."""
import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import SYNC_STATE, ic

from ._helpers import clone, new_state, set_env

pytestmark = pytest.mark.gpu

HOST_SLOTS = ("ux", "uy", "p", "psi0", "psi1", "vof")


@pytest.fixture(scope="module")
def libs():
    import oracle
    from simplebubblyflowsolver_gb300 import load_library
    return load_library(), oracle.Oracle()


def run(gpu, st, steps, link, graphs):
    gpu.set_host_link(link)
    gpu.set_use_graphs(graphs)
    dts, used = [], []
    try:
        for _ in range(steps):
            dts.append(gpu.integrate(st))
            used.append(gpu.host_link_used())
    finally:
        gpu.set_host_link(True)
        gpu.set_use_graphs(True)
    return dts, used


@pytest.mark.parametrize("graphs", [True, False], ids=["graph", "eager"])
@pytest.mark.parametrize("grid", [(256, 128), (130, 64)], ids=["256x128", "130x64"])
def test_host_linked_equals_memcpy(libs, grid, graphs):
    gpu, orc = libs
    nx, ny = grid
    wl = ic.bubble_swarm(nx, ny, nbubbles=6, seed=3)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    # poison the ghost rows of the outputs: the step must write them
    for st in (a, b):
        for s in HOST_SLOTS:
            st.field(s)[0] = np.nan
            st.field(s)[-1] = np.nan
    dta, used_a = run(gpu, a, 4, True, graphs)
    dtb, used_b = run(gpu, b, 4, False, graphs)
    assert all(used_a), "the GPU could not address the host arrays"
    assert not any(used_b)
    assert dta == dtb
    for s in HOST_SLOTS:
        fa, fb = a.field(s), b.field(s)
        assert np.array_equal(fa, fb), s
        assert np.isfinite(fa).all(), s


def test_host_linked_follows_host_changes(libs):
    """a strict-mode step starts from what the host arrays hold at the call"""
    gpu, orc = libs
    wl = ic.single_bubble(128, 64)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    run(gpu, a, 1, True, True)
    run(gpu, b, 1, False, True)
    # the caller edits its arrays between steps: both paths must see the edit
    for st in (a, b):
        st.field("ux")[...] *= 0.5
        st.field("vof")[...] = np.clip(st.field("vof") * 1.01, 0.0, 1.0)
    run(gpu, a, 2, True, True)
    run(gpu, b, 2, False, True)
    for s in HOST_SLOTS:
        assert np.array_equal(a.field(s), b.field(s)), s


def test_batch_host_linked_equals_memcpy(libs):
    """a batch copies all cases of a grid group in one launch per field"""
    gpu, orc = libs
    wls = ic.ensemble(9, seed=11, grids=((32, 16), (64, 32), (128, 64)))
    set_env(wls[0])
    for lib in (gpu, orc):
        lib.set_dt_coefs(wls[0].coef_dt_adv, wls[0].coef_dt_dif, wls[0].coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = [new_state(wl, orc) for wl in wls]
    a = [clone(s) for s in st0]
    b = [clone(s) for s in st0]
    for st in a + b:
        for s in HOST_SLOTS:
            st.field(s)[0] = np.nan
            st.field(s)[-1] = np.nan
    try:
        gpu.batch_release()
        for _ in range(3):
            dta = gpu.integrate_batch(a)
            assert gpu.host_link_used()
        gpu.batch_release()
        gpu.set_host_link(False)
        for _ in range(3):
            dtb = gpu.integrate_batch(b)
            assert not gpu.host_link_used()
    finally:
        gpu.set_host_link(True)
        gpu.batch_release()
    assert list(dta) == list(dtb)
    for k, (x, y) in enumerate(zip(a, b)):
        for s in HOST_SLOTS:
            assert np.array_equal(x.field(s), y.field(s)), (k, s)
            assert np.isfinite(x.field(s)).all(), (k, s)


def test_registered_only_link(libs):
    """without host page-table access only registered arrays are linked
    (mode 2 stands in for such a system): pinned arrays link, plain ones
    take the cudaMemcpy path, and both give the same bits"""
    gpu, orc = libs
    wl = ic.single_bubble(128, 64)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    gpu.pin_host_state(a)
    try:
        gpu.set_host_link(2)
        for _ in range(3):
            gpu.integrate(a)
            assert gpu.host_link_used()
            gpu.integrate(b)
            assert not gpu.host_link_used()
    finally:
        gpu.set_host_link(True)
        gpu.unpin_host_state(a)
    for s in HOST_SLOTS:
        assert np.array_equal(a.field(s), b.field(s)), s


@pytest.mark.parametrize("graphs", [True, False], ids=["graph", "eager"])
def test_linked_copies_follow_registration(libs, graphs):
    """a linked step moves page-locked arrays by copy engine and pageable ones
    by copy kernel, and captures its graph again when the same arrays are
    pinned or unpinned between steps: every host array, ghost rows included,
    ends as on the cudaMemcpy path"""
    gpu, orc = libs
    wl = ic.bubble_swarm(256, 128, nbubbles=6, seed=5)
    set_env(wl)
    for lib in (gpu, orc):
        lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    gpu.set_sync_mode(SYNC_STATE)
    st0 = new_state(wl, orc)
    a, b = clone(st0), clone(st0)
    for st in (a, b):
        for s in HOST_SLOTS:
            st.field(s)[0] = np.nan
            st.field(s)[-1] = np.nan
    dta = []
    try:
        dta += run(gpu, a, 2, True, graphs)[0]
        gpu.pin_host_state(a)
        dta += run(gpu, a, 2, True, graphs)[0]
        gpu.unpin_host_state(a)
        dta += run(gpu, a, 2, True, graphs)[0]
    finally:
        gpu.unpin_host_state(a)
    dtb, used_b = run(gpu, b, 6, False, graphs)
    assert not any(used_b)
    assert dta == dtb
    for s in HOST_SLOTS:
        assert np.array_equal(a.field(s), b.field(s)), s
        assert np.isfinite(a.field(s)).all(), s
