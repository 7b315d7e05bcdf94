"""GPU checks of the learned curvature closure: the BF16 tensor-core
gradient against the CPU reference network (same precision steps), batch
prediction, training, and the closure inside the time step (static drop)."""
import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import learned_curvature as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from simplebubblyflowsolver_gb300 import load_library
    return load_library()


@pytest.fixture(scope="module")
def small_set():
    st, lab, _ = L.circle_stencils(400, seed=11)
    st8 = L.symmetries(st)
    return L.features(st8), np.tile(lab, 8).astype(np.float32)


@pytest.fixture(scope="module")
def trained(lib):
    """the default training run (exact-area, advected and relaxed circles)"""
    model, params, hist = L.train_default(lib, seed=0)
    return model, params, hist


@pytest.mark.parametrize("n", [128, 1000])
def test_gradient_matches_cpu_reference(lib, small_set, n):
    X, Y = small_set
    p = L.init_params(7)
    rng = np.random.default_rng(n)
    p[L.NHID * L.NFEAT:L.NHID * L.NFEAT + L.NHID] = rng.normal(0, 0.1, L.NHID)
    p[L.NHID * L.NFEAT + L.NHID + L.NHID * L.NHID:][:L.NHID] = rng.normal(0, 0.1, L.NHID)
    rows = rng.choice(X.shape[0], n, replace=False).astype(np.int32)
    m = L.GpuCurvatureModel(lib, X, Y)
    m.set_params(p)
    g_gpu, loss_gpu = m.gradient(rows)
    _, loss_cpu, g_cpu = L.reference_forward_backward(p, X[rows].astype(np.float64), Y[rows].astype(np.float64))
    # FP32 accumulation in a different order; BF16 roundings of FP32 vs FP64
    # intermediates can differ by one bf16 ulp in rare elements
    err = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    print(f"n={n} gradient rel err {err:.2e} loss {loss_gpu:.6e} vs {loss_cpu:.6e}")
    assert err < 2e-3
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * loss_cpu
    # the padding columns of W1 get no gradient
    assert np.all(g_gpu[:L.NHID * L.NFEAT].reshape(L.NHID, L.NFEAT)[:, 11:] == 0)


def test_predict_matches_cpu_reference(lib, small_set):
    X, Y = small_set
    p = L.init_params(9)
    m = L.GpuCurvatureModel(lib, X, Y)
    m.set_params(p)
    out = m.predict(X[:1001])
    ref, _, _ = L.reference_forward_backward(p, X[:1001].astype(np.float64), Y[:1001].astype(np.float64))
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 1e-2, err  # one bf16 rounding of h1 may differ


def test_training_beats_the_plain_curvature(lib, trained):
    model, params, hist = trained
    assert hist[-1] < 0.6 * hist[0]
    st, lab, R = L.circle_stencils(20000, seed=123)  # held-out exact-area circles
    e_l = np.abs(model.predict(L.features(st)) - lab) / np.abs(lab)
    e_p = np.abs(L.plain_curvature(st) - lab) / np.abs(lab)
    print("held-out median relative error learned", np.median(e_l), "plain", np.median(e_p))
    assert np.median(e_l) < 0.5 * np.median(e_p)


@pytest.mark.parametrize("n", [64, 128, 256])
def test_static_drop_initial_curvature(lib, trained, n):
    """curvature of the static drop's interface cells (r = 0.25, exact
    kappa dx = 4 / n): learned vs the reference's -div n"""
    from simplebubblyflowsolver_gb300 import ic
    model, _, _ = trained
    st, _, _ = L.interface_stencils(ic.static_drop(n).fields()["vof"])
    ex = 4.0 / n
    e_l = np.sqrt(np.mean((model.predict(L.features(st)) - ex) ** 2)) / ex
    e_p = np.sqrt(np.mean((L.plain_curvature(st) - ex) ** 2)) / ex
    print(n, "rms relative curvature error learned", e_l, "plain", e_p)
    assert e_l < 0.5 * e_p


def test_curvature_model_switch(lib):
    with pytest.raises(Exception):
        lib.set_curvature_model(2)
    base = lib.kernels_per_step()
    lib.mlp_set_params(L.init_params(0))
    lib.set_curvature_model(1)
    try:
        assert lib.kernels_per_step() == base + 3
    finally:
        lib.set_curvature_model(0)
    assert lib.kernels_per_step() == base


@pytest.mark.parametrize("n", [64, 128, 256])
def test_static_drop_in_the_step(lib, trained, n):
    """the closure inside the time step, static drop (density ratio 1e-3, La =
    12000): the curvature the step uses and the time-averaged parasitic
    velocity, learned vs plain.  Over five training runs (1000 steps):
    kappa error learned / plain 0.20 .. 0.24 at 64^2, 0.35 .. 0.43 at 128^2,
    0.35 .. 0.47 at 256^2; parasitic velocity 0.40 .. 0.47, 0.45 .. 0.72 and
    0.70 .. 1.03 (the 256^2 bound holds on the shorter run here)."""
    _, params, _ = trained
    steps = 400 * n // 64
    a = L.evaluate_static_drop(lib, n=n, steps=steps, model=0, record_every=steps // 8)
    b = L.evaluate_static_drop(lib, n=n, steps=steps, model=1, params=params, record_every=steps // 8)
    ua = np.mean([u for _, _, u in a["umax_history"]])
    ub = np.mean([u for _, _, u in b["umax_history"]])
    print(n, "kappa rms plain", a["kappa_rms_rel_err"], "learned", b["kappa_rms_rel_err"],
          "mean parasitic velocity plain", ua, "learned", ub, "dp err", a["dp_rel_err"], b["dp_rel_err"])
    assert b["learned_cells_per_step"] > 0
    assert np.isfinite(b["umax"]) and np.isfinite(b["dp"])
    assert b["kappa_rms_rel_err"] < 0.6 * a["kappa_rms_rel_err"]
    assert ub < 0.8 * ua


def test_training_is_reproducible(lib):
    """gradients are summed in a fixed order (no atomics): two training runs
    from the same parameters and seed end bit for bit equal"""
    st, lab, _ = L.circle_stencils(4096, seed=7)
    X = L.features(L.symmetries(st))
    Y = np.tile(lab, 8).astype(np.float32)
    runs = []
    for _ in range(2):
        m = L.GpuCurvatureModel(lib, X, Y)
        m.set_params(L.init_params(5))
        m.train(epochs=2, seed=3)
        runs.append(m.params())
    assert np.array_equal(runs[0], runs[1])


def test_geometry_ahead_learned_identical(lib, trained):
    """with the learned closure the interface geometry, the closure and the
    force formed ahead of the velocity give the same bits as after the
    correction, in every array"""
    from simplebubblyflowsolver_gb300 import ic

    from ._helpers import new_state, set_env
    from .test_gpu_integrate import ahead_vs_after
    import oracle
    _, params, _ = trained
    wl = ic.bubble_swarm(512, 256, nbubbles=12, seed=3)
    set_env(wl)
    lib.set_dt_coefs(wl.coef_dt_adv, wl.coef_dt_dif, wl.coef_dt_int)
    st0 = new_state(wl, oracle.Oracle())
    lib.mlp_set_params(params)
    lib.set_curvature_model(1)
    try:
        runs = ahead_vs_after(lib, st0)
    finally:
        lib.set_curvature_model(0)
    assert runs[False][0] == runs[True][0]
    for s in runs[True][1].slots():
        assert np.array_equal(runs[False][1].field(s), runs[True][1].field(s)), s
