"""Host-side checks of the learned curvature closure: the training data
(exact-area circle stencils, labels, symmetries), the BF16 rounding used by
the CPU reference network, and that network's gradient."""
import math

import numpy as np
import pytest

from simplebubblyflowsolver_gb300 import learned_curvature as L


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.standard_normal(5000).astype(np.float32),
                        # exact ties between two bf16 values: round to even
                        (np.arange(1, 200, dtype=np.uint32) << 16 | 0x8000).view(np.float32)])
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy().astype(np.float64)
    assert np.array_equal(L.bf16(x), ref)


def test_circle_stencils_are_exact_areas_and_labels():
    st, lab, R = L.circle_stencils(4000, seed=2)
    assert st.shape[1:] == (3, 3) and st.shape[0] == lab.size == R.size
    assert np.all((st >= 0) & (st <= 1))
    assert np.all((st[:, 1, 1] > 0) & (st[:, 1, 1] < 1))
    assert np.allclose(np.abs(lab), 1.0 / R)
    assert 2.0 <= R.min() and R.max() <= 50.0
    # the inverted half: 1 - vof with the opposite curvature sign
    assert 0.4 < np.mean(lab < 0) < 0.6


def test_symmetries_keep_the_label():
    st, lab, _ = L.circle_stencils(200, seed=4)
    s8 = L.symmetries(st)
    assert s8.shape == (8 * st.shape[0], 3, 3)
    # the reference's curvature is invariant under the 8 symmetries (square cells)
    k = L.plain_curvature(s8).reshape(8, -1)
    assert np.abs(k - k[0]).max() < 1e-14
    # the cell normal turns with the stencil: its length stays 1
    f = L.features(s8)
    assert np.allclose(np.hypot(f[:, 9], f[:, 10]), 1.0, atol=1e-6)
    assert np.all(f[:, 11:] == 0)


def test_plain_curvature_of_a_large_circle_has_the_right_sign():
    st, lab, _ = L.circle_stencils(2000, rmin=2, rmax=5, seed=5)
    k = L.plain_curvature(st)
    assert np.mean(np.sign(k) == np.sign(lab)) > 0.95


def test_reference_gradient_by_finite_differences():
    rng = np.random.default_rng(0)
    st, lab, _ = L.circle_stencils(64, seed=6)
    X = L.features(st).astype(np.float64)
    y = lab
    p = L.init_params(3).astype(np.float64)
    p[L.NHID * L.NFEAT:L.NHID * L.NFEAT + L.NHID] = rng.normal(0, 0.1, L.NHID)  # non-zero b1
    _, _, g = L.reference_forward_backward(p, X, y, quantise=False)
    h = 1e-6
    for i in [0, 5, 700, 1100, 1030, 3000, 5200, L.NPARAM - 1]:
        if i < L.NHID * L.NFEAT and i % L.NFEAT >= 11:
            continue
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = L.reference_forward_backward(pp, X, y, quantise=False)[1]
        lm = L.reference_forward_backward(pm, X, y, quantise=False)[1]
        fd = (lp - lm) / (2 * h)
        assert math.isclose(fd, g[i], rel_tol=1e-5, abs_tol=1e-9), (i, fd, g[i])


def test_interface_stencils_of_a_field():
    from simplebubblyflowsolver_gb300 import ic
    wl = ic.static_drop(32)
    vof = wl.fields()["vof"]
    st, rr, cc = L.interface_stencils(vof)
    assert st.shape[0] == rr.size > 0
    assert np.all(st[:, 1, 1] == vof[rr, cc + 1])
