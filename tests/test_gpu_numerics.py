"""Accuracy of the device arithmetic helpers against exact values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_newton_raphson_reciprocal_and_rsqrt():
    from simplebubblyflowsolver_gb300 import load_library
    lib = load_library()
    rng = np.random.default_rng(0)
    x = np.concatenate([10.0 ** rng.uniform(-12, 12, 200000), rng.uniform(0.5, 2.0, 100000),
                        [1.0, 2.0, 0.1, 1e-3, 1e3, 3.0, 1.0 - 2 ** -52, 1.0 + 2 ** -52]])
    r, q = lib.check_newton_raphson(x)
    # within two units in the last place of the correctly rounded results
    ulp_r = np.abs(r - 1.0 / x) / np.spacing(1.0 / x)
    ulp_q = np.abs(q - 1.0 / np.sqrt(x)) / np.spacing(1.0 / np.sqrt(x))
    assert ulp_r.max() <= 2.0, ulp_r.max()
    assert ulp_q.max() <= 2.0, ulp_q.max()
