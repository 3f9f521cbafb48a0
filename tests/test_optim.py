"""CPU tests of the batched derivative-free optimizers (lc2_minimize): they
converge on smooth bounded problems and hand the objective batches."""
import numpy as np
import pytest

from lc2registration_gb300 import capi


def _quad(c, scale):
    c = np.asarray(c, dtype=np.float64)
    s = np.asarray(scale, dtype=np.float64)
    return lambda X: (((X - c) * s) ** 2).sum(axis=1)


@pytest.mark.parametrize("alg", ["bobyqa", "nelder_mead"])
def test_local_methods_find_interior_minimum(alg):
    c = [1.5, -2.0, 0.25, 3.0, -0.7, 0.1]
    f = _quad(c, [1.0, 0.5, 4.0, 0.3, 2.0, 1.0])
    lo, hi = np.full(6, -5.0), np.full(6, 5.0)
    x, fmin, evals, batches = capi.minimize(f, np.zeros(6), lo, hi, alg, xtol_rel=1e-7,
                                            maxeval=20000)
    assert np.allclose(x, c, atol=1e-4), x
    assert batches < evals


def test_trust_region_respects_bounds():
    f = _quad([10.0, -10.0, 0.0], [1, 1, 1])
    lo, hi = np.array([-1.0, -1.0, -1.0]), np.array([2.0, 3.0, 1.0])
    x, fmin, _, _ = capi.minimize(f, [0.5, 0.5, 0.5], lo, hi, "bobyqa", xtol_rel=1e-8)
    assert np.allclose(x, [2.0, -1.0, 0.0], atol=1e-5)


def test_direct_finds_global_basin():
    # two basins; the deeper one is away from the start and the box centre
    def f(X):
        a = ((X - 0.6) ** 2).sum(axis=1)
        b = ((X + 0.7) ** 2).sum(axis=1)
        return np.minimum(a + 0.2, b)
    lo, hi = -np.ones(3), np.ones(3)
    x, fmin, evals, batches = capi.minimize(f, np.zeros(3), lo, hi, "direct_l", xtol_rel=1e-4,
                                            maxeval=600)
    assert np.allclose(x, -0.7, atol=0.05), x
    assert evals <= 600 and batches < evals / 2


def test_maxeval_is_respected_and_errors_propagate():
    f = _quad([0.3], [1.0])
    x, fmin, evals, _ = capi.minimize(f, [0.0], [-1.0], [1.0], "bobyqa", xtol_rel=1e-12,
                                      maxeval=17)
    assert evals <= 17

    def bad(X):
        raise ValueError("objective failed")
    with pytest.raises(ValueError):
        capi.minimize(bad, [0.0], [-1.0], [1.0], "nelder_mead")
    with pytest.raises(capi.LC2Error):
        capi.minimize(f, [0.0], [1.0], [-1.0], "bobyqa")
