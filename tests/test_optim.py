"""CPU tests of the batched derivative-free optimizers (lc2_minimize): they
converge on smooth bounded problems and hand the objective batches."""
import numpy as np
import pytest

from lc2registration_gb300 import capi


def _quad(c, scale):
    c = np.asarray(c, dtype=np.float64)
    s = np.asarray(scale, dtype=np.float64)
    return lambda X: (((X - c) * s) ** 2).sum(axis=1)


@pytest.mark.parametrize("alg", ["bobyqa", "nelder_mead", "quad_tr"])
def test_local_methods_find_interior_minimum(alg):
    c = [1.5, -2.0, 0.25, 3.0, -0.7, 0.1]
    f = _quad(c, [1.0, 0.5, 4.0, 0.3, 2.0, 1.0])
    lo, hi = np.full(6, -5.0), np.full(6, 5.0)
    x, fmin, evals, batches = capi.minimize(f, np.zeros(6), lo, hi, alg, xtol_rel=1e-7,
                                            maxeval=20000)
    assert np.allclose(x, c, atol=1e-4), x
    assert batches < evals


@pytest.mark.parametrize("alg", ["bobyqa", "quad_tr"])
def test_trust_region_respects_bounds(alg):
    f = _quad([10.0, -10.0, 0.0], [1, 1, 1])
    lo, hi = np.array([-1.0, -1.0, -1.0]), np.array([2.0, 3.0, 1.0])
    x, fmin, _, _ = capi.minimize(f, [0.5, 0.5, 0.5], lo, hi, alg, xtol_rel=1e-8)
    assert np.allclose(x, [2.0, -1.0, 0.0], atol=1e-5)


# Standard test functions of derivative-free optimisation (the kind Powell
# reports BOBYQA on): Rosenbrock, ARWHEAD, Powell's singular function, and a
# scaled quadratic whose minimiser lies outside the box (bounds active).
def _rosen(X):
    return (100 * (X[:, 1:] - X[:, :-1] ** 2) ** 2 + (1 - X[:, :-1]) ** 2).sum(axis=1)


def _arwhead(X):
    return (((X[:, :-1] ** 2 + X[:, -1:] ** 2) ** 2) - 4 * X[:, :-1] + 3).sum(axis=1)


def _powell_singular(X):
    a, b, c, d = X.T
    return (a + 10 * b) ** 2 + 5 * (c - d) ** 2 + (b - 2 * c) ** 4 + 10 * (a - d) ** 4


@pytest.mark.parametrize("name,f,x0,lo,hi,xstar,fstar,tol,cap", [
    ("rosenbrock2", _rosen, [-1.2, 1.0], -2.0, 2.0, [1.0, 1.0], 0.0, 1e-6, 400),
    ("rosenbrock4", _rosen, [-1.2, 1.0, -1.2, 1.0], -2.0, 2.0, [1.0] * 4, 0.0, 1e-6, 900),
    ("arwhead8", _arwhead, [1.0] * 8, -3.0, 3.0, [1.0] * 7 + [0.0], 0.0, 1e-5, 600),
    ("powell_singular", _powell_singular, [3.0, -1.0, 0.0, 1.0], -2.0, 2.0, [0.0] * 4, 0.0,
     2e-3, 1500),
])
def test_bobyqa_on_standard_test_functions(name, f, x0, lo, hi, xstar, fstar, tol, cap):
    n = len(x0)
    x, fmin, evals, batches = capi.minimize(f, np.array(x0, float), np.full(n, lo), np.full(n, hi),
                                            "bobyqa", xtol_rel=1e-8, maxeval=5000,
                                            initial_step=0.1)
    assert np.abs(x - np.array(xstar)).max() < tol, (name, x)
    assert fmin < fstar + 1e-9
    assert evals <= cap, (name, evals)
    # the 2n+1 initial points come as one batch, then one point per iteration
    assert batches <= evals - 2 * n


def test_bobyqa_active_bounds_and_quadratic_termination():
    """A scaled quadratic whose minimiser lies outside the box: the optimum is
    the projection, reached with the bounds active; a quadratic is modelled
    exactly, so few evaluations are needed."""
    n = 12
    c = np.linspace(-1.0, 2.0, n)
    s = np.linspace(0.5, 4.0, n)
    f = lambda X: (((X - c) * s) ** 2).sum(axis=1)
    x, fmin, evals, _ = capi.minimize(f, np.full(n, 0.5), np.zeros(n), np.ones(n), "bobyqa",
                                      xtol_rel=1e-8, maxeval=2000, initial_step=0.1)
    assert np.abs(x - np.clip(c, 0, 1)).max() < 1e-7
    assert evals < 300
    x, _, evals, _ = capi.minimize(f, np.zeros(n), np.full(n, -3.0), np.full(n, 3.0), "bobyqa",
                                   xtol_rel=1e-8, maxeval=2000, initial_step=0.1)
    assert np.abs(x - c).max() < 1e-6 and evals < 300


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


def test_register_observer_sees_every_evaluation():
    """lc2_register with a CPU objective of the matrices: the observer gets
    each evaluation once, the last one being the optimum (stage rounds + 1)."""
    center = (8.0, 8.0)
    target = capi.params_to_matrix("2D", [1.5, -2.0, 3.0, 1.02, 0.98, 0.0], center)

    def lc2(M):
        d = M.reshape(-1, 9)[:, :6] - target.reshape(9)[:6]
        return np.exp(-(d * np.array([30, 30, 0.3, 30, 30, 0.3])) ** 2 @ np.ones(6) * 0.1)

    seen = []
    rounds = [(["translation", "rotation"], 1e-5), (["translation", "rotation", "scale"], 1e-5)]
    res = capi.register(None, [0, 0, 0, 1, 1, 0], [-5, -5, -8, 0.9, 0.9, -0.05],
                        [5, 5, 8, 1.1, 1.1, 0.05], center, direct_entries=["translation"],
                        direct_maxeval=40, rounds=rounds, mode="2D", lc2_of_matrices=lc2,
                        observer=lambda st, P, L: seen.append((st, P, L)))
    assert sum(len(L) for _, _, L in seen) == res["evaluations"]
    stages = [st for st, _, _ in seen]
    assert stages == sorted(stages) and stages[0] == 0 and stages[-1] == len(rounds) + 1
    assert len(seen[-1][2]) == 1 and seen[-1][2][0] == res["lc2"]
    np.testing.assert_array_equal(seen[-1][1][0], res["params"])
    assert np.abs(res["params"][:3] - [1.5, -2.0, 3.0]).max() < 0.05
