"""The measured choice of the autotuner: Kriging.autotune_precision picks the fastest precision whose LL and
gradient stay within the error budget of the FP64 path, and every choice it can make holds the budget against the
oracle."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [640, 3000])
def test_autotuned_precision_meets_the_budget(gpu_lib, n):
    lib = gpu_lib.load()
    lib.lkg_autotune_clear()
    rng = np.random.default_rng(n)
    X = rng.uniform(size=(n, 8))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = rng.uniform(0.2, 1.5, size=8)
    gamma = np.concatenate([theta, [1.0 / (1.0 + 1e-6)]])
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    s = k.autotune_precision(gamma, 1e-8, 1e-6)
    assert s in (0, 5, 6, 7) and k.precision() == s
    ll, g, _ = k.logLikelihoodFun(gamma, True)
    ll_o, g_o = O.OracleKriging(y, X, "matern5_2", noise_model="nugget").log_likelihood(gamma)
    assert rel_err(ll, ll_o) <= 1e-8
    assert rel_err(g, g_o) <= 1e-6
    # the choice is tabled: a second model of the same shape reuses it without measuring
    k2 = gpu_lib.Kriging("matern5_2", "nugget")
    k2.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    assert k2.autotune_precision(gamma, 1e-8, 1e-6) == s
    lib.lkg_autotune_clear()


def test_autotuned_lookahead_keeps_the_factor(gpu_lib):
    """autotune_lookahead times the look-ahead's SM counts and tables one for the size; evaluations with the tabled
    choice equal those without the look-ahead bit for bit."""
    lib = gpu_lib.load()
    lib.lkg_autotune_clear()
    rng = np.random.default_rng(9)
    n = 2100
    X = rng.uniform(size=(n, 8))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = rng.uniform(0.2, 1.5, size=8)
    gamma = np.concatenate([theta, [1.0 / (1.0 + 1e-6)]])
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    k.set_precision(7)
    old = lib.lkg_get_lookahead()
    try:
        lib.lkg_set_lookahead(0)
        ll0, g0, _ = k.logLikelihoodFun(gamma, True)
        lib.lkg_set_lookahead(-1)
        c = k.autotune_lookahead(gamma)
        assert c in (0, 12, 16, 24, 32)
        assert lib.lkg_autotune_lookup(("lookahead:n=%d" % n).encode(), -5) == c
        ll1, g1, _ = k.logLikelihoodFun(gamma, True)
    finally:
        lib.lkg_set_lookahead(old)
        lib.lkg_autotune_clear()
    assert ll1 == ll0 and np.array_equal(g1, g0)
