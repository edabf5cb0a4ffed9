"""GPU parity at the shapes of the Vecchia and NestedKriging configurations, larger than the unit tests':

* Vecchia: n = 2^15, d = 3, gauss, m = 30 neighbours, num_nugget 1e-6 (the configuration's jitter): the maxmin order
  and neighbour sets equal the oracle's O(n^2) restatement exactly (Kriging.cpp:736-804), and VLL / gradient at two
  theta equal the oracle's _logLikelihoodVecchia (Kriging.cpp:806-924) within 1e-10 / 1e-8.
* NestedKriging: N = 8000, d = 4, matern3_2, 8 groups of 1000 points (the configuration's median group size) at a
  fixed theta near the configuration's fitted one: the common prior (NestedKriging.cpp:273-331) within 1e-10 and gPoE
  predictions (NestedKriging.cpp:364-422) within 1e-9 (mean) / 1e-7 (stdev).
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import nested_oracle as N
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_vecchia_configuration_shape_vs_oracle(gpu_lib):
    rng = np.random.default_rng(123)
    n = 1 << 15
    X = rng.uniform(size=(n, 3))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.01 * rng.standard_normal(n)
    old = gpu_lib.get_num_nugget()
    gpu_lib.set_num_nugget(1e-6)
    try:
        k = gpu_lib.Kriging("gauss")
        k.set_vecchia_exact_commit(False)
        k.fit(y, X, "constant", False, "none", "LLVecchia(30)", {"theta": np.full((1, 3), 0.1)})
        order, nbr = k.vecchia_sets()
        o_order, o_nbr = O.vecchia_sets(X, 30)
        assert np.array_equal(order, o_order)
        assert np.array_equal(nbr, o_nbr)
        F = np.ones((n, 1), order="F")
        for th in (np.full(3, 0.1), np.array([0.3, 0.2, 0.25])):
            v, g = k.logLikelihoodVecchiaFun(th, True)
            vo, go, _, _ = O.vecchia_ll("gauss", X, y, F, th, o_order, o_nbr, num_nugget=1e-6)
            assert rel_err(v, vo) < 1e-10, (v, vo)
            assert rel_err(g, go) < 1e-8, (g, go)
    finally:
        gpu_lib.set_num_nugget(old)


def test_nested_configuration_group_size_vs_oracle(gpu_lib):
    rng = np.random.default_rng(123)
    n, d = 8000, 4
    X = rng.uniform(size=(n, d))
    y = np.sin(4 * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    perm = rng.permutation(n)
    groups = [np.sort(perm[i * 1000:(i + 1) * 1000]) for i in range(8)]
    th = np.array([0.19, 0.17, 0.15, 0.14])
    nk = gpu_lib.NestedKriging("matern3_2", aggregation="gPoE")
    nk.fit_groups(y, X, groups, optim="none", parameters={"theta": th.reshape(1, -1)})
    pr = N.fit_none(y, X, "matern3_2", groups, th)
    assert rel_err(nk.theta(), pr["theta"]) < 1e-12
    assert rel_err(nk.sigma2(), pr["sigma2"]) < 1e-10
    assert rel_err(nk.beta0(), pr["beta0"]) < 1e-10
    Xt = np.random.default_rng(124).uniform(size=(200, d))
    mean, sd = nk.predict(Xt, True)
    mo, so = N.predict_poe(y, X, "matern3_2", nk.groups(), nk.theta(), nk.sigma2(), nk.beta0(), Xt, "gPoE")
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7
