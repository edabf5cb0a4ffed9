"""GPU Vecchia path (objective LLVecchia(m)) against the oracle's restatement of make_vecchia_sets and
_logLikelihoodVecchia (src/lib/Kriging.cpp:736-924), plus the reference's own identity / FD checks
(tests/KrigingVecchiaTest.cpp:46-84)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _data(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.01 * rng.standard_normal(n)
    return X, y


@pytest.mark.parametrize("n,d,m", [(300, 3, 10), (517, 2, 30), (64, 4, 5)])
def test_sets_match_oracle(gpu_lib, n, d, m):
    X, _ = _data(n, d, n)
    order, nbr = gpu_lib.vecchia_sets(X, m)
    o_order, o_nbr = O.vecchia_sets(X, m)
    assert np.array_equal(order, o_order)
    for t in range(n):
        assert set(nbr[t][nbr[t] >= 0].tolist()) == set(o_nbr[t][o_nbr[t] >= 0].tolist()), t
        assert np.sum(nbr[t] >= 0) == min(m, t)


@pytest.mark.parametrize("case", ["uniform3", "duplicates", "flat_dim", "d8", "clustered"])
def test_grid_sets_match_oracle_beyond_the_brute_force_range(gpu_lib, case):
    """The grid-accelerated order and neighbour sets (positions above 2048 search a grid over a prefix of the order)
    equal the oracle's O(n^2) restatement exactly, including ties between duplicated points, a degenerate
    dimension, d = 8 and clustered inputs; neighbours in (squared distance, index) order."""
    rng = np.random.default_rng(11)
    n, d, m = 9000, 3, 30
    if case == "d8":
        n, d, m = 5000, 8, 16
    X = rng.uniform(size=(n, d))
    if case == "duplicates":
        X[rng.choice(n, 300, replace=False)] = X[rng.choice(n, 300, replace=False)]
    elif case == "flat_dim":
        X[:, 1] = 0.5
    elif case == "clustered":
        X = np.concatenate([0.01 * rng.standard_normal((n // 2, d)) + 0.3, rng.uniform(size=(n - n // 2, d))])
    order, nbr = gpu_lib.vecchia_sets(X, m)
    o_order, o_nbr = O.vecchia_sets(X, m)
    assert np.array_equal(order, o_order)
    assert np.array_equal(nbr, o_nbr)


@pytest.mark.parametrize("kernel", ["gauss", "matern5_2", "matern3_2", "exp"])
def test_vll_and_gradient_vs_oracle(gpu_lib, kernel):
    X, y = _data(400, 3, 7)
    k = gpu_lib.Kriging("matern5_2" if kernel == "matern5_2" else kernel)
    k.fit(y, X, "constant", False, "none", "LLVecchia(15)", {"theta": np.full((1, 3), 0.3)})
    order, nbr = k.vecchia_sets()
    ora = O.OracleKriging(y, X, kernel)
    for th in ([0.2, 0.3, 0.25], [0.5, 0.15, 0.4]):
        th = np.array(th)
        v, g = k.logLikelihoodVecchiaFun(th, True)
        vo, go, _, _ = O.vecchia_ll(kernel, ora.X, ora.y, ora.F, th, order, nbr)
        assert rel_err(v, vo) < 1e-10, (v, vo)
        assert rel_err(g, go) < 1e-8, (g, go)
        v2, _ = k.logLikelihoodVecchiaFun(th, False)
        assert v2 == v


def test_vll_full_conditioning_equals_exact_ll(gpu_lib):
    # KrigingVecchiaTest.cpp:46-61 with m = n - 1 (the GPU kernels take m <= 32)
    X, y = _data(33, 2, 3)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LLVecchia(32)", {"theta": np.array([[0.2, 0.2]])})
    for th in ([0.2, 0.2], [0.4, 0.3]):
        vll, _ = k.logLikelihoodVecchiaFun(np.array(th), False)
        ll, _, _ = k.logLikelihoodFun(np.array(th), False)
        assert abs(vll - ll) < 1e-3 * abs(ll) + 1e-3


def test_vll_gradient_vs_fd(gpu_lib):
    # KrigingVecchiaTest.cpp:63-84: n = 100, y = sin(3 x1) + cos(5 x2) + x1 x2, two theta, h = 1e-6, 1e-3
    X = np.random.default_rng(123).uniform(size=(100, 2))
    y = np.sin(3.0 * X[:, 0]) + np.cos(5.0 * X[:, 1]) + X[:, 0] * X[:, 1]
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LLVecchia(15)", {"theta": np.array([[0.2, 0.3]])})
    h = 1e-6
    for th in (np.array([0.2, 0.3]), np.array([0.5, 0.15])):
        _, g = k.logLikelihoodVecchiaFun(th, True)
        for j in range(2):
            e = np.zeros(2)
            e[j] = h
            fd = (k.logLikelihoodVecchiaFun(th + e)[0] - k.logLikelihoodVecchiaFun(th - e)[0]) / (2 * h)
            assert abs(g[j] - fd) < 1e-3 * max(1.0, abs(fd)), (th, j, g[j], fd)


@pytest.mark.parametrize("exact", [True, False])
def test_vecchia_fit(gpu_lib, exact):
    X, y = _data(300, 2, 5)
    k = gpu_lib.Kriging("matern5_2")
    k.set_vecchia_exact_commit(exact)
    k.fit(y, X, "constant", False, "BFGS", "LLVecchia(20)", {"theta": np.array([[0.3, 0.3]])})
    assert k.vecchia_neighbors() == 20
    assert k.is_vecchia_light() == (not exact)
    th = k.theta()
    v_hat, g_hat = k.logLikelihoodVecchiaFun(th, True)
    v0, _ = k.logLikelihoodVecchiaFun(np.array([0.3, 0.3]), False)
    assert v_hat >= v0
    if exact:
        mean, _, _, _, _ = k.predict(X[:10], True, False, False)
        assert np.allclose(mean, y[:10], atol=1e-3)


def test_vecchia_rejects_nugget(gpu_lib):
    X, y = _data(50, 2, 6)
    k = gpu_lib.Kriging("matern5_2", "nugget")
    with pytest.raises(gpu_lib.LibKrigingError, match="LLVecchia objective not supported"):
        k.fit(y, X, "constant", False, "BFGS", "LLVecchia(10)", {})


@pytest.mark.parametrize("kernel,reg,normalize,m", [("matern5_2", "constant", False, 20), ("gauss", "linear", True, 12),
                                                    ("exp", "constant", False, 32)])
def test_predict_vecchia_vs_oracle(gpu_lib, kernel, reg, normalize, m):
    """Kriging::predictVecchia (Kriging.cpp:950-1022): mean 1e-9, stdev 1e-7 relative to the restatement.  The
    neighbourhoods of 1500 points in the unit square are tight (cond(RN) up to ~1e8 here), so the warp solves and
    LAPACK's agree to about cond * eps; gauss is taken at shorter ranges for the same reason."""
    X, y = _data(1500, 2, 3)
    th = np.array([0.05, 0.06]) if kernel == "gauss" else np.array([0.2, 0.3])
    k = gpu_lib.Kriging(kernel)
    k.fit(y, X, reg, normalize, "none", "LL", {"theta": th.reshape(1, -1)})
    Xn = np.random.default_rng(4).uniform(size=(200, 2))
    mean, sd = k.predictVecchia(Xn, True, m)
    ora = O.OracleKriging(y, X, kernel, regmodel=reg, normalize=normalize)
    Xnn = (Xn - ora.centerX) / ora.scaleX
    Fn = O.regression_matrix(reg, Xnn)
    # the model's beta, theta and sigma2 are held in normalised units, as the reference's accessors return them
    mo, so = O.predict_vecchia(kernel, ora.X, ora.y, ora.F, k.beta(), k.theta(), k.sigma2(), Xnn, Fn, m)
    assert rel_err(mean, ora.centerY + ora.scaleY * mo) < 1e-9
    assert rel_err(sd, ora.scaleY * so) < 1e-7


def test_predict_vecchia_all_neighbours_is_kriging_mean(gpu_lib):
    """With every observation in the neighbourhood the local predictor is the kriging mean (up to num_nugget)."""
    X, y = _data(30, 2, 5)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.array([[0.3, 0.3]])})
    Xn = np.random.default_rng(6).uniform(size=(50, 2))
    mv, _ = k.predictVecchia(Xn, True, 30)
    mp, _, _, _, _ = k.predict(Xn, True, False, False)
    assert np.max(np.abs(mv - mp)) < 1e-6


def test_light_fit_predict_routes_to_predict_vecchia(gpu_lib):
    """Kriging.cpp:2242-2251: after a light Vecchia fit predict gives predictVecchia's mean and stdev."""
    X, y = _data(2000, 2, 8)
    k = gpu_lib.Kriging("gauss")
    k.set_vecchia_exact_commit(False)
    k.fit(y, X, "constant", False, "BFGS", "LLVecchia(15)", {})
    Xn = np.random.default_rng(9).uniform(size=(100, 2))
    m1, s1, _, _, _ = k.predict(Xn, True, False, False)
    m2, s2 = k.predictVecchia(Xn, True, 0)
    assert np.array_equal(m1, m2) and np.array_equal(s1, s2)
    with pytest.raises(Exception, match="light Vecchia fit"):
        k.predict(Xn, True, True, False)


def test_vecchia_shards_sum_to_the_single_evaluation(gpu_lib):
    """The sharded form's device half: two VecchiaShard ranges [0, n/2), [n/2, n) of the model's sets, their partial
    sums added on the host (what the ranks' all-reduce does), give the single evaluation's VLL and gradient."""
    from libkriging_gb300.kriging import VecchiaShard, vecchia_finish, vecchia_gls_beta
    X, y = _data(700, 3, 21)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LLVecchia(12)", {"theta": np.full((1, 3), 0.3)})
    order, nbr = k.vecchia_sets()
    th = np.array([0.25, 0.3, 0.35])
    v_ref, g_ref = k.logLikelihoodVecchiaFun(th, True)
    n, d, p = 700, 3, 1
    F = np.ones((n, 1))
    shards = [VecchiaShard("matern5_2", X, y, F, order, nbr, a, b) for a, b in ((0, 350), (350, 700))]
    s1 = sum(s.sums1(th, True)[0] for s in shards)
    beta = vecchia_gls_beta(p, s1)
    s2 = sum(s.sums2(beta, True) for s in shards)
    vll, sigma2, grad = vecchia_finish(n, d, s1[p * p + p], s2, True)
    assert rel_err(vll, v_ref) <= 1e-12
    assert rel_err(grad, g_ref) <= 1e-10
