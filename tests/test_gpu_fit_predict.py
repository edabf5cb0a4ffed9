"""GPU fit + predict against the oracle's restatement of the reference fit driver.

The plain-fit configuration (n=200, d=3, matern5_2, y = sum sin(2 pi x_j) + 0.5 x_1 x_2, theta0 = 0.5) has its
optimum on the reference's rcond boundary: at theta_hat, cond(R) ~ 4.5e14 and rcond(L)^2 ~ 1e-18 = min_rcond, so
the log-likelihood is only defined to ~1e-5 relative by ANY FP64 implementation (LAPACK builds included) and the
fitted theta moves with where the nugget-retry cliff is detected (two LAPACK builds land on different thetas, and a
single start can stop on the cliff well short of another build's optimum).  The optimum itself is checked with the
reference's own fit test (tests/KrigingFitTest.cpp: a BFGS10 fit beats a 10x10 grid of logLikelihoodFun up to
1e-3 relative); the single-start fit on this configuration is held to improving on theta0 and to committing a
self-consistent model.  Predict is compared at a
moderately conditioned theta (cond(R) ~ 1e7): mean 1e-9, stdev 1e-7 relative.
The optimiser path itself is not pinned (the reference's lbfgsb_cpp is not vendored)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _config1():
    rng = np.random.default_rng(123)
    X = rng.uniform(size=(200, 3))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.5 * X[:, 0] * X[:, 1]
    Xn = np.random.default_rng(124).uniform(size=(1000, 3))
    return X, y, Xn


def test_fit_bfgs10_beats_grid(gpu_lib):
    """tests/KrigingFitTest.cpp "BFGS finds better LL than grid search": n=20, d=2, gauss, Branin-like response,
    a 10x10 grid of logLikelihoodFun over [1e-6, 10]^2 against a BFGS10 fit, 1e-3 relative."""
    rng = np.random.default_rng(123)
    X = rng.uniform(size=(20, 2))
    x1, x2 = X[:, 0], X[:, 1]
    y = (x2 - 0.5 * x1 * x1 + 5 * x1 - 6) ** 2 + 10 * (1 - 0.1) * np.cos(x1) + 10
    kg = gpu_lib.Kriging(y, X, "gauss", "constant", False, "BFGS", "LL")
    grid = np.linspace(1e-6, 10.0, 10)
    best = -np.inf
    for t1 in grid:
        for t2 in grid:
            try:
                ll, _, _ = kg.logLikelihoodFun(np.array([t1, t2]), False)
            except RuntimeError:
                continue  # no factorisation within the nugget retries: the point has no LL
            best = max(best, ll)
    assert np.isfinite(best)
    kb = gpu_lib.Kriging(y, X, "gauss", "constant", False, "BFGS10", "LL")
    ll_b = kb.logLikelihood()
    assert ll_b >= best - abs(best) * 1e-3, (ll_b, best, kb.theta())


def test_fit_config1(gpu_lib):
    """Single-start BFGS from theta0 = 0.5 on the cliff-bound configuration: the optimiser path is decided by where
    the rcond cliff is met, so the fit is held to improving on theta0, staying in bounds and committing a model
    whose LL, sigma2 and predictions are those of theta_hat."""
    X, y, Xn = _config1()
    k = gpu_lib.Kriging(y, X, "matern5_2", "constant", False, "BFGS", "LL", {"theta": np.full((1, 3), 0.5)})
    th = k.theta()
    ora = O.OracleKriging(y, X, "matern5_2")
    # at theta_hat rcond(L)^2 sits at min_rcond, where the GPU's dlacn2 estimate and LAPACK's dtrcon can take the
    # nugget-retry branch differently: LL values are compared within the GPU implementation only
    ll_g, _, _ = k.logLikelihoodFun(th, False)
    ll_0, _, _ = k.logLikelihoodFun(np.full(3, 0.5), False)
    assert ll_0 == pytest.approx(ora.log_likelihood(np.full(3, 0.5), False)[0], rel=1e-10)
    assert ll_g > ll_0 + 1e-3 * abs(ll_0), (th, ll_g, ll_0)
    lo, hi = O.theta_bounds(ora.X, ora.y)
    assert np.all(th >= lo * (1 - 1e-12)) and np.all(th <= hi * (1 + 1e-12))
    # the committed model is self-consistent (its LL is the objective's value at theta_hat) and interpolates
    assert abs(k.logLikelihood() - ll_g) < 1e-10 * abs(ll_g)
    mean, sd, _, _, _ = k.predict(X[:25], True, False, False)
    assert np.max(np.abs(mean - y[:25])) < 1e-4
    mean, sd, _, _, _ = k.predict(Xn[:100], True, False, False)
    assert np.all(np.isfinite(mean)) and np.all(sd >= 0)


@pytest.mark.parametrize("reg,normalize", [("constant", False), ("linear", True), ("quadratic", False)])
def test_predict_vs_oracle(gpu_lib, reg, normalize):
    X, y, Xn = _config1()
    th = np.array([0.4, 0.5, 0.6])
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, reg, normalize, "none", "LL", {"theta": th.reshape(1, -1)})
    ora = O.OracleKriging(y, X, "matern5_2", regmodel=reg, normalize=normalize)
    thn = th / ora.scaleX
    m = O.populate_model("matern5_2", ora.X, ora.y, ora.F, thn, 1.0, None, False)
    assert rel_err(k.beta(), m.betahat) < 1e-10
    assert rel_err(k.sigma2(), m.SSEstar / 200) < 1e-10
    mean, sd, _, _, _ = k.predict(Xn, True, False, False)
    mo, so = ora.predict(Xn, thn, m.betahat, m.SSEstar / 200)
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7


def test_predict_cov_and_interpolation(gpu_lib):
    X, y, Xn = _config1()
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "linear", True, "none", "LL", {"theta": np.array([[0.4, 0.5, 0.6]])})
    mean, sd, cov, _, _ = k.predict(X[:20], True, True, False)
    assert np.allclose(mean, y[:20], atol=1e-7)  # interpolation at design points
    assert np.all(sd < 1e-4)
    mean2, sd2, cov2, _, _ = k.predict(Xn[:50], True, True, False)
    assert np.allclose(np.sqrt(np.clip(np.diag(cov2), 0, None)), sd2, rtol=1e-6, atol=1e-9)
    assert np.allclose(cov2, cov2.T)


def test_multistart_fit_batched(gpu_lib):
    rng = np.random.default_rng(7)
    X = rng.uniform(size=(120, 2))
    y = np.cos(3 * X).sum(axis=1) + 0.1 * rng.standard_normal(120)
    k = gpu_lib.Kriging(y, X, "gauss", "constant", False, "BFGS8", "LL", {})
    ora = O.OracleKriging(y, X, "gauss")
    th_o, ll_o = ora.fit_bfgs(multistart=8)
    ll_g = ora.log_likelihood(k.theta(), False)[0]
    # best-of-8 starts: the GPU optimum is as good as the oracle's up to 1e-6 relative
    assert ll_g >= ll_o - 1e-6 * abs(ll_o), (k.theta(), th_o, ll_g, ll_o)


def test_nugget_fit(gpu_lib):
    rng = np.random.default_rng(5)
    X = rng.uniform(size=(150, 2))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.05 * rng.standard_normal(150)
    k = gpu_lib.Kriging("matern3_2", "nugget")
    k.fit(y, X, "constant", False, "BFGS", "LL", {})
    assert 0.0 < k.nugget() < k.sigma2()
    g = np.concatenate([k.theta(), [k.sigma2() / (k.sigma2() + k.nugget())]])
    ll, grad, _ = k.logLikelihoodFun(g, True)
    ora = O.OracleKriging(y, X, "matern3_2", noise_model="nugget")
    ll_o, g_o = ora.log_likelihood(g)
    assert rel_err(ll, ll_o) < 1e-10
    assert rel_err(grad, g_o) < 1e-7


def test_predict_in_point_chunks(gpu_lib):
    """q = 10000 points at n = 4096 run in two chunks (Rstar_on of a chunk below 256 MB); each point's mean and
    stdev equal those of the same point predicted within a smaller set (per-column solves, the same operations)."""
    rng = np.random.default_rng(9)
    X = rng.uniform(size=(4096, 3))
    y = np.sin(2 * np.pi * X).sum(axis=1)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.full((1, 3), 0.4)})
    Xn = rng.uniform(size=(10000, 3))
    mean, sd, _, _, _ = k.predict(Xn, True, False, False)
    for a, b in ((0, 40), (8170, 8230), (9950, 10000)):
        m1, s1, _, _, _ = k.predict(Xn[a:b], True, False, False)
        assert rel_err(mean[a:b], m1) < 1e-13
        assert rel_err(sd[a:b], s1) < 1e-12


def test_predict_digit_solves_on_mixed_model(gpu_lib):
    """A mixed-precision model runs the solves of large predictions as digit products with L^-1 (8 seven-bit digits):
    the same means and stdevs as the FP64 triangular solve to FP64 accuracy, and the oracle's."""
    rng = np.random.default_rng(10)
    X = rng.uniform(size=(2048, 3))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.5 * X[:, 0] * X[:, 1]
    th = np.array([0.4, 0.5, 0.6])
    k64 = gpu_lib.Kriging("matern5_2")
    k64.fit(y, X, "constant", False, "none", "LL", {"theta": th.reshape(1, -1)})
    km = gpu_lib.Kriging("matern5_2")
    km.set_precision(7)
    km.fit(y, X, "constant", False, "none", "LL", {"theta": th.reshape(1, -1)})
    Xn = rng.uniform(size=(3000, 3))
    m64, s64, _, _, _ = k64.predict(Xn, True, False, False)
    mm, sm, _, _, _ = km.predict(Xn, True, False, False)
    assert rel_err(mm, m64) < 1e-11
    # the stdev comes from 1 - |Rstar_on(:, t)|^2, which cancels where points lie close to the design: two FP64
    # evaluations of it (solve with L, product with L^-1) agree to ~cond(L) eps / variance
    assert rel_err(sm, s64) < 1e-8
    ora = O.OracleKriging(y, X, "matern5_2")
    m = O.populate_model("matern5_2", ora.X, ora.y, ora.F, th, 1.0, None, False)
    mo, so = ora.predict(Xn[:300], th, m.betahat, m.SSEstar / 2048)
    assert rel_err(mm[:300], mo) < 1e-9
    assert rel_err(sm[:300], so) < 1e-7
