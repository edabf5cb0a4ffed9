"""The oracle's predict derivatives (KrigingImpl.cpp:254-296) against central finite differences of its own
predict, as the reference's tests/KrigingPredictTest.cpp checks its analytic derivatives (h = 1e-6, absolute
tolerance 1e-4 on points away from the design).  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O


def _case(kernel, reg, normalize, noise, seed=123, n=24, d=2):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(3.0 * X[:, 0]) + np.cos(5.0 * X[:, 1])
    if normalize:
        X = 100 * X - 50
        y = 1000 * (0.01 * X[:, 0] ** 2 - 0.02 * X[:, 1])
    ora = O.OracleKriging(y, X, kernel, regmodel=reg, normalize=normalize,
                          noise_model="nugget" if noise else "none")
    th = np.array([0.35, 0.45])
    alpha = 0.98 if noise else 1.0
    m = O.populate_model(kernel, ora.X, ora.y, ora.F, th, alpha, None, False)
    sigma2 = m.SSEstar / n
    Xn = rng.uniform(size=(5, d))
    if normalize:
        Xn = 100 * Xn - 50
    return ora, th, m.betahat, sigma2, alpha, Xn


@pytest.mark.parametrize("kernel", ["gauss", "exp", "matern3_2", "matern5_2"])
@pytest.mark.parametrize("reg,normalize,noise", [("constant", False, False), ("linear", True, False),
                                                 ("quadratic", False, True), ("interactive", False, False)])
def test_oracle_predict_deriv_vs_fd(kernel, reg, normalize, noise):
    ora, th, beta, s2, alpha, Xn = _case(kernel, reg, normalize, noise)
    mean, sd, dm, dsd = ora.predict(Xn, th, beta, s2, alpha, True, return_deriv=True)
    h = 1e-6 * (100.0 if normalize else 1.0)
    for i in range(Xn.shape[0]):
        for j in range(Xn.shape[1]):
            Xp, Xm = Xn[i:i + 1].copy(), Xn[i:i + 1].copy()
            Xp[0, j] += h
            Xm[0, j] -= h
            mp, sp = ora.predict(Xp, th, beta, s2, alpha, True)
            mm, sm = ora.predict(Xm, th, beta, s2, alpha, True)
            fd_m = (mp[0] - mm[0]) / (2 * h)
            fd_s = (sp[0] - sm[0]) / (2 * h)
            scale = 1.0 if not normalize else max(1.0, abs(fd_m))
            assert abs(dm[i, j] - fd_m) < 1e-4 * scale, (i, j, dm[i, j], fd_m)
            assert abs(dsd[i, j] - fd_s) < 1e-4 * max(1.0, abs(fd_s)), (i, j, dsd[i, j], fd_s)


def test_oracle_stdev_deriv_without_stdev_is_nan():
    """The reference divides by 2 sqrt(ysd2) with ysd2 = 0 when the stdev is not requested (KrigingImpl.cpp:296)."""
    ora, th, beta, s2, alpha, Xn = _case("gauss", "constant", False, False)
    _, sd, dm, dsd = ora.predict(Xn, th, beta, s2, alpha, False, return_deriv=True)
    assert sd is None and np.all(np.isfinite(dm)) and np.all(np.isnan(dsd))


def test_regression_derivative_matches_matrix():
    """dF/dx of every trend equals the finite difference of the regression matrix (Trend.cpp:34-150)."""
    x = np.array([0.3, -0.7, 1.2])
    for reg in ("none", "constant", "linear", "interactive", "quadratic"):
        DF = O.regression_derivative(reg, x)
        for k in range(3):
            e = np.zeros(3)
            e[k] = 1e-6
            fd = (O.regression_matrix(reg, (x + e).reshape(1, -1)) - O.regression_matrix(reg, (x - e).reshape(1, -1)))
            assert np.allclose(DF[k], fd[0] / 2e-6, atol=1e-8), reg
