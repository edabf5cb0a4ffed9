"""GPU predict derivatives (KrigingImpl.cpp:254-296) through the C ABI.

* Against the oracle's restatement at n = 200, d = 3 for every kernel, trend and noise model, with normalisation:
  mean derivative within 1e-9 and stdev derivative within 1e-7 (relative, the tolerances of the mean and stdev).
* The reference's own checks (tests/KrigingPredictTest.cpp): a BFGS-fitted gauss model's analytic derivatives against
  central finite differences of predict (h = 1e-6, tolerance 1e-4; and normalize = true with h = 1e-3, tolerance 1).
* Without return_stdev the stdev derivative is NaN, as the reference's division by 2 sqrt(0) makes it.
* An LMP fit predicts with sigma2 (n - p) / (n - p - 2) (Kriging.cpp:2262).
* Chunked derivative solves (n q d above 2^26 doubles) equal the unchunked ones.
"""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _config1(n=200, d=3, seed=123):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.05 * rng.standard_normal(n)
    Xn = rng.uniform(size=(40, d))
    return X, y, Xn


# ranges per kernel that keep cond(R) moderate at n = 200 (the gauss kernel at 0.4 .. 0.6 reaches cond ~1e12, where
# two FP64 evaluations of the same predictor already differ at 1e-6)
THETA = {"gauss": np.array([0.1, 0.12, 0.15]), "exp": np.array([0.4, 0.5, 0.6]),
         "matern3_2": np.array([0.4, 0.5, 0.6]), "matern5_2": np.array([0.4, 0.5, 0.6])}


@pytest.mark.parametrize("kernel", ["gauss", "exp", "matern3_2", "matern5_2"])
@pytest.mark.parametrize("reg,normalize", [("constant", False), ("linear", True), ("quadratic", False),
                                           ("interactive", True)])
def test_predict_deriv_vs_oracle(gpu_lib, kernel, reg, normalize):
    X, y, Xn = _config1()
    th = THETA[kernel]
    k = gpu_lib.Kriging(kernel)
    k.fit(y, X, reg, normalize, "none", "LL", {"theta": th.reshape(1, -1)})
    ora = O.OracleKriging(y, X, kernel, regmodel=reg, normalize=normalize)
    thn = th / ora.scaleX
    m = O.populate_model(kernel, ora.X, ora.y, ora.F, thn, 1.0, None, False)
    mean, sd, _, dm, dsd = k.predict(Xn, True, False, True)
    mo, so, dmo, dso = ora.predict(Xn, thn, m.betahat, m.SSEstar / 200, return_deriv=True)
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7
    assert dm.shape == (40, 3) and dsd.shape == (40, 3)
    assert rel_err(dm, dmo) < 1e-9, (dm, dmo)
    assert rel_err(dsd, dso) < 1e-7, (dsd, dso)


def test_predict_deriv_nugget_vs_oracle(gpu_lib):
    X, y, Xn = _config1()
    th = np.array([0.4, 0.5, 0.6])
    s2, nug = 0.5, 0.01
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "linear", False, "none", "LL",
          {"theta": th.reshape(1, -1), "sigma2": s2, "is_sigma2_estim": False, "nugget": nug,
           "is_nugget_estim": False})
    alpha = s2 / (s2 + nug)
    ora = O.OracleKriging(y, X, "matern5_2", regmodel="linear", noise_model="nugget")
    m = O.populate_model("matern5_2", ora.X, ora.y, ora.F, th, alpha, None, False)
    mean, sd, _, dm, dsd = k.predict(Xn, True, False, True)
    mo, so, dmo, dso = ora.predict(Xn, th, m.betahat, s2, alpha, return_deriv=True)
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7
    assert rel_err(dm, dmo) < 1e-9
    assert rel_err(dsd, dso) < 1e-7


def test_predict_lmp_scale_vs_oracle(gpu_lib):
    X, y, Xn = _config1()
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "BFGS", "LMP", {})
    th = k.theta()
    ora = O.OracleKriging(y, X, "matern5_2")
    m = O.populate_model("matern5_2", ora.X, ora.y, ora.F, th, 1.0, None, False)
    mean, sd, _, dm, dsd = k.predict(Xn, True, False, True)
    mo, so, dmo, dso = ora.predict(Xn, th, m.betahat, k.sigma2(), return_deriv=True, objective="LMP")
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7
    assert rel_err(dsd, dso) < 1e-7


def _fd(k, Xn, i, j, h, stdev):
    Xp, Xm = Xn[i:i + 1].copy(), Xn[i:i + 1].copy()
    Xp[0, j] += h
    Xm[0, j] -= h
    mp, sp, _, _, _ = k.predict(Xp, stdev, False, False)
    mm, sm, _, _, _ = k.predict(Xm, stdev, False, False)
    return ((sp[0] - sm[0]) if stdev else (mp[0] - mm[0])) / (2 * h)


def test_predict_deriv_vs_finite_differences(gpu_lib):
    """KrigingPredictTest.cpp:10-106: n = 20, d = 2, gauss, BFGS fit; h = 1e-6, |analytic - FD| < 1e-4."""
    rng = np.random.default_rng(123)
    X = rng.uniform(size=(20, 2))
    y = np.sin(3.0 * X[:, 0]) + np.cos(5.0 * X[:, 1])
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", False, "BFGS", "LL", {})
    Xn = rng.uniform(size=(5, 2))
    _, sd, _, dm, dsd = k.predict(Xn, True, False, True)
    for i in range(5):
        for j in range(2):
            assert abs(dm[i, j] - _fd(k, Xn, i, j, 1e-6, False)) < 1e-4, (i, j)
            assert abs(dsd[i, j] - _fd(k, Xn, i, j, 1e-6, True)) < 1e-4, (i, j)


def test_predict_deriv_normalized_vs_finite_differences(gpu_lib):
    """KrigingPredictTest.cpp:108-186: normalize = true on a wide anisotropic range, h = 1e-3, margin 1."""
    rng = np.random.default_rng(11)
    X = 100 * rng.uniform(size=(30, 2)) - 50
    y = 1000 * (0.01 * X[:, 0] ** 2 - 0.02 * X[:, 1])
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", True, "BFGS", "LL", {})
    Xn = X[:3] + 1.0
    _, sd, _, dm, dsd = k.predict(Xn, True, False, True)
    for i in range(3):
        for j in range(2):
            assert abs(dm[i, j] - _fd(k, Xn, i, j, 1e-3, False)) < 1.0, (i, j)
            if sd[i] >= 1e-6:
                assert abs(dsd[i, j] - _fd(k, Xn, i, j, 1e-3, True)) < 1.0, (i, j)


def test_stdev_deriv_without_stdev_is_nan(gpu_lib):
    X, y, Xn = _config1()
    k = gpu_lib.Kriging("matern3_2")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.array([[0.4, 0.5, 0.6]])})
    _, _, _, dm_a, dsd = k.predict(Xn, False, False, True)
    _, _, _, dm_b, _ = k.predict(Xn, True, False, True)
    assert np.all(np.isnan(dsd))
    assert np.array_equal(dm_a, dm_b)


def test_predict_deriv_chunked_equals_unchunked(gpu_lib):
    """n q d = 4000 x 2200 x 8 > 2^26: the derivative solves run in chunks of points; each point's derivatives equal
    those of the same point predicted alone, up to the rounding of triangular solves with other column counts."""
    rng = np.random.default_rng(5)
    X = rng.uniform(size=(4000, 8))
    y = np.cos(2 * X).sum(axis=1)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.full((1, 8), 1.5)})
    Xn = rng.uniform(size=(2200, 8))
    _, _, _, dm, dsd = k.predict(Xn, True, False, True)
    for i in (0, 1, 2097, 2199):
        _, _, _, dm1, dsd1 = k.predict(Xn[i:i + 1], True, False, True)
        assert rel_err(dm[i], dm1[0]) < 1e-10
        assert rel_err(dsd[i], dsd1[0]) < 1e-8
