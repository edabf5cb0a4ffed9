"""CPU tests of the NestedKriging restatement (oracle/nested_oracle.py) against the reference's own assertions
(tests/NestedKrigingTest.cpp and bindings/Python/pylibkriging/tests/pylibkriging_nested_test.py of libKriging)."""
import numpy as np
import pytest

from oracle import nested_oracle as N
from oracle import oracle as O


def _f2d(X):  # NestedKrigingTest.cpp:11-13
    return np.sin(3.0 * X[:, 0]) + np.cos(5.0 * X[:, 1]) + X[:, 0] * X[:, 1]


def _data(n, seed=123):
    X = np.random.default_rng(seed).uniform(size=(n, 2))
    return X, _f2d(X)


@pytest.mark.parametrize("method", ["kmeans", "random"])
def test_partition_covers_rows_once(method):
    X, _ = _data(150)
    groups = N.partition(X, 5, method, seed=42)
    allidx = np.sort(np.concatenate(groups))
    assert np.array_equal(allidx, np.arange(150))
    assert all(len(g) >= 4 for g in groups)
    again = N.partition(X, 5, method, seed=42)
    assert all(np.array_equal(a, b) for a, b in zip(groups, again))


def test_random_partition_is_balanced():
    X, _ = _data(103)
    sizes = sorted(len(g) for g in N.partition(X, 4, "random", seed=7))
    assert sizes[-1] - sizes[0] <= 1


def test_kmeans_falls_back_to_random_on_tiny_clusters():
    X, _ = _data(40)
    X[:38] = 0.5  # 38 coincident points: k-means leaves clusters below d + 2 points
    groups = N.partition(X, 3, "kmeans", seed=1)
    sizes = sorted(len(g) for g in groups)
    assert sizes[-1] - sizes[0] <= 1


def test_one_group_reduces_to_the_expert():
    """NestedKrigingTest.cpp:25-60: one group, NK mean = expert mean (1e-6), PoE/gPoE/BCM mean 1e-8, sd 1e-6."""
    X, y = _data(40)
    Xt = np.random.default_rng(9).uniform(size=(30, 2))
    groups = [np.arange(40)]
    th = np.array([0.15, 0.2])  # cond(R) small enough that the 1e-10 jitter of NK moves the mean by < 1e-6
    pr = N.fit_none(y, X, "gauss", groups, th)
    ora = O.OracleKriging(y, X, "gauss")
    mk, sk = ora.predict(Xt, pr["theta"], np.array([pr["beta0"]]), pr["sigma2"], fixed_beta=True)
    m_nk, s_nk = N.predict_nk(y, X, "gauss", groups, pr["theta"], pr["sigma2"], pr["beta0"], Xt)
    assert np.max(np.abs(m_nk - mk)) < 1e-6
    assert np.max(np.abs(s_nk - sk)) < 5e-2
    # rBCM is left out: its prior term (1 - beta) / sigma2 pulls a single expert's mean by ~ v / sigma2, which is
    # below 1e-8 only where the expert's variance is tiny (the reference's fitted-theta data), not at this theta
    for agg in ["PoE", "gPoE", "BCM"]:
        m1, s1 = N.predict_poe(y, X, "gauss", groups, pr["theta"], pr["sigma2"], pr["beta0"], Xt, agg)
        assert np.max(np.abs(m1 - mk)) < 1e-8
        assert np.max(np.abs(s1 - sk)) < 1e-6


def test_nk_interpolates_design_points():
    """NestedKrigingTest.cpp:62-73 / pylibkriging_nested_test.py:38-43 at a fixed common prior."""
    X, y = _data(100)
    groups = N.partition(X, 4, "kmeans", seed=123)
    pr = N.fit_none(y, X, "matern5_2", groups, np.array([0.3, 0.3]))
    mean, sd = N.predict_nk(y, X, "matern5_2", groups, pr["theta"], pr["sigma2"], pr["beta0"], X, chunk=37)
    assert np.max(np.abs(mean - y)) < 1e-3
    assert sd.max() < 1e-2


def test_nk_variance_bounded_by_prior():
    """NestedKrigingTest.cpp:141-153: NK variances <= sigma2; far away the mean returns to beta0."""
    X, y = _data(120)
    groups = N.partition(X, 4, "kmeans", seed=123)
    pr = N.fit_none(y, X, "gauss", groups, np.array([0.2, 0.2]))
    Xt = np.random.default_rng(4).uniform(size=(40, 2))
    _, sd = N.predict_nk(y, X, "gauss", groups, pr["theta"], pr["sigma2"], pr["beta0"], Xt)
    assert np.all(sd ** 2 <= pr["sigma2"] * (1 + 1e-6))
    far = np.full((3, 2), 50.0)
    mf, sf = N.predict_nk(y, X, "gauss", groups, pr["theta"], pr["sigma2"], pr["beta0"], far)
    assert np.max(np.abs(mf - pr["beta0"])) < 1e-3 * max(1.0, abs(pr["beta0"])) + 1e-6
    assert np.min(sf ** 2) > 0.5 * pr["sigma2"]
