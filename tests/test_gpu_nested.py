"""GPU NestedKriging against the restatement in oracle/nested_oracle.py and the reference's own NestedKriging tests
(tests/NestedKrigingTest.cpp, bindings/Python/pylibkriging/tests/pylibkriging_nested_test.py of libKriging).

The deterministic path (submodels fitted with optim = "none" at a given theta) is compared with the oracle to
rounding level: partition (exact), common prior (1e-12), PoE-family predictions (mean 1e-9, stdev 1e-7 relative) and
NK predictions (mean 1e-8, stdev 1e-6 relative).  The BFGS path is held to the reference's own assertions."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import nested_oracle as N
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _f2d(X):
    return np.sin(3.0 * X[:, 0]) + np.cos(5.0 * X[:, 1]) + X[:, 0] * X[:, 1]


def _data(n, seed=123, d=2):
    X = np.random.default_rng(seed).uniform(size=(n, d))
    return X, _f2d(X)


def _none_params(theta):
    return {"theta": np.asarray(theta, dtype=float).reshape(1, -1)}


@pytest.mark.parametrize("partition", ["kmeans", "random"])
def test_partition_matches_oracle(gpu_lib, partition):
    X, y = _data(300)
    nk = gpu_lib.NestedKriging(y, X, "gauss", 6, aggregation="PoE", partition=partition, seed=42, optim="none",
                               parameters=_none_params([0.2, 0.3]))
    ref = N.partition(X, 6, partition, seed=42)
    got = nk.groups()
    assert len(got) == 6
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("kernel", ["gauss", "matern5_2"])
def test_common_prior_at_fixed_theta(gpu_lib, kernel):
    X, y = _data(240)
    # gauss at longer ranges is so ill-conditioned on these groups that a 1e-10 diagonal change moves sigma2 by
    # percents (two LAPACK builds disagree at 1e-6): both kernels are compared where cond(R) stays moderate
    th = np.array([0.08, 0.1]) if kernel == "gauss" else np.array([0.15, 0.25])
    nk = gpu_lib.NestedKriging(y, X, kernel, 4, aggregation="NK", optim="none", parameters=_none_params(th))
    groups = nk.groups()
    pr = N.fit_none(y, X, kernel, groups, th)
    assert rel_err(nk.theta(), pr["theta"]) < 1e-12
    assert rel_err(nk.sigma2(), pr["sigma2"]) < 1e-10
    assert rel_err(nk.beta0(), pr["beta0"]) < 1e-10
    for g in range(nk.nb_groups()):  # NestedKrigingTest.cpp:75-92
        sub = nk.submodel(g)
        assert np.max(np.abs(sub.theta() - nk.theta())) < 1e-12
        assert abs(sub.sigma2() - nk.sigma2()) < 1e-12
        assert abs(sub.beta()[0] - nk.beta0()) < 1e-12


@pytest.mark.parametrize("agg", ["PoE", "gPoE", "BCM", "rBCM"])
def test_poe_family_matches_oracle(gpu_lib, agg):
    X, y = _data(200)
    th = np.array([0.2, 0.2])
    nk = gpu_lib.NestedKriging(y, X, "matern5_2", 4, aggregation=agg, optim="none", parameters=_none_params(th))
    Xt = np.random.default_rng(456).uniform(size=(120, 2))
    mean, sd = nk.predict(Xt, True)
    mo, so = N.predict_poe(y, X, "matern5_2", nk.groups(), nk.theta(), nk.sigma2(), nk.beta0(), Xt, agg)
    assert rel_err(mean, mo) < 1e-9
    assert rel_err(sd, so) < 1e-7


@pytest.mark.parametrize("kernel,chunk", [("matern5_2", 128), ("gauss", 37), ("exp", 64)])
def test_nk_matches_oracle(gpu_lib, kernel, chunk):
    X, y = _data(260)
    th = np.array([0.08, 0.1]) if kernel == "gauss" else np.array([0.15, 0.2])
    nk = gpu_lib.NestedKriging(y, X, kernel, 5, aggregation="NK", optim="none", parameters=_none_params(th))
    nk.set_predict_chunk(chunk)
    Xt = np.random.default_rng(456).uniform(size=(150, 2))
    mean, sd = nk.predict(Xt, True)
    mo, so = N.predict_nk(y, X, kernel, nk.groups(), nk.theta(), nk.sigma2(), nk.beta0(), Xt, chunk=chunk)
    assert rel_err(mean, mo) < 1e-8
    assert rel_err(sd, so) < 1e-6


def test_nk_groups_of_mixed_size_classes(gpu_lib):
    """Groups from 20 to 150 points (three padded size classes) given as an explicit partition."""
    X, y = _data(400, d=3)
    rng = np.random.default_rng(5)
    perm = rng.permutation(400)
    cuts = [0, 20, 70, 150, 250, 400]
    groups = [np.sort(perm[a:b]) for a, b in zip(cuts[:-1], cuts[1:])]
    th = np.array([0.3, 0.3, 0.4])
    nk = gpu_lib.NestedKriging("matern3_2")
    nk.fit_groups(y, X, groups, optim="none", parameters=_none_params(th))
    assert all(np.array_equal(a, b) for a, b in zip(nk.groups(), groups))
    Xt = np.random.default_rng(8).uniform(size=(90, 3))
    mean, sd = nk.predict(Xt, True)
    mo, so = N.predict_nk(y, X, "matern3_2", groups, nk.theta(), nk.sigma2(), nk.beta0(), Xt)
    assert rel_err(mean, mo) < 1e-8
    assert rel_err(sd, so) < 1e-6


def test_batched_submodel_fits_equal_single_fits(gpu_lib):
    """The submodel BFGS fits, batched across groups in padded size classes, give the fits of lone Kriging models:
    the common theta (weighted geometric mean of the submodel thetas) agrees to 1e-9."""
    X, y = _data(300)
    nk = gpu_lib.NestedKriging(y, X, "matern5_2", 4, aggregation="PoE")
    groups = nk.groups()
    logt = np.zeros(2)
    for g in groups:
        k = gpu_lib.Kriging(y[g], X[g], "matern5_2")
        logt += len(g) / 300.0 * np.log(k.theta())
    assert rel_err(nk.theta(), np.exp(logt)) < 1e-9


def test_log_likelihood_groups_equals_lone_models(gpu_lib):
    """The batched objective of all submodels (padded size classes) equals each group's own logLikelihoodFun."""
    X, y = _data(500, d=3)
    rng = np.random.default_rng(11)
    perm = rng.permutation(500)
    cuts = [0, 30, 100, 230, 500]
    groups = [np.sort(perm[a:b]) for a, b in zip(cuts[:-1], cuts[1:])]
    nk = gpu_lib.NestedKriging("matern5_2", aggregation="PoE")
    nk.fit_groups(y, X, groups, optim="BFGS")
    thetas = rng.uniform(0.2, 0.8, size=(4, 3))
    ll, grad = nk.logLikelihoodGroups(thetas, True)
    for g, idx in enumerate(groups):
        k = gpu_lib.Kriging(y[idx], X[idx], "matern5_2", "constant", False, "none", "LL",
                            {"theta": thetas[g].reshape(1, -1)})
        l1, g1, _ = k.logLikelihoodFun(thetas[g], True)
        assert rel_err(ll[g], l1) < 1e-12
        assert rel_err(grad[g], g1) < 1e-10


def test_log_likelihood_groups_precision_switch(gpu_lib):
    """set_precision on a fitted model switches its batched evaluations: the mixed path within 1e-8 (LL) / 1e-6
    (gradient) of FP64, and back on FP64 the values of a model fitted in FP64, bit for bit."""
    X, y = _data(1200, d=3)
    rng = np.random.default_rng(12)
    perm = rng.permutation(1200)
    groups = [np.sort(perm[a:b]) for a, b in ((0, 300), (300, 700), (700, 1200))]
    thetas = rng.uniform(0.2, 0.8, size=(3, 3))
    nk64 = gpu_lib.NestedKriging("matern5_2", aggregation="PoE")
    nk64.fit_groups(y, X, groups, optim="BFGS")
    ll64, g64 = nk64.logLikelihoodGroups(thetas, True)
    nk = gpu_lib.NestedKriging("matern5_2", aggregation="PoE")
    nk.set_precision(7)
    nk.fit_groups(y, X, groups, optim="BFGS")
    llm, gm = nk.logLikelihoodGroups(thetas, True)
    for g in range(3):
        assert rel_err(llm[g], ll64[g]) < 1e-8
        assert rel_err(gm[g], g64[g]) < 1e-6
    nk.set_precision(0)
    ll0, g0 = nk.logLikelihoodGroups(thetas, True)
    assert np.array_equal(ll0, ll64) and np.array_equal(g0, g64)


# ---- the reference's own NestedKriging tests, on the BFGS path ----
def test_one_group_reduces_to_kriging(gpu_lib):
    """NestedKrigingTest.cpp:25-60.  The NK mean of one expert is the expert's mean (1e-6) -- except where the fitted
    theta puts the expert's factor on the reference's rcond cliff (rcond(L)^2 within a factor 2 of min_rcond = 1e-18):
    there the nugget-retry branch is decided by the rcond estimate (LAPACK dtrcon in the reference, a dlacn2 estimate
    here) and the expert's mean moves with it, so the NK mean is held to the oracle's NK aggregation at that theta
    instead.  The fit's optimiser path is not pinned to the reference's, so either case can occur."""
    from oracle import nested_oracle as NO
    from scipy.linalg import lapack
    X, y = _data(40)
    Xt = np.random.default_rng(9).uniform(size=(30, 2))
    nk = gpu_lib.NestedKriging(y, X, "gauss", 1, aggregation="NK")
    m_nk, s_nk = nk.predict(Xt, True)
    m_kr, s_kr, _, _, _ = nk.submodel(0).predict(Xt, True, False, False)
    th = nk.theta()
    L, info = lapack.dpotrf(O.build_R("gauss", X, th, 1.0), lower=1, clean=1)
    on_cliff = info == 0 and 0.5e-18 < O.rcond_chol(L) < 2e-18
    if on_cliff:
        mo_nk, _ = NO.predict_nk(y, X, "gauss", [np.arange(40)], th, nk.sigma2(), nk.beta0(), Xt)
        assert np.max(np.abs(m_nk - mo_nk)) < 1e-6
    else:
        assert np.max(np.abs(m_nk - m_kr)) < 1e-6
        assert np.max(np.abs(s_nk - s_kr)) < 5e-2
    for agg in ["PoE", "gPoE", "BCM"]:
        nk1 = gpu_lib.NestedKriging(y, X, "gauss", 1, aggregation=agg)
        m1, s1 = nk1.predict(Xt, True)
        mk, sk, _, _, _ = nk1.submodel(0).predict(Xt, True, False, False)
        assert np.max(np.abs(m1 - mk)) < 1e-8
        assert np.max(np.abs(s1 - sk)) < 1e-6


def test_one_group_reduces_to_kriging_at_a_fixed_theta(gpu_lib):
    """The reference's identity (NestedKrigingTest.cpp:25-60) away from the rcond cliff: one group, theta fixed at a
    well-conditioned value, the NK mean equals the expert's to 1e-6 and the PoE family reduces to the expert."""
    X, y = _data(40)
    Xt = np.random.default_rng(9).uniform(size=(30, 2))
    P = {"theta": np.array([[0.2, 0.25]])}
    nk = gpu_lib.NestedKriging(y, X, "gauss", 1, aggregation="NK", optim="none", parameters=P)
    m_nk, s_nk = nk.predict(Xt, True)
    m_kr, s_kr, _, _, _ = nk.submodel(0).predict(Xt, True, False, False)
    assert np.max(np.abs(m_nk - m_kr)) < 1e-6
    assert np.max(np.abs(s_nk - s_kr)) < 5e-2
    for agg in ["PoE", "gPoE", "BCM"]:
        nk1 = gpu_lib.NestedKriging(y, X, "gauss", 1, aggregation=agg, optim="none", parameters=P)
        m1, s1 = nk1.predict(Xt, True)
        mk, sk, _, _, _ = nk1.submodel(0).predict(Xt, True, False, False)
        assert np.max(np.abs(m1 - mk)) < 1e-8
        assert np.max(np.abs(s1 - sk)) < 1e-6


def test_nk_interpolates(gpu_lib):
    """NestedKrigingTest.cpp:62-73."""
    X, y = _data(100)
    nk = gpu_lib.NestedKriging(y, X, "matern5_2", 4, aggregation="NK")
    mean, sd = nk.predict(X, True)
    assert np.max(np.abs(mean - y)) < 1e-3
    assert sd.max() < 1e-2


def test_close_to_full_kriging(gpu_lib):
    """NestedKrigingTest.cpp:94-121."""
    X, y = _data(400)
    Xt, yt = _data(200, seed=456)
    full = gpu_lib.Kriging(y, X, "matern5_2")
    m_full, _, _, _, _ = full.predict(Xt, True, False, False)
    rmse_full = np.sqrt(np.mean((m_full - yt) ** 2))
    sd_y = np.std(y, ddof=1)
    for agg in ["NK", "rBCM"]:
        nk = gpu_lib.NestedKriging(y, X, "matern5_2", 8, aggregation=agg)
        m_nk, s_nk = nk.predict(Xt, True)
        rmse_nk = np.sqrt(np.mean((m_nk - yt) ** 2))
        assert rmse_nk < 0.05 * sd_y + 2.0 * rmse_full
        assert np.mean(np.abs(m_nk - m_full)) < 0.05 * sd_y
        assert np.all(np.isfinite(s_nk)) and s_nk.min() >= 0.0


def test_aggregation_variances_are_sane(gpu_lib):
    """NestedKrigingTest.cpp:128-154."""
    X, y = _data(200)
    Xt = np.random.default_rng(77).uniform(size=(50, 2))
    nk = gpu_lib.NestedKriging(y, X, "gauss", 4, aggregation="NK")
    _, s_nk = nk.predict(Xt, True)
    assert np.all(s_nk ** 2 <= nk.sigma2() * (1.0 + 1e-6))
    far = np.full((3, 2), 50.0)
    m_far, s_far = nk.predict(far, True)
    assert (s_far ** 2).min() > 0.5 * nk.sigma2()
    assert np.max(np.abs(m_far - nk.beta0())) < 1e-3 * max(1.0, abs(nk.beta0())) + 1e-6


def test_reproducible_given_seed(gpu_lib):
    """NestedKrigingTest.cpp:156-170."""
    X, y = _data(150)
    Xt = np.random.default_rng(3).uniform(size=(40, 2))
    nk1 = gpu_lib.NestedKriging(y, X, "gauss", 5, aggregation="NK", partition="random", seed=42)
    nk2 = gpu_lib.NestedKriging(y, X, "gauss", 5, aggregation="NK", partition="random", seed=42)
    m1, s1 = nk1.predict(Xt, True)
    m2, s2 = nk2.predict(Xt, True)
    assert np.max(np.abs(m1 - m2)) == 0.0
    assert np.max(np.abs(s1 - s2)) == 0.0


def test_input_validation(gpu_lib):
    """NestedKrigingTest.cpp:172-196 and the Python binding's argument errors."""
    X, y = _data(50)
    with pytest.raises(Exception, match="NK aggregation requires a Constant trend"):
        gpu_lib.NestedKriging(y, X, "gauss", 2, aggregation="NK", regmodel="linear")
    with pytest.raises(Exception, match="nb_groups should be in"):
        gpu_lib.NestedKriging(y, X, "gauss", 30)
    nk = gpu_lib.NestedKriging(y, X, "gauss", 2)
    with pytest.raises(Exception, match="same number of columns"):
        nk.predict(np.zeros((3, 3)), True)
    with pytest.raises(Exception, match="Unknown aggregation"):
        gpu_lib.NestedKriging(y, X, "gauss", 2, aggregation="median")
    with pytest.raises(Exception, match="not fitted"):
        gpu_lib.NestedKriging("gauss").predict(np.zeros((2, 2)), True)
    with pytest.raises(Exception, match="WarpKriging"):
        gpu_lib.NestedKriging(y, X, "gauss", 2, warping=["kumaraswamy", "none"])


def test_llvecchia_unified_prior(gpu_lib):
    """NestedKriging.cpp:230-260: one global light Vecchia fit gives the common prior of every submodel."""
    X, y = _data(300)
    nk = gpu_lib.NestedKriging(y, X, "gauss", 3, aggregation="PoE", objective="LLVecchia(10)")
    ref = gpu_lib.Kriging("gauss")
    lib = gpu_lib.load()
    lib.lkg_kriging_set_vecchia_exact_commit(ref._h, 0)
    ref.fit(y, X, "constant", False, "BFGS", "LLVecchia(10)", {})
    assert rel_err(nk.theta(), ref.theta()) < 1e-12
    for g in range(3):
        assert rel_err(nk.submodel(g).theta(), ref.theta()) < 1e-12
    mean, sd = nk.predict(np.random.default_rng(1).uniform(size=(20, 2)), True)
    assert np.all(np.isfinite(mean)) and np.all(sd >= 0)
