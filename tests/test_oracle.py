"""CPU tests of the oracle (the CPU restatement the GPU results are compared with): pinned to the reference's known answers, plus the reference's own
finite-difference and identity checks (tests/KrigingLogLikTest.cpp, NuggetKrigingLogLikTest.cpp,
KrigingVecchiaTest.cpp:46-84 of libKriging)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

TOL_GOLDEN = 1e-12  # bindings/Python/pylibkriging/tests/binding_consistency_test.py:11


@pytest.mark.parametrize("i", range(11))
def test_oracle_matches_reference_known_answers(golden, i):
    c = golden["cases"][i]
    X, y = np.array(c["X"]), np.array(c["y"])
    k = O.OracleKriging(y, X, "gauss")
    ll, g = k.log_likelihood(golden["theta_value"] * np.ones(X.shape[1]))
    assert rel_err(ll, c["ll"]) < TOL_GOLDEN
    assert rel_err(g, c["grad"]) < TOL_GOLDEN


def _data(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.5 * X[:, 0] * X[:, -1]
    return X, y


@pytest.mark.parametrize("kernel", ["gauss", "exp", "matern3_2", "matern5_2"])
def test_oracle_gradient_vs_central_fd(kernel):
    X, y = _data(30, 2, 1)
    k = O.OracleKriging(y, X, kernel)
    th = np.array([0.4, 0.3])
    _, g = k.log_likelihood(th)
    h = 1e-6
    fd = np.array([(k.log_likelihood(th + h * e, False)[0] - k.log_likelihood(th - h * e, False)[0]) / (2 * h)
                   for e in np.eye(2)])
    assert np.all(np.abs(g - fd) / (np.abs(g) + 1e-10) < 1e-3)


@pytest.mark.parametrize("est", [(True, True), (True, False), (False, False)])
def test_oracle_nugget_gradient_vs_fd(est):
    # NuggetKrigingLogLikTest.cpp:11-80 pattern: [theta, alpha] gradient vs central FD
    X = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.5, 0.5], [0.3, 0.7]])
    y = np.array([0.0, 1.0, 1.0, 2.0, 1.0, 0.8])
    k = O.OracleKriging(y, X, "gauss", noise_model="nugget", est_sigma2=est[0], sigma2=0.5, est_nugget=est[1],
                        nugget=0.1)
    ta = np.array([0.4, 0.6, 0.45])
    _, g = k.log_likelihood(ta)
    h = 1e-7
    fd = np.array([(k.log_likelihood(ta + h * e, False)[0] - k.log_likelihood(ta - h * e, False)[0]) / (2 * h)
                   for e in np.eye(3)])
    if est == (False, False):
        assert g[2] == 0.0
        fd[2] = 0.0
    assert np.all(np.abs(g - fd) / (np.abs(g) + 1e-10) < 1e-3)


def test_oracle_vecchia_full_conditioning_equals_exact_ll():
    # KrigingVecchiaTest.cpp:46-61: VLL(n-1) ~= LL
    X, y = _data(40, 2, 3)
    k = O.OracleKriging(y, X, "matern5_2")
    order, nbr = O.vecchia_sets(k.X, 39)
    for th in ([0.2, 0.2], [0.4, 0.3]):
        vll, _, _, _ = O.vecchia_ll("matern5_2", k.X, k.y, k.F, np.array(th), order, nbr, return_grad=False)
        ll, _ = k.log_likelihood(np.array(th), False)
        assert abs(vll - ll) < 1e-3 * abs(ll) + 1e-3


def test_oracle_vecchia_gradient_vs_fd():
    # KrigingVecchiaTest.cpp:63-84
    X, y = _data(80, 2, 4)
    k = O.OracleKriging(y, X, "matern5_2")
    order, nbr = O.vecchia_sets(k.X, 15)
    th = np.array([0.2, 0.3])
    _, g, _, _ = O.vecchia_ll("matern5_2", k.X, k.y, k.F, th, order, nbr)
    h = 1e-6
    for j in range(2):
        e = np.eye(2)[j] * h
        fd = (O.vecchia_ll("matern5_2", k.X, k.y, k.F, th + e, order, nbr, return_grad=False)[0]
              - O.vecchia_ll("matern5_2", k.X, k.y, k.F, th - e, order, nbr, return_grad=False)[0]) / (2 * h)
        assert abs(g[j] - fd) < 1e-3 * max(1.0, abs(fd))


def test_oracle_vecchia_sets_properties():
    X, _ = _data(60, 3, 5)
    order, nbr = O.vecchia_sets(X, 10)
    assert sorted(order.tolist()) == list(range(60))
    pos = {int(o): t for t, o in enumerate(order)}
    for t in range(60):
        ids = [int(v) for v in nbr[t] if v >= 0]
        assert len(ids) == min(10, t)
        assert all(pos[i] < t for i in ids)  # neighbours are earlier in the ordering


def test_mt19937_stream_matches_std_uniform_real():
    # std::mt19937(123) + uniform_real_distribution<double> (libstdc++: two 32-bit draws per double)
    s = O.MT19937Stream(123)
    u = s.uniform(3)
    assert np.all((u >= 0) & (u < 1))
    # first raw outputs of std::mt19937 seeded with 123 (published reference sequence of the generator)
    raw = O.MT19937Stream(123).bg.random_raw(2)
    assert raw.tolist() == [2991312382, 3062119789]


def test_oracle_loo_gradient_matches_fd():
    """The restated _leaveOneOut gradient (Kriging.cpp:421-465) against central differences of the LOO value."""
    rng = np.random.default_rng(5)
    X = rng.uniform(size=(30, 2))
    y = np.sin(3 * X[:, 0]) + np.cos(5 * X[:, 1]) + X[:, 0] * X[:, 1]
    for kernel in ("gauss", "matern5_2"):
        ora = O.OracleKriging(y, X, kernel)
        th = np.array([0.3, 0.4])
        loo, g, _, _ = ora.leave_one_out(th, True)
        for k in range(2):
            e = np.zeros(2)
            e[k] = 1e-6
            fd = (ora.leave_one_out(th + e, False)[0] - ora.leave_one_out(th - e, False)[0]) / 2e-6
            assert abs(g[k] - fd) < 1e-5 * max(1.0, abs(fd)), (kernel, k, g[k], fd)


def test_oracle_loo_matches_reference_known_answer(golden):
    """LOO value and gradient for data1-scal at theta = 0.3 (binding_consistency_test.py:46-68)."""
    c = golden["cases"][-1]
    assert c["name"] == "data1-scal"
    X, y = np.array(c["X"]), np.array(c["y"])
    loo, g, _, _ = O.OracleKriging(y, X, "gauss").leave_one_out(golden["theta_value"] * np.ones(X.shape[1]), True)
    assert rel_err(loo, c["loo"]) < TOL_GOLDEN
    assert rel_err(g, c["loo_grad"]) < TOL_GOLDEN


@pytest.mark.parametrize("kernel", ["gauss", "matern5_2"])
def test_oracle_lmp_gradient_matches_fd(kernel):
    """The restated _logMargPost gradient (Kriging.cpp:603-626, KrigingImpl.cpp:887-921) against central
    differences, for NoiseModel None and Nugget (theta and alpha directions)."""
    rng = np.random.default_rng(7)
    X = rng.uniform(size=(30, 2))
    y = np.sin(3 * X[:, 0]) + np.cos(5 * X[:, 1]) + X[:, 0] * X[:, 1]
    cases = [(O.OracleKriging(y, X, kernel), np.array([0.3, 0.4])),
             (O.OracleKriging(y, X, kernel, noise_model="nugget", alpha=0.9), np.array([0.3, 0.4, 0.9]))]
    for ora, g0 in cases:
        v, g = ora.log_marg_post(g0, True)
        for k in range(g0.size):
            e = np.zeros(g0.size)
            e[k] = 1e-6
            fd = (ora.log_marg_post(g0 + e, False)[0] - ora.log_marg_post(g0 - e, False)[0]) / 2e-6
            assert abs(g[k] - fd) < 1e-5 * max(1.0, abs(fd)), (ora.noise_model, k, g[k], fd)


def test_oracle_lmp_fixed_sigma2_forward_differences():
    """sigma2 given: the reference takes forward differences with step 1e-6 (Kriging.cpp:629-640)."""
    rng = np.random.default_rng(8)
    X = rng.uniform(size=(25, 2))
    y = np.sin(3 * X[:, 0]) + X[:, 1]
    ora = O.OracleKriging(y, X, "gauss", est_sigma2=False, sigma2=0.5)
    th = np.array([0.3, 0.5])
    v, g = ora.log_marg_post(th, True)
    for k in range(2):
        e = np.zeros(2)
        e[k] = 1e-6
        assert g[k] == (ora.log_marg_post(th + e, False)[0] - v) / 1e-6


@pytest.mark.parametrize("no,nu", [(40, 1), (37, 13), (64, 64)])
def test_oracle_chol_block_equals_full_factor(no, nu):
    """chol_block (LinearAlgebra.cpp:254-299) on a well-conditioned matrix: the block factor is the Cholesky factor
    of the whole matrix (to rounding), no jitter is added and the fallback does not run."""
    rng = np.random.default_rng(7)
    X = rng.uniform(size=(no + nu, 3))
    C = O.build_R("matern5_2", X, np.array([0.3, 0.4, 0.5]), 1.0)
    Loo, _ = O.safe_chol_lower(C[:no, :no])
    L, inc, fb = O.chol_block(C, Loo)
    Lf, _ = O.safe_chol_lower(C)
    assert inc == 0 and not fb
    assert np.max(np.abs(L - np.tril(Lf))) < 1e-12
    assert np.max(np.abs(np.triu(L, 1))) == 0.0


def test_oracle_chol_block_jitters_the_schur_block_only():
    """A new point that duplicates an old one makes the Schur complement singular: safe_chol_lower's jitter goes on
    that block's diagonal (LinearAlgebra.cpp:286-297), so the old block of L is untouched."""
    rng = np.random.default_rng(8)
    Xo = rng.uniform(size=(30, 2))
    X = np.vstack([Xo, Xo[3:4]])
    C = O.build_R("gauss", X, np.array([0.4, 0.4]), 1.0)
    Loo, inc0 = O.safe_chol_lower(C[:30, :30])
    L, inc, fb = O.chol_block(C, Loo)
    assert not fb and inc >= 1
    assert np.array_equal(L[:30, :30], np.tril(Loo))
    Lf, incf = O.safe_chol_lower(C)  # the full factor would have jittered every diagonal entry
    assert incf >= 1


@pytest.mark.parametrize("mode", ["none", "nugget", "nugget_fixed"])
def test_full_baseline_evaluation_equals_oracle(mode):
    """oracle.baseline.eval_full (the timed CPU baseline, pair loops over all host threads) computes the oracle's
    LL exactly and its gradient up to the pair sums' order, for the three noise settings the benchmarks use."""
    from oracle import baseline as B
    rng = np.random.default_rng(21)
    n, d = 300, 4
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    th = rng.uniform(0.2, 1.0, size=d)
    if mode == "none":
        ll, g, _, _ = B.eval_full(X, y, th, "matern3_2")
        ll_o, g_o = O.OracleKriging(y, X, "matern3_2").log_likelihood(th)
    elif mode == "nugget":
        a = 1.0 / (1.0 + 1e-6)
        ll, g, _, _ = B.eval_full(X, y, th, "matern5_2", alpha=a)
        ll_o, g_o = O.OracleKriging(y, X, "matern5_2", noise_model="nugget").log_likelihood(np.r_[th, a])
    else:
        s2, nu = 0.8, 0.8e-8
        a = s2 / (s2 + nu)
        ll, g, _, _ = B.eval_full(X, y, th, "gauss", alpha=a, fixed_var=(s2, nu))
        ora = O.OracleKriging(y, X, "gauss", noise_model="nugget", est_sigma2=False, sigma2=s2, est_nugget=False,
                              nugget=nu)
        ll_o, g_o = ora.log_likelihood(th)
        g_o = g_o[:d]
        g = g[:d]
    assert ll == ll_o
    # the fixed-variance gradient is a difference of two large pair sums (cond(R) ~ 1e9 here): summation order
    # alone moves it by ~1e-9 relative
    tol = 1e-8 if mode == "nugget_fixed" else 1e-12
    assert np.max(np.abs(g - g_o)) <= tol * np.max(np.abs(g_o))
