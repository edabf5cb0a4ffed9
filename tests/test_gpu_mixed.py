"""GPU mixed path: the split-bf16 tensor-core products (error-free digit splitting) against FP64, and the mixed
likelihood against the FP64 path and the oracle.  Targets from the headline configuration: |dLL|/|LL| <= 1e-8 and
gradient relative error <= 1e-6 versus FP64."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _emulated(lk, A, B, S):
    M, K = A.shape
    N = B.shape[0]
    A = np.asfortranarray(A)
    B = np.asfortranarray(B)
    C = np.zeros((M, N), order="F")
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lk.load().lkg_ozaki_gemm_check(M, N, K, A.ctypes.data_as(dp), B.ctypes.data_as(dp), S, C.ctypes.data_as(dp))
    assert rc == 0
    return C


@pytest.mark.parametrize("S", [7, 8])
@pytest.mark.parametrize("shape", [(64, 64, 64), (200, 130, 257), (129, 300, 64)])
def test_emulated_gemm_is_fp64_accurate(gpu_lib, S, shape):
    """7-bit digits, 8 of them for S >= 7: 56-bit operands."""
    M, N, K = shape
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.standard_normal((N, K))
    C = _emulated(gpu_lib, A, B, S)
    ref = A @ B.T
    # error bound relative to |A||B|^T (the natural scale of an FP64 product)
    scale = np.abs(A) @ np.abs(B).T
    err = np.max(np.abs(C - ref) / scale)
    assert err < 4e-15, err


def test_emulated_gemm_fewer_slices_degrades_gracefully(gpu_lib):
    """Every 7-bit digit dropped costs accuracy: slices 4 .. 7 -> 5 .. 8 digits (35 .. 56-bit operands)."""
    rng = np.random.default_rng(1)
    A, B = rng.standard_normal((64, 128)), rng.standard_normal((64, 128))
    ref = A @ B.T
    scale = np.abs(A) @ np.abs(B).T
    errs = [np.max(np.abs(_emulated(gpu_lib, A, B, S) - ref) / scale) for S in (4, 5, 6, 7)]
    assert errs[0] > errs[1] > errs[2] > errs[3]
    assert errs[0] < 2.0 ** -28


def _config2_like(n, d=8, seed=123):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = rng.uniform(0.2, 1.5, size=d)
    return X, y, theta


@pytest.mark.parametrize("n", [640, 2048])
def test_mixed_loglik_vs_fp64(gpu_lib, n):
    X, y, theta = _config2_like(n)
    alpha = 1.0 / (1.0 + 1e-6)
    g = np.concatenate([theta, [alpha]])
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    ll64, g64, _ = k.logLikelihoodFun(g, True)
    k.set_precision(7)
    llm, gm, _ = k.logLikelihoodFun(g, True)
    assert k.last_slices() == 7
    assert rel_err(llm, ll64) <= 1e-8, (llm, ll64)
    assert rel_err(gm, g64) <= 1e-6, (gm, g64)
    if n <= 640:
        ll_o, g_o = O.OracleKriging(y, X, "matern5_2", noise_model="nugget").log_likelihood(g)
        assert rel_err(llm, ll_o) <= 1e-8
        assert rel_err(gm, g_o) <= 1e-6


def test_mixed_batch_matches_single(gpu_lib):
    X, y, _ = _config2_like(300, d=6)
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": np.full((1, 6), 0.3)})
    k.set_precision(7)
    thetas = np.random.default_rng(2).uniform(0.1, 0.4, size=(5, 6))
    ll_b, g_b = k.logLikelihoodFunBatch(thetas, True)
    for i in range(5):
        ll, g, _ = k.logLikelihoodFun(thetas[i], True)
        assert ll == ll_b[i]
        assert np.array_equal(g, g_b[i])


@pytest.mark.parametrize("n,ctas", [(1100, 8), (2048, 4), (3000, 16)])
def test_lookahead_factor_is_bit_identical(gpu_lib, n, ctas):
    """The look-ahead Cholesky (next panel factored on a second stream while the rest of the trailing update runs)
    performs the same operations per entry: LL and gradient equal, bit for bit, those without it."""
    lib = gpu_lib.load()
    X, y, theta = _config2_like(n)
    g = np.concatenate([theta, [1.0 / (1.0 + 1e-6)]])
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    k.set_precision(7)
    old = lib.lkg_get_lookahead()
    try:
        assert lib.lkg_set_lookahead(0) == 0
        ll0, g0, _ = k.logLikelihoodFun(g, True)
        assert lib.lkg_set_lookahead(ctas) == ctas
        ll1, g1, _ = k.logLikelihoodFun(g, True)
        ll2, g2, _ = k.logLikelihoodFun(g, True)
    finally:
        lib.lkg_set_lookahead(old)
    assert k.last_slices() == 7
    assert ll1 == ll0 and ll2 == ll0
    assert np.array_equal(g1, g0) and np.array_equal(g2, g0)
