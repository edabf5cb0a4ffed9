"""The tcgen05 kernels of the mixed path's digit products (ozaki_tc.cu) against FP64 and against the mma.sync
kernels: the same exact digit arithmetic, so the results agree to the last rounding of the per-chunk folds (bit for
bit where both fold alike)."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _emulated(lk, A, B, S):
    M, K = A.shape
    N = B.shape[0]
    A = np.asfortranarray(A)
    B = np.asfortranarray(B)
    C = np.zeros((M, N), order="F")
    dp = ctypes.POINTER(ctypes.c_double)
    rc = lk.load().lkg_ozaki_gemm_check(M, N, K, A.ctypes.data_as(dp), B.ctypes.data_as(dp), S, C.ctypes.data_as(dp))
    assert rc == 0, lk._lib.last_error()
    return C


@pytest.fixture
def tensor_path(gpu_lib):
    lib = gpu_lib.load()
    old = lib.lkg_get_tensor_path()
    yield lib
    lib.lkg_set_tensor_path(old)


@pytest.mark.parametrize("S", [4, 6, 7, 8])
@pytest.mark.parametrize("shape", [(64, 64, 64), (200, 130, 257), (129, 300, 64), (384, 256, 512)])
def test_tc_gemm_matches_fp64_and_mma_sync(gpu_lib, tensor_path, S, shape):
    M, N, K = shape
    rng = np.random.default_rng(M + N + K + S)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.standard_normal((N, K))
    assert tensor_path.lkg_set_tensor_path(0) == 0
    C_sync = _emulated(gpu_lib, A, B, S)
    assert tensor_path.lkg_set_tensor_path(1) == 1
    C_tc = _emulated(gpu_lib, A, B, S)
    scale = np.abs(A) @ np.abs(B).T
    if K <= 64 and S == 8:  # the single-stage kernel folds exactly as the mma.sync kernel does
        assert np.array_equal(C_tc, C_sync)
    else:  # the pipelined kernel rounds the chunk's exact value once instead of twice
        assert np.max(np.abs(C_tc - C_sync) / scale) < 1e-15
    if S >= 7:
        err = np.max(np.abs(C_tc - A @ B.T) / scale)
        assert err < (4e-15 if S == 7 else 2e-15), err


@pytest.mark.parametrize("S", [4, 6, 7])
@pytest.mark.parametrize("shape", [(64, 64, 64), (200, 130, 257), (129, 300, 64), (384, 256, 512), (300, 70, 1000)])
def test_oz7_gemm_matches_fp64(gpu_lib, tensor_path, S, shape):
    """Tensor path 3: 7-bit digits with one exponent per 256-wide k block; several k blocks are summed in FP64.
    S = 7 slices -> 8 digits (56-bit operands) reaches FP64-level products, S = 6 -> 7 digits (49 bits), S = 4 -> 5
    digits (35 bits) the precision of the triangular inverse and W^T W."""
    M, N, K = shape
    rng = np.random.default_rng(M + N + K + S)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.standard_normal((N, K))
    assert tensor_path.lkg_set_tensor_path(3) == 3
    C = _emulated(gpu_lib, A, B, S)
    scale = np.abs(A) @ np.abs(B).T
    err = np.max(np.abs(C - A @ B.T) / scale)
    assert err < {7: 4e-15, 6: 5e-13, 4: 2e-9}[S], err  # 2^-(7 S - 1) per operand, times the in-block spread


def _config2_like(n, d=8, seed=123):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    theta = rng.uniform(0.2, 1.5, size=d)
    return X, y, theta


@pytest.mark.parametrize("path", [1, 2, 3])
@pytest.mark.parametrize("n", [640, 2048, 1000])
def test_tc_mixed_loglik(gpu_lib, tensor_path, n, path):
    X, y, theta = _config2_like(n)
    alpha = 1.0 / (1.0 + 1e-6)
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    g = np.concatenate([theta, [alpha]])
    k.set_precision(0)
    ll64, g64, _ = k.logLikelihoodFun(g, True)
    k.set_precision(7)
    tensor_path.lkg_set_tensor_path(0)
    ll_s, g_s, _ = k.logLikelihoodFun(g, True)
    tensor_path.lkg_set_tensor_path(path)
    ll_t, g_t, _ = k.logLikelihoodFun(g, True)
    assert abs(ll_t - ll64) / abs(ll64) < 1e-8
    assert rel_err(g_t, g64) < 1e-6
    if path < 3:  # the same digits as the mma.sync kernels
        assert abs(ll_t - ll_s) / abs(ll_s) < 1e-12
        assert rel_err(g_t, g_s) < 1e-10
