"""The mixed path's digit-product kernel (ozaki7.cu: tcgen05 on 7-bit digits, 128 x 32 tiles, two TMEM accumulator
sets) against FP64 products, and the mixed likelihood it drives against the FP64 path."""
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


def test_tensor_path_is_the_7bit_kernel(gpu_lib):
    lib = gpu_lib.load()
    assert lib.lkg_get_tensor_path() == 3
    assert lib.lkg_set_tensor_path(3) == 3
    assert lib.lkg_set_tensor_path(1) == -1


@pytest.mark.parametrize("S", [4, 6, 7])
@pytest.mark.parametrize("shape", [(64, 64, 64), (200, 130, 257), (129, 300, 64), (384, 256, 512), (300, 70, 1000)])
def test_oz7_gemm_matches_fp64(gpu_lib, S, shape):
    """Tensor path 3: 7-bit digits with one exponent per 256-wide k block; several k blocks are summed in FP64.
    S = 7 slices -> 8 digits (56-bit operands) reaches FP64-level products, S = 6 -> 7 digits (49 bits), S = 4 -> 5
    digits (35 bits) the precision of the triangular inverse and W^T W."""
    M, N, K = shape
    rng = np.random.default_rng(M + N + K + S)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.standard_normal((N, K))
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


@pytest.mark.parametrize("n", [640, 2048, 1000])
def test_mixed_loglik_matches_fp64(gpu_lib, n):
    X, y, theta = _config2_like(n)
    alpha = 1.0 / (1.0 + 1e-6)
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    g = np.concatenate([theta, [alpha]])
    k.set_precision(0)
    ll64, g64, _ = k.logLikelihoodFun(g, True)
    k.set_precision(7)
    ll_t, g_t, _ = k.logLikelihoodFun(g, True)
    assert k.last_slices() == 7
    assert abs(ll_t - ll64) / abs(ll64) < 1e-8
    assert rel_err(g_t, g64) < 1e-6


@pytest.mark.parametrize("tn", [32, 64])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_both_tile_widths_give_identical_products(gpu_lib, tn, mode):
    """The 128 x 32 tiles (two accumulator sets) and the 128 x 64 tiles (one set) compute every output from the same
    exact diagonal sums with the same single rounding, so the products agree bit for bit -- for the rectangular,
    the lower (A A^T) and the W^T W forms, over several k blocks."""
    lib = gpu_lib.load()
    rng = np.random.default_rng(5 + mode)
    M, N, K = 300, 200, 700
    A = rng.standard_normal((M, K))
    if mode == 2:
        A = np.tril(rng.standard_normal((M, M)))
    B = rng.standard_normal((N, K))
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    out = {}
    old = lib.lkg_get_digit_tile()
    try:
        for t in (32, 64):
            assert lib.lkg_set_digit_tile(t) == t
            n_out = M if mode else N
            C = np.zeros((M, n_out), order="F")
            where = np.zeros(8, dtype=np.int32)
            Af, Bf = np.asfortranarray(A), np.asfortranarray(B)
            rc = lib.lkg_oz7_mode_check(mode, M, N, K, Af.ctypes.data_as(dp), Bf.ctypes.data_as(dp), 8,
                                        C.ctypes.data_as(dp), where.ctypes.data_as(ip))
            assert rc == 0, (rc, where)
            out[t] = C
    finally:
        lib.lkg_set_digit_tile(old)
    assert np.array_equal(out[32], out[64])
