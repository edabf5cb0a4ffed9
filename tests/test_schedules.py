"""CPU checks of two algebraic forms the GPU kernels rely on (no GPU, no library call).

1. k_oz7_split (csrc/ozaki7.cu) writes the balanced base-128 digits of V = round(x 2^(7 S - e)) in closed form:
   U = V + 64 (1 + 128 + ... + 128^(S-2)), digit k (least significant first) = ((U >> 7 k) & 127) - 64 for k < S - 1,
   top digit = U >> 7 (S - 1).  It must equal the digit-by-digit form (d = ((V + 64) & 127) - 64, V = (V - d) >> 7) for
   every |V| <= 2^(7 S - 1), and the bf16 bit pattern of a digit comes from FP32 arithmetic (1.5 2^23 + d - 1.5 2^23).
2. k_trsv_step (csrc/dense_fp64.cu) solves L X = B (and L^T X = B) with one launch per 64-row block: the update CTAs
   of step k form X_k = D_k^-1 B_k from the untouched B_k and update the rows below (above), while one CTA writes the
   previous step's block in place.  Run sequentially, that schedule must give the triangular solve.
"""
import random
import struct

import numpy as np
import pytest

NB = 64


def _digits_iterative(V, S):
    out = [0] * S
    for i in range(S - 1, -1, -1):
        d = V
        if i > 0:
            d = ((V + 64) & 127) - 64
            V = (V - d) >> 7
        out[i] = d
    return out


def _digits_closed(V, S):
    C = 64 * ((1 << (7 * (S - 1))) - 1) // 127
    U = V + C
    out = [0] * S
    for k in range(S):
        out[S - 1 - k] = ((U >> (7 * k)) & 127) - 64 if k < S - 1 else U >> (7 * k)
    return out


@pytest.mark.parametrize("S", [5, 6, 7, 8])
def test_closed_form_digits_equal_iterative(S):
    rng = random.Random(S)
    lim = 1 << (7 * S - 1)
    cases = [0, 1, -1, 63, 64, -64, -65, 127, 128, -128, lim - 1, -(lim - 1), lim, -lim]
    cases += [rng.randrange(-lim, lim + 1) for _ in range(20000)]
    for V in cases:
        d = _digits_closed(V, S)
        assert d == _digits_iterative(V, S), V
        assert all(-64 <= x <= 64 for x in d), V
        assert sum(x * 128 ** (S - 1 - i) for i, x in enumerate(d)) == V


def _f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", float(np.float32(x))))[0]


def test_bf16_pattern_of_small_digits():
    magic = np.float32(12582912.0)  # 1.5 2^23, bit pattern 0x4B400000
    for d in range(-64, 65):
        f = np.frombuffer(struct.pack("<I", (0x4B400000 + d) & 0xFFFFFFFF), dtype=np.float32)[0]
        got = _f32_bits(np.float32(f - magic)) >> 16
        assert got == _f32_bits(d) >> 16, d
        assert _f32_bits(d) & 0xFFFF == 0  # the value is exact in bf16


def _dinv_blocks(L):
    n = L.shape[0]
    out = []
    for k0 in range(0, n, NB):
        nb = min(NB, n - k0)
        D = np.zeros((NB, NB))
        D[:nb, :nb] = np.linalg.inv(L[k0:k0 + nb, k0:k0 + nb])
        out.append(D)
    return out


def _solve_steps(L, Dinv, B, trans):
    n = L.shape[0]
    nblk = -(-n // NB)
    B = B.copy()
    steps = range(nblk + 1) if not trans else range(nblk - 1, -2, -1)
    for k in steps:
        upd = 0 <= k < nblk
        kw = (k - 1) if not trans else (k + 1 if k + 1 < nblk else -1)
        if upd:
            k0 = k * NB
            nb = min(NB, n - k0)
            if not trans:
                X = Dinv[k][:nb, :nb] @ B[k0:k0 + nb]
                B[k0 + nb:] -= L[k0 + nb:, k0:k0 + nb] @ X
            else:
                X = Dinv[k][:nb, :nb].T @ B[k0:k0 + nb]
                B[:k0] -= L[k0:k0 + nb, :k0].T @ X
        if kw >= 0:  # the writer: no update of this step touches block kw
            w0 = kw * NB
            nbw = min(NB, n - w0)
            D = Dinv[kw][:nbw, :nbw]
            B[w0:w0 + nbw] = (D.T if trans else D) @ B[w0:w0 + nbw]
    return B


@pytest.mark.parametrize("n,r", [(1, 1), (63, 2), (64, 1), (65, 3), (200, 2), (256, 16)])
def test_one_launch_per_block_solve_schedule(n, r):
    rng = np.random.default_rng(n + r)
    A = rng.standard_normal((n, n))
    L = np.linalg.cholesky(A @ A.T + n * np.eye(n))
    B = rng.standard_normal((n, r))
    Dinv = _dinv_blocks(L)
    np.testing.assert_allclose(_solve_steps(L, Dinv, B, False), np.linalg.solve(L, B), rtol=0, atol=1e-12)
    np.testing.assert_allclose(_solve_steps(L, Dinv, B, True), np.linalg.solve(L.T, B), rtol=0, atol=1e-12)
