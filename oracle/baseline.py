"""CPU baseline: the reference's LL + gradient evaluation path restated on the host cores, timed on bounded samples.

TEST / BENCH INFRASTRUCTURE ONLY (used by bench.py's CPU-baseline leg and its ``--impl reference`` arm).

The reference cannot be compiled here (its Armadillo / lbfgsb_cpp submodules are empty), so the baseline is the
oracle's restatement of the path the reference runs for one ``logLikelihoodFun(gamma, return_grad=true)``:

1. ``LinearAlgebra::cholCov`` pair loop, serial (src/lib/LinearAlgebra.cpp:150-155)       -> oracle C, 1 thread
2. ``arma::chol`` = LAPACK dpotrf, then ``rcond_chol`` = dtrcon                             -> OpenBLAS, all cores
3. ``inv_sympd`` = two triangular solves against the n x n identity (:708-710)            -> dtrsm, all cores
4. ``F* = L \\ F``, ``y* = L \\ y``, GLS, ``E* = L \\ (y - F b)``, ``x = L' \\ E*``         -> dtrsm / numpy
5. ``compute_ll_grad_theta_vecs`` pair loop, serial (src/lib/KrigingImpl.cpp:863-884)     -> oracle C, 1 thread

At the full problem size each stage is timed on a bounded sample and scaled by its exact work ratio:
stages 1 and 5 on the last rows of the pair loop (a fixed fraction of the n(n-1)/2 pairs), stage 3 on a block of
identity columns (dtrsm's work is linear in the number of right-hand sides), stages 2 and 4 in full.  Stage 5
reads R in place of R^-1 (the loop's cost does not depend on the values).  The dX cube of compute_dX (n^2 d
doubles) is not materialised: differences are recomputed per pair with the same subtraction.
"""
from __future__ import annotations

import os
import time

import numpy as np
from scipy.linalg import blas, lapack

from . import oracle as O


def _dp(a):
    return O._dp(a)


def dense_eval_sample(X, y, theta, factor=1.0, kernel="matern5_2", pair_fraction=0.125, rhs_fraction=1.0 / 16):
    """Time one reference-restated LL+gradient evaluation.  Returns (seconds_scaled, detail dict)."""
    X = O._colmajor(X)
    n, d = X.shape
    th = np.ascontiguousarray(theta, dtype=np.float64)
    L_ = O.lib()
    kid = O.KERNELS[kernel]
    # set-up (not timed): the full covariance matrix, built over all host threads
    R = np.empty((n, n), order="F")
    L_.ora_build_R_parallel(kid, n, d, _dp(X), _dp(th), float(factor), _dp(R))
    total_pairs = n * (n - 1) / 2.0
    i0 = int(n * np.sqrt(1.0 - pair_fraction))
    sample_pairs = (n * (n - 1) - i0 * (i0 - 1)) / 2.0
    scale_pairs = total_pairs / sample_pairs
    st = {}
    # 1. covariance pair loop (rows i0..n), scaled; then R *= factor and the diagonal
    Rw = np.empty((n, n), order="F")
    t = time.perf_counter()
    L_.ora_build_R_rows(kid, n, d, _dp(X), _dp(th), i0, n, _dp(Rw))
    st["cov_pairs"] = (time.perf_counter() - t) * scale_pairs
    del Rw
    t = time.perf_counter()
    R *= 1.0  # the in-place scaling pass of "R *= factor" (factor already applied in the set-up build)
    R[np.diag_indices(n)] = 1.0
    st["cov_scale_diag"] = time.perf_counter() - t
    # 2. dpotrf + dtrcon
    t = time.perf_counter()
    Lf, info = lapack.dpotrf(R, lower=1, clean=1, overwrite_a=0)
    rc, _ = lapack.dtrcon(Lf, norm="1", uplo="L", diag="N")
    st["chol_rcond"] = time.perf_counter() - t
    if info != 0:
        raise RuntimeError("CPU baseline: dpotrf failed (info=%d)" % info)
    # 3. inv_sympd on a block of identity columns, scaled
    w = max(1, int(n * rhs_fraction))
    E = np.zeros((n, w), order="F")
    E[np.arange(w), np.arange(w)] = 1.0
    t = time.perf_counter()
    Z = blas.dtrsm(1.0, Lf, E, side=0, lower=1, trans_a=0, diag=0)
    Z = blas.dtrsm(1.0, Lf, Z, side=0, lower=1, trans_a=1, diag=0)
    st["inv_sympd"] = (time.perf_counter() - t) * (n / w)
    del E, Z
    # 4. whitening, GLS, residual, x
    t = time.perf_counter()
    F = np.ones((n, 1), order="F")
    Fs = blas.dtrsm(1.0, Lf, F, side=0, lower=1)
    ys = blas.dtrsm(1.0, Lf, np.asfortranarray(y.reshape(-1, 1)), side=0, lower=1)[:, 0]
    G = Fs.T @ Fs
    beta = np.linalg.solve(G, Fs.T @ ys)
    Es = blas.dtrsm(1.0, Lf, np.asfortranarray((y - F @ beta).reshape(-1, 1)), side=0, lower=1)[:, 0]
    sse = float(Es @ Es)
    x = blas.dtrsm(1.0, Lf, np.asfortranarray(Es.reshape(-1, 1)), side=0, lower=1, trans_a=1)[:, 0]
    logdet = 2.0 * np.sum(np.log(np.diag(Lf)))
    st["solves_gls"] = time.perf_counter() - t
    # 5. gradient pair loop (rows i0..n), scaled
    t1 = np.zeros(d)
    t2 = np.zeros(d)
    t = time.perf_counter()
    L_.ora_grad_terms_rows(kid, n, d, _dp(X), _dp(th), _dp(R), _dp(R), _dp(np.ascontiguousarray(x)), i0, n, _dp(t1),
                           _dp(t2))
    st["grad_pairs"] = (time.perf_counter() - t) * scale_pairs
    total = sum(st.values())
    detail = dict(stages_s=st, n=n, d=d, pair_fraction=sample_pairs / total_pairs, rhs_fraction=w / n,
                  sse=sse, logdet=logdet, rcond=float(rc), blas_threads=blas_threads(), host_cores=os.cpu_count())
    return total, detail


def blas_threads():
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
        v = os.environ.get(var)
        if v:
            try:
                return int(v)
            except ValueError:
                pass
    return os.cpu_count()
