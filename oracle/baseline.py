"""CPU baseline: the reference's LL + gradient evaluation path restated on the host cores, timed in full.

TEST / BENCH INFRASTRUCTURE ONLY (used by bench.py's CPU-baseline legs and its ``--impl reference`` arm).

The reference cannot be compiled here (its Armadillo / lbfgsb_cpp submodules are empty), so the baseline is the
oracle's restatement of the path the reference runs for one ``logLikelihoodFun(gamma, return_grad=true)``, every
stage at the full problem size (nothing sampled, nothing scaled):

1. ``LinearAlgebra::cholCov`` pair loop (src/lib/LinearAlgebra.cpp:150-161)               -> oracle C, `threads`
2. ``arma::chol`` = LAPACK dpotrf, then ``rcond_chol`` = dtrcon (:43-115)                  -> OpenBLAS, all cores
3. ``inv_sympd`` = two triangular solves against the n x n identity (:708-710)            -> dtrtrs, all cores
4. ``F* = L \\ F``, ``y* = L \\ y``, GLS, ``E* = L \\ (y - F b)`` (src/lib/KrigingImpl.cpp:73-125)
5. the nugget alpha terms (src/lib/Kriging.cpp:307-326) and ``x = L' \\ E*``
6. ``compute_ll_grad_theta_vecs`` pair loop (src/lib/KrigingImpl.cpp:855-885)            -> oracle C, `threads`

The reference runs the two pair loops in one thread; here they run over `threads` OpenMP threads with the identical
per-pair arithmetic (a stronger baseline than the reference as built).  The dX cube of compute_dX (n^2 d doubles,
17 GB at n = 16384, d = 8) is not materialised: differences are recomputed per pair with the same subtraction.
The LL and gradient it returns are the oracle's values at the full size (the gradient's pair sums in per-thread
order, equal to the serial loop's up to summation order).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np
from scipy.linalg import lapack

from . import oracle as O


def _dp(a):
    return O._dp(a)


def host_threads():
    """Threads the CPU legs use: OMP_NUM_THREADS when set, else every host core."""
    v = os.environ.get("OMP_NUM_THREADS")
    if v:
        try:
            return max(1, int(v))
        except ValueError:
            pass
    return os.cpu_count() or 1


def eval_full(X, y, theta, kernel="matern5_2", alpha=None, fixed_var=None, threads=None, with_grad=True):
    """One reference-restated ``logLikelihoodFun`` evaluation with constant trend, timed per stage
    (Kriging.cpp:214-341):

    * ``alpha=None``: NoiseModel None, sigma2 estimated (gamma = theta);
    * ``alpha`` given, ``fixed_var=None``: Nugget mode with sigma2 and nugget estimated (gamma = [theta, alpha]);
    * ``alpha`` and ``fixed_var=(sigma2, nugget)``: Nugget mode with both fixed (alpha = sigma2 / (sigma2 + nugget),
      the alpha-gradient is zero).

    Returns (ll, grad, seconds, detail)."""
    threads = threads or host_threads()
    X = O._colmajor(X)
    y = np.ascontiguousarray(y, dtype=np.float64)
    n, d = X.shape
    th = np.ascontiguousarray(theta, dtype=np.float64)
    L_ = O.lib()
    kid = O.KERNELS[kernel]
    factor = 1.0 if alpha is None else float(alpha)
    st = {}
    t_all = time.perf_counter()
    # 1. covariance build: R(i, j) = factor * Cov(x_i - x_j) off the diagonal, 1 on it
    t = time.perf_counter()
    R = np.empty((n, n), order="F")
    L_.ora_build_R_mt(kid, n, d, _dp(X), _dp(th), factor, None, _dp(R), int(threads))
    st["cov_pairs"] = time.perf_counter() - t
    # 2. safe_chol_lower: dpotrf + dtrcon (and the nugget retries, if any)
    t = time.perf_counter()
    L, inc = O.safe_chol_lower(R)
    st["chol_rcond"] = time.perf_counter() - t
    # 3. inv_sympd as coded: two full triangular solves against I
    Rinv = None
    if with_grad:
        t = time.perf_counter()
        Rinv = O.inv_sympd(L)
        st["inv_sympd"] = time.perf_counter() - t
    # 4. whitening, GLS, residual
    t = time.perf_counter()
    F = np.ones((n, 1), order="F")
    Fstar = O.solve_lower(L, F)
    ystar = O.solve_lower(L, y.reshape(-1, 1))[:, 0]
    Rstar, info = lapack.dpotrf(Fstar.T @ Fstar, lower=0, clean=1)
    if info != 0:
        raise RuntimeError("CPU baseline: chol(F*'F*) failed")
    rhs = Fstar.T @ ystar
    beta = lapack.dtrtrs(Rstar, lapack.dtrtrs(Rstar, rhs.reshape(-1, 1), lower=0, trans=1)[0], lower=0)[0][:, 0]
    Estar = O.solve_lower(L, (y - F @ beta).reshape(-1, 1))[:, 0]
    sse = float(Estar @ Estar)
    logdet = 2.0 * float(np.sum(np.log(np.diag(L))))
    if alpha is None:
        var = sse / n
        ll = -0.5 * (n * math.log(2 * math.pi * var) + logdet + n)
    elif fixed_var is None:
        var = sse / n
        ll = -0.5 * (n * math.log(2 * math.pi * var) + logdet + sse / var)
    else:
        var = float(fixed_var[0]) + float(fixed_var[1])
        ll = -0.5 * (n * math.log(2 * math.pi * var) + logdet + sse / var)
    st["solves_gls"] = time.perf_counter() - t
    grad = None
    if with_grad:
        # 5. x = L' \ E* and, for the estimated nugget, the alpha terms
        t = time.perf_counter()
        x = np.ascontiguousarray(O.solve_upper_t(L, Estar.reshape(-1, 1))[:, 0])
        out = np.zeros(2)
        if alpha is not None and fixed_var is None:
            L_.ora_alpha_terms_mt(n, _dp(R), _dp(Rinv), _dp(x), factor, 0.0, _dp(out), int(threads))
        st["solve_x_alpha_terms"] = time.perf_counter() - t
        # 6. gradient pair loop
        t = time.perf_counter()
        t1 = np.zeros(d)
        t2 = np.zeros(d)
        L_.ora_grad_terms_mt(kid, n, d, _dp(X), _dp(th), _dp(R), _dp(Rinv), _dp(x), _dp(t1), _dp(t2), int(threads))
        st["grad_pairs"] = time.perf_counter() - t
        grad = np.zeros(d + (0 if alpha is None else 1))
        grad[:d] = (t1 / var + t2) / 2.0
        if alpha is not None and fixed_var is None:
            grad[d] = -0.5 * (-out[0] / var + out[1])
    total = time.perf_counter() - t_all
    detail = dict(stages_s={k: round(v, 4) for k, v in st.items()}, n=n, d=d, threads=int(threads),
                  blas_threads=blas_threads(), host_cores=os.cpu_count(), nugget_increments=int(inc))
    return ll, grad, total, detail


def blas_threads():
    for var in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS"):
        v = os.environ.get(var)
        if v:
            try:
                return int(v)
            except ValueError:
                pass
    return os.cpu_count()


def predict_group_full(X, y, theta, kernel, beta0, Xq):
    """One submodel's part of a PoE-family prediction as the reference computes it (KrigingImpl.cpp:145-251, constant
    trend with a given beta, NestedKriging.cpp:364-422 per group): R = C(X, X), L = chol(R), R_on = C(X, Xq),
    Rstar_on = L \\ R_on, mean = beta + Rstar_on' z and variance 1 - colsum(Rstar_on^2).  Timed in full (the
    triangular solve with OpenBLAS on all cores).  Returns (mean, variance, seconds)."""
    X = O._colmajor(X)
    Xq = O._colmajor(Xq)
    y = np.ascontiguousarray(y, dtype=np.float64)
    t = time.perf_counter()
    R = O.build_R(kernel, X, theta)
    L, _ = O.safe_chol_lower(R)
    z = O.solve_lower(L, (y - beta0).reshape(-1, 1))[:, 0]
    Ron = O.cov_cross(kernel, X, Xq, theta)
    Rs = O.solve_lower(L, Ron)
    mean = beta0 + Rs.T @ z
    var = 1.0 - np.sum(Rs * Rs, axis=0)
    return mean, var, time.perf_counter() - t


def predict_vecchia_sample(kernel, X, resid, theta, sigma2, Xq, m=30, threads=None, num_nugget=None):
    """Kriging::predictVecchia's per-point work as the reference runs it (Kriging.cpp:950-1022): squared distances to
    every observation, a partial selection of the m nearest (std::nth_element there, numpy's argpartition here), the
    m x m local kriging system through the oracle's safe_chol_lower, mean and stdev; the points spread over `threads`
    host threads (the reference's OpenMP loop over points).  num_nugget: the jitter of the local systems (the
    numerical nugget of LinearAlgebra::set_num_nugget; the oracle's configuration when None).  Returns (mean without
    the trend, stdev, seconds)."""
    import dataclasses
    from concurrent.futures import ThreadPoolExecutor
    X = np.ascontiguousarray(X, dtype=np.float64)
    Xq = np.atleast_2d(np.asarray(Xq, dtype=np.float64))
    theta = np.asarray(theta, dtype=np.float64)
    threads = threads or host_threads()
    q = Xq.shape[0]
    mean, sd = np.empty(q), np.empty(q)
    cfg = O.CONFIG if num_nugget is None else dataclasses.replace(O.CONFIG, num_nugget=float(num_nugget))

    def one(t):
        s = ((X - Xq[t]) ** 2).sum(axis=1)
        nb = np.argpartition(s, m)[:m]
        RN = O.cov_cross(kernel, X[nb], X[nb], theta)
        RN[np.diag_indices(m)] = 1.0 + cfg.num_nugget
        r = O.cov_cross(kernel, X[nb], Xq[t:t + 1], theta)[:, 0]
        LN, _ = O.safe_chol_lower(RN, cfg)
        a = O.solve_upper_t(LN, O.solve_lower(LN, r.reshape(-1, 1)))[:, 0]
        mean[t] = a @ resid[nb]
        sd[t] = math.sqrt(sigma2 * max(0.0, 1.0 - r @ a))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, range(q)))
    return mean, sd, time.perf_counter() - t0
