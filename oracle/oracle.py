"""CPU FP64 oracle for the libKriging likelihood hot path.

TEST INFRASTRUCTURE ONLY: this module is the reference restatement the GPU results are compared with.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it; the product package never
does.  It restates the reference's algorithm in the reference's operation order:

* pair loops (covariance build, gradient loop, Vecchia conditionals) in C: ``oracle/lk_oracle.c``;
* dense linear algebra through LAPACK (scipy's bundled OpenBLAS), mirroring Armadillo's calls:
  ``arma::chol`` -> dpotrf, ``arma::rcond`` on a triangular factor -> dtrcon('1'),
  ``arma::solve(trimatl/trimatu(..), B)`` -> dtrtrs.

Reference routines restated here (paths relative to the libKriging source tree):

* ``safe_chol_lower``         src/lib/LinearAlgebra.cpp:43-98, ``rcond_chol`` :106-115
* ``populate_model``          src/lib/KrigingImpl.cpp:73-125, src/lib/LinearAlgebra.cpp:142-204, :695-714
* ``OracleKriging.log_likelihood``  src/lib/Kriging.cpp:214-341 (all NoiseModel None / Nugget branches)
* ``regression_matrix``       src/lib/Trend.cpp:34-91
* ``theta_bounds``            src/lib/Optim.cpp:179-209
* ``OracleKriging.predict``   src/lib/KrigingImpl.cpp:145-251 (mean / stdev), src/lib/Kriging.cpp:2240-2285
* ``vecchia_*``               src/lib/Kriging.cpp:736-924 (through the C restatement)

Parity pin: ``tests/golden/loglik_golden.json`` (the reference's tests/references/data2-grad-*, data1-scal
known answers, checked at 1e-12 relative in tests/test_oracle.py).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
from scipy.linalg import lapack

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SO = BUILD / "liblk_oracle.so"

KERNELS = {"gauss": 0, "exp": 1, "matern3_2": 2, "matern5_2": 3}


def build(force: bool = False) -> Path:
    """Compile lk_oracle.c into oracle/_build/liblk_oracle.so (gcc, no FMA contraction)."""
    src = HERE / "lk_oracle.c"
    if SO.exists() and not force and SO.stat().st_mtime >= src.stat().st_mtime:
        return SO
    BUILD.mkdir(exist_ok=True)
    tmp = SO.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", str(tmp), str(src),
                           "-lm"])
    os.replace(tmp, SO)
    return SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(SO))
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.ora_cov.restype = ctypes.c_double
        L.ora_cov.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int]
        L.ora_dlncov.restype = None
        L.ora_dlncov.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, dp]
        L.ora_build_R.restype = None
        L.ora_build_R.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double, dp, dp]
        L.ora_cov_cross.restype = None
        L.ora_cov_cross.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp]
        L.ora_grad_terms.restype = None
        L.ora_grad_terms.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp]
        L.ora_build_R_rows.restype = None
        L.ora_build_R_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int,
                                       dp]
        L.ora_build_R_parallel.restype = None
        L.ora_build_R_parallel.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double, dp]
        L.ora_grad_terms_rows.restype = None
        L.ora_grad_terms_rows.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_int,
                                          ctypes.c_int, dp, dp]
        L.ora_build_R_mt.restype = None
        L.ora_build_R_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, ctypes.c_double, dp, dp,
                                     ctypes.c_int]
        L.ora_grad_terms_mt.restype = None
        L.ora_grad_terms_mt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp,
                                        ctypes.c_int]
        L.ora_alpha_terms_mt.restype = None
        L.ora_alpha_terms_mt.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp,
                                         ctypes.c_int]
        L.ora_alpha_terms.restype = None
        L.ora_alpha_terms.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp]
        L.ora_vecchia_sets.restype = None
        L.ora_vecchia_sets.argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ip, ip]
        L.ora_set_rcond_check.restype = None
        L.ora_set_rcond_check.argtypes = [ctypes.c_int, ctypes.c_double]
        L.ora_vecchia_points_sample.restype = ctypes.c_int
        L.ora_vecchia_points_sample.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                                                dp, ip, ip, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                                ctypes.c_int]
        L.ora_vecchia_ll.restype = ctypes.c_double
        L.ora_vecchia_ll.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, ip, ip,
                                     ctypes.c_int, ctypes.c_double, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _colmajor(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


# --------------------------------------------------------------------------------------------------------------
# configuration statics (LinearAlgebra.cpp:33-63,100; Optim.cpp:39-139)
# --------------------------------------------------------------------------------------------------------------
@dataclass
class Config:
    num_nugget: float = 1e-10
    chol_rcond_check: bool = True
    min_rcond: float = 1e-18
    max_inc_choldiag: int = 10
    theta_lower_factor: float = 0.02
    theta_upper_factor: float = 10.0
    variogram_bounds_heuristic: bool = True


CONFIG = Config()


class CholeskyError(RuntimeError):
    pass


# --------------------------------------------------------------------------------------------------------------
# kernels and the covariance build
# --------------------------------------------------------------------------------------------------------------
def cov(kernel: str, dx, theta) -> float:
    dx = np.ascontiguousarray(dx, dtype=np.float64)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    return lib().ora_cov(KERNELS[kernel], _dp(dx), _dp(theta), dx.size)


def dlncov(kernel: str, dx, theta):
    dx = np.ascontiguousarray(dx, dtype=np.float64)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    out = np.empty(dx.size)
    lib().ora_dlncov(KERNELS[kernel], _dp(dx), _dp(theta), dx.size, _dp(out))
    return out


def dlncov_dx(kernel: str, dx, theta):
    """d ln Cov / d x at dx (Covariance.cpp:52-63 gauss, 90-100 exp, 132-145 matern3_2, 181-196 matern5_2), element by
    element in the reference's operation order."""
    out = np.empty(len(dx))
    s3, s5 = math.sqrt(3.0), math.sqrt(5.0)
    for i, (x, th) in enumerate(zip(dx, theta)):
        sg = 1.0 if x > 0 else (-1.0 if x < 0 else 0.0)
        if kernel == "gauss":
            out[i] = -x / (th * th)
        elif kernel == "exp":
            out[i] = -sg / th
        elif kernel == "matern3_2":
            t = s3 * abs(x / th)
            out[i] = -s3 * sg * t / (1.0 + t) / th
        else:
            t = s5 * abs(x / th)
            a, b = 1.0 + t, t / 3.0
            out[i] = -s5 * sg * (a * b) / (a + t * b) / th
    return out


def build_R(kernel: str, X, theta, factor: float = 1.0, diag=None):
    """cholCov's covariance build (LinearAlgebra.cpp:142-181): full symmetric n x n, column-major."""
    X = _colmajor(X)
    n, d = X.shape
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    R = np.empty((n, n), order="F")
    dg = None if diag is None else np.ascontiguousarray(diag, dtype=np.float64)
    lib().ora_build_R(KERNELS[kernel], n, d, _dp(X), _dp(theta), float(factor), _dp(dg), _dp(R))
    return R


def cov_cross(kernel: str, X1, X2, theta):
    """NestedKriging::corrMat (NestedKriging.cpp:101-115): Cov(x1_i - x2_j), n1 x n2, no coincidence rule."""
    X1, X2 = _colmajor(X1), _colmajor(X2)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    R = np.empty((X1.shape[0], X2.shape[0]), order="F")
    lib().ora_cov_cross(KERNELS[kernel], X1.shape[0], X2.shape[0], X1.shape[1], _dp(X1), _dp(X2), _dp(theta), _dp(R))
    return R


# --------------------------------------------------------------------------------------------------------------
# dense linear algebra (Armadillo -> LAPACK)
# --------------------------------------------------------------------------------------------------------------
def rcond_chol(L) -> float:
    """LinearAlgebra.cpp:106-115: arma::rcond on the (lower triangular) factor, squared."""
    rc, info = lapack.dtrcon(L, norm="1", uplo="L", diag="N")
    return float(rc) ** 2


def safe_chol_lower(A, cfg: Config = CONFIG):
    """LinearAlgebra.cpp:43-98: dpotrf; on failure or rcond^2 < min_rcond add num_nugget*10^k to the diagonal
    of a copy (cumulatively) and retry, k = 0..max_inc_choldiag.  Returns (L, increments used)."""
    X = np.array(A, order="F", dtype=np.float64, copy=True)
    inc = 0
    while True:
        L, info = lapack.dpotrf(X, lower=1, clean=1, overwrite_a=0)
        ok = info == 0
        wrong_rcond = cfg.chol_rcond_check
        if ok:
            wrong_rcond = wrong_rcond and (rcond_chol(L) < cfg.min_rcond)
        if not ok or wrong_rcond:
            if inc > cfg.max_inc_choldiag:
                raise CholeskyError("Exceed max numerical nugget (%d x 1e%g) added to force chol matrix"
                                    % (inc, math.log10(cfg.num_nugget)))
            if cfg.num_nugget <= 0.0:
                raise CholeskyError("Cannot add numerical nugget which is not strictly positive")
            X[np.diag_indices_from(X)] += cfg.num_nugget * 10.0 ** inc
            inc += 1
            continue
        return np.asfortranarray(L), inc


def predict_vecchia(kernel, X, y, F, beta, theta, sigma2, Xn, Fn, m, cfg: Config = CONFIG):
    """Kriging::predictVecchia (Kriging.cpp:950-1022) in normalised units: for each row of Xn the m nearest rows
    of X (ties of the squared distance broken by the lower index), RN = C(N, N) + num_nugget I through
    safe_chol_lower, a = RN^-1 r; mean = Fn beta + a . (y_N - F_N beta), stdev = sqrt(sigma2 max(0, 1 - r . a))."""
    X = np.asarray(X, dtype=np.float64)
    Xn = np.atleast_2d(np.asarray(Xn, dtype=np.float64))
    n = X.shape[0]
    m = min(m, n)
    resid = y - F @ beta
    mean = np.empty(Xn.shape[0])
    sd = np.empty(Xn.shape[0])
    for t in range(Xn.shape[0]):
        s = np.zeros(n)
        for k in range(X.shape[1]):
            dk = Xn[t, k] - X[:, k]
            s = s + dk * dk
        Ni = np.lexsort((np.arange(n), s))[:m]
        RN = cov_cross(kernel, X[Ni], X[Ni], theta)
        RN[np.diag_indices(m)] = 1.0 + cfg.num_nugget
        r = cov_cross(kernel, X[Ni], Xn[t:t + 1], theta)[:, 0]
        LN, _ = safe_chol_lower(RN, cfg)
        a = solve_upper_t(LN, solve_lower(LN, r.reshape(-1, 1)))[:, 0]
        mean[t] = Fn[t] @ beta + a @ resid[Ni]
        sd[t] = np.sqrt(sigma2 * max(0.0, 1.0 - r @ a))
    return mean, sd


def chol_block(C, Loo, cfg: Config = CONFIG):
    """LinearAlgebra::chol_block (LinearAlgebra.cpp:254-299): the factor of C given the factor Loo of its leading
    block.  Lou = Loo \\ C_ou, L_uo = Lou', L_uu = safe_chol_lower(C_uu - Lou' Lou) (the retry jitter lands on the
    Schur complement only); when that exceeds the retry budget, the whole C is factored instead.
    Returns (L, increments used by the accepted factorisation, True when the fallback ran)."""
    C = np.asarray(C, dtype=np.float64)
    n, no = C.shape[0], Loo.shape[0]
    Lou = solve_lower(Loo, np.asfortranarray(C[:no, no:]))
    L = np.zeros((n, n), order="F")
    L[:no, :no] = np.tril(Loo)
    L[no:, :no] = Lou.T
    try:
        Luu, inc = safe_chol_lower(C[no:, no:] - Lou.T @ Lou, cfg)
    except CholeskyError:
        Lf, inc = safe_chol_lower(C, cfg)
        return np.asfortranarray(np.tril(Lf)), inc, True
    L[no:, no:] = np.tril(Luu)
    return L, inc, False


def update_no_refit(kernel, X_old, L_old, X_new, y_all, F_all, theta, alpha=1.0, cfg: Config = CONFIG):
    """KrigingImpl::update_no_refit_impl with update_cholCov (LinearAlgebra.cpp:206-252) and populate_Model's GLS
    (KrigingImpl.cpp:73-125) in normalised units: R of the joined design (factor alpha off the diagonal, unit
    diagonal), L = chol_block(R, L_old), then F*, y*, R*, beta, E*, SSE.  Returns (KModel, fallback_used)."""
    X = np.vstack([np.asarray(X_old, dtype=np.float64), np.asarray(X_new, dtype=np.float64)])
    R = build_R(kernel, X, theta, alpha, None)
    L, inc, fb = chol_block(R, L_old, cfg)
    Fstar = solve_lower(L, F_all)
    ystar = solve_lower(L, y_all.reshape(-1, 1))[:, 0]
    FtF = Fstar.T @ Fstar
    if FtF.shape[0] > 0:
        Rstar, info = lapack.dpotrf(FtF, lower=0, clean=1)
        assert info == 0
        rhs = Fstar.T @ ystar
        beta = lapack.dtrtrs(Rstar, lapack.dtrtrs(Rstar, rhs.reshape(-1, 1), lower=0, trans=1)[0], lower=0)[0][:, 0]
    else:
        Rstar = np.zeros((0, 0))
        beta = np.zeros(0)
    Estar = solve_lower(L, (y_all - F_all @ beta).reshape(-1, 1))[:, 0]
    return KModel(R, L, None, Fstar, ystar, Rstar, beta, Estar, float(Estar @ Estar), inc), fb


def solve_lower(L, B):
    x, info = lapack.dtrtrs(L, np.asfortranarray(B, dtype=np.float64), lower=1, trans=0)
    assert info == 0
    return x


def solve_upper_t(L, B):
    """solve(trimatu(L.t()), B)."""
    x, info = lapack.dtrtrs(L, np.asfortranarray(B, dtype=np.float64), lower=1, trans=1)
    assert info == 0
    return x


def inv_sympd(L):
    """LinearAlgebra.cpp:708-710: solve(trimatu(L'), solve(trimatl(L), I)) -- two full triangular solves."""
    n = L.shape[0]
    return solve_upper_t(L, solve_lower(L, np.eye(n, order="F")))


# --------------------------------------------------------------------------------------------------------------
# trend, bounds
# --------------------------------------------------------------------------------------------------------------
def regression_matrix(regmodel: str, X):
    """Trend.cpp:34-91."""
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    cols = []
    if regmodel == "none":
        return np.zeros((n, 0), order="F")
    cols.append(np.ones(n))
    if regmodel == "constant":
        pass
    elif regmodel == "linear":
        cols += [X[:, i] for i in range(d)]
    elif regmodel == "interactive":
        for i in range(d):
            cols.append(X[:, i])
            for j in range(i):
                cols.append(X[:, i] * X[:, j])
    elif regmodel == "quadratic":
        for i in range(d):
            cols.append(X[:, i])
            for j in range(i + 1):
                cols.append(X[:, i] * X[:, j])
    else:
        raise ValueError("Cannot convert '%s' as a regression model" % regmodel)
    return np.asfortranarray(np.stack(cols, axis=1))


def regression_derivative(regmodel: str, x):
    """Trend.cpp:95-150: dF/dx at one point, d x p with DF[k, l] = d F_l / d x_k."""
    x = np.asarray(x, dtype=np.float64)
    d = x.size
    p = regression_matrix(regmodel, x.reshape(1, -1)).shape[1]
    DF = np.zeros((d, p))
    if regmodel in ("none", "constant"):
        return DF
    c = 1
    if regmodel == "linear":
        for i in range(d):
            DF[i, c] = 1.0
            c += 1
        return DF
    for i in range(d):
        DF[i, c] = 1.0
        c += 1
        for j in range(i + 1 if regmodel == "quadratic" else i):
            if i == j:
                DF[i, c] = 2.0 * x[i]
            else:
                DF[i, c] = x[j]
                DF[j, c] = x[i]
            c += 1
    return DF


def theta_bounds(X, y, cfg: Config = CONFIG):
    """Optim.cpp:179-209 with dX recomputed: [lower, upper] factors of maxdX, variogram heuristic."""
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    maxdX = X.max(axis=0) - X.min(axis=0)
    lower = cfg.theta_lower_factor * maxdX
    upper = cfg.theta_upper_factor * maxdX
    if cfg.variogram_bounds_heuristic and n > 0:
        diff = X[:, None, :] - X[None, :, :]          # (i, j, k) = X_i - X_j
        dy2 = (y[:, None] - y[None, :]) ** 2
        dx2 = (diff ** 2).sum(axis=2)
        with np.errstate(invalid="ignore", divide="ignore"):
            slope = dy2 / dx2
        slope[np.isnan(slope)] = 0.0
        wsum = slope.sum()
        if wsum > 0.0:
            w = slope / wsum
            steep = np.einsum("ijk,ij->k", np.abs(diff), w)
            lower = np.maximum(lower, cfg.theta_lower_factor * steep)
            lower = np.minimum(lower, upper)
            upper = np.maximum(lower, upper)
    return lower, upper


# --------------------------------------------------------------------------------------------------------------
# populate_Model and the log-likelihood
# --------------------------------------------------------------------------------------------------------------
@dataclass
class KModel:
    R: np.ndarray
    L: np.ndarray
    Rinv: np.ndarray | None
    Fstar: np.ndarray
    ystar: np.ndarray
    Rstar: np.ndarray
    betahat: np.ndarray
    Estar: np.ndarray
    SSEstar: float
    nugget_increments: int = 0


def populate_model(kernel, X, y, F, theta, alpha=1.0, diag=None, with_rinv=True, cfg: Config = CONFIG) -> KModel:
    """KrigingImpl.cpp:73-125 (+ cholCov LinearAlgebra.cpp:142-204)."""
    R = build_R(kernel, X, theta, alpha, diag)
    L, inc = safe_chol_lower(R, cfg)
    Rinv = inv_sympd(L) if with_rinv else None
    Fstar = solve_lower(L, F)
    ystar = solve_lower(L, y.reshape(-1, 1))[:, 0]
    FtF = Fstar.T @ Fstar
    if FtF.shape[0] > 0:
        Rstar, info = lapack.dpotrf(FtF, lower=0, clean=1)
        assert info == 0
        rhs = Fstar.T @ ystar
        beta = lapack.dtrtrs(Rstar, lapack.dtrtrs(Rstar, rhs.reshape(-1, 1), lower=0, trans=1)[0], lower=0)[0][:, 0]
    else:
        Rstar = np.zeros((0, 0))
        beta = np.zeros(0)
    residual = y - F @ beta
    Estar = solve_lower(L, residual.reshape(-1, 1))[:, 0]
    SSE = float(Estar @ Estar)
    return KModel(R, L, Rinv, Fstar, ystar, Rstar, beta, Estar, SSE, inc)


class OracleKriging:
    """The state a fitted ``Kriging`` carries into ``logLikelihoodFun`` (Kriging.hpp, KrigingImpl.hpp)."""

    def __init__(self, y, X, kernel, regmodel="constant", normalize=False, noise_model="none",
                 est_sigma2=True, sigma2=None, est_nugget=True, nugget=None, est_beta=True, beta=None,
                 alpha=1.0, cfg: Config = CONFIG):
        X = np.atleast_2d(np.asarray(X, dtype=np.float64))
        if X.shape[0] == 1 and np.size(y) != 1:
            X = X.T
        y = np.asarray(y, dtype=np.float64).reshape(-1)
        if normalize:
            cX, sX = X.min(axis=0), X.max(axis=0) - X.min(axis=0)
            cY, sY = y.min(), y.max() - y.min()
        else:
            cX, sX, cY, sY = np.zeros(X.shape[1]), np.ones(X.shape[1]), 0.0, 1.0
        self.centerX, self.scaleX, self.centerY, self.scaleY = cX, sX, cY, sY
        self.X = np.asfortranarray((X - cX) / sX)
        self.y = (y - cY) / sY
        self.kernel = kernel
        self.regmodel = regmodel
        self.F = regression_matrix(regmodel, self.X)
        self.noise_model = noise_model
        self.est_sigma2, self.sigma2 = est_sigma2, sigma2
        self.est_nugget, self.nugget = est_nugget, nugget
        self.est_beta, self.beta = est_beta, beta
        self.alpha = alpha
        self.cfg = cfg
        self.theta = None
        self.model = None

    # Kriging.cpp:214-341
    def log_likelihood(self, gamma, return_grad=True, keep_model=False):
        n, d = self.X.shape
        gamma = np.asarray(gamma, dtype=np.float64).reshape(-1)
        theta = gamma[:d]
        if gamma.size > d:
            extra = float(gamma[d])
        else:
            extra = self.alpha if self.noise_model == "nugget" else (self.sigma2 or 0.0)
        if self.noise_model == "nugget" and not self.est_sigma2 and not self.est_nugget:
            extra = self.sigma2 / (self.sigma2 + self.nugget)
        alpha = extra if self.noise_model == "nugget" else 1.0
        m = populate_model(self.kernel, self.X, self.y, self.F, theta, alpha, None, True, self.cfg)
        if not self.est_beta:
            m.betahat = np.zeros_like(m.betahat)
        logdet = 2.0 * np.sum(np.log(np.diag(m.L)))
        if self.noise_model == "nugget":
            _alpha = extra
            s2, nu = self.sigma2, self.nugget
            if self.est_sigma2:
                if self.est_nugget:
                    var = m.SSEstar / n
                    s2, nu = _alpha * var, (1.0 - _alpha) * var
                else:
                    s2 = self.nugget * _alpha / (1.0 - _alpha)
            else:
                if self.est_nugget:
                    nu = self.sigma2 * (1.0 - _alpha) / _alpha
                else:
                    _alpha = self.sigma2 / (self.sigma2 + self.nugget)
            total_var = s2 + nu
            ll = -0.5 * (n * math.log(2 * math.pi * total_var) + logdet + m.SSEstar / total_var)
            sigma2_grad = total_var
        else:
            if self.est_sigma2:
                sigma2_grad = m.SSEstar / n
                ll = -0.5 * (n * math.log(2 * math.pi * sigma2_grad) + logdet + n)
            else:
                sigma2_grad = self.sigma2
                ll = -0.5 * (n * math.log(2 * math.pi * sigma2_grad) + logdet + float(m.Estar @ m.Estar) / sigma2_grad)
        if keep_model:
            self.model = m
        if not return_grad:
            return ll, None
        x = solve_upper_t(m.L, m.Estar.reshape(-1, 1))[:, 0]
        t1 = np.zeros(d)
        t2 = np.zeros(d)
        lib().ora_grad_terms(KERNELS[self.kernel], n, d, _dp(self.X), _dp(np.ascontiguousarray(theta)),
                             _dp(m.R), _dp(m.Rinv), _dp(x), _dp(t1), _dp(t2))
        grad = np.zeros(gamma.size)
        grad[:d] = (t1 / sigma2_grad + t2) / 2.0
        if gamma.size > d and self.noise_model == "nugget":
            _alpha = extra
            out = np.zeros(2)
            if self.est_sigma2 and self.est_nugget:
                lib().ora_alpha_terms(n, _dp(m.R), _dp(m.Rinv), _dp(x), _alpha, 0.0, _dp(out))
                term1_a = -out[0] / sigma2_grad
                term2_a = out[1]
                grad[d] = -0.5 * (term1_a + term2_a)
            elif self.est_sigma2 and not self.est_nugget:
                lib().ora_alpha_terms(n, _dp(m.R), _dp(m.Rinv / sigma2_grad), _dp(x), _alpha, 1.0, _dp(out))
                term1_a = -out[0] / (sigma2_grad * sigma2_grad)
                term2_a = out[1]
                grad[d] = -0.5 * (term1_a + term2_a) * self.nugget / (1.0 - _alpha) / (1.0 - _alpha)
            else:
                grad[d] = 0.0
        return ll, grad

    # Kriging.cpp:353-468 (_leaveOneOut, NoiseModel None): B = L^-T L^-1 - A'A with A = Q*' L^-1 (Q* the thin QR
    # factor of F*), sigma2LOO = 1 / diag(B), errors = sigma2LOO * (L^-T E*), LOO = |errors|^2 / n; gradient per
    # theta_k with gradR_k = R o dlnC_k (zero diagonal).  Returns (loo, grad or None, yhat, sigma2LOO).
    def _gradR_all(self, R, theta):
        """gradR_k = R o DlnCovDtheta_k over the strict lower triangle, mirrored, zero diagonal (Kriging.cpp:430-440)."""
        n, d = self.X.shape
        G = np.zeros((d, n, n))
        for i in range(n):
            for j in range(i):
                g = R[i, j] * dlncov(self.kernel, self.X[i] - self.X[j], theta)
                G[:, i, j] = g
                G[:, j, i] = g
        return G

    def leave_one_out(self, theta, return_grad=True):
        n, d = self.X.shape
        theta = np.asarray(theta, dtype=np.float64).reshape(-1)
        alpha = self.alpha if self.noise_model == "nugget" else 1.0
        m = populate_model(self.kernel, self.X, self.y, self.F, theta, alpha, None, False, self.cfg)
        Linv = solve_lower(m.L, np.eye(n))
        By = Linv.T @ m.Estar
        Qs, _ = np.linalg.qr(m.Fstar, mode="reduced")
        A = Qs.T @ Linv
        B = Linv.T @ Linv - A.T @ A
        s2 = 1.0 / np.diag(B)
        errors = s2 * By
        loo = float(errors @ errors) / n
        grad = None
        if return_grad:
            grad = np.zeros(d)
            Gs = self._gradR_all(m.R, theta)
            for k in range(d):
                G = Gs[k]
                diagdB = -np.einsum("ij,jk,ki->i", B, G, B)
                ds2 = -s2 * s2 * diagdB
                derr = ds2 * By - s2 * (B @ (G @ By))
                grad[k] = 2.0 * float(errors @ derr) / n
        return loo, grad, self.y - errors, s2

    # Kriging.cpp:487-652 (_logMargPost, RobustGaSP's marginal likelihood + approximate reference prior) and
    # KrigingImpl.cpp:887-921 (compute_lmp_theta_ans), in the reference's order of operations.
    def log_marg_post(self, gamma, return_grad=True):
        n, d = self.X.shape
        p = self.F.shape[1]
        gamma = np.asarray(gamma, dtype=np.float64).reshape(-1)
        nug = self.noise_model == "nugget"
        if nug and gamma.size == d:
            gamma = np.append(gamma, self.alpha)
        theta = gamma[:d]
        alpha = float(gamma[d]) if nug else 1.0
        m = populate_model(self.kernel, self.X, self.y, self.F, theta, alpha, None, False, self.cfg)
        Rinv_X = solve_upper_t(m.L, m.Fstar)
        Xt_Rinv_X = self.F.T @ Rinv_X
        if p > 0:
            LX, _ = safe_chol_lower(Xt_Rinv_X, self.cfg)
            P = Rinv_X @ solve_upper_t(LX, solve_lower(LX, Rinv_X.T))
        else:
            LX, P = np.zeros((0, 0)), np.zeros((n, n))
        yt_Rinv = solve_upper_t(m.L, m.ystar.reshape(-1, 1))[:, 0]
        S_2 = float(yt_Rinv @ self.y - self.y @ P @ self.y)
        if nug:
            if self.est_sigma2 and self.est_nugget:
                sigma2 = S_2 / (n - p)
            elif self.est_sigma2 or self.est_nugget:
                sigma2 = self.sigma2 / alpha
            else:
                sigma2 = self.sigma2 + self.nugget
        elif self.est_sigma2:
            sigma2 = S_2 / (n - p)
        else:
            sigma2 = self.sigma2
        log_S_2 = math.log(sigma2 * (n - p))
        lml = -np.sum(np.log(np.diag(m.L))) - np.sum(np.log(np.diag(LX))) - (n - p) / 2.0 * log_S_2
        a = 0.2
        b = 1.0 / n ** (1.0 / d) * (a + d)
        CL = (self.X.max(axis=0) - self.X.min(axis=0)) / n ** (1.0 / d)
        t = float(np.sum(CL / theta)) + ((1.0 - alpha) / alpha if nug else 0.0)
        lp = -b * t + a * math.log(t)
        value = float(lml + lp)
        if not return_grad:
            return value, None
        grad = np.zeros(gamma.size)
        if self.est_sigma2:
            Q_output = yt_Rinv - P @ self.y
            Gs = self._gradR_all(m.R, theta)
            ans = np.zeros(d)
            for k in range(d):
                Wb = solve_upper_t(m.L, solve_lower(m.L, Gs[k])).T - Gs[k] @ P
                ans[k] = -np.trace(Wb) / 2.0 + float(self.y @ Wb.T @ Q_output) / (2.0 * sigma2)
            grad[:d] = ans - (a * CL / t - b * CL) / theta ** 2
            if nug:
                if self.est_sigma2 or self.est_nugget:
                    gR = m.R / alpha
                    np.fill_diagonal(gR, 0.0)
                    Wb = solve_upper_t(m.L, solve_lower(m.L, gR)).T - gR @ P
                    ans_d = -np.trace(Wb) / 2.0 + float(self.y @ Wb.T @ Q_output) / (2.0 * sigma2)
                    grad[d] = ans_d - (a / t - b) / alpha ** 2
        else:
            for k in range(d):
                ge = gamma.copy()
                ge[k] += 1e-6
                grad[k] = (self.log_marg_post(ge, False)[0] - value) / 1e-6
        return value, grad

    # KrigingImpl.cpp:145-300, Kriging.cpp:2240-2285 (mean, stdev and their derivatives)
    def predict(self, Xn, theta, beta, sigma2, alpha=1.0, return_stdev=True, fixed_beta=False, return_deriv=False,
                objective="LL"):
        """fixed_beta: beta is a given trend (is_beta_estim = false), so z = L \\ (y - F beta) (KrigingImpl.cpp:116).
        objective "LMP" scales sigma2 by (n - p) / (n - p - 2) (Kriging.cpp:2262).  With return_deriv the result is
        (yhat, stdev, dyhat, dstdev), the derivatives q x d with respect to the prediction points."""
        Xn = np.atleast_2d(np.asarray(Xn, dtype=np.float64))
        Xn_n = (Xn - self.centerX) / self.scaleX
        Fn = regression_matrix(self.regmodel, Xn_n)
        m = populate_model(self.kernel, self.X, self.y, self.F, theta, alpha, None, False, self.cfg)
        n_o, q = self.X.shape[0], Xn_n.shape[0]
        R_on = np.empty((n_o, q), order="F")
        for j in range(q):
            for i in range(n_o):
                dij = self.X[i] - Xn_n[j]
                if np.all(np.abs(dij) <= np.finfo(float).eps):
                    R_on[i, j] = 1.0
                else:
                    R_on[i, j] = cov(self.kernel, dij, theta) * alpha
        z = m.ystar - m.Fstar @ np.asarray(beta, dtype=np.float64) if fixed_beta else m.Estar
        Rs = solve_lower(m.L, R_on)
        beta = np.asarray(beta, dtype=np.float64)
        yhat = Fn @ beta + Rs.T @ z
        yhat = self.centerY + self.scaleY * yhat
        if not return_stdev and not return_deriv:
            return yhat, None
        E = Fn - Rs.T @ m.Fstar
        # rsolve_upper(circ, E): X * circ = E
        Ec = lapack.dtrtrs(m.Rstar, np.asfortranarray(E.T), lower=0, trans=1)[0].T if m.Rstar.size else E
        if objective == "LMP":
            p = self.F.shape[1]
            sigma2 = sigma2 * (n_o - p) / (n_o - p - 2.0)
        var_scale = sigma2 / alpha if self.noise_model == "nugget" else sigma2
        sd2 = np.zeros(q)
        if return_stdev:
            sd2 = 1.0 - np.sum(Rs * Rs, axis=0) + np.sum(Ec * Ec, axis=1)
            sd2 = np.where(np.isnan(sd2) | (sd2 < 0), 0.0, sd2)
            sd2 = sd2 * var_scale * self.scaleY * self.scaleY
        if not return_deriv:
            return yhat, np.sqrt(sd2)
        # KrigingImpl.cpp:254-296
        d = Xn_n.shape[1]
        dy = np.zeros((q, d))
        dsd2 = np.zeros((q, d))
        for i in range(q):
            DR = np.empty((n_o, d))
            for j in range(n_o):
                DR[j] = R_on[j, i] * dlncov_dx(self.kernel, Xn_n[i] - self.X[j], theta)
            DF = regression_derivative(self.regmodel, Xn_n[i])
            W = solve_lower(m.L, DR)
            dy[i] = DF @ beta + W.T @ z
            if return_stdev:
                rhs = (DF - W.T @ m.Fstar).T
                DE = lapack.dtrtrs(m.Rstar, np.asfortranarray(rhs), lower=0, trans=1)[0] if m.Rstar.size else rhs
                dsd2[i] = -2.0 * Rs[:, i] @ W + 2.0 * Ec[i] @ DE
        dy = dy * self.scaleY / self.scaleX
        dsd2 = dsd2 * var_scale * self.scaleY * self.scaleY / self.scaleX
        sd = np.sqrt(sd2)
        with np.errstate(divide="ignore", invalid="ignore"):
            dsd = dsd2 / (2.0 * sd)[:, None]
        return yhat, (sd if return_stdev else None), dy, dsd


    # Kriging.cpp:1717-2209 (BFGS[N], objective LL), with scipy's L-BFGS-B (Fortran/C port of Nocedal's 3.0 code)
    # standing in for the un-vendored lbfgsb_cpp: same bounds, starts, tolerances, restart rules and commit.
    def fit_bfgs(self, multistart=1, theta0=None, max_iter=20, pgtol=1e-3, factr=1e10, max_restart=10):
        from scipy.optimize import fmin_l_bfgs_b
        n, d = self.X.shape
        lower, upper = theta_bounds(self.X, self.y, self.cfg)
        mt = MT19937Stream(123)
        U = mt.randu_mat(multistart, d)
        rand = lower + U * (upper - lower)
        if theta0 is not None:
            t0 = np.atleast_2d(np.asarray(theta0, dtype=np.float64))
            multistart = max(multistart, t0.shape[0])
            starts = np.vstack([t0, rand])[:multistart]
        else:
            starts = rand
        glo, ghi = np.log(lower), np.log(upper)

        def ofn(g):
            th = np.exp(g)
            ll, gr = self.log_likelihood(th, True)
            return -ll, -gr * th

        best = (np.inf, None)
        for s in range(multistart):
            th_start = starts[s]
            gamma = np.log(th_start)
            lo, hi = np.minimum(gamma, glo), np.maximum(gamma, ghi)
            best_f, best_g = np.inf, gamma
            for retry in range(max_restart + 1):
                x, f, info = fmin_l_bfgs_b(ofn, gamma, bounds=list(zip(lo, hi)), m=5, factr=factr, pgtol=pgtol,
                                           maxiter=max_iter)
                if f < best_f:
                    best_f, best_g = f, x
                tp = np.exp(x)
                to_lb = np.min(np.abs(tp - lower))
                task = info["task"] if isinstance(info["task"], str) else info["task"].decode()
                if retry < max_restart and (task.startswith("ABNORMAL_TERMINATION_IN_LNSRCH") or info["nit"] <= 2
                                            or to_lb < np.finfo(float).eps or f > best_f):
                    rt = (th_start + lower) / 2.0 ** (retry + 1)
                    gamma = np.log(rt)
                    lo, hi = np.minimum(gamma, lo), np.maximum(gamma, hi)
                else:
                    break
            f_final = -self.log_likelihood(np.exp(best_g), False)[0]
            if f_final < best[0]:
                best = (f_final, np.exp(best_g))
        theta = best[1]
        m = populate_model(self.kernel, self.X, self.y, self.F, theta, 1.0, None, False, self.cfg)
        self.theta = theta
        self.beta = m.betahat
        self.sigma2 = m.SSEstar / n
        return theta, -best[0]


# --------------------------------------------------------------------------------------------------------------
# Vecchia
# --------------------------------------------------------------------------------------------------------------
def vecchia_sets(X, m):
    """Kriging.cpp:736-804 (O(n^2): small n only).  Returns (order[n], nbr[n, m]) with -1 padding."""
    X = _colmajor(X)
    n, d = X.shape
    order = np.empty(n, dtype=np.int32)
    nbr = np.empty((n, m), dtype=np.int32)
    lib().ora_vecchia_sets(n, d, _dp(X), m, _ip(order), _ip(nbr))
    return order, nbr


def vecchia_ll(kernel, X, y, F, theta, order, nbr, num_nugget=None, return_grad=True):
    """Kriging.cpp:806-924.  Returns (vll, grad or None, beta, sigma2)."""
    X = _colmajor(X)
    n, d = X.shape
    F = _colmajor(F)
    p = F.shape[1]
    y = np.ascontiguousarray(y, dtype=np.float64)
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    order = np.ascontiguousarray(order, dtype=np.int32)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    m = nbr.shape[1]
    grad = np.zeros(d) if return_grad else None
    beta = np.zeros(max(p, 1))
    s2 = np.zeros(1)
    nn = CONFIG.num_nugget if num_nugget is None else num_nugget
    v = lib().ora_vecchia_ll(KERNELS[kernel], n, d, p, _dp(X), _dp(y), _dp(F), _dp(theta), _ip(order), _ip(nbr),
                             m, nn, _dp(grad), _dp(beta), _dp(s2))
    return v, grad, beta[:p], float(s2[0])


# --------------------------------------------------------------------------------------------------------------
# mt19937 draws as the reference makes them (Random.cpp:13-49, libstdc++ uniform_real_distribution<double>)
# --------------------------------------------------------------------------------------------------------------
class MT19937Stream:
    def __init__(self, seed=123):
        self.bg = np.random.MT19937()
        self.bg._legacy_seeding(seed)

    def uniform(self, k):
        raw = self.bg.random_raw(2 * k).astype(np.float64).reshape(k, 2)
        u = (raw[:, 0] + raw[:, 1] * 4294967296.0) / 18446744073709551616.0
        return np.where(u >= 1.0, np.nextafter(1.0, 0.0), u)

    def randu_mat(self, rows, cols):
        return self.uniform(rows * cols).reshape(cols, rows).T
