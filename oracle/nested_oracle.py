"""CPU restatement of libKriging's NestedKriging (src/lib/NestedKriging.cpp) for the parity tests.

TEST INFRASTRUCTURE ONLY: the GPU NestedKriging is compared with these functions; the product package never imports
them.  Each function names the reference lines it follows.

  partition        make_partition (:124-165), with the GPU build's random source (32-bit Mersenne Twister seeded
                   with the model seed; draws u mod m) in place of Armadillo's generator, so that partitions can be
                   compared exactly
  fit_none         the plain fit path (:261-269) with optim = "none" at a given theta, then unify (:283-332)
  predict_poe      predict_poe_family (:364-422)
  predict_nk       precompute_nk (:334-347) + predict_nk (:424-498)
"""
from __future__ import annotations

import numpy as np
from scipy import linalg

from . import oracle as O

JITTER = 1e-10
TINY = 1e-12


def partition(X, nb_groups, method="kmeans", seed=123):
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    bg = np.random.MT19937()
    bg._legacy_seeding(seed)

    def draw(m):
        return int(bg.random_raw()) % m

    assignment = np.zeros(n, dtype=np.int64)
    ok = False
    if method == "kmeans" and nb_groups > 1:
        k = nb_groups
        idx = np.arange(n)
        for i in range(k):
            j = i + draw(n - i)
            idx[i], idx[j] = idx[j], idx[i]
        C = X[idx[:k]].copy()

        def assign():
            best = np.full(n, np.inf)
            bi = np.zeros(n, dtype=np.int64)
            for c in range(k):
                s = np.zeros(n)
                for q in range(d):
                    dq = X[:, q] - C[c, q]
                    s = s + dq * dq
                better = s < best
                best = np.where(better, s, best)
                bi = np.where(better, c, bi)
            return bi

        for _ in range(10):
            a = assign()
            sums = np.zeros((k, d))
            cnt = np.zeros(k, dtype=np.int64)
            for i in range(n):  # index order, as the host update
                sums[a[i]] += X[i]
                cnt[a[i]] += 1
            for c in range(k):
                if cnt[c] > 0:
                    C[c] = sums[c] / cnt[c]
        assignment = assign()
        ok = all(np.sum(assignment == g) >= d + 2 for g in range(k))
    if not ok:
        perm = np.arange(n)
        for i in range(n - 1, 0, -1):
            j = draw(i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        assignment[perm] = np.arange(n) % nb_groups
    return [np.flatnonzero(assignment == g) for g in range(nb_groups)]


def fit_none(y, X, kernel, groups, theta, regmodel="constant"):
    """Submodels fitted at the given theta (sigma2 = SSE / n_g, GLS beta), then the common prior."""
    y = np.asarray(y, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    n, d = X.shape
    theta = np.asarray(theta, dtype=np.float64)
    log_theta = np.zeros(d)
    sigma2 = 0.0
    beta0 = 0.0
    subs = []
    for g in groups:
        ora = O.OracleKriging(y[g], X[g], kernel, regmodel=regmodel)
        m = O.populate_model(kernel, ora.X, ora.y, ora.F, theta, 1.0, None, False)
        s2 = m.SSEstar / len(g)
        subs.append(dict(sigma2=s2, beta=m.betahat))
        w = len(g) / n
        log_theta = log_theta + w * np.log(theta)
        sigma2 += w * s2
        if regmodel == "constant":
            beta0 += w * m.betahat[0]
    return dict(theta=np.exp(log_theta), sigma2=sigma2, beta0=beta0, subs=subs)


def predict_poe(y, X, kernel, groups, theta, sigma2, beta0, Xn, aggregation):
    y = np.asarray(y, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    p = len(groups)
    mus, vars_ = [], []
    for g in groups:
        ora = O.OracleKriging(y[g], X[g], kernel)
        mu, sd = ora.predict(Xn, theta, np.array([beta0]), sigma2, fixed_beta=True)
        mus.append(mu)
        vars_.append(sd * sd + TINY)
    mus = np.array(mus).T
    vars_ = np.array(vars_).T
    if aggregation == "PoE":
        prec = np.sum(1.0 / vars_, axis=1)
        mean = np.sum(mus / vars_, axis=1) / prec
    elif aggregation == "gPoE":
        prec = np.sum(1.0 / vars_, axis=1) / p
        mean = (np.sum(mus / vars_, axis=1) / p) / prec
    elif aggregation == "BCM":
        prec = np.sum(1.0 / vars_, axis=1) - (p - 1.0) / sigma2
        prec = np.clip(prec, TINY, np.inf)
        mean = np.sum(mus / vars_, axis=1) / prec
    elif aggregation == "rBCM":
        beta = 0.5 * (np.log(sigma2) - np.log(vars_))
        prec = np.sum(beta / vars_, axis=1) + (1.0 - np.sum(beta, axis=1)) / sigma2
        prec = np.clip(prec, TINY, np.inf)
        mean = np.sum(beta * mus / vars_, axis=1) / prec
    else:
        raise ValueError(aggregation)
    return mean, np.sqrt(np.clip(1.0 / prec, 0.0, np.inf))


def predict_nk(y, X, kernel, groups, theta, sigma2, beta0, Xn, chunk=128):
    y = np.asarray(y, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    Xn = np.asarray(Xn, dtype=np.float64)
    p = len(groups)
    Ls, alphas = [], []
    for g in groups:
        R = O.cov_cross(kernel, X[g], X[g], theta)
        R[np.diag_indices_from(R)] += JITTER
        L = np.linalg.cholesky(R)
        r = y[g] - beta0
        alphas.append(linalg.solve_triangular(L.T, linalg.solve_triangular(L, r, lower=True), lower=False))
        Ls.append(L)
    q = Xn.shape[0]
    mean = np.zeros(q)
    var = np.zeros(q)
    for start in range(0, q, chunk):
        Xc = Xn[start:start + chunk]
        qc = Xc.shape[0]
        W, M, Kd = [], np.zeros((p, qc)), np.zeros((p, qc))
        for gi, g in enumerate(groups):
            C = O.cov_cross(kernel, X[g], Xc, theta)
            U = linalg.solve_triangular(Ls[gi], C, lower=True)
            W.append(linalg.solve_triangular(Ls[gi].T, U, lower=False))
            M[gi] = beta0 + C.T @ alphas[gi]
            Kd[gi] = np.sum(U * U, axis=0)
        cross = np.zeros((p, p, qc))
        for i in range(p):
            for j in range(i + 1, p):
                Rij = O.cov_cross(kernel, X[groups[i]], X[groups[j]], theta)
                cij = np.sum(W[i] * (Rij @ W[j]), axis=0)
                cross[i, j] = cij
                cross[j, i] = cij
        for t in range(qc):
            KM = cross[:, :, t].copy()
            KM[np.diag_indices(p)] = Kd[:, t] + JITTER
            kM = np.diag(KM).copy()
            try:
                w = linalg.cho_solve(linalg.cho_factor(KM, lower=False), kM)
            except linalg.LinAlgError:
                w = np.linalg.pinv(KM) @ kM
            mean[start + t] = beta0 + w @ (M[:, t] - beta0)
            var[start + t] = sigma2 * max(0.0, 1.0 - w @ kM)
    return mean, np.sqrt(var)
