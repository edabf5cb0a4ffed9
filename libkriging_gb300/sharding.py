"""Multi-GPU sharding of the paths that shard: multistart fits, NestedKriging submodels and the Vecchia likelihood.

One process per GPU (torch.distributed, one rank per device).  The units are independent, so there is no data-path
collective: each rank evaluates its contiguous share of the units on its own GPU, and the host exchanges a few
scalars per unit (objective, theta) to pick the winner -- the min over starts that the reference's fit loop takes
sequentially (src/lib/Kriging.cpp:2097-2114; ties go to the lowest start index, as its strict '<' does).  The dense
single evaluation does not shard (its Cholesky exchanges panels every block step): replicas only.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_items: int, rank: int, world: int):
    """Contiguous balanced share [lo, hi) of n_items for `rank` (the first n_items % world ranks get one more)."""
    base, extra = divmod(n_items, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def _gather(obj, group=None):
    import torch.distributed as dist
    world = dist.get_world_size(group)
    out = [None] * world
    dist.all_gather_object(out, obj, group=group)
    return out


def select_best(local_results, group=None):
    """local_results: list of (global_index, objective, payload) of this rank's units.  Returns the global winner
    (lowest objective, ties -> lowest global index) identically on every rank; failed units carry objective inf."""
    allres = [r for part in _gather(list(local_results), group) for r in part]
    allres.sort(key=lambda r: r[0])
    best = None
    for r in allres:
        if np.isfinite(r[1]) and (best is None or r[1] < best[1]):
            best = r
    if best is None:
        raise RuntimeError("All %d optimization attempts failed" % len(allres))
    return best


def fit_multistart_sharded(make_model, y, X, thetas, regmodel="constant", normalize=False, parameters=None,
                           group=None):
    """Fit with the given starting points (rows of `thetas`) sharded over the ranks of `group`.

    make_model() -> a fresh model exposing fit(...), theta(), logLikelihood() (a libkriging_gb300.Kriging).
    Every rank returns the same committed model: the best start over all ranks, refitted with optim="none".
    The returned index is the first start of the winning rank's share.
    """
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    thetas = np.atleast_2d(np.asarray(thetas, dtype=np.float64))
    lo, hi = shard_range(thetas.shape[0], rank, world)
    local = []
    P = dict(parameters or {})
    if hi > lo:
        # the rank's share as ONE multistart fit: every optimiser round of its starts is one batched GPU evaluation,
        # and the fit keeps the first of its best starts (the reference's strict '<' scan); across ranks the lowest
        # objective wins with ties to the lowest rank, whose starts come first -- the global first-best start
        m = make_model()
        try:
            P["theta"] = thetas[lo:hi]
            m.fit(y, X, regmodel, normalize, "BFGS%d" % (hi - lo), "LL", P)
            local.append((lo, -m.logLikelihood(), np.asarray(m.theta())))
        except Exception:  # every start of the share failed
            local.append((lo, float("inf"), None))
    idx, obj, theta = select_best(local, group)
    best = make_model()
    P["theta"] = np.asarray(theta).reshape(1, -1)
    best.fit(y, X, regmodel, normalize, "none", "LL", P)
    return best, idx, obj


def balanced_bins(sizes, world):
    """Size-balanced bins of the groups for `world` ranks: greedy longest-processing-time by n_g^3 (the
    factorisation cost), ties to the lowest rank; group indices in each bin ascending."""
    order = sorted(range(len(sizes)), key=lambda g: (-float(sizes[g]) ** 3, g))
    load = [0.0] * world
    bins = [[] for _ in range(world)]
    for g in order:
        r = min(range(world), key=lambda q: (load[q], q))
        bins[r].append(g)
        load[r] += float(sizes[g]) ** 3
    return [sorted(b) for b in bins]


def fit_nested_sharded(make_nested, y, X, groups, regmodel="constant", optim="BFGS", objective="LL",
                       parameters=None, group=None):
    """NestedKriging fit with its groups sharded over the ranks of `group` (NestedKriging.cpp:171-332):

    1. every rank fits the submodels of its size-balanced bin of groups (make_nested() -> a fresh
       libkriging_gb300.NestedKriging; fit_groups on the bin's rows),
    2. one all-reduce of (sum n_g log theta_g, sum n_g sigma2_g, sum n_g beta0_g, sum n_g) gives the common prior
       of unify_hyperparameters,
    3. every rank refits its bin at that prior (optim = "none", theta / sigma2 / beta fixed).

    Returns (local NestedKriging, global indices of its groups, (theta, sigma2, beta0)).  PoE-family predictions
    then combine per-rank partial sums (predict_poe_sharded); NK aggregation needs every pair of groups and is not
    sharded."""
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    bins = balanced_bins([len(g) for g in groups], world)
    mine = bins[rank]
    rows = np.concatenate([np.asarray(groups[g]) for g in mine]) if mine else np.zeros(0, dtype=np.int64)
    local_groups, start = [], 0
    for g in mine:
        local_groups.append(np.arange(start, start + len(groups[g])))
        start += len(groups[g])
    d = X.shape[1]
    sums = np.zeros(d + 3)
    nk = None
    if mine:
        nk = make_nested()
        nk.fit_groups(y[rows], X[rows], local_groups, regmodel, optim, objective, parameters)
        th, s2, b0 = nk.group_estimates()
        for i, g in enumerate(mine):
            ng = float(len(groups[g]))
            sums[:d] += ng * np.log(th[i])
            sums[d] += ng * s2[i]
            sums[d + 1] += ng * b0[i]
            sums[d + 2] += ng
    tot = allreduce_sums(sums, group)
    n = tot[d + 2]
    theta = np.exp(tot[:d] / n)
    sigma2 = tot[d] / n
    beta0 = tot[d + 1] / n
    if nk is not None:
        fixed = {"theta": theta.reshape(1, -1), "is_theta_estim": False, "sigma2": sigma2, "is_sigma2_estim": False}
        if regmodel == "constant":
            fixed.update(beta=np.array([beta0]), is_beta_estim=False)
        nk.fit_groups(y[rows], X[rows], local_groups, regmodel, "none", "LL", fixed)
    return nk, mine, (theta, sigma2, beta0)


def predict_poe_sharded(nk_local, Xn, aggregation, sigma2, p_total, group=None):
    """PoE / gPoE / BCM / rBCM prediction (NestedKriging.cpp:364-422) from the submodels spread over the ranks: each
    rank adds its submodels' terms, one all-reduce combines them."""
    q = np.asarray(Xn).shape[0]
    tiny = 1e-12
    acc = np.zeros((4, q))  # sum 1/v, sum mu/v, sum beta/v, sum beta
    acc_bmu = np.zeros(q)   # sum beta mu / v
    if nk_local is not None:
        for g in range(nk_local.nb_groups()):
            mu, sd, _, _, _ = nk_local.submodel(g).predict(Xn, True, False, False)
            v = sd * sd + tiny
            acc[0] += 1.0 / v
            acc[1] += mu / v
            b = 0.5 * (np.log(sigma2) - np.log(v))
            acc[2] += b / v
            acc[3] += b
            acc_bmu += b * mu / v
    tot = allreduce_sums(np.concatenate([acc.ravel(), acc_bmu]), group)
    s_iv, s_muv, s_bv, s_b = tot[:4 * q].reshape(4, q)
    s_bmu = tot[4 * q:]
    p = float(p_total)
    if aggregation == "PoE":
        prec = s_iv
        mean = s_muv / prec
    elif aggregation == "gPoE":
        prec = s_iv / p
        mean = (s_muv / p) / prec
    elif aggregation == "BCM":
        prec = np.clip(s_iv - (p - 1.0) / sigma2, tiny, np.inf)
        mean = s_muv / prec
    elif aggregation == "rBCM":
        prec = np.clip(s_bv + (1.0 - s_b) / sigma2, tiny, np.inf)
        mean = s_bmu / prec
    else:
        raise ValueError("sharded prediction supports PoE, gPoE, BCM and rBCM")
    return mean, np.sqrt(np.clip(1.0 / prec, 0.0, np.inf))


def allreduce_sums(values, group=None):
    """Sum a small float64 vector over the ranks (NestedKriging's unify step: sum w log theta, w sigma2, w beta0)."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.asarray(values, dtype=np.float64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def vecchia_ll_sharded(make_shard, n, d, p, theta, return_grad=True, group=None):
    """Vecchia log-likelihood (Kriging.cpp:806-924) with the ordered points split over the ranks of `group`.

    make_shard(t0, t1) -> an object with sums1(theta, grad) -> (s1, failed, nugget_points) and
    sums2(beta, grad) -> s2 over the ordered positions [t0, t1) (libkriging_gb300.VecchiaShard on a GPU).  Two
    exchanges of partial sums: [A (p x p), b (p), sum log v, failed] before the GLS beta, [Q, dQ_k, sum dv_k / v]
    after it.  Returns (vll, grad or None, beta, sigma2), identical on every rank."""
    import torch.distributed as dist
    from . import _lib
    from .kriging import vecchia_finish, vecchia_gls_beta
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    lo, hi = shard_range(n, rank, world)
    shard = make_shard(lo, hi)
    s1, failed, _ = shard.sums1(theta, return_grad)
    tot1 = allreduce_sums(np.concatenate([s1, [float(failed)]]), group)
    if tot1[-1] > 0:
        raise _lib.LibKrigingError("[ERROR] Exceed max numerical nugget added to force chol matrix (%d points)"
                                   % int(tot1[-1]))
    s1 = tot1[:-1]
    beta = vecchia_gls_beta(p, s1)
    s2 = allreduce_sums(shard.sums2(beta, return_grad), group)
    vll, sigma2, grad = vecchia_finish(n, d, s1[p * p + p], s2, return_grad)
    return vll, grad, beta, sigma2
