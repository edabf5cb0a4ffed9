"""Multi-GPU sharding of the paths that shard: multistart fits and NestedKriging submodels.

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
    """
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    thetas = np.atleast_2d(np.asarray(thetas, dtype=np.float64))
    lo, hi = shard_range(thetas.shape[0], rank, world)
    local = []
    P = dict(parameters or {})
    for i in range(lo, hi):
        m = make_model()
        try:
            P["theta"] = thetas[i:i + 1]
            m.fit(y, X, regmodel, normalize, "BFGS", "LL", P)
            local.append((i, -m.logLikelihood(), np.asarray(m.theta())))
        except Exception:  # a failed start, as the reference's per-start try/catch
            local.append((i, float("inf"), None))
    idx, obj, theta = select_best(local, group)
    best = make_model()
    P["theta"] = np.asarray(theta).reshape(1, -1)
    best.fit(y, X, regmodel, normalize, "none", "LL", P)
    return best, idx, obj


def allreduce_sums(values, group=None):
    """Sum a small float64 vector over the ranks (NestedKriging's unify step: sum w log theta, w sigma2, w beta0)."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.asarray(values, dtype=np.float64))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()
