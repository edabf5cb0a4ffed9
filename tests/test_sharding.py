"""CPU (gloo, world_size 2) tests of the multi-GPU sharding host logic: partition, winner selection with the
reference's tie rule, failed units, and the small all-reduce of NestedKriging's unify step."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from libkriging_gb300.sharding import shard_range


def test_shard_range_partitions():
    for n in (0, 1, 5, 64, 65):
        for w in (1, 2, 3, 8):
            spans = [shard_range(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(w - 1))
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1


class _FakeModel:
    """Stands in for a GPU model on CPU: 'fitting' from start theta0 lands on a deterministic local optimum."""

    def fit(self, y, X, regmodel, normalize, optim, objective, parameters):
        th = np.asarray(parameters["theta"], dtype=float).reshape(-1)
        if optim == "none":
            self._theta = th
            return
        if th[0] < 0:
            raise RuntimeError("start failed")
        self._theta = np.round(th, 1)  # local optimum reached from this start

    def theta(self):
        return self._theta

    def logLikelihood(self):
        return -float(np.sum((self._theta - 0.7) ** 2))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from libkriging_gb300.sharding import allreduce_sums, fit_multistart_sharded, select_best
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        starts = np.array([[0.1, 0.2], [-1.0, 0.0], [0.66, 0.74], [0.9, 0.9], [0.71, 0.69]])
        best, idx, obj = fit_multistart_sharded(_FakeModel, None, None, starts)
        # ties: starts 2 and 4 both round to (0.7, 0.7); the lowest index wins
        ties = select_best([(rank, 1.0, rank)])
        s = allreduce_sums([rank + 1.0, 2.0 * rank])
        q.put((rank, idx, obj, best.theta().tolist(), ties[0], s.tolist()))
    finally:
        dist.destroy_process_group()


def test_multistart_selection_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    for rank, idx, obj, theta, tie, s in res:
        assert idx == 2 and abs(obj) < 1e-12
        assert np.allclose(theta, [0.7, 0.7])
        assert tie == 0
        assert s == [3.0, 2.0]


class _FakeSub:
    def __init__(self, mu, sd):
        self._mu, self._sd = mu, sd

    def predict(self, Xn, return_stdev, return_cov, return_deriv):
        q = np.asarray(Xn).shape[0]
        return np.full(q, self._mu), np.full(q, self._sd), None, None, None


class _FakeNested:
    """Stands in for a GPU NestedKriging: the 'fitted' submodel of a group is a function of its rows."""

    def fit_groups(self, y, X, groups, regmodel, optim, objective, parameters):
        self._groups = [np.asarray(g) for g in groups]
        self._y = np.asarray(y)
        self._fixed = parameters if optim == "none" else None

    def group_estimates(self):
        th = np.array([[0.1 + 0.01 * len(g), 0.5] for g in self._groups])
        s2 = np.array([1.0 + float(np.mean(self._y[g])) ** 2 for g in self._groups])
        b0 = np.array([float(np.mean(self._y[g])) for g in self._groups])
        return th, s2, b0

    def nb_groups(self):
        return len(self._groups)

    def submodel(self, i):
        g = self._groups[i]
        return _FakeSub(float(np.mean(self._y[g])), 0.1 + 0.01 * len(g))


def _nested_reference(y, groups, aggregation):
    """The same pipeline in one process: unify sums over all groups, then the PoE-family formulas."""
    n = sum(len(g) for g in groups)
    th = np.array([[0.1 + 0.01 * len(g), 0.5] for g in groups])
    s2 = np.array([1.0 + float(np.mean(y[g])) ** 2 for g in groups])
    b0 = np.array([float(np.mean(y[g])) for g in groups])
    w = np.array([len(g) for g in groups], dtype=float)
    theta = np.exp((w[:, None] * np.log(th)).sum(axis=0) / n)
    sigma2 = float((w * s2).sum() / n)
    beta0 = float((w * b0).sum() / n)
    mu = np.array([np.mean(y[g]) for g in groups])
    v = np.array([(0.1 + 0.01 * len(g)) ** 2 + 1e-12 for g in groups])
    p = len(groups)
    if aggregation == "gPoE":
        prec = np.sum(1 / v) / p
        mean = (np.sum(mu / v) / p) / prec
    else:  # rBCM
        b = 0.5 * (np.log(sigma2) - np.log(v))
        prec = max(np.sum(b / v) + (1 - np.sum(b)) / sigma2, 1e-12)
        mean = np.sum(b * mu / v) / prec
    return theta, sigma2, beta0, mean, np.sqrt(1 / prec)


def _nested_worker(rank, world, port, q):
    import torch.distributed as dist
    from libkriging_gb300.sharding import fit_nested_sharded, predict_poe_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(0)
        y = rng.standard_normal(60)
        X = rng.uniform(size=(60, 2))
        perm = rng.permutation(60)
        groups = [np.sort(perm[a:b]) for a, b in [(0, 7), (7, 20), (20, 31), (31, 44), (44, 60)]]
        nk, mine, (theta, sigma2, beta0) = fit_nested_sharded(_FakeNested, y, X, groups)
        fixed = nk._fixed
        out = []
        for agg in ("gPoE", "rBCM"):
            m, s = predict_poe_sharded(nk, np.zeros((3, 2)), agg, sigma2, len(groups))
            out.append((m.tolist(), s.tolist()))
        q.put((rank, mine, theta.tolist(), sigma2, beta0, float(fixed["sigma2"]), out, y.tolist(),
               [g.tolist() for g in groups]))
    finally:
        dist.destroy_process_group()


def test_nested_sharded_fit_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 7) % 1000
    procs = [ctx.Process(target=_nested_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda r: r[0])
    bins = [r[1] for r in res]
    assert sorted(bins[0] + bins[1]) == [0, 1, 2, 3, 4] and not set(bins[0]) & set(bins[1])
    y = np.array(res[0][7])
    groups = [np.array(g) for g in res[0][8]]
    for rank, mine, theta, sigma2, beta0, fixed_s2, out, _, _ in res:
        for i, agg in enumerate(("gPoE", "rBCM")):
            t_ref, s_ref, b_ref, m_ref, sd_ref = _nested_reference(y, groups, agg)
            assert np.allclose(theta, t_ref, rtol=1e-12) and abs(sigma2 - s_ref) < 1e-12
            assert abs(beta0 - b_ref) < 1e-12 and fixed_s2 == sigma2
            assert np.allclose(out[i][0], m_ref, rtol=1e-12) and np.allclose(out[i][1], sd_ref, rtol=1e-12)
