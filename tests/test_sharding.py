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
        starts = np.atleast_2d(np.asarray(parameters["theta"], dtype=float))
        if optim == "none":
            self._theta = starts[0]
            return
        assert optim == "BFGS%d" % starts.shape[0] or (optim == "BFGS" and starts.shape[0] == 1)
        best = None
        for th in starts:  # BFGSk: every start, the first of the best kept (strict '<' on the objective)
            if th[0] < 0:
                continue  # a failed start
            opt = np.round(th, 1)  # local optimum reached from this start
            ll = -float(np.sum((opt - 0.7) ** 2))
            if best is None or -ll < -best[0]:
                best = (ll, opt)
        if best is None:
            raise RuntimeError("All optimization attempts failed")
        self._theta = best[1]

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
        # starts 2 (rank 0's share 0..2) and 4 (rank 1's share 3..4) tie at (0.7, 0.7): rank 0's share wins
        assert idx == 0 and abs(obj) < 1e-12
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


class _FakeVecchiaShard:
    """Stands in for a GPU VecchiaShard: per-point terms u, v, W and their derivatives drawn from a fixed seed (the
    host algebra of the split does not depend on where they come from)."""

    def __init__(self, n, d, p, t0, t1, seed=3):
        rng = np.random.default_rng(seed)
        self.u = rng.standard_normal(n)
        self.v = rng.uniform(0.1, 1.0, n)
        self.W = rng.standard_normal((n, p))
        self.du = rng.standard_normal((n, d))
        self.dv = 0.01 * rng.standard_normal((n, d))
        self.dW = rng.standard_normal((n, d, p))
        self.t0, self.t1, self.p, self.d = t0, t1, p, d

    def sums1(self, theta, grad):
        r = slice(self.t0, self.t1)
        W, u, v = self.W[r], self.u[r], self.v[r]
        A = (W[:, :, None] * W[:, None, :] / v[:, None, None]).sum(axis=0)
        b = (W * (u / v)[:, None]).sum(axis=0)
        return np.concatenate([A.ravel(), b, [np.log(v).sum()]]), 0, 0

    def sums2(self, beta, grad):
        r = slice(self.t0, self.t1)
        e = self.u[r] - self.W[r] @ beta
        v = self.v[r]
        de = self.du[r] - np.einsum("tkq,q->tk", self.dW[r], beta)
        dQ = (2 * e[:, None] * de / v[:, None] - (e * e / (v * v))[:, None] * self.dv[r]).sum(axis=0)
        return np.concatenate([[np.sum(e * e / v)], dQ, (self.dv[r] / v[:, None]).sum(axis=0)])


def _vecchia_worker(rank, world, port, q):
    import torch.distributed as dist
    from libkriging_gb300.sharding import vecchia_ll_sharded
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n, d, p = 1001, 3, 2
        vll, grad, beta, sigma2 = vecchia_ll_sharded(lambda t0, t1: _FakeVecchiaShard(n, d, p, t0, t1), n, d, p,
                                                     np.ones(d))
        q.put((rank, vll, grad.tolist(), beta.tolist(), sigma2))
    finally:
        dist.destroy_process_group()


def test_vecchia_sharded_gloo_world2():
    """Two ranks, each with half of the ordered points: the two partial-sum exchanges give the single-rank VLL,
    gradient, beta and sigma2 (Kriging.cpp:895-922 over all points in one loop) to 1e-12."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() + 13) % 1000
    procs = [ctx.Process(target=_vecchia_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # the same algebra over all points at once
    n, d, p = 1001, 3, 2
    f = _FakeVecchiaShard(n, d, p, 0, n)
    s1 = f.sums1(None, True)[0]
    A = s1[:p * p].reshape(p, p) + 1e-10 * np.eye(p)  # num_nugget (default 1e-10) on the GLS diagonal
    beta = np.linalg.solve(A, s1[p * p:p * p + p])
    s2 = f.sums2(beta, True)
    sigma2 = s2[0] / n
    vll = -0.5 * n * np.log(2 * np.pi * sigma2) - 0.5 * s1[-1] - 0.5 * n
    grad = -0.5 * n * s2[1:1 + d] / s2[0] - 0.5 * s2[1 + d:]
    for rank, vll_r, grad_r, beta_r, sigma2_r in res:
        assert abs(vll_r - vll) <= 1e-12 * abs(vll)
        assert np.allclose(grad_r, grad, rtol=1e-12, atol=0)
        assert np.allclose(beta_r, beta, rtol=1e-12) and abs(sigma2_r - sigma2) <= 1e-12 * sigma2
