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
