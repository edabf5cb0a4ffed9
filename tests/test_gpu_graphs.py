"""CUDA graphs of the evaluation's launch sequences (the covariance build + factorisation, and the solves, GLS,
R^-1 and adjoint sums): captured on the second run of a configuration and replayed afterwards.  Replays give the
direct launches' results bit for bit, follow changes of the entries' designs, of the precision and of the look-ahead
width, and are counted as the launches they contain."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, d, seed=5):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.1 * rng.standard_normal(n)
    return X, y, rng.uniform(0.3, 1.2, size=d)


def _launches(lib):
    need = lib.lkg_stats_report(None, 0)
    buf = ctypes.create_string_buffer(max(need, 1))
    lib.lkg_stats_report(buf, need)
    return sum(int(line.split("\t")[1]) for line in buf.value.decode().splitlines())


def _evals(k, g, times):
    return [k.logLikelihoodFun(g, True)[:2] for _ in range(times)]


@pytest.mark.parametrize("n,slices", [(300, 0), (1100, 7)])
def test_replay_is_bit_identical(gpu_lib, n, slices):
    lib = gpu_lib.load()
    X, y, th = _data(n, 4)
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": th.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    k.set_precision(slices)
    g = np.concatenate([th, [1.0 / (1.0 + 1e-6)]])
    old = lib.lkg_set_graphs(0)
    try:
        ll0, g0 = _evals(k, g, 1)[0]
        lib.lkg_set_graphs(1)
        for ll, gr in _evals(k, g, 4):  # direct, capture + launch, replay, replay
            assert ll == ll0 and np.array_equal(gr, g0)
        # another point: the replayed sequence reads theta from device memory
        g2 = g.copy()
        g2[0] *= 1.3
        ll2, gr2 = _evals(k, g2, 1)[0]
        lib.lkg_set_graphs(0)
        ll2d, gr2d = _evals(k, g2, 1)[0]
        assert ll2 == ll2d and np.array_equal(gr2, gr2d)
    finally:
        lib.lkg_set_graphs(old)


def test_replay_follows_precision_and_lookahead(gpu_lib):
    lib = gpu_lib.load()
    X, y, th = _data(1100, 4)
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": th.reshape(1, -1), "sigma2": 1.0, "nugget": 1e-6})
    g = np.concatenate([th, [1.0 / (1.0 + 1e-6)]])
    old_g, old_la = lib.lkg_set_graphs(0), lib.lkg_get_lookahead()
    try:
        ref = {}
        for s in (7, 5):
            k.set_precision(s)
            ref[s] = _evals(k, g, 1)[0]
        lib.lkg_set_graphs(1)
        for s in (7, 5, 7, 5, 7):
            k.set_precision(s)
            for ll, gr in _evals(k, g, 3):
                assert ll == ref[s][0] and np.array_equal(gr, ref[s][1])
        k.set_precision(7)
        for ctas in (8, 0, 8):
            lib.lkg_set_lookahead(ctas)
            for ll, gr in _evals(k, g, 3):
                assert ll == ref[7][0] and np.array_equal(gr, ref[7][1])
    finally:
        lib.lkg_set_graphs(old_g)
        lib.lkg_set_lookahead(old_la)


def test_replay_follows_entry_designs(gpu_lib):
    """Batched evaluations over several designs (NestedKriging size classes): the entries' designs change between
    evaluations, the replays follow them."""
    lib = gpu_lib.load()
    X, y, _ = _data(900, 3)
    rng = np.random.default_rng(8)
    perm = rng.permutation(900)
    groups = [np.sort(perm[a:b]) for a, b in ((0, 200), (200, 420), (420, 650), (650, 900))]
    nk = gpu_lib.NestedKriging("matern3_2", aggregation="PoE")
    nk.fit_groups(y, X, groups, optim="none", parameters={"theta": np.full((1, 3), 0.4)})
    thetas = [rng.uniform(0.2, 0.8, size=(4, 3)) for _ in range(3)]
    old = lib.lkg_set_graphs(0)
    try:
        ref = [nk.logLikelihoodGroups(t, True) for t in thetas]
        lib.lkg_set_graphs(1)
        for _ in range(3):
            for t, (ll0, g0) in zip(thetas, ref):
                ll, gr = nk.logLikelihoodGroups(t, True)
                assert np.array_equal(ll, ll0) and np.array_equal(gr, g0)
    finally:
        lib.lkg_set_graphs(old)


def test_replay_counts_its_launches(gpu_lib):
    lib = gpu_lib.load()
    X, y, th = _data(600, 3)
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": th.reshape(1, -1)})
    old = lib.lkg_set_graphs(0)
    try:
        k.logLikelihoodFun(th, True)
        lib.lkg_stats_reset()
        k.logLikelihoodFun(th, True)
        direct = _launches(lib)
        lib.lkg_set_graphs(1)
        for _ in range(2):
            k.logLikelihoodFun(th, True)
        lib.lkg_stats_reset()
        k.logLikelihoodFun(th, True)
        assert _launches(lib) == direct > 0
    finally:
        lib.lkg_set_graphs(old)
