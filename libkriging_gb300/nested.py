"""Python ``NestedKriging`` mirroring pylibkriging's ``NestedKriging`` (= ``WrappedPyNestedKriging``).

Constructor forms, method names and defaults as the reference binding
(bindings/Python/pylibkriging/src/_pylibkriging/pylibkriging.cpp:224-285):

    NestedKriging(kernel) / NestedKriging(y, X, kernel, nb_groups, aggregation="NK", partition="kmeans", seed=123,
                  regmodel="constant", optim="BFGS", objective="LL", parameters={}, warping=[])
    fit(y, X, nb_groups, regmodel, optim, objective, parameters, warping)
    predict(X, return_stdev=True) -> (mean, stdev)
    summary, kernel, warping, aggregation, nb_groups, groups, theta, sigma2, beta0, X, y, set_predict_chunk

plus fit_groups (a given partition), submodel(i) and set_precision (mixed-precision submodel fits).  WarpKriging
submodels (warping) are not part of this library.  Every call goes through the C ABI of include/libkriging_gb300.h.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, cstr, f64, ptr
from .kriging import Kriging, _as_X

_NK_PARAM_KEYS = ("sigma2", "is_sigma2_estim", "theta", "is_theta_estim", "beta", "is_beta_estim")


def _params(parameters):
    P = dict(parameters or {})
    bad = set(P) - set(_NK_PARAM_KEYS)
    if bad:
        raise ValueError("unknown parameters: %s" % sorted(bad))
    s2 = P.get("sigma2")
    th = P.get("theta")
    be = P.get("beta")
    s2a = np.array([float(s2)]) if s2 is not None else None
    tha = f64(np.asarray(th, dtype=np.float64).reshape(-1)) if th is not None else None
    bea = f64(np.asarray(be, dtype=np.float64).reshape(-1)) if be is not None else None
    return (s2a, int(bool(P.get("is_sigma2_estim", True))), tha, 0 if tha is None else tha.size,
            int(bool(P.get("is_theta_estim", True))), bea, 0 if bea is None else bea.size,
            int(bool(P.get("is_beta_estim", True))))


def _check_warping(warping):
    if warping:
        raise ValueError("NestedKriging: WarpKriging submodels (warping) are not supported by the GPU build")


class NestedKriging:
    def __init__(self, *args, **kwargs):
        self._h = None
        self._X = None
        self._y = None
        L = _lib.load()
        if len(args) >= 3 or "y" in kwargs:
            names = ("y", "X", "kernel", "nb_groups", "aggregation", "partition", "seed", "regmodel", "optim",
                     "objective", "parameters", "warping")
            a = dict(zip(names, args))
            a.update(kwargs)
            _check_warping(a.get("warping"))
            self._h = L.lkg_nested_kriging_new(cstr(a["kernel"]), cstr(a.get("aggregation", "NK")),
                                               cstr(a.get("partition", "kmeans")), int(a.get("seed", 123)))
            if not self._h:
                raise _lib.LibKrigingError(_lib.last_error())
            self.fit(a["y"], a["X"], a["nb_groups"], a.get("regmodel", "constant"), a.get("optim", "BFGS"),
                     a.get("objective", "LL"), a.get("parameters") or {})
        else:
            kernel = args[0] if args else kwargs["kernel"]
            self._h = L.lkg_nested_kriging_new(cstr(kernel), cstr(kwargs.get("aggregation", "NK")),
                                               cstr(kwargs.get("partition", "kmeans")), int(kwargs.get("seed", 123)))
            if not self._h:
                raise _lib.LibKrigingError(_lib.last_error())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().lkg_nested_kriging_delete(h)
            except Exception:
                pass
            self._h = None

    def fit(self, y, X, nb_groups, regmodel="constant", optim="BFGS", objective="LL", parameters=None, warping=None):
        _check_warping(warping)
        X = _as_X(X)
        y = f64(np.asarray(y, dtype=np.float64).reshape(-1))
        n, d = X.shape
        s2, s2e, th, thn, the, be, ben, bee = _params(parameters)
        check(_lib.load().lkg_nested_kriging_fit(self._h, ptr(y), y.size, ptr(X), n, d, int(nb_groups), None, 0,
                                                 cstr(regmodel), cstr(optim), cstr(objective), ptr(s2), s2e, ptr(th),
                                                 thn, the, ptr(be), ben, bee))
        self._X, self._y = X, y
        return self

    def fit_groups(self, y, X, groups, regmodel="constant", optim="BFGS", objective="LL", parameters=None):
        """Fit on a given partition: `groups` is a list of index arrays, or one label per row."""
        X = _as_X(X)
        y = f64(np.asarray(y, dtype=np.float64).reshape(-1))
        n, d = X.shape
        if len(groups) == n and np.ndim(groups[0]) == 0:
            labels = np.ascontiguousarray(np.asarray(groups, dtype=np.int32))
        else:
            labels = np.full(n, -1, dtype=np.int32)
            for g, idx in enumerate(groups):
                labels[np.asarray(idx, dtype=np.int64)] = g
        ng = int(labels.max()) + 1 if n else 0
        s2, s2e, th, thn, the, be, ben, bee = _params(parameters)
        ip = ctypes.POINTER(ctypes.c_int)
        check(_lib.load().lkg_nested_kriging_fit_groups(self._h, ptr(y), y.size, ptr(X), n, d,
                                                        labels.ctypes.data_as(ip), ng, cstr(regmodel), cstr(optim),
                                                        cstr(objective), ptr(s2), s2e, ptr(th), thn, the, ptr(be),
                                                        ben, bee))
        self._X, self._y = X, y
        return self

    def predict(self, X, return_stdev=True):
        X = _as_X(X)
        m, d = X.shape
        mean = np.zeros(m)
        sd = np.zeros(m) if return_stdev else None
        check(_lib.load().lkg_nested_kriging_predict(self._h, ptr(X), m, d, int(bool(return_stdev)), ptr(mean),
                                                     ptr(sd)))
        return mean, (sd if return_stdev else np.zeros(0))

    def summary(self):
        s = _lib.load().lkg_nested_kriging_summary(self._h)
        if s is None:
            raise _lib.LibKrigingError(_lib.last_error())
        return s.decode()

    def __repr__(self):
        return self.summary()

    def kernel(self):
        return _lib.load().lkg_nested_kriging_kernel(self._h).decode()

    def warping(self):
        return []

    def aggregation(self):
        return _lib.load().lkg_nested_kriging_aggregation(self._h).decode()

    def nb_groups(self):
        return int(_lib.load().lkg_nested_kriging_nb_groups(self._h))

    def labels(self):
        n = ctypes.c_int()
        ip = ctypes.POINTER(ctypes.c_int)
        check(_lib.load().lkg_nested_kriging_get_groups(self._h, None, ctypes.byref(n)))
        lab = np.zeros(n.value, dtype=np.int32)
        check(_lib.load().lkg_nested_kriging_get_groups(self._h, lab.ctypes.data_as(ip), ctypes.byref(n)))
        return lab

    def groups(self):
        lab = self.labels()
        return [np.flatnonzero(lab == g) for g in range(self.nb_groups())]

    def theta(self):
        n = ctypes.c_int()
        check(_lib.load().lkg_nested_kriging_get_theta(self._h, None, ctypes.byref(n)))
        out = np.zeros(n.value)
        check(_lib.load().lkg_nested_kriging_get_theta(self._h, ptr(out), ctypes.byref(n)))
        return out

    def sigma2(self):
        return float(_lib.load().lkg_nested_kriging_get_sigma2(self._h))

    def beta0(self):
        return float(_lib.load().lkg_nested_kriging_get_beta0(self._h))

    def X(self):
        return self._X

    def y(self):
        return self._y

    def set_predict_chunk(self, chunk):
        check(_lib.load().lkg_nested_kriging_set_predict_chunk(self._h, int(chunk)))

    def set_precision(self, slices):
        check(_lib.load().lkg_nested_kriging_set_precision(self._h, int(slices)))

    def logLikelihoodGroups(self, thetas, return_grad=True):
        """Concentrated LL (and theta-gradient) of every submodel at theta row g, in one batched evaluation."""
        T = np.ascontiguousarray(np.atleast_2d(np.asarray(thetas, dtype=np.float64)))
        p, d = T.shape
        ll = np.zeros(p)
        g = np.zeros((p, d)) if return_grad else None
        check(_lib.load().lkg_nested_kriging_log_likelihood_groups(self._h, ptr(T), p, d, int(bool(return_grad)),
                                                                   ptr(ll), ptr(g)))
        return ll, g

    def group_estimates(self):
        """(theta [p, d], sigma2 [p], beta0 [p]) of the submodels before the common prior replaced them."""
        p, d = ctypes.c_int(), ctypes.c_int()
        L = _lib.load()
        check(L.lkg_nested_kriging_get_group_estimates(self._h, None, None, None, ctypes.byref(p), ctypes.byref(d)))
        th = np.zeros((p.value, d.value))
        s2 = np.zeros(p.value)
        b0 = np.zeros(p.value)
        check(L.lkg_nested_kriging_get_group_estimates(self._h, ptr(th), ptr(s2), ptr(b0), ctypes.byref(p),
                                                       ctypes.byref(d)))
        return th, s2, b0

    def submodel(self, i):
        h = _lib.load().lkg_nested_kriging_submodel(self._h, int(i))
        if not h:
            raise _lib.LibKrigingError(_lib.last_error())
        return Kriging._borrowed(h, self)
