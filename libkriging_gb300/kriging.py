"""Python ``Kriging`` mirroring pylibkriging's ``Kriging`` (= ``WrappedPyKriging``).

Same constructor forms, method names, argument names / defaults and return tuples as the reference binding
(bindings/Python/pylibkriging/src/_pylibkriging/pylibkriging.cpp:120-205, Kriging_binding.cpp:260-264):

    Kriging(kernel) / Kriging(kernel, noise_model) / Kriging(y, X, kernel, regmodel="constant", normalize=False,
            optim="BFGS", objective="LL", parameters={}, noise=None)
    fit(y, X, regmodel, normalize, optim, objective, parameters)
    logLikelihoodFun(theta, return_grad=False, want_hess=False) -> (ll, grad, hess)
    predict(X, return_stdev=True, return_cov=False, return_deriv=False) -> (mean, stdev, cov, dmean, dstdev)

Every call goes through the C ABI of include/libkriging_gb300.h into the sm_103a kernels.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, cstr, f64, ptr

_PARAM_KEYS = ("sigma2", "is_sigma2_estim", "theta", "is_theta_estim", "beta", "is_beta_estim", "nugget",
               "is_nugget_estim")


def _as_X(X, n=None):
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X.reshape(-1, 1)
    return f64(X)


class Kriging:
    def __init__(self, *args, **kwargs):
        self._h = None
        L = _lib.load()
        if len(args) >= 3 or "y" in kwargs:
            names = ("y", "X", "kernel", "regmodel", "normalize", "optim", "objective", "parameters", "noise")
            a = dict(zip(names, args))
            a.update(kwargs)
            noise_model = a.pop("noise_model", "none")
            if a.get("noise") is not None:
                raise ValueError("per-observation noise is not supported by the GPU build")
            self._h = L.lkg_kriging_new(cstr(a["kernel"]), cstr(noise_model))
            if not self._h:
                raise _lib.LibKrigingError(_lib.last_error())
            self.fit(a["y"], a["X"], a.get("regmodel", "constant"), a.get("normalize", False), a.get("optim", "BFGS"),
                     a.get("objective", "LL"), a.get("parameters") or {})
        else:
            kernel = args[0] if args else kwargs["kernel"]
            noise_model = args[1] if len(args) > 1 else kwargs.get("noise_model", "none")
            self._h = L.lkg_kriging_new(cstr(kernel), cstr(noise_model))
            if not self._h:
                raise _lib.LibKrigingError(_lib.last_error())

    @classmethod
    def _borrowed(cls, handle, owner):
        """A view of a Kriging owned by another object (a NestedKriging submodel): never deleted from here."""
        k = cls.__new__(cls)
        k._h = handle
        k._owner = owner
        return k

    def __del__(self):
        h = getattr(self, "_h", None)
        if getattr(self, "_owner", None) is not None:
            self._h = None
            return
        if h:
            try:
                _lib.load().lkg_kriging_delete(h)
            except Exception:
                pass
            self._h = None

    # ---------------------------------------------------------------------------------------------------------
    def fit(self, y, X, regmodel="constant", normalize=False, optim="BFGS", objective="LL", parameters=None):
        X = _as_X(X)
        y = np.ascontiguousarray(np.asarray(y, dtype=np.float64).reshape(-1))
        n, d = X.shape
        P = dict(parameters or {})
        bad = set(P) - set(_PARAM_KEYS)
        if bad:
            raise ValueError("unknown parameters: %s" % sorted(bad))
        sigma2 = P.get("sigma2")
        nugget = P.get("nugget")
        theta = P.get("theta")
        beta = P.get("beta")
        s2 = None if sigma2 is None else np.array([sigma2], dtype=np.float64)
        nu = None if nugget is None else np.array([nugget], dtype=np.float64)
        th = None
        rows = 0
        if theta is not None:
            th = np.atleast_2d(np.asarray(theta, dtype=np.float64))
            if th.shape[1] != d and th.shape[0] == d:
                th = th.T
            rows = th.shape[0]
            th = f64(th)
        bt = None if beta is None else np.ascontiguousarray(np.asarray(beta, dtype=np.float64).reshape(-1))
        check(_lib.load().lkg_kriging_fit_params(
            self._h, ptr(y), n, ptr(X), n, d, cstr(regmodel), int(bool(normalize)), cstr(optim), cstr(objective),
            ptr(s2), int(P.get("is_sigma2_estim", True)), ptr(th), rows, int(P.get("is_theta_estim", True)),
            ptr(bt), 0 if bt is None else bt.size, int(P.get("is_beta_estim", True)), ptr(nu),
            int(P.get("is_nugget_estim", True))))
        return self

    def update(self, y_u, X_u, refit=True):
        """Kriging::update (Kriging.cpp:2433-2633): append (X_u, y_u) in original units; refit as the reference."""
        X = _as_X(X_u)
        y = np.ascontiguousarray(np.asarray(y_u, dtype=np.float64).reshape(-1))
        check(_lib.load().lkg_kriging_update(self._h, ptr(y), y.size, None, 0, ptr(X), X.shape[0], X.shape[1],
                                             int(bool(refit))))
        return self

    def save(self, filename):
        """libKriging's JSON model file, version 2 (Kriging.cpp:2691-2717)."""
        check(_lib.load().lkg_kriging_save(self._h, cstr(str(filename))))

    @staticmethod
    def load(filename):
        """A model saved by save() or by libKriging's Kriging::save (Kriging.cpp:2719-2749)."""
        L = _lib.load()
        h = L.lkg_kriging_load(cstr(str(filename)))
        if not h:
            raise _lib.LibKrigingError(_lib.last_error())
        k = Kriging.__new__(Kriging)
        k._h = h
        return k

    def copy(self):
        h = _lib.load().lkg_kriging_copy(self._h)
        if not h:
            raise _lib.LibKrigingError(_lib.last_error())
        k = Kriging.__new__(Kriging)
        k._h = h
        return k

    def covMat(self, X1, X2):
        """sigma2 C(X1, X2) in original units (KrigingImpl.cpp:60-71)."""
        A, B = _as_X(X1), _as_X(X2)
        out = np.zeros((A.shape[0], B.shape[0]), order="F")
        check(_lib.load().lkg_kriging_cov_mat(self._h, ptr(A), A.shape[0], A.shape[1], ptr(B), B.shape[0],
                                              B.shape[1], ptr(out)))
        return out

    def logLikelihoodFun(self, theta, return_grad=False, want_hess=False, bench=False):
        if want_hess:
            raise ValueError("logLikelihoodFun: the Hessian is not supported by the GPU build")
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
        ll = ctypes.c_double()
        g = np.zeros(t.size) if return_grad else None
        if bench:
            buf = ctypes.create_string_buffer(4096)
            check(_lib.load().lkg_kriging_log_likelihood_fun_bench(self._h, ptr(t), t.size, int(bool(return_grad)),
                                                                   ctypes.byref(ll), ptr(g), buf, 4096))
            self.last_bench = {kv.split("\t")[0]: float(kv.split("\t")[1])
                               for kv in buf.value.decode().split("\n") if kv}
        else:
            check(_lib.load().lkg_kriging_log_likelihood_fun(self._h, ptr(t), t.size, int(bool(return_grad)), 0,
                                                             ctypes.byref(ll), ptr(g), None))
        return ll.value, (g if return_grad else np.zeros(0)), np.zeros((0, 0))

    def logLikelihoodFunBatch(self, thetas, return_grad=True, bench=False):
        """k candidate gammas (rows) in one batched GPU evaluation -> (ll[k], grad[k, gdim]); bench=True stores the
        pass's per-stage timings (ms) in self.last_bench."""
        T = f64(np.atleast_2d(np.asarray(thetas, dtype=np.float64)))
        k, gd = T.shape
        ll = np.zeros(k)
        g = np.zeros((k, gd), order="F") if return_grad else None
        if bench:
            buf = ctypes.create_string_buffer(4096)
            check(_lib.load().lkg_kriging_log_likelihood_fun_batch_bench(
                self._h, ptr(T), k, gd, int(bool(return_grad)), ptr(ll), ptr(g), buf, 4096))
            self.last_bench = {kv.split("\t")[0]: float(kv.split("\t")[1])
                               for kv in buf.value.decode().split("\n") if kv}
        else:
            check(_lib.load().lkg_kriging_log_likelihood_fun_batch(self._h, ptr(T), k, gd, int(bool(return_grad)),
                                                                   ptr(ll), ptr(g)))
        return ll, (np.ascontiguousarray(g) if return_grad else None)

    def logLikelihood(self):
        v = _lib.load().lkg_kriging_log_likelihood(self._h)
        if np.isnan(v):
            err = _lib.last_error()
            if err:
                raise _lib.LibKrigingError(err)
        return v

    def _nan_checked(self, v):
        if np.isnan(v):
            err = _lib.last_error()
            if err:
                raise _lib.LibKrigingError(err)
        return v

    # ---- leave-one-out and marginal posterior (Kriging.hpp:135-143) ----
    def leaveOneOutFun(self, theta, return_grad=False):
        """Kriging::leaveOneOutFun -> (loo, grad); grad is empty unless return_grad."""
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
        v = ctypes.c_double()
        g = np.zeros(t.size) if return_grad else None
        check(_lib.load().lkg_kriging_leave_one_out_fun(self._h, ptr(t), t.size, int(bool(return_grad)),
                                                        ctypes.byref(v), ptr(g)))
        return v.value, (g if return_grad else np.zeros(0))

    def leaveOneOutVec(self, theta):
        """Kriging::leaveOneOutVec -> (leave-one-out means, standard deviations) in the model's units."""
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
        n = self.y().size
        yhat, sd = np.zeros(n), np.zeros(n)
        check(_lib.load().lkg_kriging_leave_one_out_vec(self._h, ptr(t), t.size, ptr(yhat), ptr(sd)))
        return yhat, sd

    def leaveOneOut(self):
        return self._nan_checked(_lib.load().lkg_kriging_leave_one_out(self._h))

    def logMargPostFun(self, theta, return_grad=False):
        """Kriging::logMargPostFun -> (lmp, grad)."""
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
        v = ctypes.c_double()
        gd = t.size + (1 if (self.noise_model() == "nugget" and t.size == self.centerX().size) else 0)
        g = np.zeros(gd) if return_grad else None
        check(_lib.load().lkg_kriging_log_marg_post_fun(self._h, ptr(t), t.size, int(bool(return_grad)),
                                                        ctypes.byref(v), ptr(g)))
        return v.value, (g if return_grad else np.zeros(0))

    def logMargPost(self):
        return self._nan_checked(_lib.load().lkg_kriging_log_marg_post(self._h))

    def predict(self, X, return_stdev=True, return_cov=False, return_deriv=False):
        X = _as_X(X)
        m, d = X.shape
        mean = np.zeros(m)
        sd = np.zeros(m) if return_stdev else None
        cov = np.zeros((m, m), order="F") if return_cov else None
        md = np.zeros((m, d), order="F") if return_deriv else None
        sdd = np.zeros((m, d), order="F") if return_deriv else None
        check(_lib.load().lkg_kriging_predict(self._h, ptr(X), m, d, int(bool(return_stdev)), int(bool(return_cov)),
                                              int(bool(return_deriv)), ptr(mean), ptr(sd), ptr(cov), ptr(md),
                                              ptr(sdd)))
        return mean, sd, cov, md, sdd

    # ---- Vecchia (Kriging.hpp:145-173) ----
    def predictVecchia(self, X, return_stdev=True, m=0):
        """Kriging::predictVecchia: each point kriged on its m nearest observations -> (mean, stdev)."""
        X = _as_X(X)
        q, d = X.shape
        mean = np.zeros(q)
        sd = np.zeros(q) if return_stdev else None
        check(_lib.load().lkg_kriging_predict_vecchia(self._h, ptr(X), q, d, int(bool(return_stdev)), int(m),
                                                      ptr(mean), ptr(sd)))
        return mean, (sd if return_stdev else np.zeros(0))

    def logLikelihoodVecchiaFun(self, theta, return_grad=False):
        t = np.ascontiguousarray(np.asarray(theta, dtype=np.float64).reshape(-1))
        v = ctypes.c_double()
        g = np.zeros(t.size) if return_grad else None
        check(_lib.load().lkg_kriging_log_likelihood_vecchia_fun(self._h, ptr(t), t.size, int(bool(return_grad)),
                                                                 ctypes.byref(v), ptr(g)))
        return v.value, (g if return_grad else np.zeros(0))

    def set_vecchia_exact_commit(self, b):
        check(_lib.load().lkg_kriging_set_vecchia_exact_commit(self._h, int(bool(b))))

    def vecchia_neighbors(self):
        return _lib.load().lkg_kriging_vecchia_neighbors(self._h)

    def is_vecchia_light(self):
        return bool(_lib.load().lkg_kriging_is_vecchia_light(self._h))

    def vecchia_sets(self):
        """(order[n], neighbours[n, m]) of the fitted Vecchia model (global row indices, -1 padded)."""
        n, m = ctypes.c_int(), ctypes.c_int()
        check(_lib.load().lkg_kriging_get_vecchia_sets(self._h, None, None, ctypes.byref(n), ctypes.byref(m)))
        order = np.zeros(n.value, dtype=np.int32)
        nbr = np.zeros((n.value, m.value), dtype=np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        check(_lib.load().lkg_kriging_get_vecchia_sets(self._h, order.ctypes.data_as(ip), nbr.ctypes.data_as(ip),
                                                       ctypes.byref(n), ctypes.byref(m)))
        return order, nbr

    def set_precision(self, slices):
        """0: FP64 path (default); 4..8: mixed path with that many bf16 digit slices (see the C header)."""
        check(_lib.load().lkg_kriging_set_precision(self._h, int(slices)))
        return self

    def precision(self):
        return _lib.load().lkg_kriging_get_precision(self._h)

    def last_slices(self):
        return _lib.load().lkg_kriging_last_slices(self._h)

    def autotune_precision(self, gamma, tol_ll=1e-8, tol_grad=1e-6):
        """Pick and set the fastest precision (0 = FP64, 5..7 mixed slices) whose LL / gradient at gamma stay within
        the tolerances of the FP64 path's (see lkg_kriging_autotune_precision); returns it."""
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        r = _lib.load().lkg_kriging_autotune_precision(self._h, ptr(g), g.size, float(tol_ll), float(tol_grad))
        if r < 0:
            raise _lib.LibKrigingError(_lib.last_error())
        return r

    def autotune_lookahead(self, gamma):
        """Time the mixed Cholesky's look-ahead with 0 / 12 / 16 / 24 / 32 SMs for the panel work on this model and table
        the fastest for its size (see lkg_kriging_autotune_lookahead); returns it."""
        g = np.ascontiguousarray(gamma, dtype=np.float64)
        r = _lib.load().lkg_kriging_autotune_lookahead(self._h, ptr(g), g.size)
        if r < 0:
            raise _lib.LibKrigingError(_lib.last_error())
        return r

    def eval_counts(self):
        """(objective evaluations, GPU evaluation launches) since this model was created."""
        ev, ro = ctypes.c_longlong(), ctypes.c_longlong()
        check(_lib.load().lkg_kriging_eval_counts(self._h, ctypes.byref(ev), ctypes.byref(ro)))
        return int(ev.value), int(ro.value)

    def summary(self):
        s = _lib.load().lkg_kriging_summary(self._h)
        return s.decode() if s else ""

    # ---- accessors (pylibkriging.cpp:196-230) ----
    def _vec(self, fn):
        n = ctypes.c_int()
        check(fn(self._h, None, ctypes.byref(n)))
        out = np.zeros(n.value)
        check(fn(self._h, ptr(out), ctypes.byref(n)))
        return out

    def _mat(self, fn):
        r, c = ctypes.c_int(), ctypes.c_int()
        check(fn(self._h, None, ctypes.byref(r), ctypes.byref(c)))
        out = np.zeros((r.value, c.value), order="F")
        check(fn(self._h, ptr(out), ctypes.byref(r), ctypes.byref(c)))
        return out

    def kernel(self):
        return _lib.load().lkg_kriging_kernel(self._h).decode()

    def optim(self):
        return _lib.load().lkg_kriging_optim(self._h).decode()

    def objective(self):
        return _lib.load().lkg_kriging_objective(self._h).decode()

    def regmodel(self):
        return _lib.load().lkg_kriging_regmodel(self._h).decode()

    def normalize(self):
        return bool(_lib.load().lkg_kriging_is_normalize(self._h))

    def X(self):
        return self._mat(_lib.load().lkg_kriging_get_X)

    def y(self):
        return self._vec(_lib.load().lkg_kriging_get_y)

    def centerX(self):
        return self._vec(_lib.load().lkg_kriging_get_centerX)

    def scaleX(self):
        return self._vec(_lib.load().lkg_kriging_get_scaleX)

    def centerY(self):
        return _lib.load().lkg_kriging_get_centerY(self._h)

    def scaleY(self):
        return _lib.load().lkg_kriging_get_scaleY(self._h)

    def F(self):
        return self._mat(_lib.load().lkg_kriging_get_F)

    def T(self):
        return self._mat(_lib.load().lkg_kriging_get_T)

    def M(self):
        return self._mat(_lib.load().lkg_kriging_get_M)

    def z(self):
        return self._vec(_lib.load().lkg_kriging_get_z)

    def beta(self):
        return self._vec(_lib.load().lkg_kriging_get_beta)

    def is_beta_estim(self):
        return bool(_lib.load().lkg_kriging_is_beta_estim(self._h))

    def theta(self):
        return self._vec(_lib.load().lkg_kriging_get_theta)

    def is_theta_estim(self):
        return bool(_lib.load().lkg_kriging_is_theta_estim(self._h))

    def sigma2(self):
        return _lib.load().lkg_kriging_get_sigma2(self._h)

    def is_sigma2_estim(self):
        return bool(_lib.load().lkg_kriging_is_sigma2_estim(self._h))

    def noise_model(self):
        return _lib.load().lkg_kriging_noise_model(self._h).decode()

    def nugget(self):
        return _lib.load().lkg_kriging_get_nugget(self._h)

    def is_nugget_estim(self):
        return bool(_lib.load().lkg_kriging_is_nugget_estim(self._h))


# ---- process-wide settings (LinearAlgebra / Optim statics) ----
def set_num_nugget(v):
    _lib.load().lkg_set_num_nugget(float(v))


def get_num_nugget():
    return _lib.load().lkg_get_num_nugget()


def check_chol_rcond(b):
    _lib.load().lkg_check_chol_rcond(int(bool(b)))


class Optim:
    @staticmethod
    def use_reparametrize(b):
        _lib.load().lkg_optim_use_reparametrize(int(bool(b)))

    @staticmethod
    def set_theta_lower_factor(f):
        _lib.load().lkg_optim_set_theta_lower_factor(float(f))

    @staticmethod
    def set_theta_upper_factor(f):
        _lib.load().lkg_optim_set_theta_upper_factor(float(f))

    @staticmethod
    def use_variogram_bounds_heuristic(b):
        _lib.load().lkg_optim_use_variogram_bounds_heuristic(int(bool(b)))

    @staticmethod
    def set_log_level(level):
        _lib.load().lkg_optim_set_log_level(int(level))

    @staticmethod
    def set_max_iteration(m):
        _lib.load().lkg_optim_set_max_iteration(int(m))

    @staticmethod
    def set_gradient_tolerance(t):
        _lib.load().lkg_optim_set_gradient_tolerance(float(t))

    @staticmethod
    def set_objective_rel_tolerance(t):
        _lib.load().lkg_optim_set_objective_rel_tolerance(float(t))

    @staticmethod
    def set_max_restart(m):
        _lib.load().lkg_optim_set_max_restart(int(m))


def vecchia_sets(X, m):
    """GPU construction of the Vecchia sets of make_vecchia_sets: (order[n], neighbours[n, m], -1 padded)."""
    X = _as_X(X)
    n, d = X.shape
    order = np.zeros(n, dtype=np.int32)
    nbr = np.zeros((n, m), dtype=np.int32)
    ip = ctypes.POINTER(ctypes.c_int)
    check(_lib.load().lkg_vecchia_sets(n, d, ptr(X), m, order.ctypes.data_as(ip), nbr.ctypes.data_as(ip)))
    return order, nbr


class VecchiaShard:
    """One rank's share of a sharded Vecchia likelihood: the ordered positions [t0, t1) of the sets (order, nbr) of
    the normalised design (X n x d, y n, F n x p).  See lkg_vecchia_shard_* in the C header."""

    def __init__(self, kernel, X, y, F, order, nbr, t0, t1):
        L = _lib.load()
        X = _as_X(X)
        n, d = X.shape
        y = f64(np.asarray(y, dtype=np.float64).reshape(-1))
        F = f64(np.asarray(F, dtype=np.float64).reshape(n, -1))
        self.d, self.p = d, F.shape[1]
        self._order = np.ascontiguousarray(order, dtype=np.int32)
        self._nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        m = self._nbr.shape[1] if self._nbr.ndim == 2 else 0
        ip = ctypes.POINTER(ctypes.c_int)
        self._h = L.lkg_vecchia_shard_new(cstr(kernel), n, d, self.p, ptr(X), ptr(y), ptr(F),
                                          self._order.ctypes.data_as(ip), self._nbr.ctypes.data_as(ip), m, int(t0),
                                          int(t1))
        if not self._h:
            raise _lib.LibKrigingError(_lib.last_error())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _lib.load().lkg_vecchia_shard_delete(h)
            except Exception:
                pass

    def sums1(self, theta, return_grad=True):
        t = np.ascontiguousarray(theta, dtype=np.float64)
        s1 = np.zeros(self.p * self.p + self.p + 1)
        npts = ctypes.c_longlong()
        failed = ctypes.c_int()
        check(_lib.load().lkg_vecchia_shard_sums1(self._h, ptr(t), int(bool(return_grad)), ptr(s1),
                                                  ctypes.byref(npts), ctypes.byref(failed)))
        return s1, int(failed.value), int(npts.value)

    def sums2(self, beta, return_grad=True):
        b = np.ascontiguousarray(beta, dtype=np.float64)
        s2 = np.zeros(1 + 2 * self.d)
        check(_lib.load().lkg_vecchia_shard_sums2(self._h, ptr(b) if b.size else None, int(bool(return_grad)),
                                                  ptr(s2)))
        return s2


def vecchia_gls_beta(p, s1):
    """The GLS beta of the summed stage-1 sums: (A + num_nugget I) beta = b (Kriging.cpp:895-905)."""
    s1 = np.ascontiguousarray(s1, dtype=np.float64)
    beta = np.zeros(p)
    check(_lib.load().lkg_vecchia_gls_beta(int(p), ptr(s1), ptr(beta) if p else None))
    return beta


def vecchia_finish(n, d, slogv, s2, return_grad=True):
    """(vll, sigma2, grad) from the summed stage-2 sums (Kriging.cpp:906-922)."""
    s2 = np.ascontiguousarray(s2, dtype=np.float64)
    vll, s2o = ctypes.c_double(), ctypes.c_double()
    g = np.zeros(d)
    check(_lib.load().lkg_vecchia_finish(int(n), int(d), float(slogv), ptr(s2), int(bool(return_grad)),
                                         ctypes.byref(vll), ctypes.byref(s2o), ptr(g)))
    return vll.value, s2o.value, (g if return_grad else None)
