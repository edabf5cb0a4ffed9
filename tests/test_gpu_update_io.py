"""GPU tests of Kriging::update (incremental data), save / load (libKriging's JSON model files, version 2), covMat
and copy.

* update(refit=false): the factor of the joined design comes from the incremental Cholesky (chol_block,
  LinearAlgebra.cpp:254-299) on the GPU; checked against the oracle's restatement of update_cholCov + chol_block
  (L 1e-12, beta / SSE 1e-10) and against a from-scratch fit at the same theta (predictions 1e-10).
* update(refit=true): the reference's own criterion (tests/KrigingUpdateTest.cpp: theta, sigma2, beta within 5 %
  and predictions within 10 % / 5 % of a fit on the joined data).
* save / load: a round trip restores every accessor and gives bit-identical predictions; the file follows the
  reference's layout (KrigingImpl.cpp:644-711: base64 little-endian column-major payloads); a file written in that
  layout from the oracle's model loads and predicts like the oracle (1e-12).
"""
import base64
import json

import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REF_KEYS = {"version", "content", "covType", "X", "centerX", "scaleX", "y", "centerY", "scaleY", "normalize",
            "regmodel", "optim", "objective", "dX", "maxdX", "F", "T", "R", "M", "star", "circ", "z", "Rinv", "beta",
            "est_beta", "theta", "est_theta", "sigma2", "est_sigma2", "noise_model", "nystrom_light"}


def _data(n, d, seed):
    rng = np.random.default_rng(seed)
    X = rng.uniform(size=(n, d))
    y = np.sin(2 * np.pi * X).sum(axis=1) + 0.3 * X[:, 0] * X[:, -1]
    return X, y


def _decode(node):
    raw = base64.b64decode(node["base64_data"])
    v = np.frombuffer(raw, dtype="<f8")
    if node["type"] == "mat":
        return v.reshape((node["n_cols"], node["n_rows"])).T
    assert v.size == node["size"]
    return v.copy()


def _encode(a, kind):
    a = np.asarray(a, dtype=np.float64)
    data = base64.b64encode(np.asfortranarray(a).ravel(order="F").astype("<f8").tobytes()).decode()
    if kind == "mat":
        a2 = np.atleast_2d(a) if a.ndim < 2 else a
        return {"type": "mat", "n_rows": int(a2.shape[0]), "n_cols": int(a2.shape[1]), "base64_data": data}
    return {"type": kind, "size": int(a.size), "base64_data": data}


@pytest.mark.parametrize("kernel,noise,no,nu", [("matern5_2", "none", 150, 37), ("gauss", "none", 128, 64),
                                                 ("exp", "nugget", 200, 1), ("matern3_2", "nugget", 97, 130)])
def test_update_norefit_is_the_block_factor(gpu_lib, kernel, noise, no, nu):
    d = 3
    X, y = _data(no + nu, d, 11)
    # gauss correlations decay fastest: a shorter range keeps this design moderately conditioned
    theta = np.array([0.35, 0.5, 0.42]) * (0.45 if kernel == "gauss" else 1.0)
    params = {"theta": theta.reshape(1, -1)}
    alpha = 1.0
    if noise == "nugget":
        params.update(sigma2=1.0, nugget=0.05)
        alpha = 1.0 / 1.05
    k = gpu_lib.Kriging(kernel, noise)
    k.fit(y[:no], X[:no], "constant", False, "none", "LL", params)
    L_old = k.T()
    k.update(y[no:], X[no:], False)
    # oracle: update_cholCov + chol_block + populate_Model's GLS
    F = O.regression_matrix("constant", X)
    m, fb = O.update_no_refit(kernel, X[:no], L_old, X[no:], y, F, theta, alpha)
    assert not fb
    T = k.T()
    kappa = np.max(np.diag(m.L)) / np.min(np.diag(m.L))  # lower bound of cond(L)
    assert np.max(np.abs(T @ T.T - m.R)) < 1e-13  # backward error of the block factor
    assert np.max(np.abs(T - m.L)) < 1e-13 * kappa
    assert rel_err(k.beta(), m.betahat) < 1e-10 * kappa
    assert rel_err(k.z(), m.Estar) < 1e-10 * kappa
    # sigma2 = SSE / n for every noise model (KrigingImpl.cpp:632-634)
    assert abs(k.sigma2() - m.SSEstar / (no + nu)) <= 1e-10 * abs(k.sigma2())
    assert np.array_equal(k.theta(), theta)
    # the same model fitted from scratch at this theta predicts the same means
    k2 = gpu_lib.Kriging(kernel, noise)
    k2.fit(y, X, "constant", False, "none", "LL", params)
    Xn = np.random.default_rng(12).uniform(size=(50, d))
    assert rel_err(k.predict(Xn, False)[0], k2.predict(Xn, False)[0]) < 1e-10


def test_update_norefit_duplicate_point_jitters_schur_block(gpu_lib):
    """A new point equal to an old one: the Schur complement is zero up to rounding.  Whether its computed value is a
    tiny positive number or <= 0 (then safe_chol_lower's jitter goes on that block alone) depends on the rounding of
    the implementation, as between LAPACK builds; in both cases the old block of the factor stays exactly as it was
    and the new row repeats row 5 of L."""
    X, y = _data(60, 2, 21)
    theta = np.array([0.4, 0.4])
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", False, "none", "LL", {"theta": theta.reshape(1, -1)})
    L_old = k.T()
    k.update(y[5:6], X[5:6], False)
    L = k.T()
    assert np.array_equal(L[:60, :60], L_old)
    Xa = np.vstack([X, X[5:6]])
    ya = np.concatenate([y, y[5:6]])
    m, fb = O.update_no_refit("gauss", X, L_old, X[5:6], ya, O.regression_matrix("constant", Xa), theta)
    assert not fb and m.nugget_increments >= 1
    # the duplicate's row of L repeats row 5 up to rounding noise (~cond(L) eps)
    assert np.max(np.abs(L[60, :60] - m.L[60, :60])) < 1e-8
    # L_uu = sqrt(S) with S either the rounding residue of the zero Schur complement or that plus the 1e-10 jitter
    assert 0.0 < L[60, 60] <= 1.1e-5
    R = O.build_R("gauss", Xa, theta, 1.0)
    D = L @ L.T - R
    assert np.max(np.abs(D[:, :60])) < 1e-12 and np.max(np.abs(D[60, :60])) < 1e-12
    assert -1e-12 < D[60, 60] < 1.1e-10


def test_update_refit_matches_combined_fit(gpu_lib):
    """tests/KrigingUpdateTest.cpp "Update with refit equals combined fit": n_old = 10, n_new = 1, d = 2, gauss,
    y = x1^2 + x2^2, BFGS; theta, sigma2 and beta within 5 %, predictions within 10 %."""
    rng = np.random.default_rng(123)
    Xo = rng.uniform(size=(10, 2))
    Xu = rng.uniform(size=(1, 2))
    f = lambda X: X[:, 0] ** 2 + X[:, 1] ** 2
    ku = gpu_lib.Kriging("gauss")
    ku.fit(f(Xo), Xo, "constant", False, "BFGS", "LL")
    ku.update(f(Xu), Xu, True)
    Xc = np.vstack([Xo, Xu])
    kc = gpu_lib.Kriging("gauss")
    kc.fit(f(Xc), Xc, "constant", False, "BFGS", "LL")
    assert np.all(np.abs(ku.theta() - kc.theta()) <= 0.05 * np.abs(kc.theta()))
    assert abs(ku.sigma2() - kc.sigma2()) <= 0.05 * abs(kc.sigma2())
    assert np.all(np.abs(ku.beta() - kc.beta()) <= 0.05 * np.abs(kc.beta()))
    Xt = rng.uniform(size=(5, 2))
    mu, mc = ku.predict(Xt, True)[0], kc.predict(Xt, True)[0]
    assert np.all(np.abs(mu - mc) <= 0.1 * np.abs(mc))
    assert ku.X().shape == (11, 2)


@pytest.mark.parametrize("kernel", ["gauss", "exp", "matern3_2", "matern5_2"])
def test_update_refit_kernels(gpu_lib, kernel):
    """tests/KrigingUpdateTest.cpp "Different kernels": predictions of the updated model within 5 % of the
    combined fit's."""
    rng = np.random.default_rng(5)
    Xo = rng.uniform(size=(10, 2))
    Xu = rng.uniform(size=(1, 2))
    f = lambda X: X[:, 0] ** 2 + X[:, 1] ** 2
    ku = gpu_lib.Kriging(kernel)
    ku.fit(f(Xo), Xo, "constant", False, "BFGS", "LL")
    ku.update(f(Xu), Xu, True)
    Xc = np.vstack([Xo, Xu])
    kc = gpu_lib.Kriging(kernel)
    kc.fit(f(Xc), Xc, "constant", False, "BFGS", "LL")
    Xt = rng.uniform(size=(3, 2))
    mu, mc = ku.predict(Xt, False)[0], kc.predict(Xt, False)[0]
    assert np.all(np.abs(mu - mc) <= 0.05 * np.abs(mc))


def test_update_refit_nugget_is_a_fit_on_joined_data(gpu_lib):
    """Kriging.cpp:2447-2468: with NoiseModel Nugget, update(refit) fits the joined data (original units) with the
    model's parameters -- the same call as a direct fit."""
    X, y = _data(40, 2, 31)
    params = {"theta": np.array([[0.3, 0.3]]), "sigma2": 1.0, "is_sigma2_estim": False, "nugget": 0.01,
              "is_nugget_estim": False}
    k = gpu_lib.Kriging("matern5_2", "nugget")
    k.fit(y[:30], X[:30], "constant", True, "BFGS", "LL", params)
    k.update(y[30:], X[30:], True)
    k2 = gpu_lib.Kriging("matern5_2", "nugget")
    ko = gpu_lib.Kriging("matern5_2", "nugget")
    ko.fit(y[:30], X[:30], "constant", True, "BFGS", "LL", params)
    # the parameters update() passes, in its own operation order (Kriging.cpp:2451-2463)
    p = {"theta": (ko.theta() * ko.scaleX()).reshape(1, -1), "sigma2": ko.sigma2() * ko.scaleY() * ko.scaleY(),
         "is_sigma2_estim": False, "nugget": ko.nugget() * ko.scaleY() * ko.scaleY(), "is_nugget_estim": False}
    k2.fit(y, X, "constant", True, "BFGS", "LL", p)
    assert rel_err(k.theta(), k2.theta()) < 1e-8
    assert abs(k.sigma2() - k2.sigma2()) <= 1e-8 * k2.sigma2()
    assert abs(k.nugget() - k2.nugget()) <= 1e-8 * k2.nugget()
    assert k.X().shape == (40, 2)


@pytest.mark.parametrize("noise,normalize", [("none", False), ("nugget", True)])
def test_save_load_roundtrip(gpu_lib, tmp_path, noise, normalize):
    """tests/KrigingTest.cpp "save & reload": the reloaded model gives the same results -- here every accessor, the
    predictions (bit for bit: the factor is restored, its diagonal-block inverses recomputed exactly) and
    logLikelihoodFun at theta = 0.5."""
    X, y = _data(120, 3, 41)
    k = gpu_lib.Kriging("matern5_2", noise)
    k.fit(y, X, "linear", normalize, "BFGS", "LL")
    f = tmp_path / "model.json"
    k.save(f)
    k2 = gpu_lib.Kriging.load(f)
    k3 = gpu_lib.load(str(f))
    for a in ("theta", "beta", "X", "y", "centerX", "scaleX", "T", "M", "z", "F"):
        assert np.array_equal(getattr(k, a)(), getattr(k2, a)()), a
        assert np.array_equal(getattr(k, a)(), getattr(k3, a)()), a
    for a in ("sigma2", "nugget", "centerY", "scaleY", "kernel", "optim", "objective", "regmodel", "noise_model",
              "normalize", "is_beta_estim", "is_theta_estim", "is_sigma2_estim"):
        assert getattr(k, a)() == getattr(k2, a)(), a
    Xn = np.random.default_rng(42).uniform(size=(64, 3))
    p1, p2 = k.predict(Xn, True, True), k2.predict(Xn, True, True)
    for a, b in zip(p1[:3], p2[:3]):
        assert np.array_equal(a, b)
    g = np.full(3, 0.5) if noise == "none" else np.array([0.5, 0.5, 0.5, 0.9])
    ll1, gr1, _ = k.logLikelihoodFun(g, True)
    ll2, gr2, _ = k2.logLikelihoodFun(g, True)
    assert ll1 == ll2 and np.array_equal(gr1, gr2)


def test_saved_file_layout(gpu_lib, tmp_path):
    """The file is the reference's version-2 layout (Kriging.cpp:2691-2717, KrigingImpl.cpp:644-675): its keys,
    base64 little-endian column-major payloads; T lower with T T' = R, R symmetric with unit diagonal, Rinv R = I,
    dX(k, i n + j) = x_i(k) - x_j(k), maxdX its row maxima."""
    X, y = _data(70, 2, 51)
    k = gpu_lib.Kriging("gauss")
    k.fit(y, X, "constant", False, "BFGS", "LL")
    f = tmp_path / "m.json"
    k.save(f)
    j = json.loads(f.read_text())
    assert set(j) == REF_KEYS
    assert j["version"] == 2 and j["content"] == "Kriging" and j["noise_model"] == "None"
    assert j["regmodel"] == "constant" and j["covType"] == "gauss"
    Xf = _decode(j["X"])
    assert np.array_equal(Xf, X)
    T, R, Rinv = _decode(j["T"]), _decode(j["R"]), _decode(j["Rinv"])
    assert np.array_equal(T, np.tril(T))
    assert np.array_equal(R, R.T) and np.all(np.diag(R) == 1.0)
    # T factors R plus the numerical nugget the retry rule added to a copy's diagonal (R itself is stored as built)
    D = T @ T.T - R
    jit = np.diag(D)
    assert np.max(np.abs(D - np.diag(jit))) < 1e-12
    assert np.all(jit > -1e-12) and np.ptp(jit) < 1e-12 and np.max(jit) < 1e-6
    assert np.array_equal(Rinv, Rinv.T)
    assert rel_err(Rinv, O.inv_sympd(T)) < 1e-8
    R_o = O.build_R("gauss", X, k.theta(), 1.0)
    assert np.max(np.abs(R - R_o)) < 1e-15  # CUDA's exp and the C library's may differ in the last bit
    dX = _decode(j["dX"])
    assert dX.shape == (2, 70 * 70)
    i, jj = 3, 17
    assert np.array_equal(dX[:, i * 70 + jj], X[i] - X[jj])
    assert np.array_equal(_decode(j["maxdX"]), X.max(axis=0) - X.min(axis=0))
    assert j["star"]["n_rows"] == 0 and j["star"]["n_cols"] == 0
    assert np.array_equal(_decode(j["theta"]), k.theta())


@pytest.mark.parametrize("noise", ["none", "nugget"])
def test_load_file_written_in_reference_layout(gpu_lib, tmp_path, noise):
    """A model file assembled in the reference's layout from the oracle's model (LAPACK factor) loads, and the
    loaded model predicts as the oracle does at that model (mean 1e-12, stdev 1e-10)."""
    X, y = _data(90, 3, 61)
    theta = np.array([0.3, 0.45, 0.6])
    alpha = 0.97 if noise == "nugget" else 1.0
    ora = O.OracleKriging(y, X, "matern3_2", noise_model=noise)
    F = O.regression_matrix("constant", ora.X)
    m = O.populate_model("matern3_2", ora.X, ora.y, F, theta, alpha, None, True)
    sigma2 = m.SSEstar / 90 * (alpha if noise == "nugget" else 1.0)
    j = {"version": 2, "content": "Kriging", "covType": "matern3_2", "X": _encode(ora.X, "mat"),
         "centerX": _encode(np.zeros(3), "rowvec"), "scaleX": _encode(np.ones(3), "rowvec"),
         "y": _encode(ora.y, "colvec"), "centerY": 0.0, "scaleY": 1.0, "normalize": False, "regmodel": "constant",
         "optim": "BFGS", "objective": "LL", "dX": _encode(np.zeros((3, 0)), "mat"),
         "maxdX": _encode(np.zeros(3), "colvec"), "F": _encode(F, "mat"), "T": _encode(m.L, "mat"),
         "R": _encode(m.R, "mat"), "M": _encode(m.Fstar, "mat"), "star": _encode(np.zeros((0, 0)), "mat"),
         "circ": _encode(m.Rstar, "mat"), "z": _encode(m.Estar, "colvec"), "Rinv": _encode(m.Rinv, "mat"),
         "beta": _encode(m.betahat, "colvec"), "est_beta": True, "theta": _encode(theta, "colvec"),
         "est_theta": True, "sigma2": sigma2, "est_sigma2": True, "noise_model": "Nugget" if noise == "nugget" else
         "None", "nystrom_light": False}
    if noise == "nugget":
        j.update(nugget=sigma2 / alpha - sigma2, est_nugget=True, alpha=alpha)
    f = tmp_path / "ref_layout.json"
    f.write_text(json.dumps(j, indent=4, sort_keys=True))
    k = gpu_lib.Kriging.load(f)
    assert np.array_equal(k.T(), m.L)
    Xn = np.random.default_rng(62).uniform(size=(40, 3))
    mean, sd, _, _, _ = k.predict(Xn, True)
    om, osd = ora.predict(Xn, theta, m.betahat, sigma2, alpha)
    assert rel_err(mean, om) < 1e-12
    assert rel_err(sd, osd) < 1e-10
    # and the loaded model takes an incremental update
    Xu, yu = _data(5, 3, 63)
    k.update(yu, Xu, False)
    assert k.X().shape == (95, 3)


def test_covmat(gpu_lib):
    """KrigingImpl::covMat (KrigingImpl.cpp:60-71): sigma2 C(X1, X2) with both inputs normalised by the model."""
    X, y = _data(50, 2, 71)
    k = gpu_lib.Kriging("matern5_2")
    k.fit(y, X * 3.0 + 1.0, "constant", True, "BFGS", "LL")
    A = np.random.default_rng(72).uniform(size=(17, 2)) * 3.0 + 1.0
    B = np.vstack([A[:4], np.random.default_rng(73).uniform(size=(9, 2)) * 3.0 + 1.0])
    C = k.covMat(A, B)
    An = (A - k.centerX()) / k.scaleX()
    Bn = (B - k.centerX()) / k.scaleX()
    Co = O.cov_cross("matern5_2", An, Bn, k.theta()) * k.sigma2()
    assert C.shape == (17, 13)
    assert rel_err(C, Co) < 1e-14


def test_copy_is_independent(gpu_lib):
    X, y = _data(80, 2, 81)
    k = gpu_lib.Kriging("exp")
    k.fit(y, X, "constant", False, "BFGS", "LL")
    c = k.copy()
    Xn = np.random.default_rng(82).uniform(size=(20, 2))
    assert np.array_equal(k.predict(Xn, True)[1], c.predict(Xn, True)[1])
    Xu, yu = _data(3, 2, 83)
    c.update(yu, Xu, False)
    assert k.X().shape == (80, 2) and c.X().shape == (83, 2)
    del k
    assert np.all(np.isfinite(c.predict(Xn, True)[0]))
