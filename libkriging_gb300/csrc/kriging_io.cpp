// kriging_io.cpp -- Kriging::update (incremental data), save / load (libKriging's JSON model files), covMat, copy.
//
//   update          Kriging.cpp:2433-2633, KrigingImpl.cpp:576-635, LinearAlgebra.cpp:206-299 (update_cholCov,
//                   chol_block)
//   save / load     Kriging.cpp:2691-2749, KrigingImpl.cpp:644-711, utils/jsonutils.cpp:66-110
//   covMat          KrigingImpl.cpp:60-71
#include <algorithm>
#include <cmath>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "common.cuh"
#include "json_io.hpp"
#include "kriging.hpp"
#include "lik_kernels.cuh"

namespace lkg {

namespace {

Mat join_rows(const std::vector<double>& A, int na, const Mat& B, int d) {  // [A (na x d); B] column-major
  Mat J;
  J.rows = na + B.rows;
  J.cols = d;
  J.v.resize((size_t)J.rows * d);
  for (int j = 0; j < d; ++j) {
    for (int i = 0; i < na; ++i) J(i, j) = A[i + (size_t)j * na];
    for (int i = 0; i < B.rows; ++i) J(na + i, j) = B(i, j);
  }
  return J;
}

struct DeviceBuf {  // scratch device array of doubles for one call
  double* p = nullptr;
  explicit DeviceBuf(size_t n) { LKG_CUDA(cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1))); }
  ~DeviceBuf() {
    if (p) cudaFree(p);
  }
  DeviceBuf(const DeviceBuf&) = delete;
  DeviceBuf& operator=(const DeviceBuf&) = delete;
};

const char* noise_to_string(Kriging::NoiseModel nm) { return nm == Kriging::NoiseModel::Nugget ? "Nugget" : "None"; }

}  // namespace

void Kriging::update(const std::vector<double>& y_u, const Mat& X_u, bool refit) {
  if (m_vecchia_light)
    throw std::runtime_error("update: not available on a light Vecchia fit (refit with set_vecchia_exact_commit(true))");
  if ((int)y_u.size() != X_u.rows)
    throw std::runtime_error("Dimension of new data should be the same:\n X: (" + std::to_string(X_u.rows) + "x" +
                             std::to_string(X_u.cols) + "), y: (" + std::to_string(y_u.size()) + ")");
  if (X_u.cols != m_d)
    throw std::runtime_error("Dimension of new data should be the same:\n X: (...x" + std::to_string(m_d) +
                             "), new X: (...x" + std::to_string(X_u.cols) + ")");
  if (m_n == 0 || (int)m_theta.size() != m_d) throw std::runtime_error("update: model is not fitted");
  if (m_service) throw std::runtime_error("update: not available on a model fitted through a shared service");
  const int d = m_d, n_old = m_n, nu = X_u.rows, n = n_old + nu;
  if (nu == 0) return;
  const bool nug = (m_noise_model == NoiseModel::Nugget);

  if (refit && m_optim != "none" && nug) {
    // full re-fit on the joined data in original units (Kriging.cpp:2447-2468)
    Mat Xo;
    Xo.rows = n_old;
    Xo.cols = d;
    Xo.v.resize((size_t)n_old * d);
    for (int j = 0; j < d; ++j)
      for (int i = 0; i < n_old; ++i) Xo(i, j) = m_X[i + (size_t)j * n_old] * m_scaleX[j] + m_centerX[j];
    Mat X_all = join_rows(Xo.v, n_old, X_u, d);
    std::vector<double> y_all(n);
    for (int i = 0; i < n_old; ++i) y_all[i] = m_y[i] * m_scaleY + m_centerY;
    for (int i = 0; i < nu; ++i) y_all[n_old + i] = y_u[i];
    Parameters params;
    if (!(m_est_beta && m_est_nugget && m_est_sigma2 && m_est_theta)) {
      params.sigma2 = m_sigma2 * m_scaleY * m_scaleY;
      params.is_sigma2_estim = m_est_sigma2;
      Mat th;
      th.rows = 1;
      th.cols = d;
      th.v.resize(d);
      for (int j = 0; j < d; ++j) th.v[j] = m_theta[j] * m_scaleX[j];
      params.theta = th;
      params.is_theta_estim = m_est_theta;
      params.nugget = m_nugget * m_scaleY * m_scaleY;
      params.is_nugget_estim = m_est_nugget;
      if (!m_est_beta) {
        std::vector<double> b(m_beta);
        for (auto& v : b) v *= m_scaleY;
        params.beta = b;
        params.is_beta_estim = false;
      }
    }
    fit(y_all, X_all, m_regmodel, m_normalize, m_optim, m_objective, params);
    return;
  }

  // the new points in the model's normalisation
  Mat Xn_u = X_u;
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < nu; ++i) Xn_u(i, j) = (X_u(i, j) - m_centerX[j]) / m_scaleX[j];
  std::vector<double> yn_all(m_y);
  yn_all.reserve(n);
  for (int i = 0; i < nu; ++i) yn_all.push_back((y_u[i] - m_centerY) / m_scaleY);
  Mat Xn_all = join_rows(m_X, n_old, Xn_u, d);

  if (refit && m_optim != "none") {
    // warm restart (Kriging.cpp:2470-2625): the joined normalised data fitted from the current theta; the fit sees
    // already-normalised data, the model keeps its normalisation
    const bool normalize = m_normalize;
    const std::vector<double> cx = m_centerX, sx = m_scaleX;
    const double cy = m_centerY, sy = m_scaleY;
    Parameters params;
    Mat th;
    th.rows = 1;
    th.cols = d;
    th.v = m_theta;
    params.theta = th;
    params.is_theta_estim = true;
    if (!m_est_sigma2) {
      params.sigma2 = m_sigma2;
      params.is_sigma2_estim = false;
    }
    if (!m_est_beta) {
      params.beta = m_beta;
      params.is_beta_estim = false;
    }
    m_warm = true;
    try {
      fit(yn_all, Xn_all, m_regmodel, false, m_optim, m_objective, params);
    } catch (...) {
      m_warm = false;
      m_normalize = normalize;
      m_centerX = cx;
      m_scaleX = sx;
      m_centerY = cy;
      m_scaleY = sy;
      throw;
    }
    m_warm = false;
    m_normalize = normalize;
    m_centerX = cx;
    m_scaleX = sx;
    m_centerY = cy;
    m_scaleY = sy;
    return;
  }

  // update without re-optimisation (KrigingImpl::update_no_refit_impl): theta (and alpha) kept, so the
  // incremental factor applies (Kriging.cpp:166-190 update_eligible)
  if (!m_model) commit(m_theta, m_alpha);
  m_X = Xn_all.v;
  m_y = yn_all;
  m_n = n;
  int p = 0;
  m_F = regression_matrix(m_regmodel, m_X, n, d, &p);
  m_p = p;
  m_eval.reset();
  m_vecchia.reset();
  auto model = std::make_unique<Engine>(m_kernel, n, d, m_p, m_X.data(), m_y.data(), m_F.data(), 1);
  const double factor = nug ? m_alpha : 1.0;
  EvalOut o;
  model->evaluate_update(*m_model, m_theta.data(), factor, o);
  if (o.status != 0) throw std::runtime_error(o.message);
  m_model = std::move(model);
  m_last_commit = o;
  if (m_est_beta) m_beta = o.beta;
  if (m_est_sigma2) m_sigma2 = o.sse / n;  // KrigingImpl.cpp:632-634, for every noise model
  if (m_vecchia_m > 0) {  // the Vecchia sets follow the data
    m_vorder.assign(n, 0);
    m_vnbr.assign((size_t)n * std::min(m_vecchia_m, VECCHIA_MAX_M), -1);
    vecchia_sets_gpu(n, d, m_X.data(), m_vecchia_m, m_vorder.data(), m_vnbr.data());
  }
}

// ---------------------------------------------------------------------------------------------------------------
void Kriging::save(const std::string& filename) const {
  if (m_vecchia_light)
    throw std::runtime_error("save: not available on a light Vecchia fit (refit with set_vecchia_exact_commit(true))");
  if (m_is_empty || !m_model || (int)m_theta.size() != m_d) throw std::runtime_error("save: model is not fitted");
  using json::Value;
  const int n = m_n, d = m_d, p = m_p;
  Value j = Value::object();
  j["version"] = Value::integer(2);
  j["content"] = Value::string("Kriging");
  // KrigingImpl::dump_common_to_json
  j["covType"] = Value::string(m_covType);
  j["X"] = json::mat_to_json(m_X.data(), n, d);
  j["centerX"] = json::rowvec_to_json(m_centerX);
  j["scaleX"] = json::rowvec_to_json(m_scaleX);
  j["y"] = json::colvec_to_json(m_y);
  j["centerY"] = Value::number(m_centerY);
  j["scaleY"] = Value::number(m_scaleY);
  j["normalize"] = Value::boolean(m_normalize);
  j["regmodel"] = Value::string(regmodel_to_string(m_regmodel));
  j["optim"] = Value::string(m_optim);
  j["objective"] = Value::string(m_objective);
  {  // dX(k, i n + j) = x_i(k) - x_j(k) (LinearAlgebra::compute_dX) and its per-dimension maximum
    std::vector<double> dX((size_t)d * n * n, 0.0), maxdX(d, 0.0);
    for (int i = 0; i < n; ++i)
      for (int jj = i + 1; jj < n; ++jj)
        for (int k = 0; k < d; ++k) {
          const double diff = m_X[i + (size_t)k * n] - m_X[jj + (size_t)k * n];
          dX[k + ((size_t)i * n + jj) * d] = diff;
          dX[k + ((size_t)jj * n + i) * d] = diff;
          maxdX[k] = std::max(maxdX[k], std::fabs(diff));
        }
    j["dX"] = json::mat_to_json(dX.data(), d, (int64_t)n * n);
    j["maxdX"] = json::colvec_to_json(maxdX);
  }
  j["F"] = json::mat_to_json(m_F.data(), n, p);
  std::vector<double> L, Fstar, ystar, Rstar, Estar, R, Rinv;
  m_model->copy_model(0, &L, &Fstar, &ystar, &Rstar, &Estar);
  const double factor = (m_noise_model == NoiseModel::Nugget) ? m_alpha : 1.0;
  m_model->model_matrices(m_theta.data(), factor, &R, &Rinv);
  j["T"] = json::mat_to_json(L.data(), n, n);
  j["R"] = json::mat_to_json(R.data(), n, n);
  j["M"] = json::mat_to_json(Fstar.data(), n, p);
  j["star"] = json::mat_to_json(nullptr, 0, 0);  // Q* is formed on demand, never stored (KrigingImpl.cpp:108-109)
  j["circ"] = json::mat_to_json(Rstar.data(), p, p);
  j["z"] = json::colvec_to_json(z());
  j["Rinv"] = json::mat_to_json(Rinv.data(), n, n);
  j["beta"] = json::colvec_to_json(m_beta);
  j["est_beta"] = Value::boolean(m_est_beta);
  j["theta"] = json::colvec_to_json(m_theta);
  j["est_theta"] = Value::boolean(m_est_theta);
  j["sigma2"] = Value::number(m_sigma2);
  j["est_sigma2"] = Value::boolean(m_est_sigma2);
  // Kriging::save
  j["noise_model"] = Value::string(noise_to_string(m_noise_model));
  if (m_noise_model == NoiseModel::Nugget) {
    j["nugget"] = Value::number(m_nugget);
    j["est_nugget"] = Value::boolean(m_est_nugget);
    j["alpha"] = Value::number(m_alpha);
  }
  j["nystrom_light"] = Value::boolean(false);
  std::ofstream f(filename, std::ios::binary);
  if (!f) throw std::runtime_error("save: cannot open '" + filename + "' for writing");
  f << json::dump(j, 4);
  if (!f) throw std::runtime_error("save: write to '" + filename + "' failed");
}

std::unique_ptr<Kriging> Kriging::load(const std::string& filename) {
  std::ifstream f(filename, std::ios::binary);
  if (!f) throw std::runtime_error("load: cannot open '" + filename + "'");
  std::stringstream ss;
  ss << f.rdbuf();
  const json::Value j = json::parse(ss.str());
  const long long version = j.at("version").as_int();
  if (version != 2)
    throw std::runtime_error("Bad version to load from '" + filename + "'; found " + std::to_string(version) +
                             ", requires 2");
  const std::string content = j.at("content").as_string();
  if (content != "Kriging")
    throw std::runtime_error("Bad content to load from '" + filename + "'; found '" + content +
                             "', requires 'Kriging'");
  NoiseModel nm = NoiseModel::None;
  if (j.contains("noise_model")) {
    const std::string s = j.at("noise_model").as_string();
    if (s == "Nugget")
      nm = NoiseModel::Nugget;
    else if (s == "Heterogeneous")
      throw std::runtime_error("load: NoiseModel Heterogeneous is not supported by the GPU build");
  }
  if (j.contains("nystrom_light") && j.at("nystrom_light").as_bool())
    throw std::runtime_error("load: Nystrom models are not supported by the GPU build");
  auto k = std::make_unique<Kriging>(j.at("covType").as_string(), nm);
  int64_t r = 0, c = 0;
  k->m_X = json::mat_from_json(j.at("X"), &r, &c);
  k->m_n = (int)r;
  k->m_d = (int)c;
  const int n = k->m_n, d = k->m_d;
  k->m_centerX = json::vec_from_json(j.at("centerX"), "rowvec");
  k->m_scaleX = json::vec_from_json(j.at("scaleX"), "rowvec");
  k->m_y = json::vec_from_json(j.at("y"), "colvec");
  k->m_centerY = j.at("centerY").as_double();
  k->m_scaleY = j.at("scaleY").as_double();
  k->m_normalize = j.at("normalize").as_bool();
  k->m_regmodel = regmodel_from_string(j.at("regmodel").as_string());
  k->m_optim = j.at("optim").as_string();
  k->m_objective = j.at("objective").as_string();
  k->m_F = json::mat_from_json(j.at("F"), &r, &c);
  k->m_p = (int)c;
  const int p = k->m_p;
  if ((int)k->m_y.size() != n || (int)k->m_centerX.size() != d || (int)k->m_scaleX.size() != d || r != n)
    throw std::runtime_error("load: inconsistent sizes in '" + filename + "'");
  std::vector<double> T = json::mat_from_json(j.at("T"), &r, &c);
  const bool has_T = (r == n && c == n);
  std::vector<double> M = json::mat_from_json(j.at("M"), &r, &c);
  std::vector<double> circ = json::mat_from_json(j.at("circ"), &r, &c);
  std::vector<double> zz = json::vec_from_json(j.at("z"), "colvec");
  k->m_beta = json::vec_from_json(j.at("beta"), "colvec");
  k->m_est_beta = j.at("est_beta").as_bool();
  k->m_theta = json::vec_from_json(j.at("theta"), "colvec");
  k->m_est_theta = j.at("est_theta").as_bool();
  k->m_sigma2 = j.at("sigma2").as_double();
  k->m_est_sigma2 = j.at("est_sigma2").as_bool();
  if (nm == NoiseModel::Nugget) {
    k->m_nugget = j.at("nugget").as_double();
    k->m_est_nugget = j.at("est_nugget").as_bool();
    k->m_alpha = j.at("alpha").as_double();
  }
  if ((int)k->m_theta.size() != d) throw std::runtime_error("load: theta has the wrong size in '" + filename + "'");
  if (k->m_objective.rfind("LLVecchia", 0) == 0) {
    k->m_vecchia_m = parse_vll_m(k->m_objective);
    k->m_vorder.assign(n, 0);
    k->m_vnbr.assign((size_t)n * std::min(k->m_vecchia_m, VECCHIA_MAX_M), -1);
    vecchia_sets_gpu(n, d, k->m_X.data(), k->m_vecchia_m, k->m_vorder.data(), k->m_vnbr.data());
  }
  k->m_is_empty = false;
  if (has_T) {
    if ((int)M.size() != n * p || (int)circ.size() != p * p || (int)zz.size() != n || (int)k->m_beta.size() != p)
      throw std::runtime_error("load: inconsistent model matrices in '" + filename + "'");
    // y* = z + M beta (z = E* with beta estimated, z = y* - M beta with beta fixed)
    std::vector<double> ystar(zz);
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < p; ++q) ystar[i] += M[i + (size_t)q * n] * k->m_beta[q];
    k->m_model = std::make_unique<Engine>(k->m_kernel, n, d, p, k->m_X.data(), k->m_y.data(), k->m_F.data(), 1);
    k->m_model->adopt_model(T.data(), M.data(), ystar.data(), circ.data(), zz.data());
    k->m_last_commit = EvalOut{};
    k->m_last_commit.beta = k->m_beta;
  }
  return k;
}

Mat Kriging::covMat(const Mat& X1, const Mat& X2) const {
  if ((int)m_theta.size() != m_d || m_d == 0) throw std::runtime_error("covMat: model is not fitted");
  if (X1.cols != m_d || X2.cols != m_d)
    throw std::invalid_argument("covMat: X1 and X2 must have " + std::to_string(m_d) + " columns");
  const int n1 = X1.rows, n2 = X2.rows, d = m_d;
  Mat R;
  R.rows = n1;
  R.cols = n2;
  R.v.assign((size_t)n1 * n2, 0.0);
  if (n1 == 0 || n2 == 0) return R;
  std::vector<double> x1((size_t)n1 * d), x2((size_t)n2 * d);
  for (int j = 0; j < d; ++j) {
    for (int i = 0; i < n1; ++i) x1[i + (size_t)j * n1] = (X1(i, j) - m_centerX[j]) / m_scaleX[j];
    for (int i = 0; i < n2; ++i) x2[i + (size_t)j * n2] = (X2(i, j) - m_centerX[j]) / m_scaleX[j];
  }
  DeviceBuf dx1(x1.size()), dx2(x2.size()), dth(d), dR((size_t)n1 * n2);
  cudaStream_t st = nullptr;
  LKG_CUDA(cudaMemcpy(dx1.p, x1.data(), sizeof(double) * x1.size(), cudaMemcpyHostToDevice));
  LKG_CUDA(cudaMemcpy(dx2.p, x2.data(), sizeof(double) * x2.size(), cudaMemcpyHostToDevice));
  LKG_CUDA(cudaMemcpy(dth.p, m_theta.data(), sizeof(double) * d, cudaMemcpyHostToDevice));
  cov_cross(m_kernel, n1, n2, d, dx1.p, dx2.p, dth.p, m_sigma2, dR.p, st, false);
  LKG_CUDA(cudaMemcpy(R.v.data(), dR.p, sizeof(double) * R.v.size(), cudaMemcpyDeviceToHost));
  return R;
}

std::unique_ptr<Kriging> Kriging::copy() const {
  auto k = std::make_unique<Kriging>(m_covType, m_noise_model);
  k->m_n = m_n;
  k->m_d = m_d;
  k->m_p = m_p;
  k->m_X = m_X;
  k->m_y = m_y;
  k->m_F = m_F;
  k->m_centerX = m_centerX;
  k->m_scaleX = m_scaleX;
  k->m_centerY = m_centerY;
  k->m_scaleY = m_scaleY;
  k->m_normalize = m_normalize;
  k->m_regmodel = m_regmodel;
  k->m_optim = m_optim;
  k->m_objective = m_objective;
  k->m_theta = m_theta;
  k->m_beta = m_beta;
  k->m_sigma2 = m_sigma2;
  k->m_nugget = m_nugget;
  k->m_alpha = m_alpha;
  k->m_est_theta = m_est_theta;
  k->m_est_sigma2 = m_est_sigma2;
  k->m_est_beta = m_est_beta;
  k->m_est_nugget = m_est_nugget;
  k->m_is_empty = m_is_empty;
  k->m_last_commit = m_last_commit;
  k->m_slices = m_slices;
  k->m_vecchia_m = m_vecchia_m;
  k->m_vorder = m_vorder;
  k->m_vnbr = m_vnbr;
  k->m_vecchia_exact_commit = m_vecchia_exact_commit;
  k->m_vecchia_light = m_vecchia_light;
  if (m_model) {
    std::vector<double> L, Fstar, ystar, Rstar, Estar;
    m_model->copy_model(0, &L, &Fstar, &ystar, &Rstar, &Estar);
    k->m_model = std::make_unique<Engine>(m_kernel, m_n, m_d, m_p, m_X.data(), m_y.data(), m_F.data(), 1);
    k->m_model->adopt_model(L.data(), Fstar.data(), ystar.data(), Rstar.data(), Estar.data());
  }
  return k;
}

}  // namespace lkg
