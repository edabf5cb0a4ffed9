// kriging.cpp -- GPU-backed Kriging facade (host C++).
//
// Restates the host logic of libKriging's Kriging class around the GPU engine:
//   fit                Kriging.cpp:1591-2215 (fit_setup_impl KrigingImpl.cpp:764-841, theta_bounds Optim.cpp:179-209,
//                      parse_method Optim.cpp:151-177, Random.cpp:13-49, make_fit_objective Kriging.cpp:1414-1470,
//                      nugget reparametrisation Kriging.cpp:676-702)
//   _logLikelihood     Kriging.cpp:214-341 (LL per noise model, gradient assembly, alpha-gradient)
//   predict            Kriging.cpp:2240-2285 -> KrigingImpl.cpp:145-300 (mean, stdev, cov, derivatives)
// The multistart runs every start's L-BFGS-B in its own host thread; their objective calls are gathered by a
// batcher into ONE batched GPU evaluation per round (the reference runs the starts one after another).
#include "kriging.hpp"

#include "autotune.hpp"
#include "engine.hpp"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <exception>
#include <limits>
#include <mutex>
#include <random>
#include <sstream>
#include <stdexcept>
#include <thread>

#include "common.cuh"
#include "dense_fp64.cuh"
#include "lbfgsb.hpp"
#include "lik_kernels.cuh"
#include "predict_kernels.cuh"

namespace lkg {

static constexpr double kNuggetAlphaLower = 1e-3;  // Kriging.cpp:680

RegressionModel regmodel_from_string(const std::string& s) {
  if (s == "none") return RegressionModel::None;
  if (s == "constant") return RegressionModel::Constant;
  if (s == "linear") return RegressionModel::Linear;
  if (s == "interactive") return RegressionModel::Interactive;
  if (s == "quadratic") return RegressionModel::Quadratic;
  throw std::invalid_argument("Cannot convert '" + s + "' as a regression model");
}

const char* regmodel_to_string(RegressionModel r) {
  static const char* names[] = {"none", "constant", "linear", "interactive", "quadratic"};
  return names[(int)r];
}

std::vector<double> regression_matrix(RegressionModel r, const std::vector<double>& X, int n, int d, int* p_out) {
  std::vector<std::vector<double>> cols;
  auto col = [&](int i) { return std::vector<double>(X.begin() + (size_t)i * n, X.begin() + (size_t)(i + 1) * n); };
  auto prod = [&](int i, int j) {
    std::vector<double> v(n);
    for (int a = 0; a < n; ++a) v[a] = X[a + (size_t)i * n] * X[a + (size_t)j * n];
    return v;
  };
  if (r != RegressionModel::None) cols.push_back(std::vector<double>(n, 1.0));
  if (r == RegressionModel::Linear) {
    for (int i = 0; i < d; ++i) cols.push_back(col(i));
  } else if (r == RegressionModel::Interactive) {
    for (int i = 0; i < d; ++i) {
      cols.push_back(col(i));
      for (int j = 0; j < i; ++j) cols.push_back(prod(i, j));
    }
  } else if (r == RegressionModel::Quadratic) {
    for (int i = 0; i < d; ++i) {
      cols.push_back(col(i));
      for (int j = 0; j <= i; ++j) cols.push_back(prod(i, j));
    }
  }
  *p_out = (int)cols.size();
  std::vector<double> F((size_t)n * cols.size());
  for (size_t q = 0; q < cols.size(); ++q) std::copy(cols[q].begin(), cols[q].end(), F.begin() + q * n);
  return F;
}

// Trend::regressionModelDerivative (src/lib/Trend.cpp:95-150): dF/dx at one point x (d values), d x p column-major,
// DF(k, l) = d F_l / d x_k, columns in regression_matrix's order
std::vector<double> regression_derivative(RegressionModel r, const double* x, int d, int p) {
  std::vector<double> DF((size_t)d * p, 0.0);
  auto at = [&](int k, int l) -> double& { return DF[k + (size_t)l * d]; };
  int l = 1;
  if (r == RegressionModel::Linear) {
    for (int i = 0; i < d; ++i) at(i, l++) = 1.0;
  } else if (r == RegressionModel::Interactive || r == RegressionModel::Quadratic) {
    const bool sq = (r == RegressionModel::Quadratic);
    for (int i = 0; i < d; ++i) {
      at(i, l++) = 1.0;
      for (int j = 0; j < (sq ? i + 1 : i); ++j, ++l) {
        if (i == j) {
          at(i, l) = 2.0 * x[i];
        } else {
          at(i, l) = x[j];
          at(j, l) = x[i];
        }
      }
    }
  }
  return DF;
}

// ---------------------------------------------------------------------------------------------------------------
// Random (Random.cpp:13-49): a process-wide mt19937 seeded with 123, re-seeded by each BFGS fit
namespace {
std::mt19937& rng_engine() {  // per thread: every fit re-seeds it first, so concurrent fits draw as sequential ones
  thread_local std::mt19937 e(123);
  return e;
}
unsigned int& rng_seed() {
  static unsigned int s = 123;
  return s;
}
Mat randu_mat(int rows, int cols) {  // column-major fill (arma imbue)
  std::uniform_real_distribution<double> dist{};
  Mat m;
  m.rows = rows;
  m.cols = cols;
  m.v.resize((size_t)rows * cols);
  for (auto& x : m.v) x = dist(rng_engine());
  return m;
}
std::vector<double> randu_vec(int n) {
  std::uniform_real_distribution<double> dist{};
  std::vector<double> v(n);
  for (auto& x : v) x = dist(rng_engine());
  return v;
}

// Optim::parse_method (Optim.cpp:151-177)
std::pair<std::string, int> parse_method(const std::string& method, const std::string& prefix) {
  if (method.rfind(prefix, 0) != 0) return {method, 1};
  size_t pos = prefix.size(), e = pos;
  while (e < method.size() && std::isdigit((unsigned char)method[e])) ++e;
  if (e == pos) return {method, 1};
  int ms = 1;
  try {
    ms = std::stoi(method.substr(pos, e - pos));
  } catch (...) {
    ms = 1;
  }
  if (ms < 1) ms = 1;
  return {prefix + method.substr(e), ms};
}

// Evaluation batcher: worker threads submit one request each and block; when every still-active worker has a
// request pending, the last arrival runs them as one batched GPU evaluation.
struct EvalRequest {
  std::vector<double> theta;
  double factor = 1.0;
  bool want_grad = false;
  bool vecchia = false;  // evaluate the Vecchia likelihood instead of the exact one
  int kind = 0;          // exact objectives: 0 LL, 1 LMP, 2 LOO
  EvalOut out;
  LooOut lout;
  VecchiaOut vout;
  std::exception_ptr err;
  bool done = false;
};

class Batcher {
 public:
  Batcher(int workers, std::function<void(std::vector<EvalRequest*>&)> run) : active_(workers), run_(std::move(run)) {}
  void submit(EvalRequest* r) {
    std::unique_lock<std::mutex> lk(mu_);
    pending_.push_back(r);
    maybe_run(lk);
    cv_.wait(lk, [&] { return r->done; });
  }
  void leave() {
    std::unique_lock<std::mutex> lk(mu_);
    active_--;
    maybe_run(lk);
  }

 private:
  void maybe_run(std::unique_lock<std::mutex>& lk) {
    if (pending_.empty() || (int)pending_.size() < active_) return;
    std::vector<EvalRequest*> batch;
    batch.swap(pending_);
    lk.unlock();
    try {
      run_(batch);
    } catch (...) {
      for (auto* r : batch) r->err = std::current_exception();
    }
    lk.lock();
    for (auto* r : batch) r->done = true;
    cv_.notify_all();
  }
  std::mutex mu_;
  std::condition_variable cv_;
  int active_;
  std::vector<EvalRequest*> pending_;
  std::function<void(std::vector<EvalRequest*>&)> run_;
};

}  // namespace

// ---------------------------------------------------------------------------------------------------------------
Kriging::Kriging(const std::string& covType, NoiseModel nm)
    : m_covType(covType), m_kernel(kernel_from_name(covType)), m_noise_model(nm) {}

Kriging::~Kriging() = default;

void Kriging::ensure_engine(int batch_cap) {
  if (m_n == 0) throw std::runtime_error("Kriging model has no data: call fit() first");
  if (!m_eval || m_eval->capacity() < batch_cap)
    m_eval = std::make_unique<Engine>(m_kernel, m_n, m_d, m_p, m_X.data(), m_y.data(), m_F.data(),
                                      std::max(batch_cap, 1));
  m_eval->set_slices(m_slices);
}

void Kriging::set_precision(int slices) {
  if (slices != 0 && (slices < 4 || slices > 8))
    throw std::invalid_argument("set_precision: slices must be 0 (FP64) or 4..8");
  m_slices = slices;
  if (m_eval) m_eval->set_slices(slices);
}

double Kriging::loglik_from(const EvalOut& o, double extra_param, std::vector<double>* grad, int gdim) const {
  if (o.status != 0) throw std::runtime_error(o.message);
  const double n = m_n;
  const int d = m_d;
  double sigma2_grad, ll;
  if (m_noise_model == NoiseModel::Nugget) {
    double a = extra_param, s2 = m_sigma2, nu = m_nugget;
    if (m_est_sigma2) {
      if (m_est_nugget) {
        const double var = o.sse / n;
        s2 = a * var;
        nu = (1.0 - a) * var;
      } else {
        s2 = m_nugget * a / (1.0 - a);
      }
    } else {
      if (m_est_nugget)
        nu = m_sigma2 * (1.0 - a) / a;
      else
        a = m_sigma2 / (m_sigma2 + m_nugget);
    }
    const double tv = s2 + nu;
    ll = -0.5 * (n * std::log(2 * M_PI * tv) + o.logdet + o.sse / tv);
    sigma2_grad = tv;
  } else {
    if (m_est_sigma2) {
      sigma2_grad = o.sse / n;
      ll = -0.5 * (n * std::log(2 * M_PI * sigma2_grad) + o.logdet + n);
    } else {
      sigma2_grad = m_sigma2;
      ll = -0.5 * (n * std::log(2 * M_PI * sigma2_grad) + o.logdet + o.sse / sigma2_grad);
    }
  }
  if (grad) {
    grad->assign(gdim, 0.0);
    const std::vector<double>& A = o.adj;  // [T1(d), T2(d), U1, U2, D1, D2]
    for (int k = 0; k < d; ++k) {
      // (term1_k / sigma2 + term2_k) / 2 with term1_k = 2 T1_k, term2_k = -2 T2_k
      (*grad)[k] = ((2.0 * A[k]) / sigma2_grad + (-2.0 * A[d + k])) / 2.0;
    }
    if (gdim > d && m_noise_model == NoiseModel::Nugget) {
      const double a = extra_param;
      const double U1 = A[2 * d], U2 = A[2 * d + 1], D1 = A[2 * d + 2], D2 = A[2 * d + 3];
      if (m_est_sigma2 && m_est_nugget) {
        const double var = sigma2_grad;
        const double term1_a = -(2.0 * U1) / var;
        const double term2_a = 2.0 * U2;
        (*grad)[d] = -0.5 * (term1_a + term2_a);
      } else if (m_est_sigma2 && !m_est_nugget) {
        const double tv = sigma2_grad;
        const double term1_a = -(2.0 * U1 + D1) / (tv * tv);
        const double term2_a = (2.0 * U2 + D2) / tv;
        (*grad)[d] = -0.5 * (term1_a + term2_a) * m_nugget / (1.0 - a) / (1.0 - a);
      } else {
        (*grad)[d] = 0.0;
      }
    }
  }
  return ll;
}

std::tuple<double, std::vector<double>> Kriging::logLikelihoodFun(const std::vector<double>& gamma, bool return_grad,
                                                                  bool bench) {
  const int d = m_d;
  if (m_n == 0) throw std::runtime_error("Kriging model has no data: call fit() first");
  if ((int)gamma.size() != d && !((int)gamma.size() == d + 1 && m_noise_model == NoiseModel::Nugget))
    throw std::invalid_argument("logLikelihoodFun: gamma should have length " + std::to_string(d) +
                                (m_noise_model == NoiseModel::Nugget ? " or " + std::to_string(d + 1) : ""));
  ensure_engine(1);
  double extra = (gamma.size() > (size_t)d) ? gamma[d] : (m_noise_model == NoiseModel::Nugget ? m_alpha : m_sigma2);
  if (m_noise_model == NoiseModel::Nugget && !m_est_sigma2 && !m_est_nugget) extra = m_sigma2 / (m_sigma2 + m_nugget);
  const double factor = (m_noise_model == NoiseModel::Nugget) ? extra : 1.0;
  std::vector<EvalOut> out;
  m_bench.clear();
  m_eval->evaluate(1, gamma.data(), &factor, return_grad, out, bench ? &m_bench : nullptr);
  m_evals++;
  m_rounds++;
  m_last_slices = out[0].slices;
  std::vector<double> grad;
  const double ll = loglik_from(out[0], extra, return_grad ? &grad : nullptr, (int)gamma.size());
  return {ll, grad};
}

int Kriging::autotune_precision(const std::vector<double>& gamma, double tol_ll, double tol_grad) {
  if (!(tol_ll > 0.0) || !(tol_grad > 0.0)) throw std::invalid_argument("autotune_precision: tolerances must be > 0");
  const int saved = m_slices;
  std::ostringstream key;
  key.precision(3);
  key << "precision:k=" << m_kernel << ":nm=" << (m_noise_model == NoiseModel::Nugget ? 1 : 0) << ":n=" << m_n
      << ":d=" << m_d << ":tol=" << tol_ll << "," << tol_grad;
  // the FP64 reference values, then each candidate timed (the second of two evaluations) and checked
  set_precision(0);
  auto [ll64, g64] = logLikelihoodFun(gamma, true, false);
  double gnorm = 0.0;
  for (double v : g64) gnorm += v * v;
  gnorm = std::sqrt(gnorm);
  auto cost = [&](int slices) -> double {
    set_precision(slices);
    double ms = 0.0;
    std::vector<double> g;
    double ll = 0.0;
    for (int rep = 0; rep < 2; ++rep) {
      auto r = logLikelihoodFun(gamma, true, true);
      ll = std::get<0>(r);
      g = std::get<1>(r);
      ms = 0.0;
      for (const auto& kv : m_bench) ms += kv.second;
    }
    if (slices == 0) return ms;
    if (m_last_slices != slices) return std::numeric_limits<double>::infinity();  // retreated to FP64
    double dg = 0.0;
    for (size_t i = 0; i < g.size(); ++i) dg += (g[i] - g64[i]) * (g[i] - g64[i]);
    const double e_ll = std::fabs(ll - ll64) / std::max(std::fabs(ll64), 1e-300);
    const double e_g = std::sqrt(dg) / std::max(gnorm, 1e-300);
    return (e_ll * 10.0 <= tol_ll && e_g * 10.0 <= tol_grad) ? ms : std::numeric_limits<double>::infinity();
  };
  const int choice = Autotuner::instance().choose(key.str(), {0, 5, 6, 7}, saved, cost);
  set_precision(choice);
  return choice;
}

int Kriging::autotune_lookahead(const std::vector<double>& gamma) {
  if (m_slices == 0) throw std::invalid_argument("autotune_lookahead: the look-ahead belongs to the mixed path");
  const int saved = lookahead_ctas_setting();
  auto cost = [&](int ctas) -> double {
    set_lookahead_ctas(ctas);
    double ms = 0.0;
    for (int rep = 0; rep < 2; ++rep) {  // the second of two evaluations (the first allocates)
      logLikelihoodFun(gamma, true, true);
      ms = 0.0;
      for (const auto& kv : m_bench) ms += kv.second;
    }
    return ms;
  };
  int choice = 16;
  try {
    const std::string key = lookahead_tune_key(m_n);
    if (Autotuner::instance().enabled()) {
      Autotuner::instance().clear_key(key);
      choice = Autotuner::instance().choose(key, {0, 12, 16, 24, 32}, 16, cost);
    }
  } catch (...) {
    set_lookahead_ctas(saved);
    throw;
  }
  set_lookahead_ctas(saved);
  return choice;
}

void Kriging::logLikelihoodFunBatch(const Mat& gammas, bool return_grad, std::vector<double>& ll,
                                    std::vector<double>& grad, bool bench) {
  const int k = gammas.rows, gd = gammas.cols, d = m_d;
  if (gd != d && !(gd == d + 1 && m_noise_model == NoiseModel::Nugget))
    throw std::invalid_argument("logLikelihoodFunBatch: gamma rows should have length " + std::to_string(d));
  ensure_engine(k);
  std::vector<double> th((size_t)k * d), fac(k), extra(k);
  for (int b = 0; b < k; ++b) {
    for (int j = 0; j < d; ++j) th[(size_t)b * d + j] = gammas(b, j);
    double e = (gd > d) ? gammas(b, d) : (m_noise_model == NoiseModel::Nugget ? m_alpha : m_sigma2);
    if (m_noise_model == NoiseModel::Nugget && !m_est_sigma2 && !m_est_nugget) e = m_sigma2 / (m_sigma2 + m_nugget);
    extra[b] = e;
    fac[b] = (m_noise_model == NoiseModel::Nugget) ? e : 1.0;
  }
  std::vector<EvalOut> out;
  m_bench.clear();
  m_eval->evaluate(k, th.data(), fac.data(), return_grad, out, bench ? &m_bench : nullptr);
  m_evals += k;
  m_rounds++;
  ll.assign(k, 0.0);
  grad.assign(return_grad ? (size_t)k * gd : 0, 0.0);
  for (int b = 0; b < k; ++b) {
    std::vector<double> g;
    ll[b] = loglik_from(out[b], extra[b], return_grad ? &g : nullptr, gd);
    if (return_grad) std::copy(g.begin(), g.end(), grad.begin() + (size_t)b * gd);
  }
}

double Kriging::logLikelihood() {
  std::vector<double> g = m_theta;
  if (m_noise_model == NoiseModel::Nugget) g.push_back(m_alpha);
  return std::get<0>(logLikelihoodFun(g, false, false));
}

// ---- leave-one-out (Kriging.cpp:353-484) ----
std::tuple<double, std::vector<double>> Kriging::leaveOneOutFun(const std::vector<double>& theta, bool return_grad) {
  if (m_n == 0) throw std::runtime_error("Kriging model has no data: call fit() first");
  if ((int)theta.size() != m_d)
    throw std::invalid_argument("leaveOneOutFun: theta should have length " + std::to_string(m_d));
  ensure_engine(1);
  const double factor = (m_noise_model == NoiseModel::Nugget) ? m_alpha : 1.0;
  std::vector<LooOut> out;
  m_eval->leave_one_out(1, theta.data(), &factor, return_grad, out);
  m_evals++;
  m_rounds++;
  if (out[0].ev.status != 0) throw std::runtime_error(out[0].ev.message);
  return {out[0].loo, return_grad ? out[0].grad : std::vector<double>()};
}

std::tuple<std::vector<double>, std::vector<double>> Kriging::leaveOneOutVec(const std::vector<double>& theta) {
  if (m_n == 0) throw std::runtime_error("Kriging model has no data: call fit() first");
  if ((int)theta.size() != m_d)
    throw std::invalid_argument("leaveOneOutVec: theta should have length " + std::to_string(m_d));
  ensure_engine(1);
  const double factor = (m_noise_model == NoiseModel::Nugget) ? m_alpha : 1.0;
  std::vector<LooOut> out;
  m_eval->leave_one_out(1, theta.data(), &factor, false, out);
  m_evals++;
  m_rounds++;
  if (out[0].ev.status != 0) throw std::runtime_error(out[0].ev.message);
  std::vector<double> yhat(m_n), sd(m_n);
  const double s = std::sqrt(m_sigma2);
  for (int i = 0; i < m_n; ++i) {
    yhat[i] = m_y[i] - out[0].errors[i];
    sd[i] = std::sqrt(out[0].s2[i]) * s;
  }
  return {yhat, sd};
}

double Kriging::leaveOneOut() { return std::get<0>(leaveOneOutFun(m_theta, false)); }

// ---- log marginal posterior (Kriging.cpp:487-665, KrigingImpl.cpp:887-921) ----
// With B = R^-1 - R^-1 F (F' R^-1 F)^-1 F' R^-1 and x = B y = L^-T E*, the reference's Wb_k = G_k B gives
// tr(Wb_k) = 2 T2_k and y' Wb_k' Q_output = x' G_k x = 2 T1_k (adjoint sums against B), and for the nugget
// direction U1, U2; S_2 = y' B y = SSE and chol(F' R^-1 F) = Rstar'.
double Kriging::lmp_from(const EvalOut& o, const double* theta, double alpha, std::vector<double>* grad,
                         int gdim) const {
  if (o.status != 0) throw std::runtime_error(o.message);
  const int n = m_n, d = m_d, p = m_p;
  const bool nug = (m_noise_model == NoiseModel::Nugget);
  double sigma2;
  if (nug) {
    if (m_est_sigma2 && m_est_nugget)
      sigma2 = o.sse / (n - p);
    else if (m_est_sigma2 || m_est_nugget)
      sigma2 = m_sigma2 / alpha;
    else
      sigma2 = m_sigma2 + m_nugget;
  } else if (m_est_sigma2) {
    sigma2 = o.sse / (n - p);
  } else {
    sigma2 = m_sigma2;
  }
  const double log_S_2 = std::log(sigma2 * (n - p));
  const double lml = -0.5 * o.logdet - o.rstar_logdet - (n - p) / 2.0 * log_S_2;
  // default prior (RobustGaSP's approximate reference prior)
  const double a = 0.2;
  const double b = 1.0 / std::pow((double)n, 1.0 / d) * (a + d);
  std::vector<double> CL(d);
  double t = 0.0;
  for (int k = 0; k < d; ++k) {
    double mn = m_X[(size_t)k * n], mx = mn;
    for (int i = 1; i < n; ++i) {
      mn = std::min(mn, m_X[i + (size_t)k * n]);
      mx = std::max(mx, m_X[i + (size_t)k * n]);
    }
    CL[k] = (mx - mn) / std::pow((double)n, 1.0 / d);
    t += CL[k] / theta[k];
  }
  t += nug ? (1.0 - alpha) / alpha : 0.0;
  const double lp = -b * t + a * std::log(t);
  if (grad) {
    grad->assign(gdim, 0.0);
    const std::vector<double>& A = o.adj;  // [T1(d), T2(d), U1, U2, D1, D2] against B
    for (int k = 0; k < d; ++k) {
      const double ans = -A[d + k] + A[k] / sigma2;
      (*grad)[k] = ans - (a * CL[k] / t - b * CL[k]) / (theta[k] * theta[k]);
    }
    if (nug && gdim > d) {
      if (m_est_sigma2 || m_est_nugget) {
        const double ans_d = -A[2 * d + 1] + A[2 * d] / sigma2;
        (*grad)[d] = ans_d - (a / t - b) / std::pow(alpha, 2.0);
      } else {
        (*grad)[d] = 0.0;
      }
    }
  }
  return lml + lp;
}

std::tuple<double, std::vector<double>> Kriging::logMargPostFun(const std::vector<double>& gamma_in,
                                                                bool return_grad) {
  if (m_n == 0) throw std::runtime_error("Kriging model has no data: call fit() first");
  const int d = m_d;
  const bool nug = (m_noise_model == NoiseModel::Nugget);
  std::vector<double> gamma = gamma_in;
  if (nug && (int)gamma.size() == d) gamma.push_back(m_alpha);
  const int gd = d + (nug ? 1 : 0);
  if ((int)gamma.size() != gd)
    throw std::invalid_argument("logMargPostFun: theta should have length " + std::to_string(d));
  const double alpha = nug ? gamma[d] : 1.0;
  const bool analytic = return_grad && m_est_sigma2;
  ensure_engine(return_grad && !m_est_sigma2 ? d + 1 : 1);
  std::vector<EvalOut> out;
  m_eval->evaluate_lmp(1, gamma.data(), &alpha, analytic, out);
  m_evals++;
  m_rounds++;
  std::vector<double> grad;
  const double lmp = lmp_from(out[0], gamma.data(), alpha, analytic ? &grad : nullptr, gd);
  if (return_grad && !m_est_sigma2) {  // forward differences, step 1e-6 in theta (Kriging.cpp:629-640)
    const double eps = 1e-6;
    std::vector<double> th((size_t)d * d), fac(d, alpha);
    for (int k = 0; k < d; ++k)
      for (int j = 0; j < d; ++j) th[(size_t)k * d + j] = gamma[j] + (j == k ? eps : 0.0);
    std::vector<EvalOut> fd;
    m_eval->evaluate_lmp(d, th.data(), fac.data(), false, fd);
    m_evals += d;
    m_rounds++;
    grad.assign(gd, 0.0);
    for (int k = 0; k < d; ++k) grad[k] = (lmp_from(fd[k], th.data() + (size_t)k * d, alpha, nullptr, gd) - lmp) / eps;
  }
  return {lmp, grad};
}

double Kriging::logMargPost() { return std::get<0>(logMargPostFun(m_theta, false)); }

// commit the model at (theta, alpha): one exact evaluation kept in the model engine (KModel -> m_T, m_M, ...)
void Kriging::commit(const std::vector<double>& theta, double alpha) {
  if (m_service) {  // batched with the other models' evaluations; no factor is kept (predict needs a plain commit)
    const double factor = (m_noise_model == NoiseModel::Nugget) ? alpha : 1.0;
    std::vector<EvalOut> out;
    m_service->evaluate(m_service_design, 1, theta.data(), &factor, false, out);
    if (out[0].status != 0) throw std::runtime_error(out[0].message);
    m_model.reset();
    m_last_commit = out[0];
    return;
  }
  if (!m_model)
    m_model = std::make_unique<Engine>(m_kernel, m_n, m_d, m_p, m_X.data(), m_y.data(), m_F.data(), 1);
  const double factor = (m_noise_model == NoiseModel::Nugget) ? alpha : 1.0;
  std::vector<EvalOut> out;
  m_model->evaluate(1, theta.data(), &factor, false, out, nullptr);
  if (out[0].status != 0) throw std::runtime_error(out[0].message);
  m_last_commit = out[0];
}

// ---------------------------------------------------------------------------------------------------------------
void Kriging::fit(const std::vector<double>& y, const Mat& Xin, RegressionModel regmodel, bool normalize,
                  const std::string& optim, const std::string& objective, const Parameters& parameters) {
  const int n = Xin.rows, d = Xin.cols;
  if ((int)y.size() != n)
    throw std::runtime_error("Dimension of new data should be the same:\n X: (" + std::to_string(n) + "x" +
                             std::to_string(d) + "), y: (" + std::to_string(y.size()) + ")");
  const bool vecchia = objective.rfind("LLVecchia", 0) == 0;
  if (!vecchia && objective != "LL" && objective != "LOO" && objective != "LMP")
    throw std::invalid_argument("Unsupported fit objective: " + objective +
                                " (supported by the GPU build are: LL, LOO, LMP, LLVecchia, LLVecchia(m))");
  const int obj_kind = (objective == "LMP") ? 1 : (objective == "LOO") ? 2 : 0;
  if (obj_kind == 2 && m_noise_model != NoiseModel::None)  // Kriging.cpp:1471-1473
    throw std::invalid_argument("LOO objective not supported for Nugget/Heterogeneous noise modes");
  if (obj_kind != 0 && m_service)
    throw std::invalid_argument("a shared evaluation service runs the LL objective only");
  if (vecchia) {
    parse_vll_m(objective);  // validate the spec early (throws on malformed), Kriging.cpp:1522-1524
    if (m_noise_model != NoiseModel::None)
      throw std::invalid_argument("LLVecchia objective not supported for Nugget/Heterogeneous noise modes");
  }
  if (d > MAX_D) throw std::invalid_argument("input dimension d > 32 is not supported by the GPU kernels");
  m_optim = optim;
  m_objective = objective;
  m_eval.reset();
  m_vecchia.reset();
  m_vecchia_light = false;
  m_model.reset();
  // ---- fit_setup_impl (KrigingImpl.cpp:764-841) ----
  m_n = n;
  m_d = d;
  m_normalize = normalize;
  m_centerX.assign(d, 0.0);
  m_scaleX.assign(d, 1.0);
  m_centerY = 0.0;
  m_scaleY = 1.0;
  if (normalize) {
    for (int j = 0; j < d; ++j) {
      double mn = Xin(0, j), mx = Xin(0, j);
      for (int i = 1; i < n; ++i) {
        mn = std::min(mn, Xin(i, j));
        mx = std::max(mx, Xin(i, j));
      }
      m_centerX[j] = mn;
      m_scaleX[j] = mx - mn;
    }
    double mn = *std::min_element(y.begin(), y.end()), mx = *std::max_element(y.begin(), y.end());
    m_centerY = mn;
    m_scaleY = mx - mn;
  }
  m_X.resize((size_t)n * d);
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < n; ++i) m_X[i + (size_t)j * n] = (Xin(i, j) - m_centerX[j]) / m_scaleX[j];
  m_y.resize(n);
  for (int i = 0; i < n; ++i) m_y[i] = (y[i] - m_centerY) / m_scaleY;
  std::vector<double> maxdX(d);
  for (int j = 0; j < d; ++j) {
    double mn = m_X[(size_t)j * n], mx = mn;
    for (int i = 1; i < n; ++i) {
      mn = std::min(mn, m_X[i + (size_t)j * n]);
      mx = std::max(mx, m_X[i + (size_t)j * n]);
    }
    maxdX[j] = mx - mn;
  }
  m_regmodel = regmodel;
  m_F = regression_matrix(regmodel, m_X, n, d, &m_p);
  m_est_beta = parameters.is_beta_estim && (m_regmodel != RegressionModel::None);
  if (!m_est_beta && parameters.beta.has_value() && !parameters.beta->empty()) {
    m_est_beta = false;
    m_beta = *parameters.beta;
    if (m_normalize)
      for (auto& b : m_beta) b /= m_scaleY;
  } else {
    m_est_beta = true;
  }
  Mat theta0;
  if (parameters.theta.has_value()) {
    theta0 = *parameters.theta;
    if (theta0.cols != d && theta0.rows == d) {  // transpose
      Mat t;
      t.rows = theta0.cols;
      t.cols = theta0.rows;
      t.v.resize(theta0.v.size());
      for (int i = 0; i < t.rows; ++i)
        for (int j = 0; j < t.cols; ++j) t(i, j) = theta0(j, i);
      theta0 = t;
    }
    if (m_normalize)
      for (int i = 0; i < theta0.rows; ++i)
        for (int j = 0; j < theta0.cols; ++j) theta0(i, j) /= m_scaleX[j];
    if (theta0.cols != d)
      throw std::runtime_error("Dimension of theta should be nx" + std::to_string(d) + " instead of " +
                               std::to_string(theta0.rows) + "x" + std::to_string(theta0.cols));
  }
  const Config& cfg = config();
  if (vecchia) {  // Kriging.cpp:1619-1624: sets built once per fit, on the GPU
    m_vecchia_m = parse_vll_m(objective);
    m_vorder.assign(n, 0);
    m_vnbr.assign((size_t)n * std::min(m_vecchia_m, VECCHIA_MAX_M), -1);
    if (m_vecchia_m > VECCHIA_MAX_M) throw std::invalid_argument("LLVecchia on the GPU supports m <= 32");
    vecchia_sets_gpu(n, d, m_X.data(), m_vecchia_m, m_vorder.data(), m_vnbr.data());
  } else {
    m_vecchia_m = 0;
    m_vorder.clear();
    m_vnbr.clear();
  }

  if (optim == "none") {  // Kriging.cpp:1633-1715
    if (!parameters.theta.has_value())
      throw std::runtime_error("Theta should be given (1x" + std::to_string(d) + ") matrix, when optim=none");
    m_theta.resize(d);
    for (int j = 0; j < d; ++j) m_theta[j] = theta0(0, j);
    m_est_theta = false;
    double sigma2 = -1;
    m_est_sigma2 = parameters.is_sigma2_estim;
    if (parameters.sigma2.has_value()) {
      sigma2 = *parameters.sigma2;
      if (m_normalize) sigma2 /= (m_scaleY * m_scaleY);
    } else {
      m_est_sigma2 = true;
    }
    double nugget_param = 0.0;
    if (m_noise_model == NoiseModel::Nugget) {
      m_est_nugget = parameters.is_nugget_estim;
      if (parameters.nugget.has_value()) {
        nugget_param = *parameters.nugget;
        if (m_normalize) nugget_param /= (m_scaleY * m_scaleY);
      }
      if (sigma2 > 0 && (sigma2 + nugget_param) > 0)
        m_alpha = sigma2 / (sigma2 + nugget_param);
      else
        m_alpha = 1.0 - kNuggetAlphaLower;
    }
    commit(m_theta, m_alpha);
    const EvalOut& m = m_last_commit;
    m_is_empty = false;
    if (m_est_beta) m_beta = m.beta;
    if (m_noise_model == NoiseModel::Nugget) {
      if (m_est_sigma2) {
        const double total_var = m.sse / n;
        m_sigma2 = m_alpha * total_var;
        m_nugget = m_est_nugget ? (1.0 - m_alpha) * total_var : nugget_param;
      } else {
        m_sigma2 = sigma2;
        m_nugget = m_est_nugget ? 0.0 : nugget_param;
      }
    } else if (m_est_sigma2) {
      m_sigma2 = m.sse / n;
    } else {
      m_sigma2 = sigma2;
    }
    return;
  }

  // ---- BFGS[N] (Kriging.cpp:1717-2209) ----
  if (optim.rfind("BFGS", 0) != 0)
    throw std::runtime_error("Unsupported optim: " + optim + " (supported are: none, BFGS[#])");
  std::vector<double> theta_lower(d), theta_upper(d);
  {
    // Optim::theta_bounds (Optim.cpp:179-209) with dX recomputed from X
    for (int j = 0; j < d; ++j) {
      theta_lower[j] = cfg.theta_lower_factor * maxdX[j];
      theta_upper[j] = cfg.theta_upper_factor * maxdX[j];
    }
    // the reference applies the heuristic only when its n^2 x d difference matrix exists, which a light Vecchia fit
    // never builds (Kriging.cpp:1610-1612, Optim.cpp:186)
    const bool dX_built = !(vecchia && !m_vecchia_exact_commit);
    if (cfg.variogram_bounds_heuristic && n > 0 && dX_built) {
      double wsum = 0.0;
      std::vector<double> steep(d, 0.0);
      std::vector<double> dx(d);
      for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
          if (i == j) continue;
          double dx2 = 0.0;
          for (int k = 0; k < d; ++k) {
            dx[k] = m_X[i + (size_t)k * n] - m_X[j + (size_t)k * n];
            dx2 += dx[k] * dx[k];
          }
          const double dyv = m_y[i] - m_y[j];
          double slope = (dyv * dyv) / dx2;
          if (std::isnan(slope)) slope = 0.0;
          wsum += slope;
          for (int k = 0; k < d; ++k) steep[k] += std::fabs(dx[k]) * slope;
        }
      }
      if (wsum > 0.0) {
        for (int k = 0; k < d; ++k) {
          const double s = steep[k] / wsum;
          theta_lower[k] = std::max(theta_lower[k], cfg.theta_lower_factor * s);
          theta_lower[k] = std::min(theta_lower[k], theta_upper[k]);
          theta_upper[k] = std::max(theta_lower[k], theta_upper[k]);
        }
      }
    }
  }
  rng_engine().seed(rng_seed());  // Random::init()
  // a warm restart (update) runs one L-BFGS-B from the given theta, without restarts (Kriging.cpp:2583-2590)
  int multistart = m_warm ? 1 : parse_method(optim, "BFGS").second;
  const int max_restart = m_warm ? 0 : cfg.max_restart;
  Mat U = randu_mat(multistart, d);
  Mat theta0_rand;
  theta0_rand.rows = multistart;
  theta0_rand.cols = d;
  theta0_rand.v.resize((size_t)multistart * d);
  for (int i = 0; i < multistart; ++i)
    for (int j = 0; j < d; ++j) theta0_rand(i, j) = theta_lower[j] + U(i, j) * (theta_upper[j] - theta_lower[j]);
  Mat starts;
  if (parameters.theta.has_value()) {
    if (!m_warm) multistart = std::max(multistart, theta0.rows);
    starts.rows = multistart;
    starts.cols = d;
    starts.v.resize((size_t)multistart * d);
    for (int i = 0; i < multistart; ++i)
      for (int j = 0; j < d; ++j) starts(i, j) = (i < theta0.rows) ? theta0(i, j) : theta0_rand(i - theta0.rows, j);
  } else {
    starts = theta0_rand;
  }
  std::vector<double> extra0;
  double extra_lower = 0.0, extra_upper = 1.0;
  if (m_noise_model == NoiseModel::Nugget) {
    extra_lower = kNuggetAlphaLower;
    extra_upper = 1.0;
    if (parameters.sigma2.has_value() && parameters.nugget.has_value()) {
      const double s = *parameters.sigma2, nu = *parameters.nugget;
      extra0 = {(s > 0 && (s + nu) > 0) ? s / (s + nu) : extra_lower + (extra_upper - extra_lower) * 0.5};
    } else {
      std::vector<double> u = randu_vec(starts.rows);
      extra0.resize(u.size());
      for (size_t i = 0; i < u.size(); ++i)
        extra0[i] = extra_lower + (extra_upper - extra_lower) * (1.0 - std::pow(u[i], 3.0));
    }
  }
  const bool nug = (m_noise_model == NoiseModel::Nugget);
  const int gd = d + (nug ? 1 : 0);
  auto reparam_to = [&](const std::vector<double>& ta) {  // nugget_reparam_to / Optim::reparam_to
    std::vector<double> g(ta.size());
    for (int j = 0; j < d; ++j) g[j] = cfg.reparametrize ? std::log(ta[j]) : ta[j];
    if (nug) g[d] = cfg.reparametrize ? -std::log(1.0 + kNuggetAlphaLower - ta[d]) : ta[d];
    return g;
  };
  auto reparam_from = [&](const std::vector<double>& g) {
    std::vector<double> ta(g.size());
    for (int j = 0; j < d; ++j) ta[j] = cfg.reparametrize ? std::exp(g[j]) : g[j];
    if (nug) ta[d] = cfg.reparametrize ? 1.0 + kNuggetAlphaLower - std::exp(-g[d]) : g[d];
    return ta;
  };
  std::vector<double> bl(gd), bu(gd);
  for (int j = 0; j < d; ++j) {
    bl[j] = theta_lower[j];
    bu[j] = theta_upper[j];
  }
  if (nug) {
    bl[d] = extra_lower;
    bu[d] = extra_upper;
  }
  const std::vector<double> gamma_lower = reparam_to(bl), gamma_upper = reparam_to(bu);
  // estimation flags (Kriging.cpp:1841-1859)
  m_est_sigma2 = parameters.is_sigma2_estim;
  if (!m_est_sigma2 && parameters.sigma2.has_value()) {
    m_sigma2 = *parameters.sigma2;
    if (m_normalize) m_sigma2 /= (m_scaleY * m_scaleY);
  } else {
    m_est_sigma2 = true;
  }
  if (nug) {
    m_est_nugget = parameters.is_nugget_estim;
    if (!m_est_nugget && parameters.nugget.has_value()) {
      m_nugget = *parameters.nugget;
      if (m_normalize) m_nugget /= (m_scaleY * m_scaleY);
    } else {
      m_est_nugget = true;
    }
  }
  if (!vecchia && !m_service) ensure_engine(multistart);
  if (vecchia) ensure_vecchia();

  // batched objective: -LL in gamma space (make_fit_objective, Kriging.cpp:1414-1470); the exact requests of one
  // round go to the GPU as one batched evaluation, Vecchia requests one after another
  Batcher batcher(multistart, [&](std::vector<EvalRequest*>& reqs) {
    std::vector<EvalRequest*> dense;
    for (auto* r : reqs) {
      if (r->vecchia) {
        r->vout = m_vecchia->evaluate(r->theta.data(), r->want_grad, m_est_beta || (int)m_beta.size() != m_p,
                                      m_beta.data());
        m_evals++;
        m_rounds++;
      } else {
        dense.push_back(r);
      }
    }
    const int k = (int)dense.size();
    if (k == 0) return;
    if (!m_service) ensure_engine(std::max(k, multistart));
    std::vector<double> th((size_t)k * d), fac(k);
    bool g = false;
    for (int b = 0; b < k; ++b) {
      std::copy(dense[b]->theta.begin(), dense[b]->theta.begin() + d, th.begin() + (size_t)b * d);
      fac[b] = dense[b]->factor;
      g = g || dense[b]->want_grad;
    }
    std::vector<EvalOut> out;
    if (obj_kind == 2) {
      std::vector<LooOut> lo;
      m_eval->leave_one_out(k, th.data(), fac.data(), g, lo);
      m_evals += k;
      m_rounds++;
      for (int b = 0; b < k; ++b) dense[b]->lout = std::move(lo[b]);
      return;
    }
    if (m_service)
      m_service->evaluate(m_service_design, k, th.data(), fac.data(), g, out);
    else if (obj_kind == 1)
      m_eval->evaluate_lmp(k, th.data(), fac.data(), g, out);
    else
      m_eval->evaluate(k, th.data(), fac.data(), g, out, nullptr);
    m_evals += k;
    m_rounds++;
    for (int b = 0; b < k; ++b) dense[b]->out = std::move(out[b]);
  });
  // The objective to maximise (LL, LMP, or -LOO) and its gradient in theta (alpha) space.
  // exact_ll: the exact likelihood even under LLVecchia (the final exact-commit evaluation, Kriging.cpp:1532-1551)
  auto eval_ll = [&](const std::vector<double>& ta, bool want_grad, std::vector<double>* grad, bool exact_ll) {
    EvalRequest req;
    req.theta.assign(ta.begin(), ta.begin() + d);
    double extra = nug ? ta[d] : m_sigma2;
    if (nug && obj_kind == 0 && !m_est_sigma2 && !m_est_nugget) extra = m_sigma2 / (m_sigma2 + m_nugget);
    req.factor = nug ? extra : 1.0;
    req.want_grad = want_grad && !(obj_kind == 1 && !m_est_sigma2);
    req.vecchia = vecchia && !exact_ll;
    req.kind = obj_kind;
    batcher.submit(&req);
    if (req.err) std::rethrow_exception(req.err);
    if (req.vecchia) {
      if (req.vout.status != 0) throw std::runtime_error(req.vout.message);
      if (grad) *grad = req.vout.grad;
      return req.vout.vll;
    }
    if (obj_kind == 2) {  // maximise -LOO
      if (req.lout.ev.status != 0) throw std::runtime_error(req.lout.ev.message);
      if (grad) {
        grad->assign(gd, 0.0);
        for (int j = 0; j < d; ++j) (*grad)[j] = -req.lout.grad[j];
      }
      return -req.lout.loo;
    }
    if (obj_kind == 1) {
      const double lmp = lmp_from(req.out, ta.data(), extra, req.want_grad ? grad : nullptr, gd);
      if (want_grad && !req.want_grad) {  // sigma2 fixed: forward differences in theta (Kriging.cpp:629-640)
        grad->assign(gd, 0.0);
        for (int k = 0; k < d; ++k) {
          EvalRequest r2;
          r2.theta = req.theta;
          r2.theta[k] += 1e-6;
          r2.factor = req.factor;
          r2.kind = 1;
          batcher.submit(&r2);
          if (r2.err) std::rethrow_exception(r2.err);
          (*grad)[k] = (lmp_from(r2.out, r2.theta.data(), extra, nullptr, gd) - lmp) / 1e-6;
        }
      }
      return lmp;
    }
    return loglik_from(req.out, extra, grad, gd);
  };
  auto fit_ofn = [&](const std::vector<double>& gamma, std::vector<double>* grad_out) {
    const std::vector<double> ta = reparam_from(gamma);
    std::vector<double> g;
    const bool exact = vecchia && grad_out == nullptr && m_vecchia_exact_commit;
    const double ll = eval_ll(ta, grad_out != nullptr, grad_out ? &g : nullptr, exact);
    if (grad_out) {
      grad_out->resize(gd);
      for (int j = 0; j < d; ++j) (*grad_out)[j] = -(cfg.reparametrize ? g[j] * ta[j] : g[j]);
      if (nug) (*grad_out)[d] = -(cfg.reparametrize ? g[d] * (1.0 + kNuggetAlphaLower - ta[d]) : g[d]);
    }
    return -ll;
  };

  struct Result {
    bool success = false;
    double objective = std::numeric_limits<double>::infinity();
    std::vector<double> theta;
    double extra = 0.0;
    std::string error;
  };
  std::vector<Result> results(multistart);
  auto worker = [&](int s) {
    Result& res = results[s];
    try {
      std::vector<double> theta_start(d);
      for (int j = 0; j < d; ++j) theta_start[j] = starts(s, j);
      std::vector<double> ta(theta_start);
      if (nug) ta.push_back(extra0[s % extra0.size()]);
      std::vector<double> gamma_tmp = reparam_to(ta);
      std::vector<double> lo(gd), hi(gd);
      for (int j = 0; j < gd; ++j) {
        lo[j] = std::min(gamma_tmp[j], gamma_lower[j]);
        hi[j] = std::max(gamma_tmp[j], gamma_upper[j]);
      }
      Lbfgsb opt(gd);
      opt.iprint = -1;
      opt.max_iter = cfg.max_iteration;
      // LOO values scale like 1 / n^2 of the likelihood's (Kriging.cpp:1953-1958)
      const double loo_scale = (obj_kind == 2) ? 1.0 / ((double)n * n) : 1.0;
      opt.pgtol = cfg.gradient_tolerance * loo_scale;
      opt.factr = cfg.objective_rel_tolerance / 1e-13 * loo_scale;
      std::vector<int> btype(gd, 2);
      int retry = 0;
      double best_f = std::numeric_limits<double>::infinity();
      std::vector<double> best_gamma = gamma_tmp;
      while (retry <= max_restart) {
        LbfgsbResult r = opt.minimize(
            [&](const std::vector<double>& x, std::vector<double>& g) { return fit_ofn(x, &g); }, gamma_tmp,
            lo.data(), hi.data(), btype.data());
        if (r.f_opt < best_f) {
          best_f = r.f_opt;
          best_gamma = gamma_tmp;
        }
        std::vector<double> tp = reparam_from(gamma_tmp);
        double sol_to_lb = std::numeric_limits<double>::infinity();
        for (int j = 0; j < d; ++j) sol_to_lb = std::min(sol_to_lb, std::fabs(tp[j] - theta_lower[j]));
        if (retry < max_restart &&
            (r.task.rfind("ABNORMAL_TERMINATION_IN_LNSRCH", 0) == 0 || r.num_iters <= 2 ||
             sol_to_lb < std::numeric_limits<double>::epsilon() || r.f_opt > best_f)) {
          std::vector<double> rt(d);
          for (int j = 0; j < d; ++j) rt[j] = (theta_start[j] + theta_lower[j]) / std::pow(2.0, retry + 1);
          std::vector<double> ta2(rt);
          if (nug) ta2.push_back(extra0[s % extra0.size()]);
          gamma_tmp = reparam_to(ta2);
          for (int j = 0; j < gd; ++j) {
            lo[j] = std::min(gamma_tmp[j], lo[j]);
            hi[j] = std::max(gamma_tmp[j], hi[j]);
          }
          retry++;
        } else {
          break;
        }
      }
      res.objective = fit_ofn(best_gamma, nullptr);  // final evaluation at the best point
      std::vector<double> ta_best = reparam_from(best_gamma);
      res.theta.assign(ta_best.begin(), ta_best.begin() + d);
      res.extra = nug ? ta_best[d] : 0.0;
      res.success = true;
    } catch (const std::exception& e) {
      res.success = false;
      res.error = e.what();
    }
    batcher.leave();
  };
  {
    std::vector<std::thread> threads;
    threads.reserve(multistart);
    for (int s = 0; s < multistart; ++s) threads.emplace_back(worker, s);
    for (auto& t : threads) t.join();
  }
  int best = -1, ok = 0;
  double min_ofn = std::numeric_limits<double>::infinity();
  for (int s = 0; s < multistart; ++s) {
    if (!results[s].success) continue;
    ok++;
    if (results[s].objective < min_ofn) {
      min_ofn = results[s].objective;
      best = s;
    }
  }
  if (ok == 0) throw std::runtime_error("All " + std::to_string(multistart) + " optimization attempts failed");
  const Result& b = results[best];
  m_theta = b.theta;
  m_est_theta = true;
  m_is_empty = false;
  if (vecchia && !m_vecchia_exact_commit) {  // light commit (Kriging.cpp:2117-2136)
    VecchiaOut vo = m_vecchia->evaluate(m_theta.data(), false, m_est_beta || (int)m_beta.size() != m_p,
                                        m_beta.data());
    if (vo.status != 0) throw std::runtime_error(vo.message);
    if (m_est_beta) m_beta = vo.beta;
    if (m_est_sigma2) m_sigma2 = vo.sigma2;
    m_vecchia_light = true;
    m_is_empty = true;
    m_last_fit_starts = multistart;
    return;
  }
  if (nug) m_alpha = b.extra;
  commit(m_theta, m_alpha);
  const EvalOut& m = m_last_commit;
  if (m_est_beta) m_beta = m.beta;
  if (nug) {
    if (m_est_sigma2) {
      if (m_est_nugget) {
        const double total_var = m.sse / n;
        m_sigma2 = m_alpha * total_var;
        if (obj_kind == 1) m_sigma2 = m_sigma2 * n / (n - m_p - 2);
        m_nugget = m_sigma2 / m_alpha - m_sigma2;
      } else {
        m_sigma2 = m_nugget * m_alpha / (1.0 - m_alpha);
      }
    } else {
      if (m_est_nugget) m_nugget = m_sigma2 * (1.0 - m_alpha) / m_alpha;
    }
  } else if (m_est_sigma2) {
    m_sigma2 = (obj_kind == 1) ? m.sse / (n - m_p) : m.sse / n;
  }
  m_last_fit_starts = multistart;
}

// ---------------------------------------------------------------------------------------------------------------
// Vecchia (Kriging.cpp:718-734 parse, :926-941 logLikelihoodVecchiaFun)
int Kriging::parse_vll_m(const std::string& objective) {
  if (objective == "LLVecchia") return 30;
  if (objective.rfind("LLVecchia(", 0) == 0 && objective.back() == ')') {
    const std::string inside = objective.substr(10, objective.size() - 11);
    try {
      size_t pos = 0;
      const long m = std::stol(inside, &pos);
      if (m >= 1) return (int)m;
    } catch (const std::exception&) {
    }
  }
  throw std::invalid_argument("Invalid Vecchia objective '" + objective +
                              "': expected \"LLVecchia\" or \"LLVecchia(m)\" with m >= 1 (e.g. \"LLVecchia(30)\")");
}

void Kriging::ensure_vecchia() {
  if (!m_vecchia) {
    const int mm = m_n > 0 ? (int)(m_vnbr.size() / m_n) : 0;
    m_vecchia = std::make_unique<VecchiaEngine>(m_kernel, m_n, m_d, m_p, m_X.data(), m_y.data(), m_F.data(),
                                                m_vorder.data(), m_vnbr.data(), mm);
  }
}

std::tuple<double, std::vector<double>> Kriging::logLikelihoodVecchiaFun(const std::vector<double>& theta,
                                                                         bool return_grad) {
  if (m_vecchia_m == 0 || (int)m_vorder.size() != m_n)
    throw std::runtime_error("logLikelihoodVecchiaFun: model was not fitted with objective=\"LLVecchia(m)\"");
  if ((int)theta.size() != m_d)
    throw std::invalid_argument("logLikelihoodVecchiaFun: theta should have length " + std::to_string(m_d));
  ensure_vecchia();
  VecchiaOut vo = m_vecchia->evaluate(theta.data(), return_grad, m_est_beta || (int)m_beta.size() != m_p,
                                      m_beta.data());
  m_evals++;
  m_rounds++;
  if (vo.status != 0) throw std::runtime_error(vo.message);
  return {vo.vll, return_grad ? vo.grad : std::vector<double>()};
}

Mat Kriging::T() const {
  Mat m;
  if (!m_model) return m;
  m.rows = m.cols = m_n;
  m_model->copy_model(0, &m.v, nullptr, nullptr, nullptr, nullptr);
  return m;
}

Mat Kriging::M() const {
  Mat m;
  if (!m_model) return m;
  m.rows = m_n;
  m.cols = m_p;
  m_model->copy_model(0, nullptr, &m.v, nullptr, nullptr, nullptr);
  return m;
}

std::vector<double> Kriging::z() const {
  std::vector<double> z;
  if (!m_model) return z;
  if (m_est_beta) {
    m_model->copy_model(0, nullptr, nullptr, nullptr, nullptr, &z);
  } else {  // m_z = ystar - M beta
    std::vector<double> ystar, Fs;
    m_model->copy_model(0, nullptr, &Fs, &ystar, nullptr, nullptr);
    z = ystar;
    for (int i = 0; i < m_n; ++i)
      for (int q = 0; q < m_p; ++q) z[i] -= Fs[i + (size_t)q * m_n] * m_beta[q];
  }
  return z;
}

// Kriging::predictVecchia (Kriging.cpp:950-1022): each point kriged on its m nearest observations, beta treated as
// known; neighbour search, local factorisations and solves on the GPU
std::tuple<std::vector<double>, std::vector<double>> Kriging::predictVecchia(const Mat& X_n, bool return_stdev,
                                                                             int m) {
  if (m_n == 0 || (int)m_theta.size() != m_d) throw std::runtime_error("predictVecchia: model is not fitted");
  const int n = m_n, d = m_d, p = m_p, q = X_n.rows;
  if (X_n.cols != d) throw std::invalid_argument("X_n should have the same number of columns as X");
  if (m <= 0) m = (m_vecchia_m > 0) ? m_vecchia_m : 30;
  m = std::min(m, n);
  Mat Xnn;
  Xnn.rows = q;
  Xnn.cols = d;
  Xnn.v.resize((size_t)q * d);
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < q; ++i) Xnn(i, j) = (X_n(i, j) - m_centerX[j]) / m_scaleX[j];
  int pn = 0;
  std::vector<double> Fn = regression_matrix(m_regmodel, Xnn.v, q, d, &pn);
  std::vector<double> resid(n);
  for (int i = 0; i < n; ++i) {
    double fb = 0.0;
    for (int k = 0; k < p; ++k) fb += m_F[i + (size_t)k * n] * m_beta[k];
    resid[i] = m_y[i] - fb;
  }
  std::vector<double> ar, ra;
  vecchia_predict_gpu(m_kernel, n, d, m_X.data(), resid.data(), m_theta.data(), q, Xnn.v.data(), m, ar, ra);
  std::vector<double> mean(q), sd;
  for (int t = 0; t < q; ++t) {
    double fb = 0.0;
    for (int k = 0; k < p; ++k) fb += Fn[t + (size_t)k * q] * m_beta[k];
    mean[t] = (fb + ar[t]) * m_scaleY + m_centerY;
  }
  if (return_stdev) {
    sd.resize(q);
    for (int t = 0; t < q; ++t) sd[t] = std::sqrt(m_sigma2 * std::max(0.0, 1.0 - ra[t])) * m_scaleY;
  }
  return {mean, sd};
}

std::tuple<std::vector<double>, std::vector<double>, Mat, Mat, Mat> Kriging::predict(const Mat& X_n, bool return_stdev,
                                                                                      bool return_cov,
                                                                                      bool return_deriv) {
  if (m_vecchia_light) {  // Kriging.cpp:2242-2251: no exact factor, mean / stdev from the local predictor
    if (return_cov || return_deriv)
      throw std::runtime_error(
          "predict: return_cov/return_deriv are not available on a light Vecchia fit "
          "(refit with set_vecchia_exact_commit(true), or use predictVecchia)");
    auto [mean, sd] = predictVecchia(X_n, return_stdev, 0);
    return {mean, sd, Mat{}, Mat{}, Mat{}};
  }
  if (m_is_empty || !m_model) throw std::runtime_error("predict: model is not fitted");
  if (X_n.cols != m_d)
    throw std::runtime_error("Predict locations have wrong dimension: " + std::to_string(X_n.cols) + " instead of " +
                             std::to_string(m_d));
  const int q = X_n.rows, d = m_d, n = m_n, p = m_p;
  const bool nug = (m_noise_model == NoiseModel::Nugget);
  // Kriging.cpp:2262-2283: an LMP fit predicts with sigma2 (n - p) / (n - p - 2)
  const double lmp_scale = (m_objective == "LMP") ? (n - p) / (n - p - 2.0) : 1.0;
  const double sigma2 = m_sigma2 * lmp_scale;
  const double R_on_factor = nug ? m_alpha : 1.0;
  const double var_scale = nug ? sigma2 / m_alpha : sigma2;
  Mat Xnn;
  Xnn.rows = q;
  Xnn.cols = d;
  Xnn.v.resize((size_t)q * d);
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < q; ++i) Xnn(i, j) = (X_n(i, j) - m_centerX[j]) / m_scaleX[j];
  int pn = 0;
  std::vector<double> Fn = regression_matrix(m_regmodel, Xnn.v, q, d, &pn);
  std::vector<double> zz = z();
  // on a mixed-precision model the solves of large predictions run as digit products with L^-1 (FP64-level)
  const bool digits = m_slices > 0 && n >= 512 && q >= 256;
  PredictOut po = predict_gpu(*m_model, Xnn.v.data(), q, m_theta.data(), R_on_factor, zz.data(), return_stdev || return_cov,
                              return_cov, nug ? m_alpha : 1.0, return_deriv, digits);
  // yhat = F_n beta + Rstar_on' z
  std::vector<double> mean(q), sd;
  for (int i = 0; i < q; ++i) {
    double fb = 0.0;
    for (int k = 0; k < p; ++k) fb += Fn[i + (size_t)k * q] * m_beta[k];
    mean[i] = m_centerY + m_scaleY * (fb + po.rz[i]);
  }
  Mat cov, md, sdd;
  std::vector<double> Rstar, Ec;
  if (return_stdev || return_cov || return_deriv) {
    // Ecirc = (F_n - Rstar_on' M) * circ^-1   (rsolve_upper)
    m_model->copy_model(0, nullptr, nullptr, nullptr, &Rstar, nullptr);
    Ec.assign((size_t)q * p, 0.0);
    for (int i = 0; i < q; ++i) {
      for (int k = 0; k < p; ++k) {
        double e = Fn[i + (size_t)k * q] - po.rm[(size_t)i * p + k];
        for (int l = 0; l < k; ++l) e -= Ec[i + (size_t)l * q] * Rstar[l + (size_t)k * p];
        Ec[i + (size_t)k * q] = e / Rstar[k + (size_t)k * p];
      }
    }
    if (return_stdev) {
      sd.resize(q);
      for (int i = 0; i < q; ++i) {
        double e2 = 0.0;
        for (int k = 0; k < p; ++k) e2 += Ec[i + (size_t)k * q] * Ec[i + (size_t)k * q];
        double v = 1.0 - po.rr[i] + e2;
        if (std::isnan(v) || v < 0) v = 0.0;
        v *= var_scale * m_scaleY * m_scaleY;
        sd[i] = std::sqrt(v);
      }
    }
    if (return_cov) {
      cov.rows = cov.cols = q;
      cov.v = po.sigma;  // R_nn - Rstar_on' Rstar_on
      for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) {
          double e = 0.0;
          for (int k = 0; k < p; ++k) e += Ec[i + (size_t)k * q] * Ec[j + (size_t)k * q];
          cov(i, j) = (cov(i, j) + e) * var_scale * m_scaleY * m_scaleY;
        }
    }
  }
  if (return_deriv) {
    // KrigingImpl.cpp:254-296, per point i with W_i = L^-1 DR_on_i (GPU) and DF_i = dF/dx at the point:
    //   Dyhat(i, :)  = (DF_i beta + W_i' z)'
    //   DEcirc_i     = circ'^-1 (DF_i - W_i' M)'                      (p x d)
    //   Dysd2(i, :)  = -2 Rstar_on(:, i)' W_i + 2 Ecirc(i, :) DEcirc_i
    // then the normalisation's chain rule and stdev_deriv = Dysd2 / (2 sqrt(ysd2)).
    md.rows = sdd.rows = q;
    md.cols = sdd.cols = d;
    md.v.assign((size_t)q * d, 0.0);
    sdd.v.assign((size_t)q * d, 0.0);
    std::vector<double> xi(d), A((size_t)p * d), DE((size_t)p * d);
    const double sd_scale = var_scale * m_scaleY * m_scaleY;
    for (int i = 0; i < q; ++i) {
      for (int k = 0; k < d; ++k) xi[k] = Xnn(i, k);
      const std::vector<double> DF = regression_derivative(m_regmodel, xi.data(), d, p);
      for (int k = 0; k < d; ++k) {
        const size_t c = (size_t)i * d + k;
        double fb = 0.0;
        for (int l = 0; l < p; ++l) fb += DF[k + (size_t)l * d] * m_beta[l];
        md.v[i + (size_t)k * q] = (fb + po.wz[c]) * m_scaleY / m_scaleX[k];
      }
      if (!return_stdev) continue;
      for (int k = 0; k < d; ++k)
        for (int l = 0; l < p; ++l)
          A[l + (size_t)k * p] = DF[k + (size_t)l * d] - po.wm[((size_t)i * d + k) * p + l];
      // forward substitution with circ' (lower): DE(l, k) = (A(l, k) - sum_{m<l} circ(m, l) DE(m, k)) / circ(l, l)
      for (int k = 0; k < d; ++k)
        for (int l = 0; l < p; ++l) {
          double e = A[l + (size_t)k * p];
          for (int m2 = 0; m2 < l; ++m2) e -= Rstar[m2 + (size_t)l * p] * DE[m2 + (size_t)k * p];
          DE[l + (size_t)k * p] = e / Rstar[l + (size_t)l * p];
        }
      for (int k = 0; k < d; ++k) {
        double ed = 0.0;
        for (int l = 0; l < p; ++l) ed += Ec[i + (size_t)l * q] * DE[l + (size_t)k * p];
        const double dysd2 = (-2.0 * po.wr[(size_t)i * d + k] + 2.0 * ed) * sd_scale / m_scaleX[k];
        sdd.v[i + (size_t)k * q] = dysd2;
      }
    }
    // the reference divides by 2 sqrt(ysd2) for every point, with ysd2 = 0 when the stdev is not requested
    for (int i = 0; i < q; ++i) {
      const double den = 2.0 * (return_stdev ? sd[i] : 0.0);
      for (int k = 0; k < d; ++k) sdd.v[i + (size_t)k * q] /= den;
    }
  }
  return {mean, sd, cov, md, sdd};
}

std::string Kriging::summary() const {
  std::ostringstream o;
  o << "* data: " << m_n << "x" << m_d << "\n";
  o << "* trend " << regmodel_to_string(m_regmodel) << (m_est_beta ? " (est.)" : "") << ": ";
  for (double b : m_beta) o << b << " ";
  o << "\n* variance" << (m_est_sigma2 ? " (est.)" : "") << ": " << m_sigma2 << "\n";
  o << "* covariance:\n  * kernel: " << m_covType << "\n  * range" << (m_est_theta ? " (est.)" : "") << ": ";
  for (double t : m_theta) o << t << " ";
  if (m_noise_model == NoiseModel::Nugget) o << "\n  * nugget" << (m_est_nugget ? " (est.)" : "") << ": " << m_nugget;
  o << "\n  * fit:\n    * objective: " << m_objective << "\n    * optim: " << m_optim << "\n";
  return o.str();
}

}  // namespace lkg
