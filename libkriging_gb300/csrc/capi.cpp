// capi.cpp -- extern "C" boundary (include/libkriging_gb300.h).
//
// Same conventions as libKriging's C ABI (bindings/Julia/jlibkriging/csrc/libkriging_c.cpp:16-41): opaque handles,
// column-major double arrays, 0 / -1 status, thread_local last error; NULL / NaN returns for pointer / double
// functions on error.
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <sstream>
#include <string>

#include "../../include/libkriging_gb300.h"
#include "common.cuh"
#include "config.hpp"
#include "kriging.hpp"
#include "vecchia.hpp"
#include "nested.hpp"

using lkg::Kriging;
using lkg::Mat;

static thread_local std::string g_last_error;

namespace lkg {
// the last-error text of this thread, for entry points implemented outside this file
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }
}  // namespace lkg

// Runs the body of one entry point.  A C++ exception never crosses the C boundary: its text becomes this thread's
// last error and the entry point returns its failure value (-1, NULL or NaN, as the header states per function).
template <class R, class Body>
R run_entry(R failure, Body&& body) noexcept {
  try {
    return body();
  } catch (const std::exception& e) {
    g_last_error = e.what();
  } catch (...) {
    g_last_error = "unexpected non-standard C++ exception";
  }
  return failure;
}

namespace {

// NoiseModel names as the reference's bindings spell them; NULL means the default ("none")
Kriging::NoiseModel parse_noise_model(const char* name) {
  const std::string key = name ? name : "none";
  struct Entry {
    const char* text;
    Kriging::NoiseModel model;
  };
  static const Entry known[] = {{"none", Kriging::NoiseModel::None}, {"nugget", Kriging::NoiseModel::Nugget}};
  for (const Entry& e : known)
    if (key == e.text) return e.model;
  if (key == "heterogeneous")
    throw std::invalid_argument("noise_model 'heterogeneous' is not supported by the GPU build");
  throw std::runtime_error("Unknown noise_model: " + key);
}

Kriging* K(void* p) {
  if (!p) throw std::invalid_argument("null Kriging handle");
  return static_cast<Kriging*>(p);
}

Mat mat_of(const double* p, int rows, int cols) {
  Mat m;
  m.rows = rows;
  m.cols = cols;
  m.v.assign(p, p + (size_t)rows * cols);
  return m;
}

lkg::Parameters make_params(const double* sigma2, int is_sigma2_estim, const double* theta, int theta_rows, int d,
                            int is_theta_estim, const double* beta, int beta_n, int is_beta_estim,
                            const double* nugget, int is_nugget_estim) {
  lkg::Parameters P;
  if (sigma2) P.sigma2 = *sigma2;
  P.is_sigma2_estim = is_sigma2_estim != 0;
  if (theta && theta_rows > 0) P.theta = mat_of(theta, theta_rows, d);
  P.is_theta_estim = is_theta_estim != 0;
  if (beta && beta_n > 0) P.beta = std::vector<double>(beta, beta + beta_n);
  P.is_beta_estim = is_beta_estim != 0;
  if (nugget) P.nugget = *nugget;
  P.is_nugget_estim = is_nugget_estim != 0;
  return P;
}

int copy_vec(const std::vector<double>& v, double* out, int* n) {
  if (n) *n = (int)v.size();
  if (out) std::memcpy(out, v.data(), sizeof(double) * v.size());
  return 0;
}

}  // namespace

extern "C" {

const char* lkg_get_last_error(void) { return g_last_error.c_str(); }

void* lkg_kriging_new(const char* kernel, const char* noise_model) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    return new Kriging(kernel ? kernel : "matern3_2", parse_noise_model(noise_model));
  });
}

void* lkg_kriging_new_fit(const double* y, int n, const double* noise, int noise_n, const double* X, int nX, int d,
                          const char* kernel, const char* noise_model, const char* regmodel, int normalize,
                          const char* optim, const char* objective, const double* sigma2, int is_sigma2_estim,
                          const double* theta, int theta_n, int is_theta_estim, const double* beta, int beta_n,
                          int is_beta_estim, const double* nugget, int is_nugget_estim) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    if (noise && noise_n > 0) throw std::invalid_argument("per-observation noise is not supported by the GPU build");
    if (n != nX) throw std::runtime_error("Dimension of new data should be the same");
    std::unique_ptr<Kriging> kr(new Kriging(kernel ? kernel : "matern3_2", parse_noise_model(noise_model)));
    // theta: one starting point (1 x theta_n), as in the reference C ABI
    lkg::Parameters P = make_params(sigma2, is_sigma2_estim, theta, (theta && theta_n > 0) ? 1 : 0, theta_n,
                                    is_theta_estim, beta, beta_n, is_beta_estim, nugget, is_nugget_estim);
    std::vector<double> yv(y, y + n);
    kr->fit(yv, mat_of(X, nX, d), lkg::regmodel_from_string(regmodel ? regmodel : "constant"), normalize != 0,
            optim ? optim : "BFGS", objective ? objective : "LL", P);
    return kr.release();  // a failed fit frees the model on the way out
  });
}

void lkg_kriging_delete(void* ptr) { delete static_cast<Kriging*>(ptr); }

int lkg_kriging_fit(void* ptr, const double* y, int n, const double* noise, int noise_n, const double* X, int nX,
                    int d, const char* regmodel, int normalize, const char* optim, const char* objective) {
  return run_entry<int>(-1, [&]() -> int {
    if (noise && noise_n > 0) throw std::invalid_argument("per-observation noise is not supported by the GPU build");
    if (n != nX) throw std::runtime_error("Dimension of new data should be the same");
    std::vector<double> yv(y, y + n);
    K(ptr)->fit(yv, mat_of(X, nX, d), lkg::regmodel_from_string(regmodel ? regmodel : "constant"), normalize != 0,
                optim ? optim : "BFGS", objective ? objective : "LL", {});
    return 0;
  });
}

int lkg_kriging_fit_params(void* ptr, const double* y, int n, const double* X, int nX, int d, const char* regmodel,
                           int normalize, const char* optim, const char* objective, const double* sigma2,
                           int is_sigma2_estim, const double* theta, int theta_rows, int is_theta_estim,
                           const double* beta, int beta_n, int is_beta_estim, const double* nugget,
                           int is_nugget_estim) {
  return run_entry<int>(-1, [&]() -> int {
    if (n != nX) throw std::runtime_error("Dimension of new data should be the same");
    lkg::Parameters P = make_params(sigma2, is_sigma2_estim, theta, theta_rows, d, is_theta_estim, beta, beta_n,
                                    is_beta_estim, nugget, is_nugget_estim);
    std::vector<double> yv(y, y + n);
    K(ptr)->fit(yv, mat_of(X, nX, d), lkg::regmodel_from_string(regmodel ? regmodel : "constant"), normalize != 0,
                optim ? optim : "BFGS", objective ? objective : "LL", P);
    return 0;
  });
}

int lkg_kriging_predict(void* ptr, const double* X_n, int m, int d, int return_stdev, int return_cov,
                        int return_deriv, double* mean_out, double* stdev_out, double* cov_out, double* mean_deriv_out,
                        double* stdev_deriv_out) {
  return run_entry<int>(-1, [&]() -> int {
    auto [mean, sd, cov, md, sdd] = K(ptr)->predict(mat_of(X_n, m, d), return_stdev != 0, return_cov != 0,
                                                    return_deriv != 0);
    if (mean_out) std::memcpy(mean_out, mean.data(), sizeof(double) * mean.size());
    if (stdev_out && return_stdev) std::memcpy(stdev_out, sd.data(), sizeof(double) * sd.size());
    if (cov_out && return_cov) std::memcpy(cov_out, cov.v.data(), sizeof(double) * cov.v.size());
    if (mean_deriv_out && return_deriv) std::memcpy(mean_deriv_out, md.v.data(), sizeof(double) * md.v.size());
    if (stdev_deriv_out && return_deriv) std::memcpy(stdev_deriv_out, sdd.v.data(), sizeof(double) * sdd.v.size());
    return 0;
  });
}

int lkg_kriging_predict_vecchia(void* ptr, const double* X_n, int q, int d, int return_stdev, int m,
                                double* mean_out, double* stdev_out) {
  return run_entry<int>(-1, [&]() -> int {
    auto [mean, sd] = K(ptr)->predictVecchia(mat_of(X_n, q, d), return_stdev != 0, m);
    if (mean_out) std::memcpy(mean_out, mean.data(), sizeof(double) * mean.size());
    if (stdev_out && return_stdev) std::memcpy(stdev_out, sd.data(), sizeof(double) * sd.size());
    return 0;
  });
}

void* lkg_kriging_copy(void* ptr) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    return K(ptr)->copy().release();
  });
}

int lkg_kriging_update(void* ptr, const double* y_u, int n, const double* noise_u, int noise_n, const double* X_u,
                       int nX, int d, int refit) {
  return run_entry<int>(-1, [&]() -> int {
    if (noise_u && noise_n > 0) throw std::runtime_error("update(y, noise, X) requires NoiseModel::Heterogeneous");
    std::vector<double> yv(y_u, y_u + n);
    K(ptr)->update(yv, mat_of(X_u, nX, d), refit != 0);
    return 0;
  });
}

int lkg_kriging_save(void* ptr, const char* filename) {
  return run_entry<int>(-1, [&]() -> int {
    if (!filename) throw std::invalid_argument("save: null filename");
    K(ptr)->save(filename);
    return 0;
  });
}

void* lkg_kriging_load(const char* filename) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    if (!filename) throw std::invalid_argument("load: null filename");
    return Kriging::load(filename).release();
  });
}

int lkg_kriging_cov_mat(void* ptr, const double* X1, int n1, int d1, const double* X2, int n2, int d2,
                        double* cov_out) {
  return run_entry<int>(-1, [&]() -> int {
    Mat R = K(ptr)->covMat(mat_of(X1, n1, d1), mat_of(X2, n2, d2));
    if (cov_out) std::memcpy(cov_out, R.v.data(), sizeof(double) * R.v.size());
    return 0;
  });
}

const char* lkg_kriging_summary(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    static thread_local std::string buf;
    buf = K(ptr)->summary();
    return buf.c_str();
  });
}

int lkg_kriging_log_likelihood_fun(void* ptr, const double* theta, int theta_n, int return_grad, int return_hess,
                                   double* ll_out, double* grad_out, double* hess_out) {
  return run_entry<int>(-1, [&]() -> int {
    (void)hess_out;
    if (return_hess) throw std::invalid_argument("logLikelihoodFun: return_hess is not supported by the GPU build");
    std::vector<double> g(theta, theta + theta_n);
    auto [ll, grad] = K(ptr)->logLikelihoodFun(g, return_grad != 0, false);
    if (ll_out) *ll_out = ll;
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    return 0;
  });
}

static void write_bench(const Kriging* k, char* bench_out, int bench_cap) {
  if (!bench_out || bench_cap <= 0) return;
  std::ostringstream o;
  o.precision(17);
  for (auto& kv : k->last_bench()) o << kv.first << "\t" << kv.second << "\n";
  const std::string s = o.str();
  std::strncpy(bench_out, s.c_str(), bench_cap - 1);
  bench_out[bench_cap - 1] = 0;
}

int lkg_kriging_log_likelihood_fun_bench(void* ptr, const double* theta, int theta_n, int return_grad, double* ll_out,
                                         double* grad_out, char* bench_out, int bench_cap) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> g(theta, theta + theta_n);
    auto [ll, grad] = K(ptr)->logLikelihoodFun(g, return_grad != 0, true);
    if (ll_out) *ll_out = ll;
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    write_bench(K(ptr), bench_out, bench_cap);
    return 0;
  });
}

int lkg_kriging_log_likelihood_fun_batch_bench(void* ptr, const double* thetas, int k, int theta_n, int return_grad,
                                               double* ll_out, double* grad_out, char* bench_out, int bench_cap) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> ll, grad;
    K(ptr)->logLikelihoodFunBatch(mat_of(thetas, k, theta_n), return_grad != 0, ll, grad, bench_out != nullptr);
    if (ll_out) std::memcpy(ll_out, ll.data(), sizeof(double) * k);
    if (grad_out && return_grad)
      for (int b = 0; b < k; ++b)
        for (int j = 0; j < theta_n; ++j) grad_out[b + (size_t)j * k] = grad[(size_t)b * theta_n + j];
    write_bench(K(ptr), bench_out, bench_cap);
    return 0;
  });
}

int lkg_kriging_log_likelihood_fun_batch(void* ptr, const double* thetas, int k, int theta_n, int return_grad,
                                         double* ll_out, double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> ll, grad;
    K(ptr)->logLikelihoodFunBatch(mat_of(thetas, k, theta_n), return_grad != 0, ll, grad);
    if (ll_out) std::memcpy(ll_out, ll.data(), sizeof(double) * k);
    if (grad_out && return_grad)  // grad is row-major per candidate -> column-major k x theta_n
      for (int b = 0; b < k; ++b)
        for (int j = 0; j < theta_n; ++j) grad_out[b + (size_t)j * k] = grad[(size_t)b * theta_n + j];
    return 0;
  });
}

double lkg_kriging_log_likelihood(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->logLikelihood();
  });
}

int lkg_kriging_leave_one_out_fun(void* ptr, const double* theta, int theta_n, int return_grad, double* loo_out,
                                  double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> t(theta, theta + theta_n);
    auto [loo, grad] = K(ptr)->leaveOneOutFun(t, return_grad != 0);
    if (loo_out) *loo_out = loo;
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    return 0;
  });
}

double lkg_kriging_leave_one_out(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->leaveOneOut();
  });
}

int lkg_kriging_leave_one_out_vec(void* ptr, const double* theta, int theta_n, double* yhat_out, double* stderr_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> t(theta, theta + theta_n);
    auto [yhat, sd] = K(ptr)->leaveOneOutVec(t);
    if (yhat_out) std::memcpy(yhat_out, yhat.data(), sizeof(double) * yhat.size());
    if (stderr_out) std::memcpy(stderr_out, sd.data(), sizeof(double) * sd.size());
    return 0;
  });
}

int lkg_kriging_log_marg_post_fun(void* ptr, const double* theta, int theta_n, int return_grad, double* lmp_out,
                                  double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> t(theta, theta + theta_n);
    auto [lmp, grad] = K(ptr)->logMargPostFun(t, return_grad != 0);
    if (lmp_out) *lmp_out = lmp;
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    return 0;
  });
}

double lkg_kriging_log_marg_post(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->logMargPost();
  });
}

const char* lkg_kriging_kernel(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return K(ptr)->kernel().c_str();
  });
}
const char* lkg_kriging_optim(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return K(ptr)->optim().c_str();
  });
}
const char* lkg_kriging_objective(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return K(ptr)->objective().c_str();
  });
}
int lkg_kriging_is_normalize(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_normalize() ? 1 : 0;
  });
}
const char* lkg_kriging_regmodel(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return lkg::regmodel_to_string(K(ptr)->regmodel());
  });
}
int lkg_kriging_get_X(void* ptr, double* out, int* n, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    Kriging* k = K(ptr);
    if (n) *n = k->n();
    if (d) *d = k->d();
    if (out) {  // original scale (m_X * scaleX + centerX), as the reference getter returns m_X un-normalised
      for (int j = 0; j < k->d(); ++j)
        for (int i = 0; i < k->n(); ++i)
          out[i + (size_t)j * k->n()] = k->X()[i + (size_t)j * k->n()] * k->scaleX()[j] + k->centerX()[j];
    }
    return 0;
  });
}
int lkg_kriging_get_centerX(void* ptr, double* out, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(K(ptr)->centerX(), out, d);
  });
}
int lkg_kriging_get_scaleX(void* ptr, double* out, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(K(ptr)->scaleX(), out, d);
  });
}
int lkg_kriging_get_y(void* ptr, double* out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    Kriging* k = K(ptr);
    if (n) *n = k->n();
    if (out)
      for (int i = 0; i < k->n(); ++i) out[i] = k->y()[i] * k->scaleY() + k->centerY();
    return 0;
  });
}
double lkg_kriging_get_centerY(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->centerY();
  });
}
double lkg_kriging_get_scaleY(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->scaleY();
  });
}
int lkg_kriging_get_F(void* ptr, double* out, int* n, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    Kriging* k = K(ptr);
    if (n) *n = k->n();
    if (d) *d = k->p();
    if (out) std::memcpy(out, k->F().data(), sizeof(double) * k->F().size());
    return 0;
  });
}

int lkg_kriging_get_T(void* ptr, double* out, int* n, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    Mat T = K(ptr)->T();
    if (n) *n = T.rows;
    if (d) *d = T.cols;
    if (out) std::memcpy(out, T.v.data(), sizeof(double) * T.v.size());
    return 0;
  });
}
int lkg_kriging_get_M(void* ptr, double* out, int* n, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    Mat M = K(ptr)->M();
    if (n) *n = M.rows;
    if (d) *d = M.cols;
    if (out) std::memcpy(out, M.v.data(), sizeof(double) * M.v.size());
    return 0;
  });
}
int lkg_kriging_get_z(void* ptr, double* out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(K(ptr)->z(), out, n);
  });
}
int lkg_kriging_get_beta(void* ptr, double* out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(K(ptr)->beta(), out, n);
  });
}
int lkg_kriging_is_beta_estim(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_beta_estim() ? 1 : 0;
  });
}
int lkg_kriging_get_theta(void* ptr, double* out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(K(ptr)->theta(), out, n);
  });
}
int lkg_kriging_is_theta_estim(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_theta_estim() ? 1 : 0;
  });
}
double lkg_kriging_get_sigma2(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->sigma2();
  });
}
int lkg_kriging_is_sigma2_estim(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_sigma2_estim() ? 1 : 0;
  });
}
const char* lkg_kriging_noise_model(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return K(ptr)->noise_model() == Kriging::NoiseModel::Nugget ? "nugget" : "none";
  });
}
double lkg_kriging_get_nugget(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return K(ptr)->nugget();
  });
}
int lkg_kriging_is_nugget_estim(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_nugget_estim() ? 1 : 0;
  });
}

void lkg_set_num_nugget(double nugget) { lkg::config().num_nugget = nugget; }
double lkg_get_num_nugget(void) { return lkg::config().num_nugget; }
void lkg_check_chol_rcond(int check) { lkg::config().chol_rcond_check = check != 0; }
void lkg_set_chol_warning(int warn) { lkg::config().warn_chol = warn != 0; }
void lkg_optim_use_reparametrize(int r) { lkg::config().reparametrize = r != 0; }
void lkg_optim_set_theta_lower_factor(double f) { lkg::config().theta_lower_factor = f; }
void lkg_optim_set_theta_upper_factor(double f) { lkg::config().theta_upper_factor = f; }
void lkg_optim_use_variogram_bounds_heuristic(int v) { lkg::config().variogram_bounds_heuristic = v != 0; }
void lkg_optim_set_log_level(int l) { lkg::config().log_level = l; }
void lkg_optim_set_max_iteration(int m) { lkg::config().max_iteration = m; }
void lkg_optim_set_gradient_tolerance(double t) { lkg::config().gradient_tolerance = t; }
void lkg_optim_set_objective_rel_tolerance(double t) { lkg::config().objective_rel_tolerance = t; }
void lkg_optim_set_max_restart(int m) { lkg::config().max_restart = m; }

}  // extern "C"

// ---- mixed precision (no counterpart in the reference) ----
extern "C" {

int lkg_kriging_set_precision(void* ptr, int slices) {
  return run_entry<int>(-1, [&]() -> int {
    K(ptr)->set_precision(slices);
    return 0;
  });
}

int lkg_kriging_get_precision(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->precision();
  });
}

int lkg_kriging_last_slices(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->last_slices();
  });
}

int lkg_kriging_autotune_precision(void* ptr, const double* gamma, int gamma_n, double tol_ll, double tol_grad) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->autotune_precision(std::vector<double>(gamma, gamma + gamma_n), tol_ll, tol_grad);
  });
}

int lkg_kriging_autotune_lookahead(void* ptr, const double* gamma, int gamma_n) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->autotune_lookahead(std::vector<double>(gamma, gamma + gamma_n));
  });
}

int lkg_kriging_eval_counts(void* ptr, long long* evaluations, long long* rounds) {
  return run_entry<int>(-1, [&]() -> int {
    const Kriging* k = K(ptr);
    if (evaluations) *evaluations = k->evaluations();
    if (rounds) *rounds = k->rounds();
    return 0;
  });
}

}  // extern "C"

// ---- Vecchia (C++ API of the reference: Kriging.hpp:145-173; its C ABI has no Vecchia entry points) ----
extern "C" {

int lkg_kriging_log_likelihood_vecchia_fun(void* ptr, const double* theta, int theta_n, int return_grad,
                                           double* vll_out, double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> t(theta, theta + theta_n);
    auto [vll, grad] = K(ptr)->logLikelihoodVecchiaFun(t, return_grad != 0);
    if (vll_out) *vll_out = vll;
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    return 0;
  });
}

int lkg_kriging_set_vecchia_exact_commit(void* ptr, int b) {
  return run_entry<int>(-1, [&]() -> int {
    K(ptr)->set_vecchia_exact_commit(b != 0);
    return 0;
  });
}

int lkg_kriging_vecchia_neighbors(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->vecchia_neighbors();
  });
}

int lkg_kriging_is_vecchia_light(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return K(ptr)->is_vecchia_light() ? 1 : 0;
  });
}

int lkg_kriging_get_vecchia_sets(void* ptr, int* order_out, int* nbr_out, int* n, int* m) {
  return run_entry<int>(-1, [&]() -> int {
    const auto& o = K(ptr)->vecchia_order();
    const auto& nb = K(ptr)->vecchia_nbr();
    const int nn = (int)o.size();
    const int mm = nn > 0 ? (int)(nb.size() / nn) : 0;
    if (n) *n = nn;
    if (m) *m = mm;
    if (order_out) std::memcpy(order_out, o.data(), sizeof(int) * o.size());
    if (nbr_out) std::memcpy(nbr_out, nb.data(), sizeof(int) * nb.size());
    return 0;
  });
}

int lkg_vecchia_sets(int n, int d, const double* X, int m, int* order_out, int* nbr_out) {
  return run_entry<int>(-1, [&]() -> int {
    if (n < 1 || d < 1 || m < 0) throw std::invalid_argument("lkg_vecchia_sets: bad sizes");
    lkg::vecchia_sets_gpu(n, d, X, m, order_out, nbr_out);
    return 0;
  });
}

void* lkg_vecchia_shard_new(const char* kernel, int n, int d, int p, const double* X, const double* y,
                            const double* F, const int* order, const int* nbr, int m, int t0, int t1) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    if (n < 1 || d < 1 || p < 0 || m < 0) throw std::invalid_argument("lkg_vecchia_shard_new: bad sizes");
    std::unique_ptr<lkg::VecchiaEngine> e(new lkg::VecchiaEngine(lkg::kernel_from_name(kernel ? kernel : ""), n, d, p,
                                                                 X, y, F, order, nbr, m));
    e->set_range(t0, t1);
    return e.release();
  });
}

void lkg_vecchia_shard_delete(void* h) { delete static_cast<lkg::VecchiaEngine*>(h); }

int lkg_vecchia_shard_sums1(void* h, const double* theta, int with_grad, double* s1_out, long long* nugget_points,
                            int* failed_points) {
  return run_entry<int>(-1, [&]() -> int {
    if (!h) throw std::invalid_argument("null Vecchia shard handle");
    auto* e = static_cast<lkg::VecchiaEngine*>(h);
    std::vector<double> s1;
    long long np = 0;
    const int failed = e->partial_sums1(theta, with_grad != 0, s1, &np);
    std::memcpy(s1_out, s1.data(), sizeof(double) * s1.size());
    if (nugget_points) *nugget_points = np;
    if (failed_points) *failed_points = failed;
    return 0;
  });
}

int lkg_vecchia_shard_sums2(void* h, const double* beta, int with_grad, double* s2_out) {
  return run_entry<int>(-1, [&]() -> int {
    if (!h) throw std::invalid_argument("null Vecchia shard handle");
    std::vector<double> s2;
    static_cast<lkg::VecchiaEngine*>(h)->partial_sums2(beta, with_grad != 0, s2);
    std::memcpy(s2_out, s2.data(), sizeof(double) * s2.size());
    return 0;
  });
}

int lkg_vecchia_gls_beta(int p, const double* s1, double* beta_out) {
  return run_entry<int>(-1, [&]() -> int {
    std::vector<double> v(s1, s1 + p * p + p + 1), beta;
    if (lkg::vecchia_gls_beta(p, v, beta) != 0)
      throw std::runtime_error("solve(): GLS system of the Vecchia likelihood is not positive definite");
    std::memcpy(beta_out, beta.data(), sizeof(double) * p);
    return 0;
  });
}

int lkg_vecchia_finish(int n, int d, double slogv, const double* s2, int with_grad, double* vll_out,
                       double* sigma2_out, double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    lkg::VecchiaOut o;
    lkg::vecchia_finish(n, d, slogv, std::vector<double>(s2, s2 + 1 + 2 * d), with_grad != 0, o);
    if (vll_out) *vll_out = o.vll;
    if (sigma2_out) *sigma2_out = o.sigma2;
    if (grad_out && with_grad) std::memcpy(grad_out, o.grad.data(), sizeof(double) * d);
    return 0;
  });
}

int lkg_vecchia_sets_noalloc(int n, int d, const double* X, int m, int* order, int* nbr, void* stream) {
  const char* err = lkg::vecchia_sets_noalloc(n, d, X, m, order, nbr, static_cast<cudaStream_t>(stream));
  if (err) {
    g_last_error = err;  // the only allocation, and only on failure
    return -1;
  }
  return 0;
}

}  // extern "C"

// ---- NestedKriging (libkriging_c.h:394-455, libkriging_c.cpp:1663-1850) ----
namespace {

lkg::NestedKriging* NK(void* p) {
  if (!p) throw std::invalid_argument("null NestedKriging handle");
  return static_cast<lkg::NestedKriging*>(p);
}

lkg::NestedKriging::Partition parse_partition(const char* s) {
  const std::string p = s ? s : "kmeans";
  if (p == "random") return lkg::NestedKriging::Partition::Random;
  if (p == "kmeans" || p.empty()) return lkg::NestedKriging::Partition::KMeans;
  throw std::invalid_argument("Unknown partition: '" + p + "'. Expected 'kmeans' or 'random'.");
}

void reject_warping(int n_warping) {
  if (n_warping > 0)
    throw std::invalid_argument("NestedKriging: WarpKriging submodels (warping) are not supported by the GPU build");
}

}  // namespace

extern "C" {

void* lkg_nested_kriging_new(const char* kernel, const char* aggregation, const char* partition, int seed) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    auto* nk = new lkg::NestedKriging(kernel ? kernel : "matern3_2");
    try {
      nk->set_aggregation(lkg::NestedKriging::aggregation_from_string(aggregation ? aggregation : "NK"));
      nk->set_partition(parse_partition(partition));
      nk->set_seed(seed);
    } catch (...) {
      delete nk;
      throw;
    }
    return nk;
  });
}

void* lkg_nested_kriging_new_fit(const double* y, int n, const double* X, int nX, int d, const char* kernel,
                                 int nb_groups, const char* aggregation, const char* partition, int seed,
                                 const char** warping, int n_warping, const char* regmodel, const char* optim,
                                 const char* objective, const double* sigma2, int is_sigma2_estim, const double* theta,
                                 int theta_n, int is_theta_estim, const double* beta, int beta_n, int is_beta_estim) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    (void)warping;
    reject_warping(n_warping);
    auto* nk = new lkg::NestedKriging(kernel ? kernel : "matern3_2");
    try {
      nk->set_aggregation(lkg::NestedKriging::aggregation_from_string(aggregation ? aggregation : "NK"));
      nk->set_partition(parse_partition(partition));
      nk->set_seed(seed);
      std::vector<double> yv(y, y + n);
      nk->fit(yv, mat_of(X, nX, d), nb_groups, lkg::regmodel_from_string(regmodel ? regmodel : "constant"),
              optim ? optim : "BFGS", objective ? objective : "LL",
              make_params(sigma2, is_sigma2_estim, theta, (theta && theta_n > 0) ? 1 : 0, theta_n, is_theta_estim,
                          beta, beta_n, is_beta_estim, nullptr, 1));
    } catch (...) {
      delete nk;
      throw;
    }
    return nk;
  });
}

void lkg_nested_kriging_delete(void* ptr) { delete static_cast<lkg::NestedKriging*>(ptr); }

int lkg_nested_kriging_fit(void* ptr, const double* y, int n, const double* X, int nX, int d, int nb_groups,
                           const char** warping, int n_warping, const char* regmodel, const char* optim,
                           const char* objective, const double* sigma2, int is_sigma2_estim, const double* theta,
                           int theta_n, int is_theta_estim, const double* beta, int beta_n, int is_beta_estim) {
  return run_entry<int>(-1, [&]() -> int {
    (void)warping;
    reject_warping(n_warping);
    std::vector<double> yv(y, y + n);
    NK(ptr)->fit(yv, mat_of(X, nX, d), nb_groups, lkg::regmodel_from_string(regmodel ? regmodel : "constant"),
                 optim ? optim : "BFGS", objective ? objective : "LL",
                 make_params(sigma2, is_sigma2_estim, theta, (theta && theta_n > 0) ? 1 : 0, theta_n, is_theta_estim,
                             beta, beta_n, is_beta_estim, nullptr, 1));
    return 0;
  });
}

int lkg_nested_kriging_fit_groups(void* ptr, const double* y, int n, const double* X, int nX, int d,
                                  const int* labels, int nb_groups, const char* regmodel, const char* optim,
                                  const char* objective, const double* sigma2, int is_sigma2_estim,
                                  const double* theta, int theta_n, int is_theta_estim, const double* beta,
                                  int beta_n, int is_beta_estim) {
  return run_entry<int>(-1, [&]() -> int {
    if (!labels || nb_groups < 1) throw std::invalid_argument("fit_groups: labels and nb_groups >= 1 required");
    std::vector<std::vector<int>> groups(nb_groups);
    for (int i = 0; i < nX; ++i) {
      if (labels[i] < 0 || labels[i] >= nb_groups)
        throw std::invalid_argument("fit_groups: labels must lie in [0, nb_groups)");
      groups[labels[i]].push_back(i);
    }
    std::vector<double> yv(y, y + n);
    NK(ptr)->fit_groups(yv, mat_of(X, nX, d), groups, lkg::regmodel_from_string(regmodel ? regmodel : "constant"),
                        optim ? optim : "BFGS", objective ? objective : "LL",
                        make_params(sigma2, is_sigma2_estim, theta, (theta && theta_n > 0) ? 1 : 0, theta_n,
                                    is_theta_estim, beta, beta_n, is_beta_estim, nullptr, 1));
    return 0;
  });
}

int lkg_nested_kriging_predict(void* ptr, const double* X_n, int m, int d, int return_stdev, double* mean_out,
                               double* stdev_out) {
  return run_entry<int>(-1, [&]() -> int {
    auto [mean, sd] = NK(ptr)->predict(mat_of(X_n, m, d), return_stdev != 0);
    if (mean_out) std::memcpy(mean_out, mean.data(), sizeof(double) * mean.size());
    if (stdev_out && return_stdev) std::memcpy(stdev_out, sd.data(), sizeof(double) * sd.size());
    return 0;
  });
}

const char* lkg_nested_kriging_summary(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    static thread_local std::string buf;
    buf = NK(ptr)->summary();
    return buf.c_str();
  });
}

const char* lkg_nested_kriging_kernel(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    return NK(ptr)->kernel().c_str();
  });
}

const char* lkg_nested_kriging_aggregation(void* ptr) {
  return run_entry<const char*>(nullptr, [&]() -> const char* {
    static thread_local std::string buf;
    buf = lkg::NestedKriging::aggregation_to_string(NK(ptr)->aggregation());
    return buf.c_str();
  });
}

int lkg_nested_kriging_nb_groups(void* ptr) {
  return run_entry<int>(-1, [&]() -> int {
    return NK(ptr)->nb_groups();
  });
}

int lkg_nested_kriging_get_theta(void* ptr, double* out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    return copy_vec(NK(ptr)->theta(), out, n);
  });
}

double lkg_nested_kriging_get_sigma2(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return NK(ptr)->sigma2();
  });
}

double lkg_nested_kriging_get_beta0(void* ptr) {
  return run_entry<double>(std::numeric_limits<double>::quiet_NaN(), [&]() -> double {
    return NK(ptr)->beta0();
  });
}

int lkg_nested_kriging_get_groups(void* ptr, int* labels_out, int* n) {
  return run_entry<int>(-1, [&]() -> int {
    const auto& G = NK(ptr)->groups();
    int total = 0;
    for (const auto& g : G) total += (int)g.size();
    if (n) *n = total;
    if (labels_out)
      for (size_t k = 0; k < G.size(); ++k)
        for (int i : G[k]) labels_out[i] = (int)k;
    return 0;
  });
}

void* lkg_nested_kriging_submodel(void* ptr, int i) {
  return run_entry<void*>(nullptr, [&]() -> void* {
    return &NK(ptr)->submodel(i);
  });
}

int lkg_nested_kriging_set_precision(void* ptr, int slices) {
  return run_entry<int>(-1, [&]() -> int {
    NK(ptr)->set_precision(slices);
    return 0;
  });
}

int lkg_nested_kriging_log_likelihood_groups(void* ptr, const double* thetas, int p, int d, int return_grad,
                                             double* ll_out, double* grad_out) {
  return run_entry<int>(-1, [&]() -> int {
    lkg::Mat T;
    T.rows = p;
    T.cols = d;
    T.v.resize((size_t)p * d);
    for (int g = 0; g < p; ++g)
      for (int k = 0; k < d; ++k) T(g, k) = thetas[(size_t)g * d + k];
    std::vector<double> ll, grad;
    NK(ptr)->log_likelihood_groups(T, return_grad != 0, ll, grad);
    if (ll_out) std::memcpy(ll_out, ll.data(), sizeof(double) * ll.size());
    if (grad_out && return_grad) std::memcpy(grad_out, grad.data(), sizeof(double) * grad.size());
    return 0;
  });
}

int lkg_nested_kriging_get_group_estimates(void* ptr, double* theta_out, double* sigma2_out, double* beta0_out,
                                           int* p, int* d) {
  return run_entry<int>(-1, [&]() -> int {
    auto* nk = NK(ptr);
    const auto& th = nk->group_theta();
    const int np = (int)nk->group_sigma2().size();
    if (p) *p = np;
    if (d) *d = np > 0 ? (int)(th.size() / np) : 0;
    if (theta_out && !th.empty()) std::memcpy(theta_out, th.data(), sizeof(double) * th.size());
    if (sigma2_out && np) std::memcpy(sigma2_out, nk->group_sigma2().data(), sizeof(double) * np);
    if (beta0_out && np) std::memcpy(beta0_out, nk->group_beta0().data(), sizeof(double) * np);
    return 0;
  });
}

int lkg_nested_kriging_set_predict_chunk(void* ptr, int chunk) {
  return run_entry<int>(-1, [&]() -> int {
    NK(ptr)->set_predict_chunk(chunk);
    return 0;
  });
}

}  // extern "C"
