// kriging.hpp -- GPU-backed Kriging facade with libKriging's Kriging API (src/lib/include/libKriging/Kriging.hpp).
//
// Same method names, argument meaning, defaults and error behaviour as the reference for the likelihood path:
//   Kriging(covType, NoiseModel)                         Kriging.hpp:78-79
//   fit(y, X, regmodel, normalize, optim, objective, P)  Kriging.hpp:113-119, Kriging.cpp:1591-2215
//   logLikelihoodFun(gamma, return_grad, bench)          Kriging.hpp:131-133, Kriging.cpp:214-349
//   predict(X_n, return_stdev, return_cov, return_deriv) Kriging.hpp:215-218, KrigingImpl.cpp:145-300
// Matrices are column-major std::vector<double> with explicit sizes (the reference uses arma::mat).
#pragma once
#include <map>
#include <memory>
#include <optional>
#include <string>
#include <tuple>
#include <vector>

#include "engine.hpp"
#include "vecchia.hpp"

namespace lkg {

enum class RegressionModel { None = 0, Constant = 1, Linear = 2, Interactive = 3, Quadratic = 4 };
RegressionModel regmodel_from_string(const std::string& s);
const char* regmodel_to_string(RegressionModel r);
// Trend::regressionModelMatrix (src/lib/Trend.cpp:34-91): X n x d column-major -> F n x p
std::vector<double> regression_matrix(RegressionModel r, const std::vector<double>& X, int n, int d, int* p_out);

struct Mat {  // column-major matrix
  int rows = 0, cols = 0;
  std::vector<double> v;
  double& operator()(int i, int j) { return v[i + (size_t)j * rows]; }
  double operator()(int i, int j) const { return v[i + (size_t)j * rows]; }
};

struct Parameters {  // KrigingParameters (Kriging.hpp:18-28)
  std::optional<double> sigma2;
  bool is_sigma2_estim = true;
  std::optional<Mat> theta;  // rows = starting points
  bool is_theta_estim = true;
  std::optional<std::vector<double>> beta;
  bool is_beta_estim = true;
  std::optional<double> nugget;
  bool is_nugget_estim = true;
};

// Exact-objective evaluations shared by the fits of several models (the submodels of a NestedKriging): evaluate()
// blocks until the service has run this model's k requests, batched with the other models' pending requests.
class DenseService {
 public:
  virtual ~DenseService() = default;
  virtual void evaluate(int design, int k, const double* thetas, const double* factors, bool with_grad,
                        std::vector<EvalOut>& out) = 0;
};

class Kriging {
 public:
  enum class NoiseModel { None, Nugget };

  explicit Kriging(const std::string& covType, NoiseModel nm = NoiseModel::None);
  ~Kriging();

  void fit(const std::vector<double>& y, const Mat& X, RegressionModel regmodel = RegressionModel::Constant,
           bool normalize = false, const std::string& optim = "BFGS", const std::string& objective = "LL",
           const Parameters& parameters = {});

  // gamma = theta (None) or [theta, alpha] (Nugget)
  std::tuple<double, std::vector<double>> logLikelihoodFun(const std::vector<double>& gamma, bool return_grad,
                                                           bool bench);
  // Batched objective: gammas rows = candidates (k x gdim).  ll[k], grad[k x gdim] (row-major per candidate).
  // bench = true records the per-stage timings of the batched pass (last_bench()).
  void logLikelihoodFunBatch(const Mat& gammas, bool return_grad, std::vector<double>& ll,
                             std::vector<double>& grad, bool bench = false);
  double logLikelihood();

  // leave-one-out (Kriging.hpp:135-143, Kriging.cpp:353-484, 666-668): theta only; R = C, or alpha C + (1 - alpha) I
  // with the model's alpha for NoiseModel Nugget
  std::tuple<double, std::vector<double>> leaveOneOutFun(const std::vector<double>& theta, bool return_grad);
  // (y - errorsLOO, sqrt(sigma2LOO) sqrt(sigma2)) in the model's (normalised) units
  std::tuple<std::vector<double>, std::vector<double>> leaveOneOutVec(const std::vector<double>& theta);
  double leaveOneOut();
  // log marginal posterior (Kriging.hpp:137-139, Kriging.cpp:487-665): gamma = theta, or [theta, alpha] (Nugget;
  // theta alone takes the model's alpha)
  std::tuple<double, std::vector<double>> logMargPostFun(const std::vector<double>& gamma, bool return_grad);
  double logMargPost();

  // Vecchia (objective "LLVecchia" / "LLVecchia(m)"; Kriging.hpp:145-173, Kriging.cpp:718-924)
  std::tuple<double, std::vector<double>> logLikelihoodVecchiaFun(const std::vector<double>& theta, bool return_grad);
  void set_vecchia_exact_commit(bool b) { m_vecchia_exact_commit = b; }
  bool vecchia_exact_commit() const { return m_vecchia_exact_commit; }
  int vecchia_neighbors() const { return m_vecchia_m; }
  bool is_vecchia_light() const { return m_vecchia_light; }
  const std::vector<int32_t>& vecchia_order() const { return m_vorder; }
  const std::vector<int32_t>& vecchia_nbr() const { return m_vnbr; }
  static int parse_vll_m(const std::string& objective);

  // mean, stdev, cov, mean_deriv, stdev_deriv
  std::tuple<std::vector<double>, std::vector<double>, Mat, Mat, Mat> predict(const Mat& X_n, bool return_stdev,
                                                                                bool return_cov, bool return_deriv);
  // Kriging.hpp:163-173: local prediction on the m nearest observations (m = 0: vecchia_neighbors() or 30)
  std::tuple<std::vector<double>, std::vector<double>> predictVecchia(const Mat& X_n, bool return_stdev = true,
                                                                      int m = 0);

  // update (Kriging.hpp:255-257, Kriging.cpp:2433-2633): append (X_u, y_u) in the model's original units.
  //   refit and optim != "none", NoiseModel Nugget: a full fit on the joined data with the model's parameters;
  //   refit and optim != "none", NoiseModel None: one L-BFGS-B run warm-started at the current theta, bounds from
  //     the joined data, the normalisation kept;
  //   otherwise: theta kept, the factor extended by the incremental Cholesky (chol_block) on the GPU, beta and
  //     sigma2 = SSE / n re-estimated when they are estimated (KrigingImpl.cpp:576-635).
  void update(const std::vector<double>& y_u, const Mat& X_u, bool refit = true);
  // libKriging's JSON model file, version 2 (Kriging.cpp:2691-2749, KrigingImpl.cpp:644-711)
  void save(const std::string& filename) const;
  static std::unique_ptr<Kriging> load(const std::string& filename);
  // sigma2 * C(X1, X2) in the original units (KrigingImpl.cpp:60-71); X1 n1 x d, X2 n2 x d -> n1 x n2
  Mat covMat(const Mat& X1, const Mat& X2) const;
  // deep copy (Kriging(const Kriging&, ExplicitCopySpecifier)): the data, parameters and committed model
  std::unique_ptr<Kriging> copy() const;

  // accessors (KrigingImpl.hpp:40-60, Kriging.hpp:94-97)
  const std::string& kernel() const { return m_covType; }
  NoiseModel noise_model() const { return m_noise_model; }
  const std::vector<double>& theta() const { return m_theta; }
  double sigma2() const { return m_sigma2; }
  const std::vector<double>& beta() const { return m_beta; }
  double nugget() const { return m_nugget; }
  double alpha() const { return m_alpha; }
  bool is_sigma2_estim() const { return m_est_sigma2; }
  bool is_theta_estim() const { return m_est_theta; }
  bool is_beta_estim() const { return m_est_beta; }
  bool is_nugget_estim() const { return m_est_nugget; }
  bool is_normalize() const { return m_normalize; }
  const std::string& optim() const { return m_optim; }
  const std::string& objective() const { return m_objective; }
  RegressionModel regmodel() const { return m_regmodel; }
  int n() const { return m_n; }
  int d() const { return m_d; }
  int p() const { return m_p; }
  const std::vector<double>& X() const { return m_X; }
  const std::vector<double>& y() const { return m_y; }
  const std::vector<double>& F() const { return m_F; }
  const std::vector<double>& centerX() const { return m_centerX; }
  const std::vector<double>& scaleX() const { return m_scaleX; }
  double centerY() const { return m_centerY; }
  double scaleY() const { return m_scaleY; }
  // committed factor and whitened quantities (m_T, m_M, m_z, m_circ) copied to host on demand
  Mat T() const;
  Mat M() const;
  std::vector<double> z() const;
  std::string summary() const;

  // per-stage timings of the last logLikelihoodFun(..., bench=true) call (Bench keys of the reference)
  const std::map<std::string, double>& last_bench() const { return m_bench; }
  // total evaluations performed by the engine since construction (objective calls, batched entries counted once each)
  long long evaluations() const { return m_evals; }
  // GPU evaluation launches since construction: a batched round of a multistart fit counts once
  long long rounds() const { return m_rounds; }
  // 0: FP64 path (default); 4..8: mixed path with that many bf16 digit slices for the O(n^3) products of the
  // objective evaluations (logLikelihoodFun and the fit); the committed model used by predict stays FP64.
  void set_precision(int slices);
  int precision() const { return m_slices; }
  // mixed-path bookkeeping of the last logLikelihoodFun: slices used (0 = FP64, also after a retreat)
  int last_slices() const { return m_last_slices; }
  // The fastest precision (0 = FP64, or 5..7 slices of the mixed path) whose logLikelihoodFun(gamma, grad) stays
  // within tol_ll / tol_grad (relative) of the FP64 path's, measured on this model (CUDA-event timings, errors with a
  // 10x margin); tabled by the autotuner under the problem's shape and the tolerances, then set as the precision.
  int autotune_precision(const std::vector<double>& gamma, double tol_ll, double tol_grad);
  // The SMs kept for the mixed Cholesky's look-ahead at this model's size (0 = none, 12, 16, 24, 32), chosen by timing
  // logLikelihoodFun(gamma, grad) on the mixed path for each (the factor is identical for all); tabled by the
  // autotuner under the matrix size and used by every later evaluation of that size.  Returns the choice.
  int autotune_lookahead(const std::vector<double>& gamma);
  // route the fit's objective evaluations through a shared service (design = this model's index there); nullptr
  // restores the model's own engine
  void attach_service(DenseService* s, int design) {
    m_service = s;
    m_service_design = design;
  }

 private:
  double loglik_from(const EvalOut& o, double extra_param, std::vector<double>* grad, int gdim) const;
  // log marginal posterior at (theta, alpha) from an evaluate_lmp result; grad (gdim) only when sigma2 is estimated
  double lmp_from(const EvalOut& o, const double* theta, double alpha, std::vector<double>* grad, int gdim) const;
  void ensure_engine(int batch_cap);
  // fit() on data that is already normalised with the model's centre / scale, restarted from theta_warm only
  // (update's warm restart, Kriging.cpp:2467-2625): one start, no restarts, normalisation kept
  bool m_warm = false;
  void commit(const std::vector<double>& theta, double alpha);

  std::string m_covType;
  int m_kernel;
  NoiseModel m_noise_model;
  int m_n = 0, m_d = 0, m_p = 0;
  std::vector<double> m_X, m_y, m_F;  // normalised
  std::vector<double> m_centerX, m_scaleX;
  double m_centerY = 0.0, m_scaleY = 1.0;
  bool m_normalize = false;
  RegressionModel m_regmodel = RegressionModel::Constant;
  std::string m_optim = "BFGS", m_objective = "LL";
  std::vector<double> m_theta, m_beta;
  double m_sigma2 = 0.0, m_nugget = 0.0, m_alpha = 1.0;
  bool m_est_theta = false, m_est_sigma2 = false, m_est_beta = true, m_est_nugget = false;
  bool m_is_empty = true;
  std::unique_ptr<Engine> m_eval;   // objective evaluations (batch capacity grows as needed)
  std::unique_ptr<Engine> m_model;  // committed model (predict)
  std::map<std::string, double> m_bench;
  long long m_evals = 0;
  long long m_rounds = 0;
  EvalOut m_last_commit;
  int m_last_fit_starts = 0;
  int m_slices = 0;
  int m_last_slices = 0;
  DenseService* m_service = nullptr;
  int m_service_design = 0;
  // Vecchia state: maxmin order and neighbour sets (global row indices, -1 padded), GPU engine
  int m_vecchia_m = 0;
  std::vector<int32_t> m_vorder, m_vnbr;
  bool m_vecchia_exact_commit = true;
  bool m_vecchia_light = false;
  std::unique_ptr<VecchiaEngine> m_vecchia;
  void ensure_vecchia();
};

}  // namespace lkg
