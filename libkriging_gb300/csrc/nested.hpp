// nested.hpp -- NestedKriging with libKriging's API (src/lib/include/libKriging/NestedKriging.hpp).
//
//   NestedKriging(covType)                                      NestedKriging.hpp:63
//   fit(y, X, nb_groups, regmodel, optim, objective, params)    NestedKriging.hpp:94-101, NestedKriging.cpp:171-281
//   predict(X_n, return_stdev) -> (mean, stdev)                 NestedKriging.hpp:105, NestedKriging.cpp:351-498
//   aggregations PoE / gPoE / BCM / rBCM / NK, partitions KMeans / Random (NestedKriging.cpp:124-165)
// The submodel fits run concurrently: every submodel's optimiser lives in its own host thread and each round of
// objective evaluations goes to the GPU as one batched launch sequence per size class (groups padded to a
// multiple of 64 points with the identity).  The plain (Kriging submodels) and LLVecchia-unified paths are
// provided; WarpKriging submodels are not part of this library.
#pragma once
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "kriging.hpp"

namespace lkg {

class NestedService;

class NestedKriging {
 public:
  enum class Aggregation { PoE, gPoE, BCM, rBCM, NK };
  enum class Partition { Random, KMeans };
  static Aggregation aggregation_from_string(const std::string& s);
  static std::string aggregation_to_string(Aggregation a);

  explicit NestedKriging(const std::string& covType);
  ~NestedKriging();

  void set_aggregation(Aggregation a) { m_aggregation = a; }
  void set_partition(Partition p) { m_partition = p; }
  void set_seed(int s) { m_seed = s; }
  void set_predict_chunk(int c);
  // digit slices of the submodel objective evaluations: 0 = FP64 (default), 4..8 = mixed path
  void set_precision(int slices);

  void fit(const std::vector<double>& y, const Mat& X, int nb_groups,
           RegressionModel regmodel = RegressionModel::Constant, const std::string& optim = "BFGS",
           const std::string& objective = "LL", const Parameters& parameters = {});
  // the same with the partition given (row indices; every row in exactly one group, groups of >= d + 2 rows)
  void fit_groups(const std::vector<double>& y, const Mat& X, const std::vector<std::vector<int>>& groups,
                  RegressionModel regmodel = RegressionModel::Constant, const std::string& optim = "BFGS",
                  const std::string& objective = "LL", const Parameters& parameters = {});

  std::tuple<std::vector<double>, std::vector<double>> predict(const Mat& X_n, bool return_stdev);

  // The submodel fit objective of every group in one batched evaluation: the concentrated log-likelihood
  // (sigma2 = SSE / n_g, GLS trend) of group g at theta row g (thetas p x d), and its theta-gradient (p x d,
  // row-major) when return_grad.  No counterpart in the reference (there each submodel's logLikelihoodFun runs
  // alone); available after a fit on the plain path.
  void log_likelihood_groups(const Mat& thetas, bool return_grad, std::vector<double>& ll,
                             std::vector<double>& grad);

  const std::string& kernel() const { return m_covType; }
  Aggregation aggregation() const { return m_aggregation; }
  Partition partition() const { return m_partition; }
  int seed() const { return m_seed; }
  int nb_groups() const { return (int)m_groups.size(); }
  const std::vector<std::vector<int>>& groups() const { return m_groups; }
  Kriging& submodel(int i);
  const std::vector<double>& theta() const { return m_theta; }
  double sigma2() const { return m_sigma2; }
  double beta0() const { return m_beta0; }
  const Mat& X() const { return m_X; }
  const std::vector<double>& y() const { return m_y; }
  int predict_chunk() const { return m_chunk; }
  // the submodel estimates before the common prior replaced them (plain path): theta p x d (row g = group g),
  // sigma2 and beta0 per group -- the inputs of unify_hyperparameters, for a fit whose groups are sharded
  const std::vector<double>& group_theta() const { return m_gtheta; }
  const std::vector<double>& group_sigma2() const { return m_gsigma2; }
  const std::vector<double>& group_beta0() const { return m_gbeta0; }
  bool is_fitted() const { return m_is_fitted; }
  std::string summary() const;

 private:
  void make_partition(int nb_groups);
  void fit_partitioned(RegressionModel regmodel, const std::string& optim, const std::string& objective,
                       const Parameters& parameters);
  void unify_hyperparameters(const std::string& objective);
  void precompute_nk();
  std::tuple<std::vector<double>, std::vector<double>> predict_poe_family(const Mat& X_n, bool return_stdev);
  std::tuple<std::vector<double>, std::vector<double>> predict_nk(const Mat& X_n, bool return_stdev);
  Mat group_rows(const Mat& A, const std::vector<int>& idx) const;

  std::string m_covType;
  int m_kernel;
  Aggregation m_aggregation = Aggregation::NK;
  Partition m_partition = Partition::KMeans;
  int m_seed = 123;
  int m_chunk = 128;
  int m_slices = 0;
  Mat m_X;
  std::vector<double> m_y;
  RegressionModel m_regmodel = RegressionModel::Constant;
  std::vector<std::vector<int>> m_groups;
  std::vector<std::unique_ptr<Kriging>> m_submodels;
  std::vector<double> m_theta;
  double m_sigma2 = -1.0;
  double m_beta0 = 0.0;
  bool m_is_fitted = false;
  // NK precomputations: per size class, one engine holding L_g of R_g + jitter I for each of its groups
  struct NkClass;
  std::vector<std::unique_ptr<NkClass>> m_nk;
  // batched submodel evaluations of the last plain-path fit (kept for log_likelihood_groups)
  std::unique_ptr<NestedService> m_service;
  std::vector<int> m_group_n;
  std::vector<double> m_gtheta, m_gsigma2, m_gbeta0;
};

}  // namespace lkg
