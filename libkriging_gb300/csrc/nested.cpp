// nested.cpp -- NestedKriging (nested.hpp): partition, batched submodel fits, common prior, PoE-family and NK
// aggregation (src/lib/NestedKriging.cpp of libKriging).
#include "nested.hpp"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdlib>
#include <cmath>
#include <condition_variable>
#include <exception>
#include <limits>
#include <mutex>
#include <random>
#include <sstream>
#include <stdexcept>
#include <thread>

#include "common.cuh"
#include "dense_fp64.cuh"
#include "nested_kernels.cuh"

namespace lkg {

namespace {

constexpr double kJitter = 1e-10;   // NestedKriging.hpp: jitter of the NK factorisations and of K_M
constexpr double kTiny = 1e-12;     // NestedKriging.cpp:366 (predict_poe_family)
constexpr int kClassGrain = 64;     // size classes: groups padded to a multiple of 64 points
constexpr int kMaxFitThreads = 1024;

int class_size(int n) { return ceil_div(n, kClassGrain) * kClassGrain; }

int starts_of(const std::string& optim, const Parameters& P) {
  int ms = 1;
  if (optim.rfind("BFGS", 0) == 0) {
    size_t e = 4;
    while (e < optim.size() && std::isdigit((unsigned char)optim[e])) ++e;
    if (e > 4) ms = std::max(1, std::atoi(optim.substr(4, e - 4).c_str()));
  }
  if (P.theta.has_value()) ms = std::max(ms, P.theta->rows);
  return ms;
}

// run f(i) for i in [0, count) on at most `width` threads at a time; the first exception is rethrown
template <typename F>
void parallel_for(int count, int width, F f) {
  std::atomic<int> next{0};
  std::exception_ptr err;
  std::mutex emu;
  auto body = [&]() {
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= count) return;
      try {
        f(i);
      } catch (...) {
        std::lock_guard<std::mutex> g(emu);
        if (!err) err = std::current_exception();
      }
    }
  };
  std::vector<std::thread> th;
  const int w = std::max(1, std::min(width, count));
  th.reserve(w);
  for (int t = 0; t < w; ++t) th.emplace_back(body);
  for (auto& t : th) t.join();
  if (err) std::rethrow_exception(err);
}

// Uniform draw in [0, m) from a 32-bit Mersenne Twister (the partition's random choices)
uint32_t draw_below(std::mt19937& g, uint32_t m) { return g() % m; }

struct Design {
  std::vector<double> X, y, F;  // column-major, n rows
  int n = 0;
};

// padded design arrays of one size class
void pack_class(const std::vector<Design>& ds, const std::vector<int>& members, int n_pad, int d, int p,
                std::vector<double>& X, std::vector<double>& y, std::vector<double>& F, std::vector<int>& nv) {
  const size_t ne = members.size();
  X.assign(ne * n_pad * d, 0.0);
  y.assign(ne * n_pad, 0.0);
  F.assign(ne * n_pad * std::max(p, 1), 0.0);
  nv.assign(ne, 0);
  for (size_t e = 0; e < ne; ++e) {
    const Design& g = ds[members[e]];
    nv[e] = g.n;
    for (int k = 0; k < d; ++k)
      std::copy(g.X.begin() + (size_t)k * g.n, g.X.begin() + (size_t)(k + 1) * g.n,
                X.begin() + e * n_pad * d + (size_t)k * n_pad);
    std::copy(g.y.begin(), g.y.end(), y.begin() + e * n_pad);
    for (int k = 0; k < p; ++k)
      std::copy(g.F.begin() + (size_t)k * g.n, g.F.begin() + (size_t)(k + 1) * g.n,
                F.begin() + e * n_pad * p + (size_t)k * n_pad);
  }
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------------
// Batched objective evaluations of the submodel fits: every round, the pending requests of all active fits are
// grouped by size class and each class runs as one batched evaluation (classes concurrently, one stream each).
class NestedService : public DenseService {
 public:
  NestedService(int kernel, int d, int p, const std::vector<Design>& ds, int starts, int slices) : d_(d) {
    const int G = (int)ds.size();
    class_of_.assign(G, -1);
    local_of_.assign(G, -1);
    std::vector<int> order(G);
    for (int g = 0; g < G; ++g) order[g] = g;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ds[a].n < ds[b].n; });
    for (int g : order) {
      const int np = class_size(ds[g].n);
      if (classes_.empty() || classes_.back().n_pad != np) classes_.push_back(Class{np, {}, nullptr, 0});
      class_of_[g] = (int)classes_.size() - 1;
      local_of_[g] = (int)classes_.back().designs.size();
      classes_.back().designs.push_back(g);
    }
    // batch capacity per class: every design x starts entries, scaled down to ~70% of the free device memory
    size_t free_b = 0, total_b = 0;
    LKG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const double per_n2 = slices > 0 ? 38.0 : 25.0;  // bytes per n^2 per entry (A, W, R^-1, digit planes)
    double need = 0.0;
    for (auto& c : classes_) need += per_n2 * (double)c.n_pad * c.n_pad * c.designs.size() * starts;
    const double scale = std::min(1.0, 0.7 * (double)free_b / std::max(need, 1.0));
    for (auto& c : classes_) {
      c.cap = std::max(1, (int)std::floor(scale * c.designs.size() * starts));
      std::vector<double> X, y, F;
      std::vector<int> nv;
      pack_class(ds, c.designs, c.n_pad, d, p, X, y, F, nv);
      c.eng = std::make_unique<Engine>(kernel, c.n_pad, d, p, (int)c.designs.size(), X.data(), y.data(), F.data(),
                                       nv.data(), c.cap);
      c.eng->set_slices(slices);
    }
  }

  void set_active(int a) {
    std::lock_guard<std::mutex> g(mu_);
    active_ = a;
  }

  // precision of the batched evaluations from now on (0: FP64, 4..8: mixed)
  void set_slices(int s) {
    for (auto& c : classes_) c.eng->set_slices(s);
  }

  void leave() {
    std::unique_lock<std::mutex> lk(mu_);
    active_--;
    maybe_run(lk);
  }

  void evaluate(int design, int k, const double* thetas, const double* factors, bool with_grad,
                std::vector<EvalOut>& out) override {
    Req r{design, k, thetas, factors, with_grad, &out};
    std::unique_lock<std::mutex> lk(mu_);
    pending_.push_back(&r);
    maybe_run(lk);
    cv_.wait(lk, [&] { return r.done; });
    lk.unlock();
    if (r.err) std::rethrow_exception(r.err);
  }

  int classes() const { return (int)classes_.size(); }

  // one entry per design (thetas: designs x d row-major), run directly without the worker barrier
  void evaluate_all(const double* thetas, bool with_grad, std::vector<EvalOut>& out) {
    const int G = (int)class_of_.size();
    std::vector<std::vector<EvalOut>> outs(G);
    std::vector<double> one(G, 1.0);
    std::vector<Req> reqs(G);
    std::vector<Req*> ptrs(G);
    for (int g = 0; g < G; ++g) {
      reqs[g] = Req{g, 1, thetas + (size_t)g * d_, &one[g], with_grad, &outs[g]};
      ptrs[g] = &reqs[g];
    }
    std::lock_guard<std::mutex> lock(run_mu_);
    run(ptrs);
    out.resize(G);
    for (int g = 0; g < G; ++g) {
      if (reqs[g].err) std::rethrow_exception(reqs[g].err);
      out[g] = std::move(outs[g][0]);
    }
  }

 private:
  struct Class {
    int n_pad;
    std::vector<int> designs;
    std::unique_ptr<Engine> eng;
    int cap;
  };
  struct Req {
    int design, k;
    const double* th;
    const double* fac;
    bool grad;
    std::vector<EvalOut>* out;
    bool done = false;
    std::exception_ptr err;
  };

  void maybe_run(std::unique_lock<std::mutex>& lk) {
    if (pending_.empty() || (int)pending_.size() < active_) return;
    std::vector<Req*> batch;
    batch.swap(pending_);
    lk.unlock();
    run(batch);
    lk.lock();
    for (auto* r : batch) r->done = true;
    cv_.notify_all();
  }

  void run(std::vector<Req*>& reqs) {
    std::vector<std::vector<Req*>> per(classes_.size());
    for (auto* r : reqs) {
      r->out->assign(r->k, EvalOut{});
      per[class_of_[r->design]].push_back(r);
    }
    std::vector<std::thread> th;
    for (size_t c = 0; c < classes_.size(); ++c) {
      if (per[c].empty()) continue;
      th.emplace_back([this, c, &per]() {
        try {
          run_class(classes_[c], per[c]);
        } catch (...) {
          for (auto* r : per[c]) r->err = std::current_exception();
        }
      });
    }
    for (auto& t : th) t.join();
  }

  void run_class(Class& c, std::vector<Req*>& reqs) {
    struct Slot {
      Req* r;
      int j;
    };
    std::vector<Slot> slots;
    bool grad = false;
    for (auto* r : reqs) {
      for (int j = 0; j < r->k; ++j) slots.push_back({r, j});
      grad = grad || r->grad;
    }
    const int d = d_;
    for (size_t s0 = 0; s0 < slots.size(); s0 += c.cap) {
      const int k = (int)std::min<size_t>(c.cap, slots.size() - s0);
      std::vector<double> th((size_t)k * d), fac(k);
      std::vector<int> des(k);
      for (int b = 0; b < k; ++b) {
        const Slot& s = slots[s0 + b];
        std::copy(s.r->th + (size_t)s.j * d, s.r->th + (size_t)(s.j + 1) * d, th.begin() + (size_t)b * d);
        fac[b] = s.r->fac[s.j];
        des[b] = local_of_[s.r->design];
      }
      std::vector<EvalOut> out;
      c.eng->evaluate(k, th.data(), fac.data(), grad, out, nullptr, des.data());
      for (int b = 0; b < k; ++b) {
        const Slot& s = slots[s0 + b];
        (*s.r->out)[s.j] = std::move(out[b]);
      }
    }
  }

  int d_;
  std::vector<Class> classes_;
  std::vector<int> class_of_, local_of_;
  std::mutex run_mu_;
  std::mutex mu_;
  std::condition_variable cv_;
  int active_ = 0;
  std::vector<Req*> pending_;
};

// ---------------------------------------------------------------------------------------------------------------
struct NestedKriging::NkClass {
  int n_pad = 0;
  std::vector<int> groups;
  std::unique_ptr<Engine> eng;
  double* dz = nullptr;  // z_e = L_e \ (y_e - beta0), n_pad per entry
  int* dnv = nullptr;    // valid sizes per entry
  ~NkClass() {
    if (dz) cudaFree(dz);
    if (dnv) cudaFree(dnv);
  }
};

NestedKriging::Aggregation NestedKriging::aggregation_from_string(const std::string& s) {
  if (s == "PoE") return Aggregation::PoE;
  if (s == "gPoE") return Aggregation::gPoE;
  if (s == "BCM") return Aggregation::BCM;
  if (s == "rBCM") return Aggregation::rBCM;
  if (s == "NK") return Aggregation::NK;
  throw std::invalid_argument("Unknown aggregation: " + s + " (expected PoE, gPoE, BCM, rBCM or NK)");
}

std::string NestedKriging::aggregation_to_string(Aggregation a) {
  switch (a) {
    case Aggregation::PoE: return "PoE";
    case Aggregation::gPoE: return "gPoE";
    case Aggregation::BCM: return "BCM";
    case Aggregation::rBCM: return "rBCM";
    case Aggregation::NK: return "NK";
  }
  return "?";
}

NestedKriging::NestedKriging(const std::string& covType) : m_covType(covType), m_kernel(kernel_from_name(covType)) {}

NestedKriging::~NestedKriging() = default;

void NestedKriging::set_predict_chunk(int c) {
  if (c < 1) throw std::invalid_argument("set_predict_chunk: chunk must be >= 1");
  m_chunk = c;
}

void NestedKriging::set_precision(int slices) {
  if (slices != 0 && (slices < 4 || slices > 8))
    throw std::invalid_argument("set_precision: slices must be 0 (FP64) or 4..8");
  m_slices = slices;
  if (m_service) m_service->set_slices(slices);  // a fitted model's batched evaluations follow the setting
}

Kriging& NestedKriging::submodel(int i) {
  if (i < 0 || i >= (int)m_submodels.size()) throw std::out_of_range("submodel: index out of range");
  return *m_submodels[i];
}

Mat NestedKriging::group_rows(const Mat& A, const std::vector<int>& idx) const {
  Mat r;
  r.rows = (int)idx.size();
  r.cols = A.cols;
  r.v.resize((size_t)r.rows * r.cols);
  for (int j = 0; j < A.cols; ++j)
    for (int i = 0; i < r.rows; ++i) r(i, j) = A(idx[i], j);
  return r;
}

// NestedKriging::make_partition (NestedKriging.cpp:124-165): k-means (random-subset seeding, 10 Lloyd iterations)
// with a balanced random split as fallback when a cluster has fewer than d + 2 points.  The random choices come
// from a 32-bit Mersenne Twister seeded with the model seed (Armadillo's generator is not reproduced).
void NestedKriging::make_partition(int nb_groups) {
  const int n = m_X.rows, d = m_X.cols;
  const int min_group_size = d + 2;
  std::mt19937 gen((uint32_t)m_seed);
  std::vector<int> assignment(n, 0);
  bool kmeans_ok = false;
  if (m_partition == Partition::KMeans && nb_groups > 1) {
    if (d > 8) throw std::invalid_argument("NestedKriging: the k-means partition supports d <= 8");
    const int k = nb_groups;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    for (int i = 0; i < k; ++i) std::swap(idx[i], idx[i + draw_below(gen, (uint32_t)(n - i))]);
    std::vector<double> C((size_t)k * d);  // k x d row-major
    for (int c = 0; c < k; ++c)
      for (int j = 0; j < d; ++j) C[(size_t)c * d + j] = m_X(idx[c], j);
    cudaStream_t st;
    LKG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    double *dX = nullptr, *dC = nullptr;
    int* dA = nullptr;
    auto cleanup = [&]() {
      if (dX) cudaFree(dX);
      if (dC) cudaFree(dC);
      if (dA) cudaFree(dA);
      cudaStreamDestroy(st);
    };
    try {
      LKG_CUDA(cudaMalloc(&dX, sizeof(double) * (size_t)n * d));
      LKG_CUDA(cudaMalloc(&dC, sizeof(double) * (size_t)k * d));
      LKG_CUDA(cudaMalloc(&dA, sizeof(int) * (size_t)n));
      LKG_CUDA(cudaMemcpyAsync(dX, m_X.v.data(), sizeof(double) * (size_t)n * d, cudaMemcpyHostToDevice, st));
      auto assign = [&]() {
        LKG_CUDA(cudaMemcpyAsync(dC, C.data(), sizeof(double) * (size_t)k * d, cudaMemcpyHostToDevice, st));
        kmeans_assign(n, d, dX, k, dC, dA, st);
        LKG_CUDA(cudaMemcpyAsync(assignment.data(), dA, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
        LKG_CUDA(cudaStreamSynchronize(st));
      };
      std::vector<double> sum((size_t)k * d);
      std::vector<int> cnt(k);
      for (int it = 0; it < 10; ++it) {
        assign();
        std::fill(sum.begin(), sum.end(), 0.0);
        std::fill(cnt.begin(), cnt.end(), 0);
        for (int i = 0; i < n; ++i) {
          const int c = assignment[i];
          cnt[c]++;
          for (int j = 0; j < d; ++j) sum[(size_t)c * d + j] += m_X(i, j);
        }
        for (int c = 0; c < k; ++c)
          if (cnt[c] > 0)
            for (int j = 0; j < d; ++j) C[(size_t)c * d + j] = sum[(size_t)c * d + j] / cnt[c];
      }
      assign();
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    kmeans_ok = true;
    std::vector<int> size(nb_groups, 0);
    for (int i = 0; i < n; ++i) size[assignment[i]]++;
    for (int g = 0; g < nb_groups; ++g)
      if (size[g] < min_group_size) kmeans_ok = false;
  }
  if (!kmeans_ok) {  // balanced random split: assignment(perm(i)) = i % nb_groups
    std::vector<int> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int i = n - 1; i > 0; --i) std::swap(perm[i], perm[draw_below(gen, (uint32_t)(i + 1))]);
    for (int i = 0; i < n; ++i) assignment[perm[i]] = i % nb_groups;
  }
  m_groups.assign(nb_groups, {});
  for (int i = 0; i < n; ++i) m_groups[assignment[i]].push_back(i);
}

void NestedKriging::fit(const std::vector<double>& y, const Mat& X, int nb_groups, RegressionModel regmodel,
                        const std::string& optim, const std::string& objective, const Parameters& parameters) {
  if ((int)y.size() != X.rows) throw std::invalid_argument("y and X should have the same number of rows");
  if (nb_groups < 1 || nb_groups > X.rows / (X.cols + 2))
    throw std::invalid_argument("nb_groups should be in [1, n/(d+2)]");
  if (m_aggregation == Aggregation::NK && regmodel != RegressionModel::Constant)
    throw std::invalid_argument("NK aggregation requires a Constant trend; use PoE/gPoE/BCM/rBCM otherwise");
  m_is_fitted = false;
  m_X = X;
  m_y = y;
  m_regmodel = regmodel;
  make_partition(nb_groups);
  fit_partitioned(regmodel, optim, objective, parameters);
}

void NestedKriging::fit_groups(const std::vector<double>& y, const Mat& X, const std::vector<std::vector<int>>& groups,
                               RegressionModel regmodel, const std::string& optim, const std::string& objective,
                               const Parameters& parameters) {
  const int n = X.rows, d = X.cols;
  if ((int)y.size() != n) throw std::invalid_argument("y and X should have the same number of rows");
  if (groups.empty() || (int)groups.size() > n / (d + 2))
    throw std::invalid_argument("nb_groups should be in [1, n/(d+2)]");
  if (m_aggregation == Aggregation::NK && regmodel != RegressionModel::Constant)
    throw std::invalid_argument("NK aggregation requires a Constant trend; use PoE/gPoE/BCM/rBCM otherwise");
  std::vector<char> seen(n, 0);
  for (const auto& g : groups) {
    if ((int)g.size() < d + 2) throw std::invalid_argument("fit_groups: every group needs at least d + 2 points");
    for (int i : g) {
      if (i < 0 || i >= n || seen[i]) throw std::invalid_argument("fit_groups: groups must partition 0..n-1");
      seen[i] = 1;
    }
  }
  for (int i = 0; i < n; ++i)
    if (!seen[i]) throw std::invalid_argument("fit_groups: groups must partition 0..n-1");
  m_is_fitted = false;
  m_X = X;
  m_y = y;
  m_regmodel = regmodel;
  m_groups = groups;
  for (auto& g : m_groups) std::sort(g.begin(), g.end());
  fit_partitioned(regmodel, optim, objective, parameters);
}

void NestedKriging::fit_partitioned(RegressionModel regmodel, const std::string& optim,
                                    const std::string& objective, const Parameters& parameters) {
  const int p = (int)m_groups.size();
  const int d = m_X.cols;
  const bool vll_unified = objective.rfind("LLVecchia", 0) == 0;
  m_submodels.clear();
  m_nk.clear();
  m_service.reset();
  m_group_n.clear();
  m_gtheta.clear();
  m_gsigma2.clear();
  m_gbeta0.clear();
  std::vector<Mat> Xg(p);
  std::vector<std::vector<double>> yg(p);
  for (int g = 0; g < p; ++g) {
    Xg[g] = group_rows(m_X, m_groups[g]);
    yg[g].resize(m_groups[g].size());
    for (size_t i = 0; i < m_groups[g].size(); ++i) yg[g][i] = m_y[m_groups[g][i]];
  }
  for (int g = 0; g < p; ++g) {
    m_submodels.push_back(std::make_unique<Kriging>(m_covType));
    m_submodels.back()->set_precision(m_slices);
  }

  if (vll_unified) {
    // LLVecchia-unified path (NestedKriging.cpp:230-260): one global light Vecchia fit gives the common prior,
    // then every submodel is fitted in closed form on it
    Kriging ref(m_covType);
    ref.set_vecchia_exact_commit(false);
    ref.fit(m_y, m_X, regmodel, false, optim, objective, parameters);
    m_theta = ref.theta();
    m_sigma2 = ref.sigma2();
    m_beta0 = (regmodel == RegressionModel::Constant) ? ref.beta()[0] : 0.0;
    Parameters fixed;
    Mat th;
    th.rows = 1;
    th.cols = d;
    th.v = m_theta;
    fixed.theta = th;
    fixed.is_theta_estim = false;
    fixed.sigma2 = m_sigma2;
    fixed.is_sigma2_estim = false;
    fixed.beta = ref.beta();
    fixed.is_beta_estim = false;
    parallel_for(p, 16, [&](int g) { m_submodels[g]->fit(yg[g], Xg[g], regmodel, false, "none", "LL", fixed); });
  } else {
    // plain path (NestedKriging.cpp:261-269): independent submodel fits, here concurrent and batched
    std::vector<Design> ds(p);
    int pcols = 0;
    for (int g = 0; g < p; ++g) {
      ds[g].n = Xg[g].rows;
      ds[g].X = Xg[g].v;
      ds[g].y = yg[g];
      ds[g].F = regression_matrix(regmodel, ds[g].X, ds[g].n, d, &pcols);
    }
    m_service = std::make_unique<NestedService>(m_kernel, d, pcols, ds, starts_of(optim, parameters), m_slices);
    NestedService& service = *m_service;
    m_group_n.resize(p);
    for (int g = 0; g < p; ++g) m_group_n[g] = ds[g].n;
    std::vector<std::exception_ptr> errs(p);
    for (int w0 = 0; w0 < p; w0 += kMaxFitThreads) {
      const int w1 = std::min(p, w0 + kMaxFitThreads);
      service.set_active(w1 - w0);
      std::vector<std::thread> th;
      th.reserve(w1 - w0);
      for (int g = w0; g < w1; ++g)
        th.emplace_back([&, g]() {
          try {
            m_submodels[g]->attach_service(&service, g);
            m_submodels[g]->fit(yg[g], Xg[g], regmodel, false, optim, objective, parameters);
          } catch (...) {
            errs[g] = std::current_exception();
          }
          m_submodels[g]->attach_service(nullptr, 0);
          service.leave();
        });
      for (auto& t : th) t.join();
    }
    for (auto& e : errs)
      if (e) std::rethrow_exception(e);
    unify_hyperparameters(objective);
  }
  if (m_aggregation == Aggregation::NK) precompute_nk();
  m_is_fitted = true;
}

// NestedKriging::unify_hyperparameters (NestedKriging.cpp:283-332): group-size weighted geometric mean of theta,
// weighted means of sigma2 and beta0, then every submodel refitted with optim = "none" on that common prior
void NestedKriging::unify_hyperparameters(const std::string& objective) {
  const int p = (int)m_groups.size();
  const int d = m_X.cols;
  const double n = (double)m_X.rows;
  std::vector<double> log_theta(d, 0.0);
  double sigma2 = 0.0, beta0 = 0.0;
  m_gtheta.assign((size_t)p * d, 0.0);
  m_gsigma2.assign(p, 0.0);
  m_gbeta0.assign(p, 0.0);
  for (int g = 0; g < p; ++g) {
    std::copy(m_submodels[g]->theta().begin(), m_submodels[g]->theta().end(), m_gtheta.begin() + (size_t)g * d);
    m_gsigma2[g] = m_submodels[g]->sigma2();
    m_gbeta0[g] = m_submodels[g]->beta().empty() ? 0.0 : m_submodels[g]->beta()[0];
  }
  for (int g = 0; g < p; ++g) {
    const double w = (double)m_groups[g].size() / n;
    const std::vector<double>& th = m_submodels[g]->theta();
    for (int k = 0; k < d; ++k) log_theta[k] += w * std::log(th[k]);
    sigma2 += w * m_submodels[g]->sigma2();
    if (m_regmodel == RegressionModel::Constant) beta0 += w * m_submodels[g]->beta()[0];
  }
  m_theta.resize(d);
  for (int k = 0; k < d; ++k) m_theta[k] = std::exp(log_theta[k]);
  m_sigma2 = sigma2;
  m_beta0 = beta0;
  Parameters fixed;
  Mat th;
  th.rows = 1;
  th.cols = d;
  th.v = m_theta;
  fixed.theta = th;
  fixed.is_theta_estim = false;
  fixed.sigma2 = m_sigma2;
  fixed.is_sigma2_estim = false;
  if (m_regmodel == RegressionModel::Constant) {
    fixed.beta = std::vector<double>{m_beta0};
    fixed.is_beta_estim = false;
  }
  parallel_for(p, 16, [&](int g) {
    Mat Xg = group_rows(m_X, m_groups[g]);
    std::vector<double> yg(m_groups[g].size());
    for (size_t i = 0; i < yg.size(); ++i) yg[i] = m_y[m_groups[g][i]];
    m_submodels[g]->fit(yg, Xg, m_regmodel, false, "none", objective, fixed);
  });
}

// NestedKriging::precompute_nk (NestedKriging.cpp:334-347): L_g = chol(R_g + jitter I) under the common prior and
// z_g = L_g \ (y_g - beta0), per size class in one batched factorisation
void NestedKriging::precompute_nk() {
  const int p = (int)m_groups.size();
  const int d = m_X.cols;
  std::vector<Design> ds(p);
  for (int g = 0; g < p; ++g) {
    Mat Xg = group_rows(m_X, m_groups[g]);
    ds[g].n = Xg.rows;
    ds[g].X = Xg.v;
    ds[g].y.resize(ds[g].n);
    for (int i = 0; i < ds[g].n; ++i) ds[g].y[i] = m_y[m_groups[g][i]];
    ds[g].F.assign(ds[g].n, 1.0);
  }
  std::vector<int> order(p);
  for (int g = 0; g < p; ++g) order[g] = g;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ds[a].n < ds[b].n; });
  m_nk.clear();
  for (int g : order) {
    const int np = class_size(ds[g].n);
    if (m_nk.empty() || m_nk.back()->n_pad != np) {
      m_nk.push_back(std::make_unique<NkClass>());
      m_nk.back()->n_pad = np;
    }
    m_nk.back()->groups.push_back(g);
  }
  for (auto& c : m_nk) {
    const int ne = (int)c->groups.size(), np = c->n_pad;
    std::vector<double> X, y, F;
    std::vector<int> nv;
    pack_class(ds, c->groups, np, d, 1, X, y, F, nv);
    c->eng = std::make_unique<Engine>(m_kernel, np, d, 1, ne, X.data(), y.data(), F.data(), nv.data(), ne);
    c->eng->set_plain_chol(true, 1.0 + kJitter);
    std::vector<double> th((size_t)ne * d), fac(ne, 1.0);
    std::vector<int> des(ne);
    for (int e = 0; e < ne; ++e) {
      std::copy(m_theta.begin(), m_theta.end(), th.begin() + (size_t)e * d);
      des[e] = e;
    }
    std::vector<EvalOut> out;
    c->eng->evaluate(ne, th.data(), fac.data(), false, out, nullptr, des.data());
    for (int e = 0; e < ne; ++e)
      if (out[e].status != 0) throw std::runtime_error("chol(): decomposition failed");
    std::vector<double> z((size_t)ne * np, 0.0);
    for (int e = 0; e < ne; ++e) {
      std::vector<double> Fs, ys;
      c->eng->copy_model(e, nullptr, &Fs, &ys, nullptr, nullptr);
      for (int i = 0; i < np; ++i) z[(size_t)e * np + i] = ys[i] - m_beta0 * Fs[i];
    }
    LKG_CUDA(cudaMalloc(&c->dz, sizeof(double) * z.size()));
    LKG_CUDA(cudaMalloc(&c->dnv, sizeof(int) * ne));
    LKG_CUDA(cudaMemcpy(c->dz, z.data(), sizeof(double) * z.size(), cudaMemcpyHostToDevice));
    LKG_CUDA(cudaMemcpy(c->dnv, nv.data(), sizeof(int) * ne, cudaMemcpyHostToDevice));
  }
}

std::tuple<std::vector<double>, std::vector<double>> NestedKriging::predict(const Mat& X_n, bool return_stdev) {
  if (!m_is_fitted) throw std::runtime_error("NestedKriging is not fitted");
  if (X_n.cols != m_X.cols) throw std::invalid_argument("X_n should have the same number of columns as X");
  if (m_aggregation == Aggregation::NK) return predict_nk(X_n, return_stdev);
  return predict_poe_family(X_n, return_stdev);
}

void NestedKriging::log_likelihood_groups(const Mat& thetas, bool return_grad, std::vector<double>& ll,
                                          std::vector<double>& grad) {
  if (!m_service) throw std::runtime_error("log_likelihood_groups: needs a NestedKriging fitted on the plain path");
  const int p = (int)m_groups.size(), d = m_X.cols;
  if (thetas.rows != p || thetas.cols != d)
    throw std::invalid_argument("log_likelihood_groups: thetas should be " + std::to_string(p) + " x " +
                                std::to_string(d));
  std::vector<double> th((size_t)p * d);
  for (int g = 0; g < p; ++g)
    for (int k = 0; k < d; ++k) th[(size_t)g * d + k] = thetas(g, k);
  std::vector<EvalOut> out;
  m_service->evaluate_all(th.data(), return_grad, out);
  ll.assign(p, 0.0);
  grad.assign(return_grad ? (size_t)p * d : 0, 0.0);
  for (int g = 0; g < p; ++g) {
    const EvalOut& o = out[g];
    if (o.status != 0) throw std::runtime_error(o.message);
    // Kriging.cpp:290-306 (sigma2 estimated): the concentrated log-likelihood and its theta-gradient
    const double n = m_group_n[g];
    const double s2 = o.sse / n;
    ll[g] = -0.5 * (n * std::log(2 * M_PI * s2) + o.logdet + n);
    if (return_grad)
      for (int k = 0; k < d; ++k) grad[(size_t)g * d + k] = ((2.0 * o.adj[k]) / s2 + (-2.0 * o.adj[d + k])) / 2.0;
  }
}

// NestedKriging::predict_poe_family (NestedKriging.cpp:364-422)
std::tuple<std::vector<double>, std::vector<double>> NestedKriging::predict_poe_family(const Mat& X_n,
                                                                                      bool return_stdev) {
  const int q = X_n.rows, p = (int)m_groups.size();
  const double prior_var = m_sigma2;
  std::vector<std::vector<double>> mus(p), vars(p);
  parallel_for(p, 8, [&](int g) {
    auto [mu, sd, cov, dmu, dsd] = m_submodels[g]->predict(X_n, true, false, false);
    mus[g] = std::move(mu);
    vars[g].resize(q);
    for (int t = 0; t < q; ++t) vars[g][t] = sd[t] * sd[t] + kTiny;
  });
  std::vector<double> mean(q), var(q);
  const double pd = (double)p;
  for (int t = 0; t < q; ++t) {
    switch (m_aggregation) {
      case Aggregation::PoE: {
        double prec = 0.0, num = 0.0;
        for (int g = 0; g < p; ++g) prec += 1.0 / vars[g][t];
        for (int g = 0; g < p; ++g) num += mus[g][t] / vars[g][t];
        mean[t] = num / prec;
        var[t] = 1.0 / prec;
      } break;
      case Aggregation::gPoE: {
        double prec = 0.0, num = 0.0;
        for (int g = 0; g < p; ++g) prec += 1.0 / vars[g][t];
        prec /= pd;
        for (int g = 0; g < p; ++g) num += mus[g][t] / vars[g][t];
        mean[t] = (num / pd) / prec;
        var[t] = 1.0 / prec;
      } break;
      case Aggregation::BCM: {
        double prec = 0.0, num = 0.0;
        for (int g = 0; g < p; ++g) prec += 1.0 / vars[g][t];
        prec -= (pd - 1.0) / prior_var;
        prec = std::max(prec, kTiny);
        for (int g = 0; g < p; ++g) num += mus[g][t] / vars[g][t];
        mean[t] = num / prec;
        var[t] = 1.0 / prec;
      } break;
      case Aggregation::rBCM: {
        const double lp = std::log(prior_var);
        double sbv = 0.0, sb = 0.0, num = 0.0;
        for (int g = 0; g < p; ++g) {
          const double beta = 0.5 * (lp - std::log(vars[g][t]));
          sbv += beta / vars[g][t];
          sb += beta;
          num += beta * mus[g][t] / vars[g][t];
        }
        double prec = sbv + (1.0 - sb) / prior_var;
        prec = std::max(prec, kTiny);
        mean[t] = num / prec;
        var[t] = 1.0 / prec;
      } break;
      default:
        throw std::logic_error("unreachable");
    }
  }
  if (!return_stdev) return {mean, {}};
  std::vector<double> sd(q);
  for (int t = 0; t < q; ++t) sd[t] = std::sqrt(std::max(var[t], 0.0));
  return {mean, sd};
}

namespace {

// Solve K w = k for a symmetric p x p matrix (upper triangle used, column-major): Cholesky, else LU with
// partial pivoting, else the pseudo-inverse from a cyclic Jacobi eigendecomposition (arma::solve with
// likely_sympd, then arma::pinv, NestedKriging.cpp:484-486)
std::vector<double> solve_sym(int p, std::vector<double> K, const std::vector<double>& k) {
  auto A = [&](std::vector<double>& M, int i, int j) -> double& { return M[i + (size_t)j * p]; };
  for (int j = 0; j < p; ++j)
    for (int i = j + 1; i < p; ++i) A(K, i, j) = A(K, j, i);
  {  // Cholesky
    std::vector<double> L = K;
    bool ok = true;
    for (int j = 0; j < p && ok; ++j) {
      double s = A(L, j, j);
      for (int m = 0; m < j; ++m) s -= A(L, j, m) * A(L, j, m);
      if (!(s > 0.0)) {
        ok = false;
        break;
      }
      const double ljj = std::sqrt(s);
      A(L, j, j) = ljj;
      for (int i = j + 1; i < p; ++i) {
        double v = A(L, i, j);
        for (int m = 0; m < j; ++m) v -= A(L, i, m) * A(L, j, m);
        A(L, i, j) = v / ljj;
      }
    }
    if (ok) {
      std::vector<double> w(k);
      for (int i = 0; i < p; ++i) {
        double v = w[i];
        for (int m = 0; m < i; ++m) v -= A(L, i, m) * w[m];
        w[i] = v / A(L, i, i);
      }
      for (int i = p - 1; i >= 0; --i) {
        double v = w[i];
        for (int m = i + 1; m < p; ++m) v -= A(L, m, i) * w[m];
        w[i] = v / A(L, i, i);
      }
      return w;
    }
  }
  {  // LU with partial pivoting
    std::vector<double> M = K, w(k);
    bool ok = true;
    for (int c = 0; c < p && ok; ++c) {
      int piv = c;
      for (int i = c + 1; i < p; ++i)
        if (std::fabs(A(M, i, c)) > std::fabs(A(M, piv, c))) piv = i;
      if (A(M, piv, c) == 0.0) {
        ok = false;
        break;
      }
      if (piv != c) {
        for (int j = 0; j < p; ++j) std::swap(A(M, c, j), A(M, piv, j));
        std::swap(w[c], w[piv]);
      }
      for (int i = c + 1; i < p; ++i) {
        const double f = A(M, i, c) / A(M, c, c);
        for (int j = c; j < p; ++j) A(M, i, j) -= f * A(M, c, j);
        w[i] -= f * w[c];
      }
    }
    if (ok) {
      for (int i = p - 1; i >= 0; --i) {
        double v = w[i];
        for (int j = i + 1; j < p; ++j) v -= A(M, i, j) * w[j];
        w[i] = v / A(M, i, i);
      }
      return w;
    }
  }
  // pseudo-inverse (cyclic Jacobi), singular values below p * eps * max kept out
  std::vector<double> M = K, V((size_t)p * p, 0.0);
  for (int i = 0; i < p; ++i) A(V, i, i) = 1.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int j = 0; j < p; ++j)
      for (int i = 0; i < j; ++i) off += A(M, i, j) * A(M, i, j);
    if (off < 1e-300) break;
    for (int a = 0; a < p; ++a)
      for (int b = a + 1; b < p; ++b) {
        const double apq = A(M, a, b);
        if (apq == 0.0) continue;
        const double tau = (A(M, b, b) - A(M, a, a)) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int i = 0; i < p; ++i) {
          const double mia = A(M, i, a), mib = A(M, i, b);
          A(M, i, a) = c * mia - s * mib;
          A(M, i, b) = s * mia + c * mib;
        }
        for (int j = 0; j < p; ++j) {
          const double maj = A(M, a, j), mbj = A(M, b, j);
          A(M, a, j) = c * maj - s * mbj;
          A(M, b, j) = s * maj + c * mbj;
        }
        for (int i = 0; i < p; ++i) {
          const double via = A(V, i, a), vib = A(V, i, b);
          A(V, i, a) = c * via - s * vib;
          A(V, i, b) = s * via + c * vib;
        }
      }
  }
  double emax = 0.0;
  for (int i = 0; i < p; ++i) emax = std::max(emax, std::fabs(A(M, i, i)));
  const double tol = p * std::numeric_limits<double>::epsilon() * emax;
  std::vector<double> w(p, 0.0);
  for (int e = 0; e < p; ++e) {
    const double lam = A(M, e, e);
    if (std::fabs(lam) <= tol) continue;
    double vk = 0.0;
    for (int i = 0; i < p; ++i) vk += A(V, i, e) * k[i];
    for (int i = 0; i < p; ++i) w[i] += A(V, i, e) * vk / lam;
  }
  return w;
}

}  // namespace

// NestedKriging::predict_nk (NestedKriging.cpp:424-498): per chunk of m_chunk points, C_g, U_g = L_g \ C_g,
// W_g = L_g' \ U_g, M_g, k_g and all pair cross-covariances on the GPU; the p x p aggregation per point on the host
std::tuple<std::vector<double>, std::vector<double>> NestedKriging::predict_nk(const Mat& X_n, bool return_stdev) {
  const int q = X_n.rows, p = (int)m_groups.size(), d = m_X.cols;
  std::vector<double> mean(q), var(return_stdev ? q : 0);
  const int chunk = std::min(m_chunk, std::max(q, 1));
  cudaStream_t st;
  LKG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  std::vector<void*> bufs;
  auto dmalloc = [&](size_t bytes) {
    void* ptr = nullptr;
    LKG_CUDA(cudaMalloc(&ptr, std::max<size_t>(bytes, 8)));
    bufs.push_back(ptr);
    return ptr;
  };
  try {
    double* dtheta = (double*)dmalloc(sizeof(double) * d);
    double* dXc = (double*)dmalloc(sizeof(double) * (size_t)chunk * d);
    std::vector<double*> dW(m_nk.size());
    std::vector<int> slot_of(p);  // group -> position in M / K
    int slot = 0;
    for (size_t c = 0; c < m_nk.size(); ++c) {
      const NkClass& nc = *m_nk[c];
      dW[c] = (double*)dmalloc(sizeof(double) * nc.groups.size() * nc.n_pad * chunk);
      for (int g : nc.groups) slot_of[g] = slot++;
    }
    double* dM = (double*)dmalloc(sizeof(double) * (size_t)p * chunk);
    double* dK = (double*)dmalloc(sizeof(double) * (size_t)p * chunk);
    const long long npairs = (long long)p * (p - 1) / 2;
    double* dcross = (double*)dmalloc(sizeof(double) * (size_t)std::max<long long>(npairs, 1) * chunk);
    std::vector<NkGroup> G(p);
    for (size_t c = 0; c < m_nk.size(); ++c) {
      const NkClass& nc = *m_nk[c];
      for (size_t e = 0; e < nc.groups.size(); ++e) {
        const int g = nc.groups[e];
        G[g] = NkGroup{nc.eng->dX_design((int)e), nc.n_pad, dW[c] + e * (size_t)nc.n_pad * chunk, nc.n_pad,
                       nc.eng->n_valid((int)e)};
      }
    }
    NkGroup* dG = (NkGroup*)dmalloc(sizeof(NkGroup) * p);
    LKG_CUDA(cudaMemcpyAsync(dG, G.data(), sizeof(NkGroup) * p, cudaMemcpyHostToDevice, st));
    LKG_CUDA(cudaMemcpyAsync(dtheta, m_theta.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st));
    std::vector<double> M((size_t)p * chunk), Kd((size_t)p * chunk), cross((size_t)std::max<long long>(npairs, 1) * chunk);
    std::vector<double> Xc((size_t)chunk * d);
    for (int start = 0; start < q; start += chunk) {
      const int qc = std::min(chunk, q - start);
      for (int k = 0; k < d; ++k)
        for (int t = 0; t < qc; ++t) Xc[t + (size_t)k * qc] = X_n(start + t, k);
      LKG_CUDA(cudaMemcpyAsync(dXc, Xc.data(), sizeof(double) * (size_t)qc * d, cudaMemcpyHostToDevice, st));
      int off = 0;
      for (size_t c = 0; c < m_nk.size(); ++c) {
        const NkClass& nc = *m_nk[c];
        const int ne = (int)nc.groups.size(), np = nc.n_pad;
        const Engine& eng = *nc.eng;
        nk_corr_entries(m_kernel, np, d, eng.dX(), (int64_t)np * d, nc.dnv, ne, dtheta, dXc, qc, dW[c],
                        (int64_t)np * chunk, st);
        trsm_lower_left(eng.dL(0), eng.lda(), eng.mstride(), np, eng.dDinv(0), dW[c], np, (int64_t)np * chunk, qc,
                        ne, st);
        nk_moments(np, qc, dW[c], (int64_t)np * chunk, nc.dz, np, m_beta0, ne, dM + (size_t)off * chunk,
                   dK + (size_t)off * chunk, chunk, st);
        trsm_lower_left_t(eng.dL(0), eng.lda(), eng.mstride(), np, eng.dDinv(0), dW[c], np, (int64_t)np * chunk,
                          qc, ne, st);
        off += ne;
      }
      nk_cross(m_kernel, d, p, dG, dtheta, qc, dcross, st);
      LKG_CUDA(cudaMemcpyAsync(M.data(), dM, sizeof(double) * (size_t)p * chunk, cudaMemcpyDeviceToHost, st));
      LKG_CUDA(cudaMemcpyAsync(Kd.data(), dK, sizeof(double) * (size_t)p * chunk, cudaMemcpyDeviceToHost, st));
      if (npairs > 0)
        LKG_CUDA(cudaMemcpyAsync(cross.data(), dcross, sizeof(double) * (size_t)npairs * qc, cudaMemcpyDeviceToHost,
                                 st));
      LKG_CUDA(cudaStreamSynchronize(st));
      // aggregate per point (NestedKriging.cpp:476-492)
      auto point = [&](int t) {
        std::vector<double> KM((size_t)p * p, 0.0), kM(p), Mt(p);
        long long kk = 0;
        for (int i = 0; i < p; ++i)
          for (int j = i + 1; j < p; ++j, ++kk) KM[i + (size_t)j * p] = cross[(size_t)kk * qc + t];
        for (int g = 0; g < p; ++g) {
          KM[g + (size_t)g * p] = Kd[(size_t)slot_of[g] * chunk + t] + kJitter;
          kM[g] = KM[g + (size_t)g * p];
          Mt[g] = M[(size_t)slot_of[g] * chunk + t];
        }
        const std::vector<double> w = solve_sym(p, KM, kM);
        double dm = 0.0, dk = 0.0;
        for (int g = 0; g < p; ++g) dm += w[g] * (Mt[g] - m_beta0);
        mean[start + t] = m_beta0 + dm;
        if (return_stdev) {
          for (int g = 0; g < p; ++g) dk += w[g] * kM[g];
          var[start + t] = m_sigma2 * std::max(0.0, 1.0 - dk);
        }
      };
      const int width = (p >= 64) ? 16 : 1;
      parallel_for(qc, width, point);
    }
  } catch (...) {
    for (void* ptr : bufs) cudaFree(ptr);
    cudaStreamDestroy(st);
    throw;
  }
  for (void* ptr : bufs) cudaFree(ptr);
  cudaStreamDestroy(st);
  if (!return_stdev) return {mean, {}};
  std::vector<double> sd(q);
  for (int t = 0; t < q; ++t) sd[t] = std::sqrt(var[t]);
  return {mean, sd};
}

std::string NestedKriging::summary() const {
  std::ostringstream oss;
  if (!m_is_fitted) {
    oss << "* covariance: " << m_covType << " (not fitted)";
    return oss.str();
  }
  oss << "* data: " << m_X.rows << " x " << m_X.cols << " -> " << m_y.size() << "\n";
  oss << "* groups: " << m_groups.size() << " (";
  for (size_t g = 0; g < m_groups.size(); ++g) oss << (g ? "," : "") << m_groups[g].size();
  oss << ")\n";
  oss << "* aggregation: " << aggregation_to_string(m_aggregation) << "\n";
  oss << "* trend (constant): " << m_beta0 << "\n";
  oss << "* variance: " << m_sigma2 << "\n";
  oss << "* covariance: " << m_covType << ", range:";
  for (double t : m_theta) oss << " " << t;
  return oss.str();
}

}  // namespace lkg
