// engine.cpp -- device-resident evaluation engine (host orchestration of the sm_103a kernels).
//
// Order of operations per evaluation follows KrigingImpl::populate_Model (src/lib/KrigingImpl.cpp:73-125):
//   R = factor * C(X; theta), diag = 1 (+ numerical nugget on retry)      LinearAlgebra::cholCov  (:142-204)
//   L = chol(R) with the rcond / nugget-retry rules                        safe_chol_lower_retry   (:68-98)
//   [F* y*] = L \ [F y]; R* = chol(F*'F*); beta = R* \ (R*' \ F*'y*); E* = y* - F* beta; SSE = E*'E*
// and, when a gradient is requested, the adjoint sums of compute_ll_grad_theta_vecs (KrigingImpl.cpp:855-885)
// with x = L' \ E* and R^-1 = (L^-1)' L^-1.
#include "engine.hpp"

#include "autotune.hpp"

#include <algorithm>
#include <cmath>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <string>

#include "common.cuh"
#include "dense_fp64.cuh"
#include "lik_kernels.cuh"
#include "ozaki7.cuh"
#include "stats.hpp"

namespace lkg {

namespace {

template <typename T>
T env_or(const char* name, T def) {
  const char* v = std::getenv(name);
  if (!v) return def;
  try {
    if constexpr (std::is_same_v<T, int>) return std::stoi(v);
    else if constexpr (std::is_same_v<T, double>) return std::stod(v);
    else if constexpr (std::is_same_v<T, bool>) {
      std::string s(v);
      return s == "1" || s == "true" || s == "TRUE" || s == "True";
    }
  } catch (...) {
  }
  return def;
}

struct Timer {
  cudaStream_t st;
  std::map<std::string, double>* bench;
  cudaEvent_t e0 = nullptr;
  Timer(cudaStream_t s, std::map<std::string, double>* b) : st(s), bench(b) {
    if (bench) {
      LKG_CUDA(cudaEventCreate(&e0));
      LKG_CUDA(cudaEventRecord(e0, st));
    }
  }
  ~Timer() {
    if (e0) cudaEventDestroy(e0);
  }
  void lap(const char* key) {
    if (!bench) return;
    cudaEvent_t e1;
    LKG_CUDA(cudaEventCreate(&e1));
    LKG_CUDA(cudaEventRecord(e1, st));
    LKG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    LKG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    (*bench)[key] += ms;
    LKG_CUDA(cudaEventDestroy(e0));
    e0 = e1;
  }
};

template <typename P>
void dalloc(P** p, size_t count) {
  LKG_CUDA(cudaMalloc((void**)p, sizeof(P) * std::max<size_t>(count, 1)));
}

}  // namespace

Config& config() {
  static Config c = [] {
    Config x;
    x.reparametrize = env_or("LK_REPARAMETRIZE", true);
    x.theta_lower_factor = env_or("LK_THETA_LOWER_FACTOR", 0.02);
    x.theta_upper_factor = env_or("LK_THETA_UPPER_FACTOR", 10.0);
    x.variogram_bounds_heuristic = env_or("LK_VARIOGRAM_BOUNDS_HEURISTIC", true);
    x.log_level = env_or("LK_LOG_LEVEL", 0);
    x.max_restart = env_or("LK_MAX_RESTART", 10);
    x.max_iteration = env_or("LK_MAX_ITERATION", 20);
    x.gradient_tolerance = env_or("LK_GRADIENT_TOLERANCE", 0.001);
    x.objective_rel_tolerance = env_or("LK_OBJECTIVE_REL_TOLERANCE", 0.001);
    return x;
  }();
  return c;
}

Engine::Engine(int kernel, int n, int d, int p, const double* X, const double* y, const double* F, int batch_cap)
    : Engine(kernel, n, d, p, 1, X, y, F, nullptr, batch_cap) {}

Engine::Engine(int kernel, int n, int d, int p, int ndesign, const double* X, const double* y, const double* F,
               const int* n_valid, int batch_cap)
    : kernel_(kernel), n_(n), d_(d), p_(p), cap_(batch_cap), ndesign_(ndesign) {
  if (n < 1 || d < 1 || d > MAX_D || p < 0 || p > 64 || batch_cap < 1 || ndesign < 1)
    throw std::invalid_argument("Engine: unsupported sizes n=" + std::to_string(n) + " d=" + std::to_string(d) +
                                " p=" + std::to_string(p));
  nvalid_.assign(ndesign, n);
  if (n_valid)
    for (int e = 0; e < ndesign; ++e) {
      if (n_valid[e] < 1 || n_valid[e] > n) throw std::invalid_argument("Engine: design size out of range");
      nvalid_[e] = n_valid[e];
    }
  LKG_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
  lda_ = ((int64_t)n + 7) / 8 * 8;  // 64-byte aligned columns
  mstride_ = lda_ * n;
  const int nblk = ceil_div(n, NB);
  dstride_ = (int64_t)nblk * NB * NB;
  fystride_ = (int64_t)n * (p + 1);
  gram_stride_ = (p + 1) * (p + 1) + 1;
  const size_t nd = (size_t)ndesign;
  dalloc(&dX_, nd * n * d);
  dalloc(&dY_, nd * n);
  dalloc(&dF_, nd * n * std::max(p, 1));
  LKG_CUDA(cudaMemcpyAsync(dX_, X, sizeof(double) * nd * n * d, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dY_, y, sizeof(double) * nd * n, cudaMemcpyHostToDevice, st_));
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(dF_, F, sizeof(double) * nd * n * p, cudaMemcpyHostToDevice, st_));
  if (ndesign > 1 || n_valid) {
    dalloc(&dXe_, (size_t)cap_ * n * d);
    dalloc(&dnv_, cap_);
  }
  dalloc(&dA_, (size_t)mstride_ * cap_);
  dalloc(&dDinv_, (size_t)dstride_ * cap_);
  dalloc(&dFY_, (size_t)fystride_ * cap_);
  dalloc(&dEstar_, (size_t)n * cap_);
  dalloc(&dxv_, (size_t)n * cap_);
  dalloc(&dvec_, (size_t)n * cap_);
  dalloc(&dcol_, (size_t)n * cap_);
  dalloc(&dtheta_, (size_t)d * cap_);
  dalloc(&dfactor_, cap_);
  dalloc(&ddiag_, cap_);
  dalloc(&dgram_, (size_t)gram_stride_ * cap_);
  dalloc(&dbeta_, (size_t)std::max(p, 1) * cap_);
  dalloc(&drstar_, (size_t)std::max(p * p, 1) * cap_);
  dalloc(&dsse_, cap_);
  dalloc(&dadj_, (size_t)adjoint_nacc(d) * cap_);
  dalloc(&dinfo_, cap_);
  dalloc(&dgls_info_, cap_);
  LKG_CUDA(cudaStreamSynchronize(st_));
}

Engine::~Engine() {
  clear_graphs();
  for (double* p : {dX_, dY_, dF_, dA_, dDinv_, dW_, dRinv_, dFY_, dEstar_, dxv_, dtheta_, dfactor_, ddiag_, dgram_,
                    dbeta_, drstar_, dsse_, dpart_, dadj_, dvec_, dcol_, dloo_m_, dloo_at_, dloo_vec_, dWp_})
    if (p) cudaFree(p);
  if (dinfo_) cudaFree(dinfo_);
  if (dgls_info_) cudaFree(dgls_info_);
  if (dXe_) cudaFree(dXe_);
  if (dnv_) cudaFree(dnv_);
  for (void* p : {dpanel_, drowblk_, dwfull_, dside_})
    if (p) cudaFree(p);
  for (int* p : {dpanel_exp_, drowblk_exp_, dwfull_exp_, dside_exp_})
    if (p) cudaFree(p);
  if (ev_strip_) cudaEventDestroy(ev_strip_);
  if (ev_panel_) cudaEventDestroy(ev_panel_);
  if (side_st_) cudaStreamDestroy(side_st_);
  if (st_) cudaStreamDestroy(st_);
}

void Engine::set_slices(int s) {
  if (s != 0 && (s < 4 || s > 8)) throw std::invalid_argument("mixed precision: slices must be 0 (FP64) or 4..8");
  slices_ = s;
}

// SMs kept for the mixed Cholesky's look-ahead panel work (0: no look-ahead).  An explicit setting
// (LKG_LOOKAHEAD_CTAS, lkg_set_lookahead) applies to every size; otherwise (-1) the autotuner's choice for the matrix
// size is used ("lookahead:n=<n>", see Kriging::autotune_lookahead), else kLookaheadDefault.
namespace {
constexpr int kLookaheadDefault = 16;
std::atomic<int> g_lookahead_ctas{[] {
  const char* v = std::getenv("LKG_LOOKAHEAD_CTAS");
  if (!v) return -1;
  const int x = std::atoi(v);
  return x >= 0 && x <= 64 ? x : -1;
}()};
}  // namespace

void set_lookahead_ctas(int c) {
  if (c < -1 || c > 64) throw std::invalid_argument("look-ahead: SMs for the panel work must be -1 .. 64");
  g_lookahead_ctas = c;
}
int lookahead_ctas_setting() { return g_lookahead_ctas; }

std::string lookahead_tune_key(int n) { return "lookahead:n=" + std::to_string(n); }

int lookahead_ctas_for(int n) {
  const int c = g_lookahead_ctas;
  if (c >= 0) return c;
  return Autotuner::instance().lookup(lookahead_tune_key(n), kLookaheadDefault);
}

namespace {
std::atomic<bool> g_graphs{[] {
  const char* v = std::getenv("LKG_GRAPHS");
  return !(v && std::strcmp(v, "0") == 0);
}()};
}  // namespace

void set_graphs_enabled(bool on) { g_graphs = on; }
bool graphs_enabled() { return g_graphs; }

void Engine::clear_graphs() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  graph_launches_.clear();
  graph_seen_.clear();
  graph_refused_.clear();
}

void Engine::buffers_changed() {
  ++buf_gen_;
  clear_graphs();
}

void Engine::run_phase(const std::string& key, const std::function<void()>& launch, bool allow) {
  if (!allow || !graphs_enabled() || stats_enabled() || graph_refused_.count(key)) {
    launch();
    return;
  }
  auto it = graphs_.find(key);
  if (it != graphs_.end()) {
    LKG_CUDA(cudaGraphLaunch(it->second, st_));
    stats_add_launches(graph_launches_[key], +1);
    return;
  }
  // the first run of a configuration goes direct: kernel attributes, module loading and lazily sized buffers are
  // settled before anything is captured
  if (graph_seen_.insert(key).second) {
    launch();
    return;
  }
  const auto before = stats_thread_launch_counts();
  auto delta = [&] {
    std::map<std::string, long long> d;
    for (auto& kv : stats_thread_launch_counts()) {
      const auto b = before.find(kv.first);
      const long long c = kv.second - (b == before.end() ? 0 : b->second);
      if (c) d[kv.first] = c;
    }
    return d;
  };
  LKG_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
  bool captured = true;
  try {
    launch();
  } catch (...) {
    captured = false;
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(st_, &g);
  cudaGraphExec_t ex = nullptr;
  if (captured && e == cudaSuccess && g) e = cudaGraphInstantiate(&ex, g, 0);
  if (g) cudaGraphDestroy(g);
  const auto d = delta();
  if (!captured || e != cudaSuccess || !ex) {
    // nothing ran: forget the capture's counts, keep this configuration on direct launches
    (void)cudaGetLastError();
    if (ex) cudaGraphExecDestroy(ex);
    stats_add_launches(d, -1);
    graph_refused_.insert(key);
    launch();
    return;
  }
  graphs_[key] = ex;
  graph_launches_[key] = d;  // the capture counted this execution's launches already
  LKG_CUDA(cudaGraphLaunch(ex, st_));
}

// the look-ahead pays when the matrix has several 256-wide panels
bool Engine::lookahead_enabled() const { return n_ >= 4 * OZ7_KB && lookahead_ctas_for(n_) > 0; }

int Engine::lookahead_ctas() const { return lookahead_ctas_for(n_); }

void Engine::ensure_mixed_buffers(bool with_grad) {
  if (mixed_alloc_slices_ != slices_) {
    buffers_changed();
    for (void** p : {&dpanel_, &drowblk_, &dwfull_, &dside_})
      if (*p) {
        cudaFree(*p);
        *p = nullptr;
      }
    for (int** p : {&dpanel_exp_, &drowblk_exp_, &dwfull_exp_, &dside_exp_})
      if (*p) {
        cudaFree(*p);
        *p = nullptr;
      }
    mixed_alloc_slices_ = slices_;
  }
  // up to 8 7-bit digits of a 256-wide panel per batch entry (ozaki7.cuh)
  const size_t pe = oz7_plane_elems(n_, OZ7_KB, 8) * cap_;
  const size_t ee = oz7_exp_elems(n_, OZ7_KB, OZ7_KB) * cap_;
  if (!dpanel_) {
    buffers_changed();
    LKG_CUDA(cudaMalloc(&dpanel_, pe * 2));
    LKG_CUDA(cudaMalloc(&drowblk_, pe * 2));
    dalloc(&dpanel_exp_, ee);
    dalloc(&drowblk_exp_, ee);
  }
  // the look-ahead's own panel splits (single-matrix evaluations of a size where it pays)
  if (lookahead_enabled() && !dside_) {
    buffers_changed();
    const size_t pe1 = oz7_plane_elems(n_, OZ7_KB, 8), ee1 = oz7_exp_elems(n_, OZ7_KB, OZ7_KB);
    LKG_CUDA(cudaMalloc(&dside_, pe1 * 2));
    dalloc(&dside_exp_, ee1);
    if (!side_st_) {
      LKG_CUDA(cudaStreamCreateWithFlags(&side_st_, cudaStreamNonBlocking));
      LKG_CUDA(cudaEventCreateWithFlags(&ev_strip_, cudaEventDisableTiming));
      LKG_CUDA(cudaEventCreateWithFlags(&ev_panel_, cudaEventDisableTiming));
    }
  }
  if (with_grad && !dwfull_) {
    buffers_changed();
    LKG_CUDA(cudaMalloc(&dwfull_, oz7_plane_elems(n_, n_, std::min(8, slices_ + 1)) * cap_ * 2));
    dalloc(&dwfull_exp_, oz7_exp_elems(n_, n_, OZ7_KB) * cap_);
  }
}

void Engine::ensure_grad_buffers() {
  if (dW_) return;
  buffers_changed();
  dalloc(&dW_, (size_t)mstride_ * cap_);
  dalloc(&dRinv_, (size_t)mstride_ * cap_);
  part_size_ = adjoint_partials_size(n_, d_, cap_);
  dalloc(&dpart_, part_size_);
}

const double* Engine::factor_inverse() {
  if (!dWp_) {
    buffers_changed();
    dalloc(&dWp_, (size_t)mstride_);
  }
  if (!wp_valid_) {
    trtri_blocked(dA_, lda_, mstride_, n_, dDinv_, dWp_, lda_, mstride_, 1, st_);
    wp_valid_ = true;
  }
  return dWp_;
}

void Engine::solve_lower_inplace(int b, double* dB, int64_t ldb, int r) const {
  trsm_lower_left(dA_ + (size_t)b * mstride_, lda_, mstride_, n_, dDinv_ + (size_t)b * dstride_, dB, ldb, 0, r, 1,
                  st_);
}

// dtrcon('1', 'L', 'N') style estimate (LAPACK dlacn2 iteration of Hager / Higham) of rcond(L)^2 for every entry,
// with the triangular solves of all entries batched into the same launches.
void Engine::rcond_batch(int batch, std::vector<double>& rc2, const std::vector<int>& nvb) {
  rcond_core(batch, rc2, nvb, dA_, lda_, mstride_, n_, dDinv_);
}

void Engine::rcond_core(int batch, std::vector<double>& rc2, const std::vector<int>& nvb, const double* A,
                        int64_t lda, int64_t mstride, int n, const double* Dinv) {
  // every vector of the estimator lives on the entry's valid block (the padded identity stays out of it), so a
  // padded entry follows exactly the iteration of its unpadded matrix
  std::vector<double> colsum((size_t)n * batch);
  lower_colsum_abs(n, A, lda, mstride, dcol_, batch, st_);
  LKG_CUDA(cudaMemcpyAsync(colsum.data(), dcol_, sizeof(double) * n * batch, cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaStreamSynchronize(st_));
  std::vector<double> anorm(batch, 0.0);
  for (int b = 0; b < batch; ++b)
    for (int j = 0; j < nvb[b]; ++j) anorm[b] = std::max(anorm[b], colsum[(size_t)b * n + j]);

  // per-entry state machine of dlacn2
  struct St {
    int phase = 0;  // 0: x=1/n pending kind1; 1: sign pending kind2; 2: e_j pending kind1; 3: altsgn kind1; 4 done
    int iter = 0, j = 0;
    double est = 0.0;
    std::vector<double> xi;
    bool first_done = false;
  };
  std::vector<St> S(batch);
  std::vector<double> vec((size_t)n * batch);
  auto set_x = [&](int b, int phase) {
    double* x = vec.data() + (size_t)b * n;
    const int m = nvb[b];
    std::fill(x, x + n, 0.0);
    if (phase == 0) {
      for (int i = 0; i < m; ++i) x[i] = 1.0 / m;
    } else if (phase == 1) {
      for (int i = 0; i < m; ++i) x[i] = S[b].xi[i];
    } else if (phase == 2) {
      x[S[b].j] = 1.0;
    } else if (phase == 3) {
      double altsgn = 1.0;
      for (int i = 0; i < m; ++i) {
        x[i] = altsgn * (1.0 + (m > 1 ? (double)i / (double)(m - 1) : 0.0));
        altsgn = -altsgn;
      }
    }
  };
  for (int b = 0; b < batch; ++b) {
    S[b].xi.assign(n, 0.0);
    set_x(b, 0);
    if (!(anorm[b] > 0.0)) S[b].phase = 4;
  }
  auto kind_of = [](int phase) { return phase == 1 ? 2 : 1; };
  for (int round = 0; round < 64; ++round) {
    bool any1 = false, any2 = false;
    for (int b = 0; b < batch; ++b)
      if (S[b].phase < 4) (kind_of(S[b].phase) == 1 ? any1 : any2) = true;
    if (!any1 && !any2) break;
    const int kind = any1 ? 1 : 2;
    LKG_CUDA(cudaMemcpyAsync(dvec_, vec.data(), sizeof(double) * n * batch, cudaMemcpyHostToDevice, st_));
    if (kind == 1)
      trsm_lower_left(A, lda, mstride, n, Dinv, dvec_, n, n, 1, batch, st_);
    else
      trsm_lower_left_t(A, lda, mstride, n, Dinv, dvec_, n, n, 1, batch, st_);
    std::vector<double> res((size_t)n * batch);
    LKG_CUDA(cudaMemcpyAsync(res.data(), dvec_, sizeof(double) * n * batch, cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    for (int b = 0; b < batch; ++b) {
      St& s = S[b];
      if (s.phase >= 4 || kind_of(s.phase) != kind) continue;
      const double* y = res.data() + (size_t)b * n;
      const int m = nvb[b];
      double l1 = 0.0;
      for (int i = 0; i < m; ++i) l1 += std::fabs(y[i]);
      if (s.phase == 0) {
        s.est = l1;
        if (m == 1) {
          s.phase = 4;
          continue;
        }
        for (int i = 0; i < m; ++i) s.xi[i] = (y[i] >= 0.0) ? 1.0 : -1.0;
        s.phase = 1;
        s.iter = 2;
        s.first_done = true;
      } else if (s.phase == 1) {
        int jlast = s.j;
        int jm = 0;
        for (int i = 1; i < m; ++i)
          if (std::fabs(y[i]) > std::fabs(y[jm])) jm = i;
        if (s.first_done) {
          s.first_done = false;
          s.j = jm;
          s.phase = 2;
        } else {
          s.j = jm;
          if (y[jlast] != std::fabs(y[jm]) && s.iter < 5) {
            s.iter++;
            s.phase = 2;
          } else {
            s.phase = 3;
          }
        }
      } else if (s.phase == 2) {
        const double estold = s.est;
        s.est = l1;
        bool same = true;
        for (int i = 0; i < m && same; ++i) same = (((y[i] >= 0.0) ? 1.0 : -1.0) == s.xi[i]);
        if (same || s.est <= estold) {
          s.phase = 3;
        } else {
          for (int i = 0; i < m; ++i) s.xi[i] = (y[i] >= 0.0) ? 1.0 : -1.0;
          s.phase = 1;
        }
      } else if (s.phase == 3) {
        const double temp = 2.0 * l1 / (3.0 * m);
        if (temp > s.est) s.est = temp;
        s.phase = 4;
      }
      if (s.phase < 4) set_x(b, s.phase);
    }
  }
  rc2.assign(batch, 0.0);
  for (int b = 0; b < batch; ++b) {
    double rc = 0.0;
    if (anorm[b] > 0.0 && S[b].est > 0.0) rc = (1.0 / anorm[b]) / S[b].est;
    rc2[b] = rc * rc;
  }
}

void Engine::evaluate(int batch, const double* thetas, const double* factors, bool with_grad,
                      std::vector<EvalOut>& out, std::map<std::string, double>* bench, const int* designs) {
  if (batch < 1 || batch > cap_) throw std::invalid_argument("Engine::evaluate: batch out of range");
  wp_valid_ = false;
  if (ndesign_ > 1 && !designs) throw std::invalid_argument("Engine::evaluate: design of each entry required");
  const Config& cfg = config();
  const int n = n_, d = d_, p = p_;
  out.assign(batch, EvalOut{});
  Timer tm(st_, bench);
  LKG_CUDA(cudaMemcpyAsync(dtheta_, thetas, sizeof(double) * d * batch, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dfactor_, factors, sizeof(double) * batch, cudaMemcpyHostToDevice, st_));
  // design of every entry: X gathered per entry and valid sizes for the identity padding (several designs only)
  entry_design_.assign(batch, 0);
  const double* dXb = dX_;
  int64_t xbs = 0;
  const int* dnv = nullptr;
  std::vector<int> nv_entry(batch, n);
  if (dXe_) {
    for (int b = 0; b < batch; ++b) {
      const int e = designs ? designs[b] : 0;
      if (e < 0 || e >= ndesign_) throw std::invalid_argument("Engine::evaluate: design index out of range");
      entry_design_[b] = e;
      nv_entry[b] = nvalid_[e];
      LKG_CUDA(cudaMemcpyAsync(dXe_ + (size_t)b * n * d, dX_ + (size_t)e * n * d, sizeof(double) * n * d,
                               cudaMemcpyDeviceToDevice, st_));
    }
    LKG_CUDA(cudaMemcpyAsync(dnv_, nv_entry.data(), sizeof(int) * batch, cudaMemcpyHostToDevice, st_));
    dXb = dXe_;
    xbs = (int64_t)n * d;
    dnv = dnv_;
  }

  // ---- R, L with the numerical-nugget retry rules (LinearAlgebra.cpp:68-98) ----
  std::vector<double> diag(batch, base_diag_);
  const bool rcond_check = cfg.chol_rcond_check && !plain_chol_;
  std::vector<int> inc(batch, 0);
  std::vector<char> dead(batch, 0);
  std::vector<int> info(batch, 0);
  std::vector<double> rc2(batch, -1.0);
  MixedWorkspace mw;
  if (slices_ > 0) {
    ensure_mixed_buffers(with_grad);
    mw.slices = slices_;
    // L^-1 and R^-1 feed only the gradient (tolerance 1e-6): two slices fewer than the factorisation, each slice
    // dropped costing about two decimal digits of the gradient
    mw.slices_inv = std::max(4, slices_ - 2);
    mw.n = n;
    mw.panel = dpanel_;
    mw.panel_exp = dpanel_exp_;
    mw.rowblk = drowblk_;
    mw.rowblk_exp = drowblk_exp_;
    mw.wfull = dwfull_;
    mw.wfull_exp = dwfull_exp_;
    if (batch == 1 && dside_ && lookahead_enabled()) {
      mw.side_stream = side_st_;
      mw.ev_strip = ev_strip_;
      mw.ev_panel = ev_panel_;
      mw.side = dside_;
      mw.side_exp = dside_exp_;
      mw.side_ctas = lookahead_ctas();
    }
  }
  bool retreated = false;
  bool w_valid = false;  // W = L^-1 of the accepted factor is already in dW_
  // the covariance build and the factorisation as one launch sequence (a CUDA graph after its first run): its
  // inputs -- theta, factor, diagonal -- are read from device memory
  const bool graphs_ok = (bench == nullptr);
  auto factor_phase = [&](bool mixed) {
    const std::string key = "factor:b=" + std::to_string(batch) + ":m=" + std::to_string(mixed ? slices_ : 0) +
                            ":xe=" + std::to_string(dXb == dXe_) + ":la=" +
                            std::to_string(mixed && mw.side_stream ? mw.side_ctas : 0) + ":t=" +
                            std::to_string(oz7_tile()) + ":g=" + std::to_string(buf_gen_);
    run_phase(key, [&] {
      cov_build_lower(kernel_, n, d, dXb, xbs, dtheta_, dfactor_, ddiag_, dA_, lda_, mstride_, batch, st_, mixed,
                      dnv);
      if (mixed)
        potrf_blocked_mixed(dA_, lda_, mstride_, n, dDinv_, dinfo_, batch, mw, st_);
      else
        potrf_blocked(dA_, lda_, mstride_, n, dDinv_, dinfo_, batch, st_);
    }, graphs_ok);
  };
  for (int attempt = 0;; ++attempt) {
    LKG_CUDA(cudaMemcpyAsync(ddiag_, diag.data(), sizeof(double) * batch, cudaMemcpyHostToDevice, st_));
    if (slices_ > 0 && !retreated) {
      factor_phase(true);
      LKG_CUDA(cudaMemcpyAsync(info.data(), dinfo_, sizeof(int) * batch, cudaMemcpyDeviceToHost, st_));
      LKG_CUDA(cudaStreamSynchronize(st_));
      bool any_fail = false;
      for (int b = 0; b < batch; ++b) any_fail = any_fail || (info[b] != 0 && !dead[b]);
      if (any_fail) {  // retreat: redo this factorisation on the FP64 path before the nugget-retry rules apply
        retreated = true;
        factor_phase(false);
      }
    } else {
      factor_phase(false);
    }
    LKG_CUDA(cudaMemcpyAsync(info.data(), dinfo_, sizeof(int) * batch, cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    w_valid = false;
    if (rcond_check) {
      if (with_grad) {
        // The gradient needs W = L^-1 anyway: rcond_exact = 1 / (|L|_1 |L^-1|_1) <= the dlacn2 estimate, so
        // rcond_exact^2 >= min_rcond already decides "no retry"; only entries below it run the estimator.
        ensure_grad_buffers();
        if (slices_ > 0 && !retreated)
          trtri_blocked_mixed(dA_, lda_, mstride_, n, dDinv_, dW_, lda_, mstride_, batch, mw, st_);
        else
          trtri_blocked(dA_, lda_, mstride_, n, dDinv_, dW_, lda_, mstride_, batch, st_);
        w_valid = true;
        std::vector<double> cl((size_t)n * batch), cw((size_t)n * batch);
        lower_colsum_abs(n, dA_, lda_, mstride_, dcol_, batch, st_);
        LKG_CUDA(cudaMemcpyAsync(cl.data(), dcol_, sizeof(double) * n * batch, cudaMemcpyDeviceToHost, st_));
        lower_colsum_abs(n, dW_, lda_, mstride_, dvec_, batch, st_);
        LKG_CUDA(cudaMemcpyAsync(cw.data(), dvec_, sizeof(double) * n * batch, cudaMemcpyDeviceToHost, st_));
        LKG_CUDA(cudaStreamSynchronize(st_));
        bool need_est = false;
        for (int b = 0; b < batch; ++b) {
          double an = 0.0, wn = 0.0;
          for (int j = 0; j < nv_entry[b]; ++j) {  // the valid block's columns only
            an = std::max(an, cl[(size_t)b * n + j]);
            wn = std::max(wn, cw[(size_t)b * n + j]);
          }
          const double rc = (an > 0.0 && wn > 0.0 && std::isfinite(wn)) ? (1.0 / an) / wn : 0.0;
          rc2[b] = rc * rc;
          if (info[b] == 0 && !dead[b] && !(rc2[b] >= cfg.min_rcond)) need_est = true;
        }
        if (need_est) {
          std::vector<double> est;
          rcond_batch(batch, est, nv_entry);
          for (int b = 0; b < batch; ++b)
            if (!(rc2[b] >= cfg.min_rcond)) rc2[b] = est[b];
        }
      } else {
        rcond_batch(batch, rc2, nv_entry);
      }
    }
    bool retry = false;
    for (int b = 0; b < batch; ++b) {
      if (dead[b]) continue;
      const bool ok = info[b] == 0;
      const bool wrong = rcond_check && ok && rc2[b] < cfg.min_rcond;
      if (!ok || wrong) {
        if (plain_chol_) {
          dead[b] = 1;
          out[b].status = 1;
          out[b].message = "chol(): decomposition failed";
        } else if (inc[b] > cfg.max_inc_choldiag) {
          dead[b] = 1;
          out[b].status = 1;
          out[b].message = "[ERROR] Exceed max numerical nugget (" + std::to_string(inc[b]) + " x 1e" +
                           std::to_string(std::log10(cfg.num_nugget)) + ") added to force chol matrix";
        } else if (cfg.num_nugget <= 0.0) {
          dead[b] = 1;
          out[b].status = 1;
          out[b].message = "[ERROR] Cannot add numerical nugget which is not strictly positive: " +
                           std::to_string(cfg.num_nugget);
        } else {
          diag[b] += cfg.num_nugget * std::pow(10.0, inc[b]);
          inc[b]++;
          retry = true;
        }
      }
    }
    if (!retry) break;
  }
  for (int b = 0; b < batch; ++b) {
    out[b].nugget_increments = inc[b];
    out[b].rcond = rc2[b];
    out[b].slices = retreated ? 0 : slices_;
    out[b].retreated = retreated;
  }
  tm.lap("R = _Cov(dX) & L = Chol(R)");

  // ---- [F* y*] = L \ [F y], GLS, E*, SSE, and the gradient's R^-1 and adjoint sums: one launch sequence (a CUDA
  // graph after its first run) ----
  if (with_grad) ensure_grad_buffers();
  const bool mixed_post = slices_ > 0 && !retreated;
  const std::string post_key = "post:b=" + std::to_string(batch) + ":m=" + std::to_string(mixed_post ? slices_ : 0) +
                               ":gr=" + std::to_string(with_grad) + ":w=" + std::to_string(w_valid) + ":sa=" +
                               std::to_string(skip_adjoint_) + ":xe=" + std::to_string(dXb == dXe_) + ":t=" +
                               std::to_string(oz7_tile()) + ":g=" + std::to_string(buf_gen_);
  // [F y] of every entry's design (outside the sequence: the entries' designs change between evaluations)
  for (int b = 0; b < batch; ++b) {
    double* fy = dFY_ + (size_t)b * fystride_;
    const size_t e = entry_design_[b];
    if (p > 0)
      LKG_CUDA(cudaMemcpyAsync(fy, dF_ + e * n * p, sizeof(double) * n * p, cudaMemcpyDeviceToDevice, st_));
    LKG_CUDA(cudaMemcpyAsync(fy + (size_t)n * p, dY_ + e * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
  }
  run_phase(post_key, [&] {
    trsm_lower_left(dA_, lda_, mstride_, n, dDinv_, dFY_, n, fystride_, p + 1, batch, st_);
    tm.lap("F* = L \\ F, y* = L \\ y");
    gram_and_logdet(n, p + 1, dFY_, n, fystride_, dA_, lda_, mstride_, dgram_, gram_stride_, batch, st_);
    if (p > 0) {
      gls_solve(p, dgram_, gram_stride_, dbeta_, p, drstar_, p * p, dgls_info_, batch, st_);
    } else {
      LKG_CUDA(cudaMemsetAsync(dgls_info_, 0, sizeof(int) * batch, st_));
    }
    tm.lap("^b = R*^-1 R*'^-1 F*'y*");
    residual_sse(n, p, dFY_, n, fystride_, dbeta_, std::max(p, 1), dEstar_, n, dsse_, 1, batch, st_);
    tm.lap("z = L \\ (y - F*b), SSE = z'z");

    if (with_grad) {
      LKG_CUDA(cudaMemcpyAsync(dxv_, dEstar_, sizeof(double) * n * batch, cudaMemcpyDeviceToDevice, st_));
      trsm_lower_left_t(dA_, lda_, mstride_, n, dDinv_, dxv_, n, n, 1, batch, st_);
      tm.lap("x = tL \\ z");
      if (slices_ > 0 && !retreated) {
        if (!w_valid) trtri_blocked_mixed(dA_, lda_, mstride_, n, dDinv_, dW_, lda_, mstride_, batch, mw, st_);
        wtw_lower_mixed(dW_, lda_, mstride_, n, dRinv_, lda_, mstride_, batch, mw, st_);
      } else {
        if (!w_valid) trtri_blocked(dA_, lda_, mstride_, n, dDinv_, dW_, lda_, mstride_, batch, st_);
        wtw_lower(dW_, lda_, mstride_, n, dRinv_, lda_, mstride_, batch, st_);
      }
      tm.lap("R^-1 = L^-T * L^-1");
      if (lmp_mode_ && p > 0) {  // B = R^-1 - A'A in the lower triangle of R^-1
        build_At(batch);
        sub_aat_lower(n, p, dloo_at_, (int64_t)n * p, dRinv_, lda_, mstride_, batch, st_);
        tm.lap("B = R^-1 - RiF (F'RiF)^-1 F'Ri");
      }
      if (!skip_adjoint_) {
        adjoint_sums(kernel_, n, d, dXb, xbs, dtheta_, dfactor_, dxv_, n, dRinv_, lda_, mstride_, dpart_, dadj_, batch,
                     st_);
        tm.lap("gradR computation [optimized]");
      }
    }
  }, graphs_ok && !lmp_mode_);

  // ---- results to host ----
  std::vector<double> gram((size_t)gram_stride_ * batch), sse(batch), beta((size_t)std::max(p, 1) * batch);
  std::vector<int> gls(batch);
  std::vector<double> adj;
  LKG_CUDA(cudaMemcpyAsync(gram.data(), dgram_, sizeof(double) * gram.size(), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(sse.data(), dsse_, sizeof(double) * batch, cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(beta.data(), dbeta_, sizeof(double) * beta.size(), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(gls.data(), dgls_info_, sizeof(int) * batch, cudaMemcpyDeviceToHost, st_));
  std::vector<double> rstar((size_t)p * p * batch);
  if (p > 0)
    LKG_CUDA(cudaMemcpyAsync(rstar.data(), drstar_, sizeof(double) * rstar.size(), cudaMemcpyDeviceToHost, st_));
  const int nacc = adjoint_nacc(d);
  const bool adj_out = with_grad && !skip_adjoint_;
  if (adj_out) {
    adj.resize((size_t)nacc * batch);
    LKG_CUDA(cudaMemcpyAsync(adj.data(), dadj_, sizeof(double) * adj.size(), cudaMemcpyDeviceToHost, st_));
  }
  LKG_CUDA(cudaStreamSynchronize(st_));
  if (slices_ > 0 && oz7_error_and_reset())
    throw std::runtime_error("mixed path: a tensor-core digit product did not complete (timed out)");
  for (int b = 0; b < batch; ++b) {
    EvalOut& o = out[b];
    if (o.status == 0 && gls[b] != 0) {
      o.status = 2;
      o.message = "chol(): decomposition failed (F*'F* not positive definite)";
    }
    o.logdet = 2.0 * gram[(size_t)b * gram_stride_ + (p + 1) * (p + 1)];
    o.sse = sse[b];
    o.rstar_logdet = 0.0;
    for (int j = 0; j < p; ++j) o.rstar_logdet += std::log(rstar[(size_t)b * p * p + j + (size_t)j * p]);
    o.beta.assign(beta.begin() + (size_t)b * std::max(p, 1), beta.begin() + (size_t)b * std::max(p, 1) + p);
    if (adj_out) {
      o.adj.assign(adj.begin() + (size_t)b * nacc, adj.begin() + (size_t)(b + 1) * nacc);
      o.adj[2 * d + 3] -= (double)(n - nv_entry[b]);  // padded R^-1 diagonal entries are exactly 1
    }
  }
}

void Engine::ensure_loo_buffers(bool with_product) {
  if (!dloo_at_) {
    buffers_changed();
    dalloc(&dloo_at_, (size_t)cap_ * n_ * std::max(p_, 1));
  }
  if (with_product && !dloo_m_) {
    buffers_changed();
    dalloc(&dloo_m_, (size_t)mstride_);
    dalloc(&dloo_vec_, (size_t)n_ * (2 * d_ + 2));
  }
}

// A' = L^-T Q* with Q* = F* Rstar^-1 (the thin QR of F*; A'A does not depend on the signs of Q*'s columns)
void Engine::build_At(int batch) {
  const int n = n_, p = p_;
  ensure_loo_buffers(false);
  for (int b = 0; b < batch; ++b)
    LKG_CUDA(cudaMemcpyAsync(dloo_at_ + (size_t)b * n * p, dFY_ + (size_t)b * fystride_, sizeof(double) * n * p,
                             cudaMemcpyDeviceToDevice, st_));
  trsm_lower_left_t(dA_, lda_, mstride_, n, dDinv_, dloo_at_, n, (int64_t)n * p, p, batch, st_);
  right_solve_upper(n, p, dloo_at_, (int64_t)n * p, drstar_, batch, st_);
}

void Engine::evaluate_lmp(int batch, const double* thetas, const double* factors, bool with_grad,
                          std::vector<EvalOut>& out) {
  if (ndesign_ != 1) throw std::invalid_argument("evaluate_lmp: engine holds several designs");
  lmp_mode_ = true;
  try {
    evaluate(batch, thetas, factors, with_grad, out, nullptr);
  } catch (...) {
    lmp_mode_ = false;
    throw;
  }
  lmp_mode_ = false;
}

void Engine::leave_one_out(int batch, const double* thetas, const double* factors, bool want_grad,
                           std::vector<LooOut>& out) {
  if (ndesign_ != 1) throw std::invalid_argument("leave_one_out: engine holds several designs");
  const int n = n_, d = d_, p = p_;
  std::vector<EvalOut> ev;
  const int saved_slices = slices_;
  slices_ = 0;
  skip_adjoint_ = true;
  try {
    evaluate(batch, thetas, factors, true, ev, nullptr);
  } catch (...) {
    slices_ = saved_slices;
    skip_adjoint_ = false;
    throw;
  }
  slices_ = saved_slices;
  skip_adjoint_ = false;
  ensure_loo_buffers(true);
  if (p > 0) build_At(batch);
  out.assign(batch, LooOut());
  for (int b = 0; b < batch; ++b) {
    LooOut& o = out[b];
    o.ev = ev[b];
    if (ev[b].status != 0) continue;
    double* Bm = dW_ + (size_t)b * mstride_;     // L^-1 is not needed any more: B goes here
    double* G = dRinv_ + (size_t)b * mstride_;   // R^-1 is consumed by B: G_k goes here
    const double* By = dxv_ + (size_t)b * n;     // L^-T E*
    double* vdiag = dloo_vec_;                   // diag(B)
    double* vby = dloo_vec_ + n;                 // By
    loo_build_B(n, p, G, lda_, dloo_at_ + (size_t)b * n * p, Bm, lda_, st_);
    LKG_CUDA(cudaMemcpy2DAsync(vdiag, sizeof(double), Bm, sizeof(double) * (lda_ + 1), sizeof(double), n,
                               cudaMemcpyDeviceToDevice, st_));
    LKG_CUDA(cudaMemcpyAsync(vby, By, sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
    if (want_grad) {
      const double* th = dtheta_ + (size_t)b * d;
      for (int k = 0; k < d; ++k) {
        loo_gradR(kernel_, n, d, dX_, th, factors[b], k, G, lda_, st_);
        gemm_tiles(n, n, n, 1.0, MatView{G, 1, lda_, 0}, MatView{Bm, 1, lda_, 0}, 0.0, dloo_m_, lda_, 0, 1, false,
                   st_);
        col_dot(n, Bm, lda_, dloo_m_, lda_, dloo_vec_ + (size_t)(2 + 2 * k) * n, st_);  // diag(B G_k B)
        col_dot(n, By, 0, dloo_m_, lda_, dloo_vec_ + (size_t)(3 + 2 * k) * n, st_);     // (G_k B)' By
      }
    }
    const int nvec = want_grad ? 2 * d + 2 : 2;
    std::vector<double> hv((size_t)n * nvec);
    LKG_CUDA(cudaMemcpyAsync(hv.data(), dloo_vec_, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    // host assembly (Kriging.cpp:411-465), n-vectors only
    const double* dg = hv.data();
    const double* by = hv.data() + n;
    o.s2.resize(n);
    o.errors.resize(n);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) {
      o.s2[i] = 1.0 / dg[i];
      o.errors[i] = o.s2[i] * by[i];
      acc += o.errors[i] * o.errors[i];
    }
    o.loo = acc / n;
    if (want_grad) {
      o.grad.assign(d, 0.0);
      for (int k = 0; k < d; ++k) {
        const double* bgb = hv.data() + (size_t)(2 + 2 * k) * n;
        const double* bgy = hv.data() + (size_t)(3 + 2 * k) * n;
        double s = 0.0;
        for (int i = 0; i < n; ++i) {
          const double diagdB = -bgb[i];
          const double ds2 = -o.s2[i] * o.s2[i] * diagdB;
          const double derr = ds2 * by[i] - o.s2[i] * bgy[i];
          s += o.errors[i] * derr;
        }
        o.grad[k] = 2.0 * s / n;
      }
    }
  }
}

void Engine::evaluate_update(const Engine& old, const double* theta, double factor, EvalOut& out) {
  wp_valid_ = false;
  const int n = n_, d = d_, p = p_, no = old.n(), nu = n_ - old.n();
  if (ndesign_ != 1 || old.ndesign() != 1 || nu < 1 || old.d() != d || old.p() != p || old.kernel() != kernel_)
    throw std::invalid_argument("Engine::evaluate_update: the new design must extend the old one");
  const Config& cfg = config();
  out = EvalOut{};
  const double one = base_diag_;
  LKG_CUDA(cudaMemcpyAsync(dtheta_, theta, sizeof(double) * d, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dfactor_, &factor, sizeof(double), cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(ddiag_, &one, sizeof(double), cudaMemcpyHostToDevice, st_));
  // R (lower) of the whole design; its leading block is then replaced by the old factor (update_cholCov restores
  // R_old there and chol_block keeps L_oo)
  cov_build_lower(kernel_, n, d, dX_, 0, dtheta_, dfactor_, ddiag_, dA_, lda_, mstride_, 1, st_, false, nullptr);
  LKG_CUDA(cudaStreamSynchronize(old.stream()));
  LKG_CUDA(cudaMemcpy2DAsync(dA_, sizeof(double) * lda_, old.dL(0), sizeof(double) * old.lda(), sizeof(double) * no,
                             no, cudaMemcpyDeviceToDevice, st_));
  double* Auo = dA_ + no;                       // rows no.., columns 0..no-1: C_uo, then L_uo
  double* Auu = dA_ + no + (int64_t)no * lda_;  // trailing block: C_uu, then S, then L_uu
  const int nbs = ceil_div(nu, NB);
  double *dT = nullptr, *dS = nullptr, *dDs = nullptr;
  struct Free {
    double** p[3];
    ~Free() {
      for (double** q : p)
        if (*q) cudaFree(*q);
    }
  } guard{{&dT, &dS, &dDs}};
  LKG_CUDA(cudaMalloc(&dT, sizeof(double) * (size_t)no * nu));
  LKG_CUDA(cudaMalloc(&dS, sizeof(double) * (size_t)nu * nu));
  LKG_CUDA(cudaMalloc(&dDs, sizeof(double) * (size_t)nbs * NB * NB));
  // Lou = L_oo \ C_ou (n_o x n_u), then L_uo = Lou'
  transpose_copy(Auo, lda_, dT, no, nu, no, st_);
  trsm_lower_left(old.dL(0), old.lda(), 0, no, old.dDinv(0), dT, no, 0, nu, 1, st_);
  transpose_copy(dT, no, Auo, lda_, no, nu, st_);
  // S = C_uu - L_uo L_uo'
  MatView a{Auo, 1, lda_, 0}, bt{Auo, lda_, 1, 0};
  gemm_tiles(nu, nu, no, -1.0, a, bt, 1.0, Auu, lda_, 0, 1, true, st_);
  LKG_CUDA(cudaMemcpy2DAsync(dS, sizeof(double) * nu, Auu, sizeof(double) * lda_, sizeof(double) * nu, nu,
                             cudaMemcpyDeviceToDevice, st_));
  // L_uu = safe_chol_lower(S): cumulative 1e-10 * 10^k jitter on S's diagonal (LinearAlgebra.cpp:68-98)
  const bool rcond_check = cfg.chol_rcond_check && !plain_chol_;
  double jitter = 0.0;
  int inc = 0, info = 0;
  double rc2 = -1.0;
  bool fallback = false;
  for (;;) {
    if (inc > 0) {
      LKG_CUDA(cudaMemcpy2DAsync(Auu, sizeof(double) * lda_, dS, sizeof(double) * nu, sizeof(double) * nu, nu,
                                 cudaMemcpyDeviceToDevice, st_));
      add_diag(Auu, lda_, nu, jitter, st_);
    }
    potrf_blocked(Auu, lda_, 0, nu, dDs, dinfo_, 1, st_);
    LKG_CUDA(cudaMemcpyAsync(&info, dinfo_, sizeof(int), cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    rc2 = -1.0;
    if (info == 0 && rcond_check) {
      std::vector<double> r;
      rcond_core(1, r, std::vector<int>{nu}, Auu, lda_, 0, nu, dDs);
      rc2 = r[0];
    }
    const bool wrong = rcond_check && info == 0 && rc2 < cfg.min_rcond;
    if (info == 0 && !wrong) break;
    if (plain_chol_ || inc > cfg.max_inc_choldiag || cfg.num_nugget <= 0.0) {
      fallback = true;
      break;
    }
    jitter += cfg.num_nugget * std::pow(10.0, inc);
    inc++;
  }
  if (fallback) {  // chol_block: "falling back to a full Cholesky factorization"
    std::vector<EvalOut> o;
    evaluate(1, theta, &factor, false, o, nullptr);
    out = o[0];
    return;
  }
  zero_upper(dA_, lda_, mstride_, n, 1, st_);
  trtri_diag_blocks(dA_, lda_, mstride_, n, dDinv_, 1, st_);
  out.nugget_increments = inc;
  out.rcond = rc2;
  entry_design_.assign(1, 0);
  // [F* y*] = L \ [F y], GLS, E*, SSE (as in evaluate)
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(dFY_, dF_, sizeof(double) * n * p, cudaMemcpyDeviceToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dFY_ + (size_t)n * p, dY_, sizeof(double) * n, cudaMemcpyDeviceToDevice, st_));
  trsm_lower_left(dA_, lda_, mstride_, n, dDinv_, dFY_, n, fystride_, p + 1, 1, st_);
  gram_and_logdet(n, p + 1, dFY_, n, fystride_, dA_, lda_, mstride_, dgram_, gram_stride_, 1, st_);
  if (p > 0)
    gls_solve(p, dgram_, gram_stride_, dbeta_, p, drstar_, p * p, dgls_info_, 1, st_);
  else
    LKG_CUDA(cudaMemsetAsync(dgls_info_, 0, sizeof(int), st_));
  residual_sse(n, p, dFY_, n, fystride_, dbeta_, std::max(p, 1), dEstar_, n, dsse_, 1, 1, st_);
  std::vector<double> gram((size_t)gram_stride_), beta((size_t)std::max(p, 1)), rstar((size_t)p * p);
  int gls = 0;
  LKG_CUDA(cudaMemcpyAsync(gram.data(), dgram_, sizeof(double) * gram.size(), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(&out.sse, dsse_, sizeof(double), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(beta.data(), dbeta_, sizeof(double) * beta.size(), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(&gls, dgls_info_, sizeof(int), cudaMemcpyDeviceToHost, st_));
  if (p > 0)
    LKG_CUDA(cudaMemcpyAsync(rstar.data(), drstar_, sizeof(double) * rstar.size(), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaStreamSynchronize(st_));
  if (gls != 0) {
    out.status = 2;
    out.message = "chol(): decomposition failed (F*'F* not positive definite)";
  }
  out.logdet = 2.0 * gram[(size_t)(p + 1) * (p + 1)];
  for (int j = 0; j < p; ++j) out.rstar_logdet += std::log(rstar[j + (size_t)j * p]);
  out.beta.assign(beta.begin(), beta.begin() + p);
}

void Engine::adopt_model(const double* L, const double* Fstar, const double* ystar, const double* Rstar,
                         const double* Estar) {
  if (ndesign_ != 1) throw std::invalid_argument("Engine::adopt_model: one design only");
  wp_valid_ = false;
  const int n = n_, p = p_;
  LKG_CUDA(cudaMemcpy2DAsync(dA_, sizeof(double) * lda_, L, sizeof(double) * n, sizeof(double) * n, n,
                             cudaMemcpyHostToDevice, st_));
  zero_upper(dA_, lda_, mstride_, n, 1, st_);
  trtri_diag_blocks(dA_, lda_, mstride_, n, dDinv_, 1, st_);
  if (p > 0) {
    LKG_CUDA(cudaMemcpyAsync(dFY_, Fstar, sizeof(double) * n * p, cudaMemcpyHostToDevice, st_));
    LKG_CUDA(cudaMemcpyAsync(drstar_, Rstar, sizeof(double) * p * p, cudaMemcpyHostToDevice, st_));
  }
  LKG_CUDA(cudaMemcpyAsync(dFY_ + (size_t)n * p, ystar, sizeof(double) * n, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dEstar_, Estar, sizeof(double) * n, cudaMemcpyHostToDevice, st_));
  entry_design_.assign(1, 0);
  LKG_CUDA(cudaStreamSynchronize(st_));
}

void Engine::model_matrices(const double* theta, double factor, std::vector<double>* R, std::vector<double>* Rinv) {
  if (ndesign_ != 1) throw std::invalid_argument("Engine::model_matrices: one design only");
  const int n = n_;
  ensure_grad_buffers();
  auto mirror = [n](std::vector<double>& M) {  // lower triangle -> full symmetric
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < j; ++i) M[i + (size_t)j * n] = M[j + (size_t)i * n];
  };
  if (R) {
    const double one = 1.0;
    LKG_CUDA(cudaMemcpyAsync(dtheta_, theta, sizeof(double) * d_, cudaMemcpyHostToDevice, st_));
    LKG_CUDA(cudaMemcpyAsync(dfactor_, &factor, sizeof(double), cudaMemcpyHostToDevice, st_));
    LKG_CUDA(cudaMemcpyAsync(ddiag_, &one, sizeof(double), cudaMemcpyHostToDevice, st_));
    cov_build_lower(kernel_, n, d_, dX_, 0, dtheta_, dfactor_, ddiag_, dW_, lda_, mstride_, 1, st_, false, nullptr);
    R->assign((size_t)n * n, 0.0);
    LKG_CUDA(cudaMemcpy2DAsync(R->data(), sizeof(double) * n, dW_, sizeof(double) * lda_, sizeof(double) * n, n,
                               cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    mirror(*R);
  }
  if (Rinv) {
    trtri_blocked(dA_, lda_, mstride_, n, dDinv_, dW_, lda_, mstride_, 1, st_);
    wtw_lower(dW_, lda_, mstride_, n, dRinv_, lda_, mstride_, 1, st_);
    Rinv->assign((size_t)n * n, 0.0);
    LKG_CUDA(cudaMemcpy2DAsync(Rinv->data(), sizeof(double) * n, dRinv_, sizeof(double) * lda_, sizeof(double) * n,
                               n, cudaMemcpyDeviceToHost, st_));
    LKG_CUDA(cudaStreamSynchronize(st_));
    mirror(*Rinv);
  }
}

void Engine::copy_model(int b, std::vector<double>* L, std::vector<double>* Fstar, std::vector<double>* ystar,
                        std::vector<double>* Rstar, std::vector<double>* Estar) const {
  const int n = n_, p = p_;
  if (L) {
    L->assign((size_t)n * n, 0.0);
    LKG_CUDA(cudaMemcpy2DAsync(L->data(), sizeof(double) * n, dA_ + (size_t)b * mstride_, sizeof(double) * lda_,
                               sizeof(double) * n, n, cudaMemcpyDeviceToHost, st_));
  }
  if (Fstar) {
    Fstar->resize((size_t)n * p);
    if (p > 0)
      LKG_CUDA(cudaMemcpyAsync(Fstar->data(), dFY_ + (size_t)b * fystride_, sizeof(double) * n * p,
                               cudaMemcpyDeviceToHost, st_));
  }
  if (ystar) {
    ystar->resize(n);
    LKG_CUDA(cudaMemcpyAsync(ystar->data(), dFY_ + (size_t)b * fystride_ + (size_t)n * p, sizeof(double) * n,
                             cudaMemcpyDeviceToHost, st_));
  }
  if (Rstar) {
    Rstar->resize((size_t)p * p);
    if (p > 0)
      LKG_CUDA(cudaMemcpyAsync(Rstar->data(), drstar_ + (size_t)b * p * p, sizeof(double) * p * p,
                               cudaMemcpyDeviceToHost, st_));
  }
  if (Estar) {
    Estar->resize(n);
    LKG_CUDA(cudaMemcpyAsync(Estar->data(), dEstar_ + (size_t)b * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                             st_));
  }
  LKG_CUDA(cudaStreamSynchronize(st_));
  if (L)  // zero the (unreferenced) upper triangle so that the host copy is trimatl(L)
    for (int j = 1; j < n; ++j)
      for (int i = 0; i < j; ++i) (*L)[i + (size_t)j * n] = 0.0;
}

}  // namespace lkg
