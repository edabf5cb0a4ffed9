// engine.hpp -- device-resident evaluation engine for the exact (dense) likelihood.
//
// One Engine holds one design (X, y, F) in HBM and evaluates populate_Model + the log-likelihood building blocks
// for a batch of theta values in the same launches (multistart).  It replaces, for the GPU, the seam
// KrigingImpl::populate_Model + compute_ll_grad_theta_vecs (src/lib/KrigingImpl.cpp:73-125, :855-885).
#pragma once
#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "config.hpp"

namespace lkg {

struct EvalOut {
  int status = 0;              // 0 ok; 1 Cholesky failed after max nugget increments; 2 GLS factor failed
  std::string message;         // reference-style error text when status != 0
  int nugget_increments = 0;   // numerical nugget increments used (safe_chol_lower_retry)
  double logdet = 0.0;         // 2 * sum log L_ii
  double sse = 0.0;            // Estar' Estar
  std::vector<double> beta;    // GLS beta (p)
  std::vector<double> adj;     // adjoint sums [T1(d), T2(d), U1, U2, D1, D2] (with_grad)
  double rcond = -1.0;         // rcond(L)^2 of the accepted factor (when the check ran)
  int slices = 0;              // 0: FP64 path; > 0: tensor-core digit slices used for the O(n^3) products
  bool retreated = false;      // the mixed factorisation hit a non-positive pivot and was redone in FP64
  double rstar_logdet = 0.0;   // sum log Rstar_jj, Rstar = chol_upper(F*'F*) (= chol(F' R^-1 F) of the LMP)
};

struct LooOut {
  EvalOut ev;                  // the populate_Model part (status, beta, SSE, ...)
  double loo = 0.0;            // sum(errors^2) / n
  std::vector<double> grad;    // dLOO/dtheta (want_grad)
  std::vector<double> errors;  // sigma2LOO * By
  std::vector<double> s2;      // sigma2LOO = 1 / diag(B)
};

// SMs kept for the panel work of the mixed Cholesky's look-ahead (0 turns it off, -1 = the autotuned or default
// choice per matrix size); process-wide
void set_lookahead_ctas(int c);
int lookahead_ctas_setting();
// CUDA graphs for the launch sequences of Engine::evaluate (on by default; LKG_GRAPHS=0 turns them off)
void set_graphs_enabled(bool on);
bool graphs_enabled();
std::string lookahead_tune_key(int n);
int lookahead_ctas_for(int n);

class Engine {
 public:
  // X: n x d column-major, y: n, F: n x p column-major (all host, copied to HBM).  batch_cap: max thetas per call.
  Engine(int kernel, int n, int d, int p, const double* X, const double* y, const double* F, int batch_cap);
  // ndesign designs of one size class: design e has n_valid[e] <= n points, stored as the first rows of its n-row
  // blocks X + e*n*d (n x d column-major, ld n), y + e*n, F + e*n*p, the remaining rows zero.  Every design's
  // matrices are padded to n x n with the identity, which leaves L, the solves, the log-determinant and the
  // adjoint sums of the valid block unchanged (the padded R^-1 diagonal is removed from D2).
  Engine(int kernel, int n, int d, int p, int ndesign, const double* X, const double* y, const double* F,
         const int* n_valid, int batch_cap);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  // thetas: batch x d (row b = theta of entry b); factors: batch (alpha, 1 for NoiseModel None).
  // The accepted factor L of every entry stays in HBM until the next call (see copy_model).
  // designs (host, batch entries; required when the engine holds several designs): entry b evaluates design
  // designs[b]; several entries may name the same design.
  void evaluate(int batch, const double* thetas, const double* factors, bool with_grad, std::vector<EvalOut>& out,
                std::map<std::string, double>* bench = nullptr, const int* designs = nullptr);

  // Leave-one-out objective (Kriging::_leaveOneOut, Kriging.cpp:353-468) at each theta with R = factor C + (1 -
  // factor) I (factor 1 for NoiseModel None), on the FP64 path: By = L^-T E*, A' = L^-T F* Rstar^-1, B = R^-1 - A'A, sigma2LOO = 1 / diag(B),
  // errors = sigma2LOO * By; with want_grad, per dimension k: G_k = R o dlnC_k (zero diagonal), M = G_k B,
  // diag(B G_k B) = column dots of B and M, B G_k By = M' By.  One design only.  Leaves the factor of every
  // entry in HBM like evaluate() (R^-1 and L^-1 are overwritten).
  void leave_one_out(int batch, const double* thetas, const double* factors, bool want_grad,
                     std::vector<LooOut>& out);

  // evaluate() for the marginal-posterior objective (Kriging::_logMargPost, Kriging.cpp:487-652): with with_grad the
  // adjoint sums are taken against B = R^-1 - R^-1 F (F' R^-1 F)^-1 F' R^-1 instead of R^-1, which turns
  // T2_k into tr(G_k B) / 2 and U2 into tr(C B) / 2 (compute_lmp_theta_ans, KrigingImpl.cpp:887-921).
  void evaluate_lmp(int batch, const double* thetas, const double* factors, bool with_grad, std::vector<EvalOut>& out);

  // populate_Model with the incremental factor of update_cholCov / chol_block (src/lib/LinearAlgebra.cpp:206-299).
  // The first n_o = old.n() points of this engine's design are old's, and old's entry 0 holds the factor L_oo of
  // the same (theta, factor).  L_uo = C_uo L_oo^-T; S = C_uu - L_uo L_uo^T is factored with the retry rules of
  // safe_chol_lower applied to S alone; when S cannot be factored within the retry budget the whole matrix is
  // factored from scratch instead (chol_block's fallback).  One entry, no gradient; the factor stays in entry 0
  // like evaluate().  The O(n^3) work shrinks to O(n_u n_o^2 + n_u^2 n_o + n_u^3) for n_u = n - n_o new points.
  void evaluate_update(const Engine& old, const double* theta, double factor, EvalOut& out);

  // Entry 0 takes a committed model given on the host (a loaded model file): L (n x n lower, column-major), F* (n x
  // p), y* (n), R* (p x p upper), E* (n).  The diagonal-block inverses are recomputed from L.
  void adopt_model(const double* L, const double* Fstar, const double* ystar, const double* Rstar,
                   const double* Estar);

  // Model matrices of a saved model file (host, n x n, full symmetric): R = factor C(X; theta) with unit diagonal,
  // and R^-1 = (L^-1)' L^-1 from entry 0's factor (FP64 path).
  void model_matrices(const double* theta, double factor, std::vector<double>* R, std::vector<double>* Rinv);

  // Copies of the last evaluation's state for batch entry b (host, column-major):
  //   L (n x n lower, upper part zero), Fstar (n x p), ystar (n), Rstar (p x p upper), Estar (n)
  void copy_model(int b, std::vector<double>* L, std::vector<double>* Fstar, std::vector<double>* ystar,
                  std::vector<double>* Rstar, std::vector<double>* Estar) const;

  int n() const { return n_; }
  int ndesign() const { return ndesign_; }
  int n_valid(int e) const { return nvalid_[e]; }
  int d() const { return d_; }
  int p() const { return p_; }
  int kernel() const { return kernel_; }
  int capacity() const { return cap_; }
  // plain factorisation of R with diagonal base_diag (NestedKriging's chol(R + jitter I)): no rcond check and no
  // numerical-nugget retries; a failed factorisation gives status 1
  void set_plain_chol(bool on, double base_diag = 1.0) {
    plain_chol_ = on;
    base_diag_ = base_diag;
  }
  // 0 selects the FP64 path; 4..8 the mixed path with that many bf16 digit slices (7 ~ FP64-level products)
  void set_slices(int s);
  bool lookahead_enabled() const;
  int lookahead_ctas() const;
  int slices() const { return slices_; }
  cudaStream_t stream() const { return st_; }

  // device pointers (batch entry 0 layout) for predict: factor, diagonal-block inverses, Fstar, Estar
  const double* dL(int b = 0) const { return dA_ + (size_t)b * mstride_; }
  const double* dDinv(int b = 0) const { return dDinv_ + (size_t)b * dstride_; }
  const double* dX() const { return dX_; }
  const double* dX_design(int e) const { return dX_ + (size_t)e * n_ * d_; }
  int64_t lda() const { return lda_; }
  int64_t mstride() const { return mstride_; }
  const double* dFY(int b = 0) const { return dFY_ + (size_t)b * fystride_; }
  const double* dEstar(int b = 0) const { return dEstar_ + (size_t)b * n_; }
  // solve L Z = B in place for entry b (B device, n x r, ldb)
  void solve_lower_inplace(int b, double* dB, int64_t ldb, int r) const;
  // W = L^-1 of the (single-matrix) factor, formed once per factor on the FP64 path and kept for predictions whose
  // solves run as digit products (W R_on)
  const double* factor_inverse();

 private:
  void ensure_grad_buffers();
  void ensure_loo_buffers(bool with_product);
  // A' = L^-T F* Rstar^-1 (n x p per entry, stride n p) into dloo_at_ for entries [0, batch)
  void build_At(int batch);
  void ensure_mixed_buffers(bool with_grad);
  // rcond(L)^2 per entry, dtrcon('1') style estimate on each entry's first nvb[b] rows / columns
  void rcond_batch(int batch, std::vector<double>& rc2, const std::vector<int>& nvb);
  // the same estimate for the n x n lower factors at A (lda, mstride) with diagonal-block inverses Dinv
  void rcond_core(int batch, std::vector<double>& rc2, const std::vector<int>& nvb, const double* A, int64_t lda,
                  int64_t mstride, int n, const double* Dinv);

  // Runs launch(): directly the first time a key is seen, then captured once into a CUDA graph and replayed on the
  // engine's stream (the key names everything the launch sequence depends on besides device memory contents).
  // Off when allow is false, when graphs are disabled, and while per-launch timing is on.
  void run_phase(const std::string& key, const std::function<void()>& launch, bool allow);
  void clear_graphs();
  void buffers_changed();  // a device buffer was (re)allocated: every captured graph may hold a stale address

  int kernel_, n_, d_, p_, cap_;
  int ndesign_ = 1;
  double* dWp_ = nullptr;  // factor_inverse()
  bool wp_valid_ = false;
  std::map<std::string, cudaGraphExec_t> graphs_;
  std::map<std::string, std::map<std::string, long long>> graph_launches_;
  std::set<std::string> graph_seen_, graph_refused_;
  long long buf_gen_ = 0;
  bool skip_adjoint_ = false;                      // leave_one_out needs R^-1 but not the adjoint sums
  bool lmp_mode_ = false;                          // evaluate_lmp: adjoint sums against B
  double *dloo_m_ = nullptr, *dloo_at_ = nullptr;  // leave-one-out scratch: n x n product, A' (n x p per entry)
  double* dloo_vec_ = nullptr;                     // diag(B), By and per-dimension column dots (n x (2 d + 2))
  bool plain_chol_ = false;
  double base_diag_ = 1.0;
  std::vector<int> nvalid_;               // valid points per design
  std::vector<int> entry_design_;         // design of each entry of the last evaluate
  double* dXe_ = nullptr;                 // per-entry copy of its design's X (several designs only)
  int* dnv_ = nullptr;                    // per-entry valid sizes on the device (several designs only)
  int slices_ = 0;
  void *dpanel_ = nullptr, *drowblk_ = nullptr, *dwfull_ = nullptr, *dside_ = nullptr;
  int *dpanel_exp_ = nullptr, *drowblk_exp_ = nullptr, *dwfull_exp_ = nullptr, *dside_exp_ = nullptr;
  cudaStream_t side_st_ = nullptr;  // look-ahead stream of the mixed Cholesky (single-matrix evaluations)
  cudaEvent_t ev_strip_ = nullptr, ev_panel_ = nullptr;
  int mixed_alloc_slices_ = 0;
  int64_t lda_, mstride_, dstride_, fystride_;
  cudaStream_t st_ = nullptr;
  double *dX_ = nullptr, *dY_ = nullptr, *dF_ = nullptr;
  double *dA_ = nullptr, *dDinv_ = nullptr, *dW_ = nullptr, *dRinv_ = nullptr;
  double *dFY_ = nullptr, *dEstar_ = nullptr, *dxv_ = nullptr;
  double *dtheta_ = nullptr, *dfactor_ = nullptr, *ddiag_ = nullptr;
  double *dgram_ = nullptr, *dbeta_ = nullptr, *drstar_ = nullptr, *dsse_ = nullptr;
  double *dpart_ = nullptr, *dadj_ = nullptr, *dvec_ = nullptr, *dcol_ = nullptr;
  int *dinfo_ = nullptr, *dgls_info_ = nullptr;
  size_t part_size_ = 0;
  int gram_stride_ = 0;
};

}  // namespace lkg
