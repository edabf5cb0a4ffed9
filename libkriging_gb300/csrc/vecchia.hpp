// vecchia.hpp -- Vecchia approximated log-likelihood (objective "LLVecchia(m)") on the GPU.
//
// Reference: Kriging::make_vecchia_sets (src/lib/Kriging.cpp:736-804) and Kriging::_logLikelihoodVecchia
// (src/lib/Kriging.cpp:806-924).  One warp per ordered point builds its (m x m) conditional block, factors it with
// the numerical-nugget retry and rcond rules of safe_chol_lower, and produces u, v, W and their theta-derivatives;
// deterministic block reductions then give the GLS beta, sigma2, VLL and the envelope-theorem gradient.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace lkg {

constexpr int VECCHIA_MAX_M = 32;

struct VecchiaOut {
  double vll = 0.0, sigma2 = 0.0;
  std::vector<double> beta, grad;
  int status = 0;  // 0 ok, 1 a conditional block stayed non-SPD after the nugget increments
  std::string message;
  long long nugget_points = 0;  // conditionals that needed numerical-nugget increments
};

class VecchiaEngine {
 public:
  // X n x d column-major (normalised), y n, F n x p column-major; order[n], nbr[n * m] (-1 padded), host arrays.
  VecchiaEngine(int kernel, int n, int d, int p, const double* X, const double* y, const double* F,
                const int32_t* order, const int32_t* nbr, int m);
  ~VecchiaEngine();
  VecchiaEngine(const VecchiaEngine&) = delete;
  VecchiaEngine& operator=(const VecchiaEngine&) = delete;

  // est_beta = false uses beta_fixed (p values), as the reference when m_est_beta is false and m_beta has p entries
  VecchiaOut evaluate(const double* theta, bool with_grad, bool est_beta, const double* beta_fixed);

  // One share of a sharded evaluation (Kriging.cpp:895-922 sums over the ordered points, split by position):
  // evaluate only the ordered positions [t0, t1) (default: all).
  void set_range(int t0, int t1);
  // stage 1 over the range: s1 = [A (p x p, row-major), b (p), sum log v] with A = sum W W'/v, b = sum W u / v;
  // returns the number of points whose conditional stayed non-SPD after the nugget increments and adds the points
  // that needed increments to *nugget_points
  int partial_sums1(const double* theta, bool with_grad, std::vector<double>& s1, long long* nugget_points);
  // stage 2 over the range, given beta (the last partial_sums1's theta): s2 = [Q, dQ_k (d), sum dv_k / v (d)]
  void partial_sums2(const double* beta, bool with_grad, std::vector<double>& s2);
  int n() const { return n_; }
  int m() const { return m_; }
  cudaStream_t stream() const { return st_; }

 private:
  int kernel_, n_, d_, p_, m_;
  cudaStream_t st_ = nullptr;
  double *dX_ = nullptr, *dY_ = nullptr, *dF_ = nullptr, *dth_ = nullptr;
  int32_t *dorder_ = nullptr, *dnbr_ = nullptr;
  double *du_ = nullptr, *dv_ = nullptr, *dW_ = nullptr, *ddu_ = nullptr, *ddv_ = nullptr, *ddW_ = nullptr;
  int* dstatus_ = nullptr;
  double *dpart_ = nullptr, *dbeta_ = nullptr;
  int nblk_red_ = 0;
  int t0_ = 0, t1_ = 0;
};

// the host steps between and after the partial sums (shared by evaluate and the sharded form): the GLS beta from the
// summed stage-1 sums (A + num_nugget I) beta = b (0, or -1 when not positive definite); sigma2 = Q / n, VLL and its
// gradient from the summed sums; the reference's message for a conditional that stayed non-SPD
int vecchia_gls_beta(int p, const std::vector<double>& s1, std::vector<double>& beta);
void vecchia_finish(int n, int d, double slogv, const std::vector<double>& s2, bool with_grad, VecchiaOut& out);
std::string vecchia_failure_message();

// GPU construction of the Vecchia sets, same definition as make_vecchia_sets: maxmin ordering from the point closest
// to the centroid (argmin / argmax ties -> lowest index), then the min(m, t) nearest earlier-ordered points by
// (squared distance, index).  X n x d column-major on the host; outputs host arrays order[n], nbr[n * m].
void vecchia_sets_gpu(int n, int d, const double* X, int m, int32_t* order, int32_t* nbr);

// The same sets from X on the device (n x d column-major; hX its host copy, for the grids' bounding box) with the
// maxmin order started at `first`, on uniform grids (vecchia_grid.cu): dorder[n], dnbr[n x min(m, n - 1)].
// Synchronises `st` before returning (its temporary buffers are freed).
void vecchia_sets_grid(int n, int d, const double* hX, const double* dX, int first, int m, int32_t* dorder,
                       int32_t* dnbr, cudaStream_t st);

// predictVecchia's local kriging (Kriging.cpp:950-1022) on the GPU: for each of the q points of Xq (q x d
// column-major, normalised), the m nearest of the n observations X (n x d column-major) by (squared distance,
// index), RN = C(N, N) + num_nugget I under the safe_chol_lower rules, a = RN^-1 r; ar[t] = a . resid_N and
// ra[t] = r . a (resid = y - F beta, n).  Throws the reference's error when a factorisation exceeds the retries.
void vecchia_predict_gpu(int kernel, int n, int d, const double* X, const double* resid, const double* theta, int q,
                         const double* Xq, int m, std::vector<double>& ar, std::vector<double>& ra);

// The same sets from device buffers, with every intermediate in one fixed device array of this library
// (SETS_SCRATCH_DOUBLES doubles) instead of allocated memory; all work is queued on `stream`, nothing is
// synchronised.  Returns nullptr on success, else a message that stays valid until the calling thread's next call.
constexpr long long SETS_SCRATCH_DOUBLES = 1LL << 20;  // 8 MiB
const char* vecchia_sets_noalloc(int n, int d, const double* X, int m, int32_t* order, int32_t* nbr,
                                 cudaStream_t stream);

}  // namespace lkg
