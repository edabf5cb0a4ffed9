// lik_kernels.cuh -- covariance build, adjoint gradient and likelihood reductions (sm_103a).
#pragma once
#include "common.cuh"

namespace lkg {

// Number of adjoint accumulators for input dimension d:
//   [0, d)      T1_k = sum_{i>j} x_i x_j R_ij dlnC_k
//   [d, 2d)     T2_k = sum_{i>j} Rinv_ij R_ij dlnC_k
//   2d          U1   = sum_{i>j} x_i x_j C_ij          (C = correlation without the nugget factor)
//   2d+1        U2   = sum_{i>j} Rinv_ij C_ij
//   2d+2        D1   = sum_i x_i^2
//   2d+3        D2   = sum_i Rinv_ii
inline int adjoint_nacc(int d) { return 2 * d + 4; }

// Lower triangle (and diagonal) of R = factor * C(X) with R_ii = diag[b], for each batch entry b (theta stride d).
// X: n x d column-major (ldx = n), shared by the batch when x_bstride = 0.  fast = false evaluates the reference's
// formulas in its operation order (FP64 path); fast = true the division- and log1p-free forms (mixed path).
// nvalid (device, per entry, optional): entry b uses only its first nvalid[b] points; rows and columns beyond are
// written as the identity, so that the factor, solves and log-determinant of the padded matrix equal those of the
// valid block.
void cov_build_lower(int kernel, int n, int d, const double* X, int64_t x_bstride, const double* theta,
                     const double* factor, const double* diag, double* A, int64_t lda, int64_t mstride, int batch,
                     cudaStream_t st, bool fast = false, const int* nvalid = nullptr);

// Rectangular cross-correlation R_on(i, j) = factor * C(Xo_i - Xn_j) (n_o x q, column-major, ldr = n_o);
// with snap_coincident, coincident points (all |dx| <= eps) get 1.0 as in KrigingImpl::predict_impl; without it
// every entry is the formula (LinearAlgebra::covMat_rect).
void cov_cross(int kernel, int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta,
               double factor, double* R, cudaStream_t st, bool snap_coincident = true);

// Derivatives of R_on with respect to the new points: DR(j, c d + k) = R_on(j, c) dlnC/dx_k (Xn_c - Xo_j), n_o x (q d)
// column-major (ld n_o), R_on as cov_cross forms it with snap_coincident.
void dcov_cross(int kernel, int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta,
                double factor, double* DR, cudaStream_t st);

// Adjoint partial sums over the strict lower triangle (+ diagonal terms), one partial per 64x64 tile,
// then a deterministic fixed-order reduction into out[b * nacc + a].
void adjoint_sums(int kernel, int n, int d, const double* X, int64_t x_bstride, const double* theta,
                  const double* factor, const double* xv, int64_t xv_bstride, const double* Rinv, int64_t ldr,
                  int64_t rstride, double* partials, double* out, int batch, cudaStream_t st);
size_t adjoint_partials_size(int n, int d, int batch);  // doubles

// All column-pair dot products of M (n x ncols, ldm, batch stride mstride): out[b][q1 * ncols + q2] for q1 >= q2,
// plus out[b][ncols * ncols] = sum_i log(L_ii) of the factor L (ldl, lstride).  Deterministic.
void gram_and_logdet(int n, int ncols, const double* Mat, int64_t ldm, int64_t mstride, const double* L, int64_t ldl,
                     int64_t lstride, double* out, int64_t out_bstride, int batch, cudaStream_t st);

// GLS on the (p+1) x (p+1) Gram matrix [F* y*]'[F* y*] held in gram (row q1, col q2, q1 >= q2 filled):
// Rstar = chol_upper(F*'F*), beta = Rstar \ (Rstar' \ F*'y*).  res[b*res_stride + 0..p) = beta, Rstar to rstar.
void gls_solve(int p, const double* gram, int64_t gram_bstride, double* beta, int64_t beta_bstride, double* rstar,
               int64_t rstar_bstride, int* gls_info, int batch, cudaStream_t st);

// Estar = y* - F* beta, and sse[b] = Estar . Estar (deterministic).
void residual_sse(int n, int p, const double* FY, int64_t ldfy, int64_t fystride, const double* beta,
                  int64_t beta_bstride, double* Estar, int64_t estride, double* sse, int64_t sse_bstride, int batch,
                  cudaStream_t st);

// 1-norm of each column of the lower-triangular L (for the 1-norm condition estimate): colsum[b*n + j].
void lower_colsum_abs(int n, const double* L, int64_t ldl, int64_t lstride, double* colsum, int batch,
                      cudaStream_t st);

// ---- leave-one-out (Kriging.cpp:353-468) ----
// G(i, j) = R(i, j) dlnC/dtheta_k (x_i - x_j) for i != j with R(i, j) = factor C(x_i - x_j), G(i, i) = 0;
// full n x n, ld ldg; the reference's formulas.
void loo_gradR(int kernel, int n, int d, const double* X, const double* theta, double factor, int k, double* G,
               int64_t ldg, cudaStream_t st);
// full symmetric B = R^-1 - A'A from the lower triangle of R^-1 (ldr) and At = A' (n x p, column-major, ld n)
void loo_build_B(int n, int p, const double* Rinv, int64_t ldr, const double* At, double* B, int64_t ldb,
                 cudaStream_t st);
// At = H Rstar^-1 in place (H n x p, ld n, batch stride hstride; Rstar p x p upper, column-major, batch stride p*p)
void right_solve_upper(int n, int p, double* H, int64_t hstride, const double* Rstar, int batch, cudaStream_t st);
// lower triangle of C (ldc, batch stride cstride) -= At At' (At n x p, ld n, batch stride atstride)
void sub_aat_lower(int n, int p, const double* At, int64_t atstride, double* C, int64_t ldc, int64_t cstride,
                   int batch, cudaStream_t st);
// out[i] = sum_j B(j, i) M(j, i) (one warp per column, fixed order)
void col_dot(int n, const double* B, int64_t ldb, const double* M, int64_t ldm, double* out, cudaStream_t st);

}  // namespace lkg
