// dense_fp64.cuh -- FP64 dense kernels for the blocked Cholesky, triangular inverse and R^-1 (sm_103a).
//
// Measured on GB300: DFMA peaks at ~1.19 TFLOP/s while DMMA (mma.sync f64) peaks at ~1.04 TFLOP/s, so the FP64
// tiles are register-blocked DFMA.  Every kernel takes a batch index from blockIdx.z and per-matrix strides so
// that multistart evaluations of one design run in the same launch.
#pragma once
#include "common.cuh"

namespace lkg {

constexpr int NB = 64;  // block size of the blocked factorisations (also the GEMM tile edge)

// Operand view for a tile GEMM: element (row r, col c) of the logical operand is p[r*sr + c*sc].
struct MatView {
  const double* p;
  int64_t sr, sc;      // element strides
  int64_t batch;       // element stride between batch entries (0 = shared)
};

// ---- launch helpers (implemented in dense_fp64.cu) ----
// C(M x N) = beta*C + alpha * A(M x K) * B(K x N)  with A, B generic views; C column-major (ldc) in place.
// lower_only: skip tiles strictly above the diagonal and write only r >= c (diagonal offset c_off - r_off).
void gemm_tiles(int M, int N, int K, double alpha, MatView A, MatView B, double beta, double* C, int64_t ldc,
                int64_t c_batch, int batch, bool lower_only, cudaStream_t st);

// One Cholesky step on the diagonal block at (k0, k0) of each batch matrix (lda, stride mstride):
// factors the nb x nb block in place and writes its inverse into Dinv (NB*NB per block, block index blk).
void potrf_diag(double* A, int64_t lda, int64_t mstride, int k0, int nb, double* Dinv, int64_t dinv_bstride,
                int blk, int* info, int batch, cudaStream_t st);

// Full blocked lower Cholesky of each batch matrix (n x n, lower triangle referenced), keeping the inverses of
// the diagonal blocks in Dinv (nblk * NB * NB per matrix).  info[b] = 1-based column of the first non-positive
// pivot, 0 on success.
void potrf_blocked(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                   cudaStream_t st);

// W = L^-1 (lower, out of place, zero above the diagonal) from L and the diagonal-block inverses.
void trtri_blocked(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W,
                   int64_t ldw, int64_t wstride, int batch, cudaStream_t st);

// C = W^T W, lower triangle (= R^-1 when W = L^-1).
void wtw_lower(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
               int batch, cudaStream_t st);

// W(k0:k0+nb, k0:k0+nb) = Dinv block blk (full NB x NB block with its zero upper part).
void copy_dinv_block(const double* Dinv, int64_t dinv_bstride, int blk, double* W, int64_t ldw, int64_t wstride,
                     int k0, int nb, int batch, cudaStream_t st);

// Mixed-precision variants (trailing updates, trtri updates and W^T W on the bf16 tensor cores by error-free
// splitting into 7-bit digit planes, see ozaki7.cuh); the diagonal blocks stay FP64.
struct MixedWorkspace {
  int slices = 7;      // digit slices of the Cholesky's trailing updates
  int slices_inv = 6;  // digit slices of the triangular inverse and W^T W (gradient only)
  void* panel = nullptr;  // bf16 planes, oz7_plane_elems(n, 256, 8) per batch entry
  int* panel_exp = nullptr;
  void* rowblk = nullptr;  // bf16 planes, same size
  int* rowblk_exp = nullptr;
  void* wfull = nullptr;  // bf16 planes, oz7_plane_elems(n, n, digits) per batch entry
  int* wfull_exp = nullptr;
  int n = 0;
  // look-ahead of the blocked Cholesky (single matrix): the next panel is factored on side_stream, on side_ctas SMs
  // kept free by the trailing update, with its splits in side / side_exp (the size of panel); off when null
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_strip = nullptr, ev_panel = nullptr;
  void* side = nullptr;
  int* side_exp = nullptr;
  int side_ctas = 0;
};
void potrf_blocked_mixed(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                         const MixedWorkspace& ws, cudaStream_t st);
void trtri_blocked_mixed(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W,
                         int64_t ldw, int64_t wstride, int batch, const MixedWorkspace& ws, cudaStream_t st);
void wtw_lower_mixed(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
                     int batch, const MixedWorkspace& ws, cudaStream_t st);

// Dinv blocks (nblk * NB * NB per matrix) of an existing lower factor L: the inverses of its NB x NB diagonal
// blocks, computed exactly as potrf_diag computes them.
void trtri_diag_blocks(const double* L, int64_t lda, int64_t mstride, int n, double* Dinv, int batch,
                       cudaStream_t st);
// D(c, r) = S(r, c) for r < rows, c < cols (column-major, leading dimensions lds, ldd)
void transpose_copy(const double* S, int64_t lds, double* D, int64_t ldd, int rows, int cols, cudaStream_t st);
// A(i, i) += v for i < n
void add_diag(double* A, int64_t lda, int n, double v, cudaStream_t st);
// A(i, j) = 0 for i < j < n in every batch matrix
void zero_upper(double* A, int64_t lda, int64_t mstride, int n, int batch, cudaStream_t st);

// Solve L X = B in place (B n x r column-major, ldb, batch stride bstride).
void trsm_lower_left(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* B,
                     int64_t ldb, int64_t bstride, int r, int batch, cudaStream_t st);
// Solve L^T X = B in place.
void trsm_lower_left_t(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* B,
                       int64_t ldb, int64_t bstride, int r, int batch, cudaStream_t st);

}  // namespace lkg
