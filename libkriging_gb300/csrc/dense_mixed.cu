// dense_mixed.cu -- blocked Cholesky / triangular inverse / W^T W with the O(n^3) products on the bf16 tensor cores
// (error-free splitting into 7-bit digits, ozaki7.cuh).  The diagonal-block factorisations and inverses stay FP64.
#include "dense_fp64.cuh"
#include "ozaki7.cuh"

namespace lkg {

namespace {

// digits of the 7-bit split of the factorisation for a given count of 8-bit slices: the same operand precision, one
// digit more (6 .. 8)
int oz7_digits(int slices) { return std::min(8, std::max(6, slices + 1)); }
// digits of the triangular inverse and of W^T W, which feed only the gradient: as many 7-bit digits as the inverse
// has 8-bit slices (5 .. 8)
int oz7_inv_digits(int slices_inv) { return std::min(8, std::max(5, slices_inv)); }

// Two-level blocked Cholesky: 256-wide panels factored in 64-wide steps (FP64 diagonal block; panel solve and the update
// of the panel's remaining columns as 64-deep digit products), then one rank-256 trailing update per panel.  Every
// product reads split copies of its operands, so the in-place ones (the panel solve) are safe.
//
// Look-ahead (single matrix, ws.side_stream set): the trailing update of panel p is cut into the strip of panel p + 1's
// columns and the rest.  After the strip, panel p + 1 is factored on the side stream -- its diagonal blocks, splits
// and small products on ws.side_ctas SMs -- while the rest of the update runs on the other SMs; the main stream
// waits for the panel before splitting it.  Every entry receives the same operations either way, so the factor is
// bit-identical with and without the look-ahead.
void factor_panel7(double* A, int64_t lda, int64_t mstride, int n, int K0, double* Dinv, int* info, int batch,
                   Split7& SA, Split7& SD, int max_ctas, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  const int W = std::min(OZ7_KB, n - K0);
  for (int k0 = K0; k0 < K0 + W; k0 += NB) {
    const int nb = std::min(NB, n - k0), k = k0 / NB;
    potrf_diag(A, lda, mstride, k0, nb, Dinv, dstride, k, info, batch, st);
    const int M = n - k0 - nb;
    if (M <= 0) continue;
    double* A21 = A + (k0 + nb) + (int64_t)k0 * lda;
    // L21 = A21 Dinv_k^T: B rows are the rows of Dinv_k
    oz7_split2(M, nb, A21, 1, lda, mstride, SA, nb, nb, Dinv + (int64_t)k * NB * NB, 1, NB, dstride, SD, batch, st);
    oz7_gemm_ex(M, nb, 0, 1, 1.0, SA, 0, SD, 0, 0.0, A21, lda, mstride, batch, false, max_ctas, st);
    const int wr = K0 + W - (k0 + nb);  // panel columns right of this block
    if (wr > 0) {  // A(k0+nb:, k0+nb:K0+W) -= L21 L21(0:wr, :)^T (the strict upper part written is never read)
      oz7_split(M, nb, A21, 1, lda, mstride, batch, SA, st);
      oz7_gemm_ex(M, wr, 0, 1, -1.0, SA, 0, SA, 0, 1.0, A21 + (int64_t)nb * lda, lda, mstride, batch, false,
                  max_ctas, st);
    }
  }
}

void potrf_blocked_mixed7(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                          const MixedWorkspace& ws, cudaStream_t st) {
  LKG_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
  const int S = oz7_digits(ws.slices);
  Split7 P = oz7_buffer(ws.panel, ws.panel_exp, S, ws.n, OZ7_KB, OZ7_KB);
  Split7 SA = oz7_buffer(ws.panel, ws.panel_exp, S, ws.n, NB, NB);
  Split7 SD = oz7_buffer(ws.rowblk, ws.rowblk_exp, S, ws.n, NB, NB);
  const bool ahead = ws.side_stream && batch == 1;
  if (!ahead) {
    for (int K0 = 0; K0 < n; K0 += OZ7_KB) {
      const int W = std::min(OZ7_KB, n - K0);
      factor_panel7(A, lda, mstride, n, K0, Dinv, info, batch, SA, SD, 0, st);
      const int M2 = n - K0 - W;
      if (M2 <= 0) continue;
      // A22 -= P2 P2^T, P2 = L(K0+W:, K0:K0+W), one 256-wide k block
      double* P2 = A + (K0 + W) + (int64_t)K0 * lda;
      oz7_split(M2, W, P2, 1, lda, mstride, batch, P, st);
      oz7_gemm(M2, M2, 0, 1, -1.0, P, P, 1.0, P2 + (int64_t)W * lda, lda, mstride, batch, true, st);
    }
    return;
  }
  // the side stream's panel splits have their own buffer: the main stream's trailing update still reads P (the
  // Dinv splits in rowblk are used by one stream at a time)
  Split7 SAs = oz7_buffer(ws.side, ws.side_exp, S, ws.n, NB, NB);
  const int rest_ctas = std::max(1, oz7_sm_count() - ws.side_ctas);
  factor_panel7(A, lda, mstride, n, 0, Dinv, info, batch, SA, SD, 0, st);
  for (int K0 = 0; K0 < n; K0 += OZ7_KB) {
    const int W = std::min(OZ7_KB, n - K0);
    const int M2 = n - K0 - W;
    if (M2 <= 0) break;
    double* P2 = A + (K0 + W) + (int64_t)K0 * lda;
    oz7_split(M2, W, P2, 1, lda, mstride, batch, P, st);
    const int W1 = std::min(OZ7_KB, M2);  // the next panel's width
    // the strip of the next panel's columns: A(K0+W:, K0+W:K0+W+W1) -= P2 P2(0:W1, :)^T
    oz7_gemm_ex(M2, W1, 0, 1, -1.0, P, 0, P, 0, 1.0, P2 + (int64_t)W * lda, lda, mstride, batch, false, 0, st);
    const int M3 = M2 - W1;
    if (M3 <= 0) {  // the last panel: nothing left to overlap with
      factor_panel7(A, lda, mstride, n, K0 + W, Dinv, info, batch, SA, SD, 0, st);
      continue;
    }
    LKG_CUDA(cudaEventRecord(ws.ev_strip, st));
    LKG_CUDA(cudaStreamWaitEvent(ws.side_stream, ws.ev_strip, 0));
    factor_panel7(A, lda, mstride, n, K0 + W, Dinv, info, batch, SAs, SD, ws.side_ctas, ws.side_stream);
    LKG_CUDA(cudaEventRecord(ws.ev_panel, ws.side_stream));
    // the rest of the update, lower: A(K0+W+W1:, K0+W+W1:) -= P2(W1:, :) P2(W1:, :)^T
    oz7_gemm_ex(M3, M3, 0, 1, -1.0, P, W1, P, W1, 1.0, P2 + W1 + (int64_t)(W + W1) * lda, lda, mstride, batch, true,
                rest_ctas, st);
    LKG_CUDA(cudaStreamWaitEvent(st, ws.ev_panel, 0));
  }
}

// The 64-wide steps of one 256-row block of the triangular inverse (rows K0 .. K0 + Wd): D^-1 blocks onto the
// diagonal, W(k0:k0+nb, 0:k0) = -Dinv_k Acc(k0:k0+nb, 0:k0), then the block's rows below accumulate
// L(k0+nb:, k0:k0+nb) W(k0:k0+nb, 0:k0+nb).
void trtri_block7(const double* L, int64_t lda, int64_t mstride, int n, int K0, int Wd, const double* Dinv,
                  int64_t dstride, double* W, int64_t ldw, int64_t wstride, int batch, Split7& SA, Split7& SB,
                  cudaStream_t st) {
  for (int k0 = K0; k0 < K0 + Wd; k0 += NB) {
    const int nb = std::min(NB, n - k0), k = k0 / NB;
    copy_dinv_block(Dinv, dstride, k, W, ldw, wstride, k0, nb, batch, st);
    if (k0 > 0) {  // W(k0:k0+nb, 0:k0) = -Dinv_k Acc(k0:k0+nb, 0:k0): B rows are the columns of Acc
      oz7_split2(nb, nb, Dinv + (int64_t)k * NB * NB, 1, NB, dstride, SA, k0, nb, W + k0, ldw, 1, wstride, SB,
                 batch, st);
      oz7_gemm(nb, k0, 0, 1, -1.0, SA, SB, 0.0, W + k0, ldw, wstride, batch, false, st);
    }
    const int mr = K0 + Wd - (k0 + nb);  // rows of this 256-row block below the 64-row one
    if (mr > 0) {  // Acc(k0+nb:K0+Wd, 0:k0+nb) += L(k0+nb:K0+Wd, k0:k0+nb) W(k0:k0+nb, 0:k0+nb)
      oz7_split2(mr, nb, L + (k0 + nb) + (int64_t)k0 * lda, 1, lda, mstride, SA, k0 + nb, nb, W + k0, ldw, 1,
                 wstride, SB, batch, st);
      oz7_gemm(mr, k0 + nb, 0, 1, 1.0, SA, SB, 1.0, W + k0 + nb, ldw, wstride, batch, false, st);
    }
  }
}

// Two-level triangular inverse: inside a 256-row block the 64-wide steps, below it one rank-256 update of the
// accumulated rows; every product on the digit kernel.  (A look-ahead like the Cholesky's -- the next block's 64-wide
// steps on a side stream while the rest of the update runs -- measured 1.9 ms slower per n = 16384 evaluation: the
// steps' wide products need most of the SMs, so it is not used here.)
void trtri_blocked_mixed7(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W,
                          int64_t ldw, int64_t wstride, int batch, const MixedWorkspace& ws, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  for (int b = 0; b < batch; ++b)
    LKG_CUDA(cudaMemset2DAsync(W + b * wstride, ldw * sizeof(double), 0, n * sizeof(double), n, st));
  const int S = oz7_inv_digits(ws.slices_inv);
  Split7 SL = oz7_buffer(ws.panel, ws.panel_exp, S, ws.n, OZ7_KB, OZ7_KB);
  Split7 SR = oz7_buffer(ws.rowblk, ws.rowblk_exp, S, ws.n, OZ7_KB, OZ7_KB);
  Split7 SA = oz7_buffer(ws.panel, ws.panel_exp, S, ws.n, NB, NB);
  Split7 SB = oz7_buffer(ws.rowblk, ws.rowblk_exp, S, ws.n, NB, NB);
  for (int K0 = 0; K0 < n; K0 += OZ7_KB) {
    const int Wd = std::min(OZ7_KB, n - K0);
    trtri_block7(L, lda, mstride, n, K0, Wd, Dinv, dstride, W, ldw, wstride, batch, SA, SB, st);
    const int M2 = n - K0 - Wd;
    if (M2 <= 0) continue;
    // Acc(K0+Wd:, 0:N) += L(K0+Wd:, K0:K0+Wd) W(K0:K0+Wd, 0:N), N = K0 + Wd
    const int N = K0 + Wd;
    oz7_split2(M2, Wd, L + (K0 + Wd) + (int64_t)K0 * lda, 1, lda, mstride, SL, N, Wd, W + K0, ldw, 1, wstride, SR,
               batch, st);
    oz7_gemm(M2, N, 0, 1, 1.0, SL, SR, 1.0, W + K0 + Wd, ldw, wstride, batch, false, st);
  }
}

void wtw_lower_mixed7(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
                      int batch, const MixedWorkspace& ws, cudaStream_t st) {
  Split7 SW = oz7_buffer(ws.wfull, ws.wfull_exp, oz7_inv_digits(ws.slices_inv), ws.n, ws.n, OZ7_KB);
  oz7_split(n, n, W, ldw, 1, wstride, batch, SW, st);  // rows of the split = columns of W, k = rows of W
  oz7_wtw(n, SW, C, ldc, cstride, batch, st);
}

}  // namespace

void potrf_blocked_mixed(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                         const MixedWorkspace& ws, cudaStream_t st) {
  potrf_blocked_mixed7(A, lda, mstride, n, Dinv, info, batch, ws, st);
}

void trtri_blocked_mixed(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W,
                         int64_t ldw, int64_t wstride, int batch, const MixedWorkspace& ws, cudaStream_t st) {
  trtri_blocked_mixed7(L, lda, mstride, n, Dinv, W, ldw, wstride, batch, ws, st);
}

void wtw_lower_mixed(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
                     int batch, const MixedWorkspace& ws, cudaStream_t st) {
  wtw_lower_mixed7(W, ldw, wstride, n, C, ldc, cstride, batch, ws, st);
}

}  // namespace lkg
