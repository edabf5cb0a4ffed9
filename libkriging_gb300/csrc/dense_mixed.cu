// dense_mixed.cu -- blocked Cholesky / triangular inverse / W^T W with the O(n^3) products on the bf16 tensor cores
// (error-free digit splitting, ozaki.cuh).  Same block algorithms and NB = 64 blocking as dense_fp64.cu: the
// diagonal-block factorisations and inverses, the panel solves and the small row-block products stay FP64.
#include "dense_fp64.cuh"
#include "ozaki.cuh"

namespace lkg {

namespace {

SplitBuf make_split(void* planes, int* exps, int S, int rows_cap, int K_cap) {
  SplitBuf s;
  s.planes = static_cast<__nv_bfloat16*>(planes);
  s.exps = exps;
  s.S = S;
  s.plane_bstride = (int64_t)split_plane_elems(rows_cap, K_cap, S);
  s.exp_bstride = (int64_t)split_exp_elems(rows_cap, K_cap);
  return s;
}

}  // namespace

void potrf_blocked_mixed(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                         const MixedWorkspace& ws, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  LKG_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
  SplitBuf P = make_split(ws.panel, ws.panel_exp, ws.slices, ws.n, NB);
  for (int k = 0; k < nblk; ++k) {
    const int k0 = k * NB, nb = std::min(NB, n - k0);
    potrf_diag(A, lda, mstride, k0, nb, Dinv, dstride, k, info, batch, st);
    const int M = n - k0 - nb;
    if (M <= 0) continue;
    double* A21 = A + (k0 + nb) + (int64_t)k0 * lda;
    MatView a{A21, 1, lda, mstride};
    MatView bt{Dinv + (int64_t)k * NB * NB, NB, 1, dstride};
    gemm_tiles(M, nb, nb, 1.0, a, bt, 0.0, A21, lda, mstride, batch, false, st);
    // A22 -= L21 L21^T on the tensor cores
    ozaki_split(M, nb, A21, 1, lda, mstride, batch, P, st);
    ozaki_gemm(M, M, 0, 1, -1.0, P, 0, P, 0, 1.0, A21 + (int64_t)nb * lda, lda, mstride, batch, true, st);
  }
}

void trtri_blocked_mixed(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W,
                         int64_t ldw, int64_t wstride, int batch, const MixedWorkspace& ws, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  for (int b = 0; b < batch; ++b)
    LKG_CUDA(cudaMemset2DAsync(W + b * wstride, ldw * sizeof(double), 0, n * sizeof(double), n, st));
  SplitBuf SL = make_split(ws.panel, ws.panel_exp, ws.slices_inv, ws.n, NB);
  SplitBuf SR = make_split(ws.rowblk, ws.rowblk_exp, ws.slices_inv, ws.n, NB);
  for (int k = 0; k < nblk; ++k) {
    const int k0 = k * NB, nb = std::min(NB, n - k0);
    copy_dinv_block(Dinv, dstride, k, W, ldw, wstride, k0, nb, batch, st);
    if (k0 > 0) {
      MatView d{Dinv + (int64_t)k * NB * NB, 1, NB, dstride};
      MatView acc{W + k0, 1, ldw, wstride};
      gemm_tiles(nb, k0, nb, -1.0, d, acc, 0.0, W + k0, ldw, wstride, batch, false, st);
    }
    const int M2 = n - k0 - nb;
    if (M2 > 0) {
      // Acc(k0+nb:, 0:k0+nb) += L(k0+nb:, k0:k0+nb) W(k0:k0+nb, 0:k0+nb) on the tensor cores
      const int N = k0 + nb;
      ozaki_split(M2, nb, L + (k0 + nb) + (int64_t)k0 * lda, 1, lda, mstride, batch, SL, st);
      ozaki_split(N, nb, W + k0, ldw, 1, wstride, batch, SR, st);
      ozaki_gemm(M2, N, 0, 1, 1.0, SL, 0, SR, 0, 1.0, W + k0 + nb, ldw, wstride, batch, false, st);
    }
  }
}

void wtw_lower_mixed(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
                     int batch, const MixedWorkspace& ws, cudaStream_t st) {
  SplitBuf SW = make_split(ws.wfull, ws.wfull_exp, ws.slices_inv, ws.n, ws.n);
  // rows of the split = columns of W, k = rows of W
  ozaki_split(n, n, W, ldw, 1, wstride, batch, SW, st);
  ozaki_wtw(n, SW, C, ldc, cstride, batch, st);
}

}  // namespace lkg
