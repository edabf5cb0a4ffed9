// ozaki.cuh -- FP64 GEMM emulated on the bf16 tensor cores by error-free splitting (mixed-precision path).
//
// Method: Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix multiplication by using fast routines of
// matrix multiplication and its applications", Numer. Algorithms 59 (2012); the slices are taken here as balanced
// base-2^8 digits of a per-(row, 64-wide k chunk) scaled fixed-point representation:
//   x = 2^e * sum_{i=1..S} d_i 2^{-8 i},   d_i integer in [-128, 128]  (exact in bf16),
// so that every digit product is exact and every sum of at most S * 64 products stays below 2^24 -- exact in the
// FP32 accumulators of mma.sync.  Products of digits with i + j <= S + 1 are formed (S (S + 1) / 2 bf16 GEMMs per
// 64-chunk), grouped by i + j in FP32, and folded into an FP64 accumulator once per chunk.  With S = 7 the
// truncation is ~2^-52 relative to max|a_row| max|b_col| per chunk, the level of an FP64 dot product.
//
// GB300 rates that motivate it: DFMA ~1.25 TFLOP/s, bf16 mma.sync ~605 TFLOP/s (both measured).
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace lkg {

constexpr int OZ_CHUNK = 64;  // k chunk of one exponent / one FP64 fold
constexpr int OZ_MAX_SLICES = 8;

struct SplitBuf {  // planes [batch][S][nchunk][rows_pad][64] bf16, exps [batch][nchunk][rows_pad] int
  __nv_bfloat16* planes = nullptr;
  int* exps = nullptr;
  int S = 0, nchunk = 0, rows_pad = 0;
  int64_t plane_bstride = 0, exp_bstride = 0;
};

size_t split_plane_elems(int rows, int K, int S);  // bf16 elements per batch entry
size_t split_exp_elems(int rows, int K);            // ints per batch entry

// Split rows x K operand (element (r, k) at p[b*bstride + r*s_r + k*s_k]) into S digit planes.
void ozaki_split(int rows, int K, const double* p, int64_t s_r, int64_t s_k, int64_t bstride, int batch, SplitBuf& out,
                 cudaStream_t st);

// C(M x N) = beta C + alpha A B^T where A rows come from SA (M rows) and B rows from SB (N rows), over chunks
// [c0, c1) of the shared k dimension.  lower_only: skip tiles above the diagonal and write r >= c only.
void ozaki_gemm(int M, int N, int c0, int c1, double alpha, const SplitBuf& SA, int a_row0, const SplitBuf& SB,
                int b_row0, double beta, double* C, int64_t ldc, int64_t c_batch, int batch, bool lower_only,
                cudaStream_t st);

// R^-1 = W^T W lower tiles with W split by columns (SW rows = columns of W, k = rows of W):
// tile (I, J) sums chunks I .. nblk-1.
void ozaki_wtw(int n, const SplitBuf& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st);

// The same two products on the tcgen05 tensor cores (ozaki_tc.cu): 128 x 64 output tiles, TMEM accumulators.
// ozaki_gemm / ozaki_wtw route here when the tensor path is 1 (ozaki_set_tensor_path, or LK_OZAKI_TC=1).
void ozaki_gemm_tc(int M, int N, int c0, int c1, double alpha, const SplitBuf& SA, const SplitBuf& SB, double beta,
                   double* C, int64_t ldc, int64_t c_batch, int batch, bool lower_only, cudaStream_t st);
void ozaki_wtw_tc(int n, const SplitBuf& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st);
void ozaki_set_tensor_path(int tc);  // 0: mma.sync kernels, 1: tcgen05 kernels
int ozaki_tensor_path();
// 1 if a tcgen05 CTA gave up waiting for its products since the last call (then reset); synchronous
int ozaki_tc_error_and_reset();

}  // namespace lkg
