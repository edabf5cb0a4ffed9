// ozaki7.cuh -- FP64 products on the tcgen05 tensor cores by error-free splitting into 7-bit digits with one exponent
// per (row, k block of up to 256 columns); see ozaki7.cu for the method and the kernel.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"

namespace lkg {

constexpr int OZ7_SUB = 64;      // k sub-chunk of one staged digit image (128 bytes per row)
constexpr int OZ7_MAX_SPB = 4;   // sub-chunks per exponent block: at most 256 columns (exact FP32 sums)
constexpr int OZ7_KB = 256;      // the k block of the trailing updates and of W^T W

// planes [batch][S][nsub][rows_pad / 128][128 x 64 bf16 swizzled image]; exps [batch][nblk][rows_pad]
struct Split7 {
  __nv_bfloat16* planes = nullptr;
  int* exps = nullptr;
  int S = 0, sub_per_blk = 0, nsub = 0, nblk = 0, rows_pad = 0;
  int64_t plane_bstride = 0, exp_bstride = 0;
};

struct Oz7Args {
  int M, N, kb0, kb1;
  double alpha, beta;
  Split7 SA, SB;
  double* C;
  int64_t ldc, c_batch;
  int lower;  // square lower product: tiles on or below the diagonal, entries r >= c
  int wtw;    // R^-1 = W^T W (lower): tile (I, J) sums the k blocks from the one holding row 128 I
  int a_row0, b_row0;  // first operand rows of A and B in their splits (multiples of 128)
};

size_t oz7_plane_elems(int rows, int K, int S);     // bf16 elements per batch entry
size_t oz7_exp_elems(int rows, int K, int kb);      // ints per batch entry
// a split descriptor over caller-owned buffers sized for rows_cap x K_cap, exponent block kb (64 .. 256)
Split7 oz7_buffer(void* planes, int* exps, int S, int rows_cap, int K_cap, int kb);

// rows x K operand, element (r, k) at p[b*bstride + r*s_r + k*s_k], into out.S digit planes
void oz7_split(int rows, int K, const double* p, int64_t s_r, int64_t s_k, int64_t bstride, int batch, Split7& out,
               cudaStream_t st);
// two operands split by one launch (the same digit count); an operand with no rows is skipped
void oz7_split2(int rows0, int K0, const double* p0, int64_t s_r0, int64_t s_k0, int64_t bstride0, Split7& out0,
                int rows1, int K1, const double* p1, int64_t s_r1, int64_t s_k1, int64_t bstride1, Split7& out1,
                int batch, cudaStream_t st);
// C(M x N) = beta C + alpha A B^T over the k blocks [kb0, kb1) (A rows from SA, B rows from SB)
void oz7_gemm(int M, int N, int kb0, int kb1, double alpha, const Split7& SA, const Split7& SB, double beta, double* C,
              int64_t ldc, int64_t c_batch, int batch, bool lower, cudaStream_t st);
// the same with the operands' rows starting at a_row0 / b_row0 of their splits (multiples of 128) and at most
// max_ctas persistent CTAs per batch entry (0: one per SM), so that work on another stream keeps some SMs
void oz7_gemm_ex(int M, int N, int kb0, int kb1, double alpha, const Split7& SA, int a_row0, const Split7& SB,
                 int b_row0, double beta, double* C, int64_t ldc, int64_t c_batch, int batch, bool lower, int max_ctas,
                 cudaStream_t st);
int oz7_sm_count();
// C = W^T W (lower) with W split by columns (rows of SW = columns of W, k = rows of W)
void oz7_wtw(int n, const Split7& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st);
// output tile width of the digit products: 32 (two TMEM accumulator sets, the default) or 64 (one set)
void oz7_set_tile(int tn);
int oz7_tile();
// 1 if a CTA gave up waiting since the last call (then reset); synchronous.  where (8 ints, optional): the first
// expired wait -- role (1, 2 producer B / A; 3, 4, 5 MMA TMEM / B / A; 6 + 16 warp epilogue), tile, k block,
// sub-chunk, digit and the role's counters
int oz7_error_and_reset(int* where = nullptr);

}  // namespace lkg
