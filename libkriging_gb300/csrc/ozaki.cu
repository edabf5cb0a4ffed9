// ozaki.cu -- FP64 GEMM emulated with bf16 mma.sync by error-free digit splitting (see ozaki.cuh for the method).
#include "ozaki.cuh"

#include "stats.hpp"

namespace lkg {

namespace {


__global__ void k_oz_split(int rows, int K, const double* __restrict__ p, int64_t s_r, int64_t s_k, int64_t bstride,
                           SplitBuf out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + warp, c = blockIdx.y;
  const int64_t b = blockIdx.z;
  if (r >= out.rows_pad) return;
  double x0 = 0.0, x1 = 0.0;
  const int k0 = c * OZ_CHUNK + lane, k1 = k0 + 32;
  if (r < rows) {
    const double* pb = p + b * bstride + (int64_t)r * s_r;
    if (k0 < K) x0 = pb[(int64_t)k0 * s_k];
    if (k1 < K) x1 = pb[(int64_t)k1 * s_k];
  }
  // Integer arithmetic on the IEEE-754 bits throughout (FP64 instructions are scarce on this part).  The chunk
  // exponent e = E + 1 with max|x| = f 2^E, f in [1/2, 1), so |x| 2^-e < 1/2; every x becomes the integer
  // V = round(x 2^(8S - e)), |V| < 2^(8S - 1), cut into S balanced base-256 digits, each in [-128, 128].
  const unsigned long long b0 = (unsigned long long)__double_as_longlong(x0) & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long b1 = (unsigned long long)__double_as_longlong(x1) & 0x7FFFFFFFFFFFFFFFull;
  unsigned long long bm = b0 > b1 ? b0 : b1;  // |x| orders as its bit pattern
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, bm, o);
    bm = ob > bm ? ob : bm;
  }
  int e = 0;
  if (bm != 0) {
    const int bx = (int)(bm >> 52);
    // E of max|x| = f 2^E: biased exponent - 1022 for a normal number; subnormals from their leading bit
    const int E = bx ? bx - 1022 : (64 - __clzll((long long)(bm & 0xFFFFFFFFFFFFFull))) - 1074;
    e = E + 1;
  }
  const int S = out.S;
  auto to_fixed = [&](double x) -> long long {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const unsigned long long ab = bits & 0x7FFFFFFFFFFFFFFFull;
    if (ab == 0) return 0;
    const int bx = (int)(ab >> 52);
    const unsigned long long mant = bx ? ((ab & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : (ab & 0xFFFFFFFFFFFFFull);
    const int ex = bx ? bx - 1075 : -1074;  // x = mant 2^ex
    const int sh = ex + 8 * S - e;          // V = mant 2^sh
    long long V;
    if (sh >= 0)
      V = (long long)(mant << sh);  // |V| < 2^(8S - 1) <= 2^63
    else if (sh > -64)
      V = (long long)((mant + (1ull << (-sh - 1))) >> (-sh));
    else
      V = 0;
    return (bits >> 63) ? -V : V;
  };
  long long V0 = to_fixed(x0), V1 = to_fixed(x1);
  __nv_bfloat16* base = out.planes + b * out.plane_bstride;
  for (int i = S - 1; i >= 0; --i) {  // least significant digit first
    const long long d0 = (i == 0) ? V0 : ((V0 + 128) & 255) - 128;
    const long long d1 = (i == 0) ? V1 : ((V1 + 128) & 255) - 128;
    V0 = (V0 - d0) >> 8;
    V1 = (V1 - d1) >> 8;
    __nv_bfloat16* row = base + (((int64_t)i * out.nchunk + c) * out.rows_pad + r) * OZ_CHUNK;
    row[lane] = __float2bfloat16_rn((float)d0);
    row[lane + 32] = __float2bfloat16_rn((float)d1);
  }
  if (lane == 0) out.exps[b * out.exp_bstride + (int64_t)c * out.rows_pad + r] = e;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::);
}

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(s));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// exact (h * 2^E) as a double for |h| < 2^53, by building the IEEE bits
__device__ __forceinline__ double ll_scaled_to_double(long long h, int E) {
  if (h == 0) return 0.0;
  const unsigned long long sgn = (h < 0) ? 0x8000000000000000ull : 0ull;
  const unsigned long long a = (unsigned long long)(h < 0 ? -h : h);
  const int lz = __clzll((long long)a);
  const int fld = (63 - lz) + 1023 + E;
  if (fld <= 0 || fld >= 2047) return ldexp((double)h, E);
  const unsigned long long mant = ((a << lz) << 1) >> 12;  // drop the leading one, keep 52 fraction bits
  return __longlong_as_double((long long)(sgn | ((unsigned long long)fld << 52) | mant));
}

struct OzArgs {
  int M, N, c0, c1;
  double alpha, beta;
  SplitBuf SA, SB;
  int a_row0, b_row0;
  double* C;
  int64_t ldc, c_batch;
  bool lower_only;
  int wtw_n;  // > 0: R^-1 = W^T W tile mode over n
};

template <int S>
__global__ void __launch_bounds__(128) k_oz_gemm(OzArgs g) {
  // [S][64 rows][64 k] bf16 per operand; the 16-byte chunk c of row r is stored at chunk c ^ (r & 7), so the
  // eight row addresses of every ldmatrix phase and of the cp.async stores hit distinct bank groups
  extern __shared__ __align__(16) unsigned char oz_smem[];
  __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(oz_smem);
  __nv_bfloat16* sB = sA + (size_t)S * 64 * 64;
  int* sea = reinterpret_cast<int*>(sB + (size_t)S * 64 * 64);  // [64]
  int* seb = sea + 64;                                          // [64]
  int m0, n0, c0 = g.c0, arow, brow;
  bool diag_tile;
  if (g.wtw_n > 0) {
    const int64_t x = blockIdx.x;
    int I = (int)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
    while ((int64_t)(I + 1) * (I + 2) / 2 <= x) ++I;
    while ((int64_t)I * (I + 1) / 2 > x) --I;
    const int J = (int)(x - (int64_t)I * (I + 1) / 2);
    m0 = I * 64;
    n0 = J * 64;
    c0 = I;
    arow = m0;
    brow = n0;
    diag_tile = (I == J);
  } else {
    m0 = blockIdx.x * 64;
    n0 = blockIdx.y * 64;
    if (g.lower_only && m0 + 63 < n0) return;
    arow = g.a_row0 + m0;
    brow = g.b_row0 + n0;
    diag_tile = g.lower_only;
  }
  const int64_t b = blockIdx.z;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int wm = w & 1, wn = w >> 1;
  const int gq = lane >> 2, tig = lane & 3;
  const __nv_bfloat16* pa = g.SA.planes + b * g.SA.plane_bstride;
  const __nv_bfloat16* pb = g.SB.planes + b * g.SB.plane_bstride;
  const int* ea = g.SA.exps + b * g.SA.exp_bstride;
  const int* eb = g.SB.exps + b * g.SB.exp_bstride;

  double acc64[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc64[i][j][q] = 0.0;

  for (int c = c0; c < g.c1; ++c) {
    // ---- stage the S digit planes of A rows [arow, arow+64) and B rows [brow, brow+64) for chunk c ----
    for (int idx = t; idx < S * 64 * 8; idx += 128) {
      const int i = idx / 512, rem = idx % 512, row = rem >> 3, seg = rem & 7;
      const __nv_bfloat16* ga = pa + (((int64_t)i * g.SA.nchunk + c) * g.SA.rows_pad + arow + row) * OZ_CHUNK + seg * 8;
      const __nv_bfloat16* gb = pb + (((int64_t)i * g.SB.nchunk + c) * g.SB.rows_pad + brow + row) * OZ_CHUNK + seg * 8;
      cp_async16(sA + ((size_t)i * 64 + row) * 64 + ((seg ^ (row & 7)) * 8), ga);
      cp_async16(sB + ((size_t)i * 64 + row) * 64 + ((seg ^ (row & 7)) * 8), gb);
    }
    if (t < 64) {
      sea[t] = ea[(int64_t)c * g.SA.rows_pad + arow + t];
      seb[t] = eb[(int64_t)c * g.SB.rows_pad + brow + t];
    }
    cp_async_wait_all();
    __syncthreads();
    int er[2][2], ec[4][2];
#pragma unroll
    for (int mb = 0; mb < 2; ++mb) {
      er[mb][0] = sea[wm * 32 + mb * 16 + gq];
      er[mb][1] = sea[wm * 32 + mb * 16 + gq + 8];
    }
#pragma unroll
    for (int nb = 0; nb < 4; ++nb) {
      ec[nb][0] = seb[wn * 32 + nb * 8 + 2 * tig];
      ec[nb][1] = seb[wn * 32 + nb * 8 + 2 * tig + 1];
    }
    // ---- diagonals dg = i + j of the digit products ----
    // Each diagonal's FP32 sum is an exact integer below 2^23; diagonals are chained in int64 by Horner in base
    // 256 over groups [2..5] and [6..S+1] (below 2^48, exact as a double) and each group is folded into the FP64
    // accumulator with one add: 2 FP64 operations per element per chunk instead of S.
    long long hacc[2][4][4];
#pragma unroll 1
    for (int dg = 2; dg <= S + 1; ++dg) {
      float acc[2][4][4];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
      const int ilo = dg - S > 1 ? dg - S : 1, ihi = dg - 1 < S ? dg - 1 : S;
#pragma unroll 1
      for (int i = ilo; i <= ihi; ++i) {
        const int j = dg - i;
        const __nv_bfloat16* A = sA + (size_t)(i - 1) * 64 * 64;
        const __nv_bfloat16* B = sB + (size_t)(j - 1) * 64 * 64;
#pragma unroll
        for (int kk = 0; kk < 64; kk += 16) {
          unsigned af[2][4], bf[4][2];
#pragma unroll
          for (int mb = 0; mb < 2; ++mb) {
            const int row = wm * 32 + mb * 16 + (lane & 7) + ((lane >> 3) & 1) * 8;
            const int chunk = (kk >> 3) + ((lane >> 4) & 1);
            ldsm_x4(af[mb][0], af[mb][1], af[mb][2], af[mb][3], A + (size_t)row * 64 + ((chunk ^ (row & 7)) * 8));
          }
#pragma unroll
          for (int nb = 0; nb < 4; nb += 2) {
            const int row = wn * 32 + nb * 8 + (lane & 7) + ((lane >> 4) & 1) * 8;
            const int chunk = (kk >> 3) + ((lane >> 3) & 1);
            ldsm_x4(bf[nb][0], bf[nb][1], bf[nb + 1][0], bf[nb + 1][1],
                    B + (size_t)row * 64 + ((chunk ^ (row & 7)) * 8));
          }
#pragma unroll
          for (int mb = 0; mb < 2; ++mb)
#pragma unroll
            for (int nb = 0; nb < 4; ++nb) mma_bf16(acc[mb][nb], af[mb], bf[nb][0], bf[nb][1]);
        }
      }
      const bool gstart = (dg == 2) || (dg == 6);
      const bool gend = (dg == 5) || (dg == S + 1);
#pragma unroll
      for (int mb = 0; mb < 2; ++mb)
#pragma unroll
        for (int nb = 0; nb < 4; ++nb)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const long long v = (long long)__float2int_rn(acc[mb][nb][q]);
            hacc[mb][nb][q] = gstart ? v : hacc[mb][nb][q] * 256 + v;
            if (gend)
              acc64[mb][nb][q] += ll_scaled_to_double(hacc[mb][nb][q], er[mb][q >> 1] + ec[nb][q & 1] - 8 * dg);
          }
    }
    __syncthreads();
  }
  // ---- epilogue ----
  double* Cb = g.C + b * g.c_batch;
  const int mrow0 = (g.wtw_n > 0) ? m0 : m0, ncol0 = n0;
#pragma unroll
  for (int mb = 0; mb < 2; ++mb)
#pragma unroll
    for (int nb = 0; nb < 4; ++nb)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = mrow0 + wm * 32 + mb * 16 + gq + (q >> 1) * 8;
        const int c = ncol0 + wn * 32 + nb * 8 + 2 * tig + (q & 1);
        if (r < g.M && c < g.N && (!diag_tile || r >= c)) {
          double* cp = Cb + r + (int64_t)c * g.ldc;
          const double v = acc64[mb][nb][q];
          *cp = (g.beta == 0.0) ? g.alpha * v : fma(g.alpha, v, g.beta * *cp);
        }
      }
}

template <int S>
void launch_oz(const OzArgs& a, dim3 grid, cudaStream_t st) {
  const size_t smem = (size_t)2 * S * 64 * 64 * sizeof(__nv_bfloat16) + 128 * sizeof(int);
  static bool attr = false;
  if (!attr) {
    LKG_CUDA(cudaFuncSetAttribute(k_oz_gemm<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  k_oz_gemm<S><<<grid, 128, smem, st>>>(a);
  LKG_LAUNCH("k_oz_gemm");
}

void dispatch_oz(int S, const OzArgs& a, dim3 grid, cudaStream_t st) {
  switch (S) {
    case 4: launch_oz<4>(a, grid, st); break;
    case 5: launch_oz<5>(a, grid, st); break;
    case 6: launch_oz<6>(a, grid, st); break;
    case 7: launch_oz<7>(a, grid, st); break;
    case 8: launch_oz<8>(a, grid, st); break;
    default: throw std::invalid_argument("ozaki: number of slices must be in [4, 8]");
  }
}

}  // namespace

// rows padded to a multiple of 128: the tcgen05 kernel stages 128-row tiles of A
size_t split_plane_elems(int rows, int K, int S) {
  const int rp = ceil_div(rows, 128) * 128, nc = ceil_div(K, OZ_CHUNK);
  return (size_t)S * nc * rp * OZ_CHUNK;
}

size_t split_exp_elems(int rows, int K) { return (size_t)ceil_div(K, OZ_CHUNK) * ceil_div(rows, 128) * 128; }

// default 3: 7-bit digits in 256-wide k blocks on tcgen05 with two-level blocked factorisations (527 ms per n = 16384
// LL + gradient evaluation, against 866 ms for path 1: tcgen05 64-wide updates with W^T W on mma.sync)
int& oz_tc_flag() {
  static int f = [] {
    const char* e = std::getenv("LK_OZAKI_TC");
    return e ? std::atoi(e) : 3;
  }();
  return f;
}

void ozaki_set_tensor_path(int tc) { oz_tc_flag() = (tc < 0 || tc > 3) ? 1 : tc; }
int ozaki_tensor_path() { return oz_tc_flag(); }

void ozaki_split(int rows, int K, const double* p, int64_t s_r, int64_t s_k, int64_t bstride, int batch, SplitBuf& out,
                 cudaStream_t st) {
  out.rows_pad = ceil_div(rows, 128) * 128;
  out.nchunk = ceil_div(K, OZ_CHUNK);
  if (out.plane_bstride == 0) out.plane_bstride = (int64_t)split_plane_elems(rows, K, out.S);
  if (out.exp_bstride == 0) out.exp_bstride = (int64_t)split_exp_elems(rows, K);
  dim3 grid(out.rows_pad / 8, out.nchunk, batch);
  LaunchTimer lt("k_oz_split", st, 0.0, ((double)rows * K * (8.0 + 2.0 * out.S)) * batch);
  k_oz_split<<<grid, 256, 0, st>>>(rows, K, p, s_r, s_k, bstride, out);
  LKG_LAUNCH("k_oz_split");
}

void ozaki_gemm(int M, int N, int c0, int c1, double alpha, const SplitBuf& SA, int a_row0, const SplitBuf& SB,
                int b_row0, double beta, double* C, int64_t ldc, int64_t c_batch, int batch, bool lower_only,
                cudaStream_t st) {
  if (M <= 0 || N <= 0 || c1 <= c0) return;
  if (SA.S != SB.S) throw std::invalid_argument("ozaki_gemm: operands split with different slice counts");
  if (oz_tc_flag() && a_row0 == 0 && b_row0 == 0) {
    ozaki_gemm_tc(M, N, c0, c1, alpha, SA, SB, beta, C, ldc, c_batch, batch, lower_only, st);
    return;
  }
  OzArgs a{M, N, c0, c1, alpha, beta, SA, SB, a_row0, b_row0, C, ldc, c_batch, lower_only, 0};
  dim3 grid(ceil_div(M, 64), ceil_div(N, 64), batch);
  const double K = (double)(c1 - c0) * OZ_CHUNK;
  const double fl = (lower_only && M == N) ? K * M * (M + 1.0) : 2.0 * M * N * K;
  // flops recorded = the bf16 tensor work executed: S (S + 1) / 2 digit GEMMs of the FP64-equivalent product
  LaunchTimer lt("k_oz_gemm", st, fl * batch * SA.S * (SA.S + 1) / 2.0,
                 8.0 * ((beta == 0.0) ? 1.0 : 2.0) * M * N * batch);
  dispatch_oz(SA.S, a, grid, st);
}

void ozaki_wtw(int n, const SplitBuf& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st) {
  // W^T W sums many chunks per tile, which the mma.sync kernel folds in registers; the tcgen05 form adds every
  // chunk into C and measured slower (209 vs 150 ms at n = 16384), so it is used only on request (tensor path 2)
  if (oz_tc_flag() == 2) {
    ozaki_wtw_tc(n, SW, C, ldc, cstride, batch, st);
    return;
  }
  const int nblk = ceil_div(n, 64);
  const int64_t ntiles = (int64_t)nblk * (nblk + 1) / 2;
  OzArgs a{n, n, 0, SW.nchunk, 1.0, 0.0, SW, SW, 0, 0, C, ldc, cstride, false, n};
  LaunchTimer lt("k_oz_wtw", st, (double)n * (n + 1.0) * (n + 2.0) / 3.0 * batch * SW.S * (SW.S + 1) / 2.0,
                 8.0 * n * (n + 1.0) * batch);
  dispatch_oz(SW.S, a, dim3((unsigned)ntiles, 1, batch), st);
}

}  // namespace lkg
