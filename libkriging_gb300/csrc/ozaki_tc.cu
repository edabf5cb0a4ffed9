// ozaki_tc.cu -- the digit-product GEMM of the mixed path on the 5th-generation tensor cores (tcgen05).
//
// Same split operands and the same exact arithmetic as k_oz_gemm (ozaki.cu): per 64-wide k chunk, digit products
// with i + j <= S + 1 accumulate per diagonal i + j in FP32 (exact integers), and every diagonal is folded into
// FP64 with the chunk's row and column exponents.  Here one CTA (4 warps) owns a 128 x 64 output tile:
//   * all 128 threads stage the S digit planes of A (128 rows) and B (64 rows) with cp.async, in the 128-byte
//     swizzled K-major layout (16-byte chunk c of row r at c ^ (r & 7), 1024-byte aligned 8-row atoms),
//   * one thread issues tcgen05.mma (M = 128, N = 64, K = 16, bf16 -> FP32) with the S diagonal accumulators in
//     TMEM (S x 64 columns) and commits them to an mbarrier,
//   * the 4 warps read their 32 TMEM lanes (rows) with tcgen05.ld, fold the diagonals (int64 Horner groups
//     [2..5], [6..S+1]) and add the chunk's contribution into C.
// Every wait on the mbarrier is bounded: on expiry the CTA records an error, frees its TMEM and returns.
#include "ozaki.cuh"

#include "stats.hpp"

namespace lkg {

namespace {

constexpr int TC_M = 128, TC_N = 64;
constexpr uint32_t kWaitLimit = 1u << 24;  // mbarrier polls before a CTA gives up (each poll may suspend)

__device__ int g_oz_tc_error;  // set to 1 by a CTA whose mbarrier wait expired

// instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TC_N >> 3) << 17) |
                            ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle (layout type 2), stride between 8-row atoms 1024 B,
// leading-byte offset unused by this layout (0), descriptor version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(1024u >> 4) << 32) | ((uint64_t)1u << 46) |
         ((uint64_t)2u << 61);
}

__device__ __forceinline__ void cp16(uint32_t s, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(g));
}

__device__ __forceinline__ void mma_issue(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_poll(uint32_t m, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(m), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(uint32_t m, uint32_t phase) {
  for (uint32_t it = 0; it < kWaitLimit; ++it)
    if (mbar_poll(m, phase)) return true;
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ double ll_to_double(long long h, int E) {  // exact h * 2^E for |h| < 2^53
  if (h == 0) return 0.0;
  const unsigned long long sgn = (h < 0) ? 0x8000000000000000ull : 0ull;
  const unsigned long long a = (unsigned long long)(h < 0 ? -h : h);
  const int lz = __clzll((long long)a);
  const int fld = (63 - lz) + 1023 + E;
  if (fld <= 0 || fld >= 2047) return ldexp((double)h, E);
  const unsigned long long mant = ((a << lz) << 1) >> 12;
  return __longlong_as_double((long long)(sgn | ((unsigned long long)fld << 52) | mant));
}

struct TcArgs {
  int M, N, c0, c1;
  double alpha, beta;
  SplitBuf SA, SB;
  double* C;
  int64_t ldc, c_batch;
  bool lower_only;
  int wtw_n;  // > 0: R^-1 = W^T W lower tiles (linear tile index, chunks from the tile's row block)
};

template <int S>
__global__ void __launch_bounds__(128, 1) k_oz_tc(TcArgs g) {
  constexpr int NCOLS = (S * TC_N <= 256) ? 256 : 512;
  extern __shared__ unsigned char tc_raw[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  // 1024-byte aligned operand area
  const uint32_t raw = su32(tc_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char* smp = tc_raw + (base - raw);
  const uint32_t sA = base;                                // S x 128 rows x 128 B
  const uint32_t sB = base + (uint32_t)S * TC_M * 128;     // S x 64 rows x 128 B
  int* sea = reinterpret_cast<int*>(smp + (size_t)S * (TC_M + TC_N) * 128);
  int* seb = sea + TC_M;

  int m0, n0, c0 = g.c0;
  if (g.wtw_n > 0) {
    // lower tiles in row-major order: row block I (128 rows) holds column blocks J = 0 .. 2I+1 (64 columns)
    const long long x = blockIdx.x;
    int I = (int)((sqrt(4.0 * (double)x + 1.0) - 1.0) * 0.5);
    while ((long long)(I + 1) * (I + 2) <= x) ++I;
    while ((long long)I * (I + 1) > x) --I;
    m0 = I * TC_M;
    n0 = (int)(x - (long long)I * (I + 1)) * TC_N;
    c0 = 2 * I;
  } else {
    m0 = blockIdx.x * TC_M;
    n0 = blockIdx.y * TC_N;
  }
  if (m0 >= g.M || n0 >= g.N) return;
  if ((g.lower_only || g.wtw_n > 0) && m0 + TC_M - 1 < n0) return;
  const bool lower = g.lower_only || g.wtw_n > 0;
  const int64_t b = blockIdx.z;
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const __nv_bfloat16* pa = g.SA.planes + b * g.SA.plane_bstride;
  const __nv_bfloat16* pb = g.SB.planes + b * g.SB.plane_bstride;
  const int* ea = g.SA.exps + b * g.SA.exp_bstride;
  const int* eb = g.SB.exps + b * g.SB.exp_bstride;
  const uint32_t mb = su32(&mbar);

  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(&tslot)),
                 "r"(NCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tslot;

  double* Cb = g.C + b * g.c_batch;
  const int row = m0 + 32 * w + lane;
  uint32_t phase = 0;
  bool failed = false;
  for (int c = c0; c < g.c1 && !failed; ++c) {
    // ---- stage the digit planes of chunk c (zero rows beyond the split's padding never occur: rows_pad is a
    // multiple of 128) ----
    for (int idx = t; idx < S * (TC_M + TC_N) * 8; idx += 128) {
      const int seg = idx & 7;
      const int rr = idx >> 3;  // operand row over [S x 128 A rows][S x 64 B rows]
      const __nv_bfloat16* src;
      uint32_t dst;
      if (rr < S * TC_M) {
        const int i = rr / TC_M, r = rr % TC_M;
        src = pa + (((int64_t)i * g.SA.nchunk + c) * g.SA.rows_pad + m0 + r) * OZ_CHUNK + seg * 8;
        dst = sA + (uint32_t)(i * TC_M + r) * 128u + (uint32_t)((seg ^ (r & 7)) * 16);
      } else {
        const int q = rr - S * TC_M, i = q / TC_N, r = q % TC_N;
        src = pb + (((int64_t)i * g.SB.nchunk + c) * g.SB.rows_pad + n0 + r) * OZ_CHUNK + seg * 8;
        dst = sB + (uint32_t)(i * TC_N + r) * 128u + (uint32_t)((seg ^ (r & 7)) * 16);
      }
      cp16(dst, src);
    }
    if (t < TC_M) sea[t] = ea[(int64_t)c * g.SA.rows_pad + m0 + t];
    if (t < TC_N) seb[t] = eb[(int64_t)c * g.SB.rows_pad + n0 + t];
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    // ---- digit products on the tensor cores ----
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll 1
      for (int dg = 2; dg <= S + 1; ++dg) {
        const uint32_t d = tmem + (uint32_t)((dg - 2) * TC_N);
        const int ilo = dg - S > 1 ? dg - S : 1, ihi = dg - 1 < S ? dg - 1 : S;
        uint32_t acc = 0;
#pragma unroll 1
        for (int i = ilo; i <= ihi; ++i) {
          const int j = dg - i;
          const uint32_t a0 = sA + (uint32_t)((i - 1) * TC_M) * 128u;
          const uint32_t b0 = sB + (uint32_t)((j - 1) * TC_N) * 128u;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            mma_issue(d, sdesc(a0 + kk * 32u), sdesc(b0 + kk * 32u), acc);
            acc = 1;
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mb)
                   : "memory");
    }
    // the CTA agrees on the outcome, so that the warp-collective TMEM loads below run on all lanes or on none
    failed = __syncthreads_or(mbar_wait(mb, phase) ? 0 : 1) != 0;
    if (failed) {
      if (t == 0) atomicExch(&g_oz_tc_error, 1);
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // ---- fold the diagonals of this warp's 32 rows into C ----
    const int er = sea[32 * w + lane];
    const bool first = (c == c0);
#pragma unroll 1
    for (int cg = 0; cg < TC_N / 16; ++cg) {
      long long h[16];
      double out[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) out[q] = 0.0;
#pragma unroll 1
      for (int dg = 2; dg <= S + 1; ++dg) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)((dg - 2) * TC_N + cg * 16), v);
        const bool gstart = (dg == 2) || (dg == 6);
        const bool gend = (dg == 5) || (dg == S + 1);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const long long iv = (long long)__float2int_rn(v[q]);
          h[q] = gstart ? iv : h[q] * 256 + iv;
          if (gend) out[q] += ll_to_double(h[q], er + seb[cg * 16 + q] - 8 * dg);
        }
      }
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int col = n0 + cg * 16 + q;
        if (row < g.M && col < g.N && (!lower || row >= col)) {
          double* cp = Cb + row + (int64_t)col * g.ldc;
          if (first)
            *cp = (g.beta == 0.0) ? g.alpha * out[q] : fma(g.alpha, out[q], g.beta * *cp);
          else
            *cp = fma(g.alpha, out[q], *cp);
        }
      }
    }
    // TMEM and the operand buffers are reused by the next chunk
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  if (failed) {
    // give the committed products a last bounded chance to finish before the accumulators are freed
    (void)mbar_wait(mb, phase);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(NCOLS));
}

// ---------------------------------------------------------------------------------------------------------------
// Pipelined form (S <= 7): a persistent CTA runs a sequence of jobs = (128 x 64 tile, 64-chunk) with three roles
//   warps 0-7   epilogue: warp e reads TMEM lanes 32 (e % 4) .. +31 (rows), columns 32 (e / 4) .. +31
//   warps 8-10  producers: cp.async of the digit planes; B (S x 64 rows) double-buffered per job, A in S one-digit
//               slots refilled as soon as the products of that digit retire
//   warp 11     TMEM allocation; its lane 0 issues the products, A-digit major: digit i meets B digits
//               1 .. S+1-i, then a commit to adone[i].  Diagonal i + 1 is complete once adone[i] fires, so the
//               epilogue folds it while the products of later digits run.
// Each mbarrier is at most one phase ahead of any waiter (every producer / consumer pair is ordered through the
// previous job), so parity waits are unambiguous.  All waits are bounded.

struct PipeBars {
  uint64_t full_a[8], adone[8], full_b[2], jobdone[2], tmemfree;
};

__device__ __forceinline__ void mbar_arrive(uint32_t m) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(m) : "memory");
}

__device__ __forceinline__ bool warp_wait(uint32_t m, uint32_t parity) {
  const bool ok = mbar_wait(m, parity);
  return __all_sync(0xffffffffu, ok);
}

// exact value of the signed 128-bit integer H times 2^E, rounded to nearest (ties to even)
__device__ __forceinline__ double i128_scaled_to_double(__int128 H, int E) {
  if (H == 0) return 0.0;
  const bool neg = H < 0;
  unsigned __int128 u = neg ? (unsigned __int128)(-H) : (unsigned __int128)H;
  const unsigned long long hi = (unsigned long long)(u >> 64), lo = (unsigned long long)u;
  const int p = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);  // position of the top bit
  unsigned long long mant;
  int e = p;
  if (p <= 52) {
    mant = lo << (52 - p);
  } else {
    const int sh = p - 52;
    mant = (unsigned long long)(u >> sh);
    const unsigned __int128 rem = u & (((unsigned __int128)1 << sh) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant >> 53) {
        mant >>= 1;
        ++e;
      }
    }
  }
  const int fld = e + E + 1023;
  if (fld <= 0 || fld >= 2047) return ldexp(neg ? -(double)u : (double)u, E);
  return __longlong_as_double(
      (long long)((neg ? 0x8000000000000000ull : 0ull) | ((unsigned long long)fld << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

struct TileJob {
  int m0, n0, c0, c1;
};

__device__ __forceinline__ bool tile_at(const TcArgs& g, long long t, TileJob& T) {
  if (g.wtw_n > 0) {
    int I = (int)((sqrt(4.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)(I + 1) * (I + 2) <= t) ++I;
    while ((long long)I * (I + 1) > t) --I;
    T.m0 = I * TC_M;
    T.n0 = (int)(t - (long long)I * (I + 1)) * TC_N;
    T.c0 = 2 * I;
    T.c1 = g.SA.nchunk;
  } else {
    const int tx = (g.M + TC_M - 1) / TC_M;
    T.m0 = (int)(t % tx) * TC_M;
    T.n0 = (int)(t / tx) * TC_N;
    T.c0 = g.c0;
    T.c1 = g.c1;
  }
  if (T.m0 >= g.M || T.n0 >= g.N || T.c1 <= T.c0) return false;
  if ((g.lower_only || g.wtw_n > 0) && T.m0 + TC_M - 1 < T.n0) return false;
  return true;
}

template <int S>
__global__ void __launch_bounds__(384, 1) k_oz_tcp(TcArgs g, long long ntiles) {
  constexpr int NCOLS = (S * TC_N <= 256) ? 256 : 512;
  constexpr uint32_t A_SLOT = TC_M * 128, B_DIGIT = TC_N * 128, B_BUF = S * B_DIGIT;
  extern __shared__ unsigned char tcp_raw[];
  __shared__ PipeBars bars;
  __shared__ uint32_t tslot;
  const uint32_t raw = su32(tcp_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u;  // S slots of one A digit (128 rows)
  const uint32_t sB = sA + S * A_SLOT;          // 2 buffers of S B digits (64 rows)
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const int64_t b = blockIdx.z;
  const __nv_bfloat16* pa = g.SA.planes + b * g.SA.plane_bstride;
  const __nv_bfloat16* pb = g.SB.planes + b * g.SB.plane_bstride;
  const int* ea = g.SA.exps + b * g.SA.exp_bstride;
  const int* eb = g.SB.exps + b * g.SB.exp_bstride;
  auto bar = [&](const uint64_t& x) { return su32(&x); };

  if (t == 0) {
    for (int i = 0; i < S; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 32;\n" ::"r"(bar(bars.full_a[i])));  // its owner warp
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(bars.adone[i])));
    }
    for (int q = 0; q < 2; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 96;\n" ::"r"(bar(bars.full_b[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar(bars.jobdone[q])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 256;\n" ::"r"(bar(bars.tmemfree)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (w == 11) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(&tslot)),
                 "r"(NCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tslot;
  bool ok = true;

  if (w >= 8 && w <= 10) {
    // ---------------- producers: warp pw owns the digits i = pw (mod 3), of A and of B ----------------
    // the three warps stream different digits at the same time, so a job's staging latency is that of about
    // S / 3 dependent copies instead of S
    const int pw = w - 8;
    int job = 0;
    for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
      TileJob T;
      if (!tile_at(g, ti, T)) continue;
      for (int c = T.c0; c < T.c1 && ok; ++c, ++job) {
        const int bb = job & 1;
        if (job >= 2 && !warp_wait(bar(bars.jobdone[bb]), ((job - 2) >> 1) & 1)) {
          ok = false;
          break;
        }
        const uint32_t bdst = sB + bb * B_BUF;
        for (int i = pw; i < S; i += 3)
          for (int idx = lane; idx < TC_N * 8; idx += 32) {
            const int seg = idx & 7, r = idx >> 3;
            cp16(bdst + (uint32_t)(i * TC_N + r) * 128u + (uint32_t)((seg ^ (r & 7)) * 16),
                 pb + (((int64_t)i * g.SB.nchunk + c) * g.SB.rows_pad + T.n0 + r) * OZ_CHUNK + seg * 8);
          }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        bool b_announced = false;
        for (int i = pw; i < S; i += 3) {
          if (job >= 1 && !warp_wait(bar(bars.adone[i]), (job - 1) & 1)) {
            ok = false;
            break;
          }
          const uint32_t adst = sA + i * A_SLOT;
          for (int idx = lane; idx < TC_M * 8; idx += 32) {
            const int seg = idx & 7, r = idx >> 3;
            cp16(adst + (uint32_t)r * 128u + (uint32_t)((seg ^ (r & 7)) * 16),
                 pa + (((int64_t)i * g.SA.nchunk + c) * g.SA.rows_pad + T.m0 + r) * OZ_CHUNK + seg * 8);
          }
          asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          if (!b_announced) {
            mbar_arrive(bar(bars.full_b[bb]));
            b_announced = true;
          }
          mbar_arrive(bar(bars.full_a[i]));
        }
        if (ok && !b_announced) {  // a warp without A digits (S < 3) still owes its share of B
          asm volatile("cp.async.wait_group 0;\n" ::: "memory");
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          mbar_arrive(bar(bars.full_b[bb]));
        }
      }
    }
    if (!ok) atomicExch(&g_oz_tc_error, 1);
  } else if (w == 11) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      int job = 0;
      for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        TileJob T;
        if (!tile_at(g, ti, T)) continue;
        for (int c = T.c0; c < T.c1 && ok; ++c, ++job) {
          const int bb = job & 1;
          if (!mbar_wait(bar(bars.full_b[bb]), (job >> 1) & 1) ||
              (job >= 1 && !mbar_wait(bar(bars.tmemfree), (job - 1) & 1))) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t bbase = sB + bb * B_BUF;
          for (int i = 1; i <= S; ++i) {
            if (!mbar_wait(bar(bars.full_a[i - 1]), job & 1)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = sA + (i - 1) * A_SLOT;
            for (int j = 1; j <= S + 1 - i; ++j) {
              const uint32_t d = tmem + (uint32_t)((i + j - 2) * TC_N);
              const uint32_t b0 = bbase + (j - 1) * B_DIGIT;
#pragma unroll
              for (int kk = 0; kk < 4; ++kk) mma_issue(d, sdesc(a0 + kk * 32u), sdesc(b0 + kk * 32u),
                                                       (i > 1 || kk > 0) ? 1u : 0u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             bar(bars.adone[i - 1]))
                         : "memory");
          }
          if (!ok) break;
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                           bar(bars.jobdone[bb]))
                       : "memory");
        }
      }
      if (!ok) atomicExch(&g_oz_tc_error, 1);
    }
  } else {
    // ---------------- epilogue (warps 0-7) ----------------
    const int quarter = w & 3, half = w >> 2;
    const uint32_t tl = tmem + ((uint32_t)(32 * quarter) << 16);
    double* Cb = g.C + b * g.c_batch;
    const bool lower = g.lower_only || g.wtw_n > 0;
    int job = 0;
    for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
      TileJob T;
      if (!tile_at(g, ti, T)) continue;
      const int row = T.m0 + 32 * quarter + lane;
      for (int c = T.c0; c < T.c1 && ok; ++c, ++job) {
        const int er = ea[(int64_t)c * g.SA.rows_pad + T.m0 + 32 * quarter + lane];
        const bool first = (c == T.c0);
        const bool need_c = !(first && g.beta == 0.0);
        const double cscale = first ? g.beta : 1.0;
#pragma unroll 1
        for (int cg = 0; cg < 2 && ok; ++cg) {
          const int col0 = 32 * half + 16 * cg;
          // operands of this column group's update, loaded together (before the products retire for cg 0)
          int ec[16];
          double cold[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int col = T.n0 + col0 + q;
            ec[q] = eb[(int64_t)c * g.SB.rows_pad + col];
            const bool inside = row < g.M && col < g.N && (!lower || row >= col);
            cold[q] = (inside && need_c) ? Cb[row + (int64_t)col * g.ldc] : 0.0;
          }
          long long h1[16], h2[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) h2[q] = 0;
#pragma unroll 1
          for (int i = 1; i <= S; ++i) {  // diagonal dg = i + 1 is complete after adone[i]
            if (cg == 0 && !warp_wait(bar(bars.adone[i - 1]), job & 1)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const int dg = i + 1;
            float v[16];
            tmem_ld16(tl + (uint32_t)((dg - 2) * TC_N + col0), v);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
              const long long iv = (long long)__float2int_rn(v[q]);
              if (dg <= 5)
                h1[q] = (dg == 2) ? iv : h1[q] * 256 + iv;
              else
                h2[q] = (dg == 6) ? iv : h2[q] * 256 + iv;
            }
          }
          if (!ok) break;
          if (cg == 1) {  // the job's last TMEM read: the next job's products may start now
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            mbar_arrive(bar(bars.tmemfree));
          }
          // H = h1 256^(S-4) + h2 holds the chunk's exact product in units of 2^(er + ec - 8 (S + 1))
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            const int col = T.n0 + col0 + q;
            const __int128 H = ((__int128)h1[q] << (8 * (S - 4))) + (__int128)h2[q];
            const double val = i128_scaled_to_double(H, er + ec[q] - 8 * (S + 1));
            if (row < g.M && col < g.N && (!lower || row >= col)) {
              // one FP64 operation per element where the update allows it (the FP64 pipe is the scarce one here)
              double outv;
              if (!need_c)
                outv = g.alpha * val;
              else if (cscale == 1.0 && g.alpha == -1.0)
                outv = cold[q] - val;
              else if (cscale == 1.0 && g.alpha == 1.0)
                outv = cold[q] + val;
              else
                outv = fma(g.alpha, val, cscale * cold[q]);
              Cb[row + (int64_t)col * g.ldc] = outv;
            }
          }
        }
        if (!ok) break;
      }
    }
    if (!ok && lane == 0) atomicExch(&g_oz_tc_error, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (w == 11) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(NCOLS));
}

template <int S>
void launch_tcp(const TcArgs& a, long long ntiles, int batch, cudaStream_t st) {
  const size_t smem = (size_t)S * (TC_M + 2 * TC_N) * 128 + 1024;
  static bool attr = false;
  if (!attr) {
    LKG_CUDA(cudaFuncSetAttribute(k_oz_tcp<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    LKG_CUDA(cudaGetDevice(&dev));
    LKG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  const long long gx = std::min<long long>(ntiles, std::max(1, nsm / std::max(1, batch)));
  k_oz_tcp<S><<<dim3((unsigned)gx, 1, batch), 384, smem, st>>>(a, ntiles);
  LKG_LAUNCH("k_oz_tcp");
}

bool dispatch_tcp(int S, const TcArgs& a, long long ntiles, int batch, cudaStream_t st) {
  switch (S) {
    case 4: launch_tcp<4>(a, ntiles, batch, st); return true;
    case 5: launch_tcp<5>(a, ntiles, batch, st); return true;
    case 6: launch_tcp<6>(a, ntiles, batch, st); return true;
    case 7: launch_tcp<7>(a, ntiles, batch, st); return true;
    default: return false;  // S = 8 does not fit a double-buffered B: the single-stage kernel
  }
}

template <int S>
void launch_tc(const TcArgs& a, dim3 grid, cudaStream_t st) {
  // operands + exponents + 1024 B for the alignment; at least 120 KB so that one CTA (one TMEM allocation) is
  // resident per SM
  const size_t need = (size_t)S * (TC_M + TC_N) * 128 + (TC_M + TC_N) * sizeof(int) + 1024;
  const size_t smem = need < 120 * 1024 ? 120 * 1024 : need;
  static bool attr = false;
  if (!attr) {
    LKG_CUDA(cudaFuncSetAttribute(k_oz_tc<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  k_oz_tc<S><<<grid, 128, smem, st>>>(a);
  LKG_LAUNCH("k_oz_tc");
}

void dispatch_tc(int S, const TcArgs& a, dim3 grid, cudaStream_t st) {
  switch (S) {
    case 4: launch_tc<4>(a, grid, st); break;
    case 5: launch_tc<5>(a, grid, st); break;
    case 6: launch_tc<6>(a, grid, st); break;
    case 7: launch_tc<7>(a, grid, st); break;
    case 8: launch_tc<8>(a, grid, st); break;
    default: throw std::invalid_argument("ozaki: number of slices must be in [4, 8]");
  }
}

}  // namespace

void ozaki_gemm_tc(int M, int N, int c0, int c1, double alpha, const SplitBuf& SA, const SplitBuf& SB, double beta,
                   double* C, int64_t ldc, int64_t c_batch, int batch, bool lower_only, cudaStream_t st) {
  if (M <= 0 || N <= 0 || c1 <= c0) return;
  if (SA.S != SB.S) throw std::invalid_argument("ozaki_gemm: operands split with different slice counts");
  if (SA.rows_pad % TC_M || SB.rows_pad % TC_M) throw std::logic_error("ozaki_gemm_tc: split rows not padded to 128");
  TcArgs a{M, N, c0, c1, alpha, beta, SA, SB, C, ldc, c_batch, lower_only, 0};
  dim3 grid(ceil_div(M, TC_M), ceil_div(N, TC_N), batch);
  const double K = (double)(c1 - c0) * OZ_CHUNK;
  const double fl = (lower_only && M == N) ? K * M * (M + 1.0) : 2.0 * M * N * K;
  LaunchTimer lt("k_oz_tc", st, fl * batch * SA.S * (SA.S + 1) / 2.0,
                 8.0 * ((beta == 0.0) ? 1.0 : 2.0) * M * N * batch);
  if (!dispatch_tcp(SA.S, a, (long long)grid.x * grid.y, batch, st)) dispatch_tc(SA.S, a, grid, st);
}

void ozaki_wtw_tc(int n, const SplitBuf& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st) {
  if (SW.rows_pad % TC_M) throw std::logic_error("ozaki_wtw_tc: split rows not padded to 128");
  const int I = ceil_div(n, TC_M);
  const int64_t ntiles = (int64_t)I * (I + 1);
  TcArgs a{n, n, 0, SW.nchunk, 1.0, 0.0, SW, SW, C, ldc, cstride, false, n};
  LaunchTimer lt("k_oz_tc_wtw", st, (double)n * (n + 1.0) * (n + 2.0) / 3.0 * batch * SW.S * (SW.S + 1) / 2.0,
                 8.0 * n * (n + 1.0) * batch);
  if (!dispatch_tcp(SW.S, a, ntiles, batch, st)) dispatch_tc(SW.S, a, dim3((unsigned)ntiles, 1, batch), st);
}

int ozaki_tc_error_and_reset() {
  int e = 0, z = 0;
  LKG_CUDA(cudaMemcpyFromSymbol(&e, g_oz_tc_error, sizeof(int)));
  if (e) LKG_CUDA(cudaMemcpyToSymbol(g_oz_tc_error, &z, sizeof(int)));
  return e;
}

}  // namespace lkg
