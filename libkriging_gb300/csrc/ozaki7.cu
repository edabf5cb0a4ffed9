// ozaki7.cu -- FP64 products on the tcgen05 tensor cores by error-free splitting into 7-bit digits, with one
// exponent per (row, 256-wide k block).
//
// Method (Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59, 2012), in the form used here: every FP64 operand row is
// scaled, per k block of KB = 256 columns, by a power of two 2^e with max |x| 2^-e < 1/2 and written as
//   x = 2^e sum_{i=1..S} d_i 2^(-7 i),   d_i integer in [-64, 64]  (exact in bf16),
// so a digit product is below 2^12 in magnitude and the sum over i + j = g of up to S products over the 256 columns
// of a block stays below S * 256 * 2^12 <= 2^23: every FP32 tensor-core accumulator is an exact integer.  Products
// with i + j <= S + 1 are formed (S (S + 1) / 2 bf16 GEMMs per block), one accumulator per diagonal g, and the S
// diagonals are folded into FP64 once per block: adjacent diagonals paired in int32, the exact sum split into two
// integers below 2^46 that are exact doubles, one correctly rounded FP64 addition.  S = 8 gives 56-bit operands
// (FP64-level products); S = 5
// (35 bits) serves the triangular inverse and W^T W, which feed only the gradient.
//
// Data layout: the split writes each (digit, 64-wide k sub-chunk, 128-row tile) as the 16 KB shared-memory image of
// a K-major tile with the 128-byte swizzle (16-byte chunk c of row r at chunk c ^ (r & 7)), so the kernel moves it
// with one bulk copy; a 64-row tile is the first or second half of an image.
//
// k_oz7_gemm (one persistent CTA per SM, 18 warps):
//   warp 0        one thread streams the digit images: per sub-chunk all S digits of B (64 rows, double-buffered),
//                 then the S digits of A (128 rows) through a 6-7-stage ring; bulk copies complete on mbarriers
//   warp 1        TMEM allocation (512 columns = S diagonals x 64 columns); one thread issues tcgen05.mma
//                 (M 128, N 64 k, K 16): A digit i against up to 4 adjacent B digits at once, and releases each A
//                 stage and B buffer with tcgen05.commit
//   warps 2..17   epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (rows) and 8 columns, 4 at a time:
//                 folds the S diagonals exactly (int32 pairs, two exact doubles, one rounded FP64 addition) and
//                 updates C, then releases its accumulator set to the next block (18 warps leave 96 registers a
//                 thread: a sub-partition holds 5 warps of its 16K registers)
// All mbarrier waits are bounded; on expiry the CTA records an error (oz7_error_and_reset), drains what it issued and
// returns.
#include "ozaki7.cuh"

#include "stats.hpp"

namespace lkg {

void set_last_error(const char* msg);

namespace {

constexpr int TM = 128;
constexpr int NA_MAX = 10;                     // A ring stages at most
constexpr uint32_t A_BYTES = TM * 128;         // one digit of a 128-row tile, one 64-wide sub-chunk: 16 KB
constexpr uint64_t kWaitNs = 200000000ull;     // an mbarrier wait gives up after 200 ms

// Output tiles are 128 x TN.  TN = 32: two accumulator sets of S x 32 TMEM columns, so the fold of one tile overlaps
// the products of the next; TN = 64: one set of S x 64 columns (each A digit image serves twice the columns, the fold
// waits for the products).  The tile width is chosen per launch (oz7_set_tile).
template <int TN>
constexpr uint32_t b_bytes() { return TN * 128; }  // one digit of a TN-row B tile, one 64-wide sub-chunk
template <int S, int TN>
constexpr int nsets() { return 2 * S * TN <= 512 ? 2 : 1; }

// A ring depth: what 227 KB of shared memory holds beside the two B buffers (10 for TN = 32, 6 for TN = 64 at
// S = 8); a deep ring keeps enough digit images in flight to cover the L2 latency at the rate the MMAs consume them
template <int S, int TN>
constexpr int ring_depth() {
  return (int)((227u * 1024u - 1024u - 2u * S * b_bytes<TN>()) / A_BYTES) < NA_MAX
             ? (int)((227u * 1024u - 1024u - 2u * S * b_bytes<TN>()) / A_BYTES)
             : NA_MAX;
}
constexpr int NTHREADS = 576;                  // 18 warps

__device__ int g_oz7_error;
__device__ int g_oz7_where[8];  // first expired wait: role, tile, k block, sub-chunk, digit, and the role's counters

// instruction descriptor of tcgen05.mma kind::f16: D FP32, A and B bf16, both K-major, M = 128, N = TN k (k B
// digits side by side, up to N = 256)
__host__ __device__ constexpr uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {  // K-major, 128-byte swizzle, 8-row atoms 1024 B apart
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(1024u >> 4) << 32) | ((uint64_t)1u << 46) |
         ((uint64_t)2u << 61);
}

__device__ __forceinline__ void mbar_init(uint32_t m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(m), "r"(count));
}

__device__ __forceinline__ bool mbar_poll(uint32_t m, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(m), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;\n" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t m, uint32_t parity) {
  if (mbar_poll(m, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_poll(m, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

__device__ __forceinline__ void record_expiry(int role, long long tile, int kb, int s, int i, uint32_t c0, uint32_t c1,
                                              uint32_t c2) {
  if (atomicCAS(&g_oz7_error, 0, 1) == 0) {
    g_oz7_where[0] = role;
    g_oz7_where[1] = (int)tile;
    g_oz7_where[2] = kb;
    g_oz7_where[3] = s;
    g_oz7_where[4] = i;
    g_oz7_where[5] = (int)c0;
    g_oz7_where[6] = (int)c1;
    g_oz7_where[7] = (int)c2;
  }
}

__device__ __forceinline__ void mbar_arrive(uint32_t m) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(m) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(m), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

__device__ __forceinline__ void mma_issue(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}

// x 2^e for an integer |x| < 2^53, built from its bits with integer instructions (FP64 issue is scarce on this
// part): exact whenever the result is a normal number; the rare out-of-range case goes through ldexp
__device__ __forceinline__ double exact_scaled(long long x, int e) {
  if (x == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)x & 0x8000000000000000ull;
  const unsigned long long u = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
  const int p = 63 - __clzll((long long)u);  // top bit (<= 52)
  const int fld = p + e + 1023;
  if (fld <= 0 || fld >= 2047) return ldexp((double)x, e);
  return __longlong_as_double(
      (long long)(sgn | ((unsigned long long)fld << 52) | ((u << (52 - p)) & 0xFFFFFFFFFFFFFull)));
}

// The block's exact product H = sum_g v_g 128^(S + 1 - g) (v_g the FP32 diagonal sums, g = 2 .. S + 1, exact
// integers with |v_g| <= (g - 1) 2^20) times 2^E, correctly rounded: adjacent diagonals first combine in int32
// (v_g 128 + v_(g+1) < 2^31), then H = hi 2^28 + lo with lo the last four diagonals and hi the first S - 4, both
// below 2^46 and so exact as doubles; one FP64 addition rounds their sum once (ties to even).
template <int S>
__device__ __forceinline__ double fold_diagonals(const uint32_t (&v)[S][4], int q, int E) {
  int iv[S];
#pragma unroll
  for (int j = 0; j < S; ++j) iv[j] = __float2int_rn(__uint_as_float(v[j][q]));
  const long long lo = ((long long)(iv[S - 4] * 128 + iv[S - 3]) << 14) + (iv[S - 2] * 128 + iv[S - 1]);
  long long hi;
  if constexpr (S == 8)
    hi = ((long long)(iv[0] * 128 + iv[1]) << 14) + (iv[2] * 128 + iv[3]);
  else if constexpr (S == 7)
    hi = ((long long)iv[0] << 14) + (iv[1] * 128 + iv[2]);
  else if constexpr (S == 6)
    hi = iv[0] * 128 + iv[1];
  else
    hi = iv[0];
  return exact_scaled(hi, E + 28) + exact_scaled(lo, E);
}

// ---------------------------------------------------------------------------------------------------------------
// bf16 bit pattern of a small integer d (|d| <= 64): 1.5 2^23 + d is exact in FP32, so subtracting 1.5 2^23 gives d
// as a float whose low 16 bits are zero (at most 7 significant bits), and its high half is the bf16 value
__device__ __forceinline__ uint32_t bf16_bits_of_small(int d) {
  const float f = __int_as_float(0x4B400000 + d) - 12582912.0f;
  return (uint32_t)__float_as_int(f) >> 16;
}

// one operand of a split launch: element (r, k) of batch entry b at p[b * bstride + r * s_r + k * s_k]
struct SplitJob {
  int rows, K;
  const double* p;
  int64_t s_r, s_k, bstride;
  Split7 out;
};

// split: one warp per (row, k block); lane l holds the column pairs 2 l, 2 l + 1 of every 64-wide sub-chunk.  One
// launch serves two operands: CTAs x < nx0 the first, the rest the second.
template <int S>
__global__ void __launch_bounds__(256) k_oz7_split(SplitJob j0, SplitJob j1, int nx0) {
  const bool second = (int)blockIdx.x >= nx0;
  const int rows = second ? j1.rows : j0.rows, K = second ? j1.K : j0.K;
  const double* __restrict__ p = second ? j1.p : j0.p;
  const int64_t s_r = second ? j1.s_r : j0.s_r, s_k = second ? j1.s_k : j0.s_k;
  const int64_t bstride = second ? j1.bstride : j0.bstride;
  const Split7 out = second ? j1.out : j0.out;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = ((int)blockIdx.x - (second ? nx0 : 0)) * 8 + warp, kb = blockIdx.y;
  const int64_t b = blockIdx.z;
  if (r >= out.rows_pad || kb >= out.nblk) return;
  const int spb = out.sub_per_blk;
  double x[2 * OZ7_MAX_SPB];
#pragma unroll
  for (int q = 0; q < 2 * OZ7_MAX_SPB; ++q) x[q] = 0.0;
  const double* pr = p + b * bstride + (int64_t)r * s_r;
#pragma unroll
  for (int q = 0; q < OZ7_MAX_SPB; ++q) {
    if (q >= spb) break;
    const int k = (kb * spb + q) * 64 + 2 * lane;
    if (r < rows) {
      if (k < K) x[2 * q] = pr[(int64_t)k * s_k];
      if (k + 1 < K) x[2 * q + 1] = pr[(int64_t)(k + 1) * s_k];
    }
  }
  // block exponent from the largest |x| (IEEE bit patterns order like the magnitudes): |x| 2^-e < 1/2
  unsigned long long bm = 0;
#pragma unroll
  for (int q = 0; q < 2 * OZ7_MAX_SPB; ++q) {
    const unsigned long long a = (unsigned long long)__double_as_longlong(x[q]) & 0x7FFFFFFFFFFFFFFFull;
    bm = a > bm ? a : bm;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, bm, o);
    bm = ob > bm ? ob : bm;
  }
  int e = 0;
  if (bm != 0) {
    const int bx = (int)(bm >> 52);
    const int E = bx ? bx - 1022 : (64 - __clzll((long long)(bm & 0xFFFFFFFFFFFFFull))) - 1074;
    e = E + 1;
  }
  const int ntile = out.rows_pad / 128, t = r >> 7, rr = r & 127;
  __nv_bfloat16* base = out.planes + b * out.plane_bstride;
#pragma unroll
  for (int q = 0; q < OZ7_MAX_SPB; ++q) {
    if (q >= spb) break;
    const int s = kb * spb + q;
    if (s >= out.nsub) break;
    long long V[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // V = round(x 2^(7 S - e)), |V| < 2^(7 S - 1)
      const unsigned long long bits = (unsigned long long)__double_as_longlong(x[2 * q + h]);
      const unsigned long long ab = bits & 0x7FFFFFFFFFFFFFFFull;
      long long v = 0;
      if (ab != 0) {
        const int bx = (int)(ab >> 52);
        const unsigned long long mant = bx ? ((ab & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : (ab & 0xFFFFFFFFFFFFFull);
        const int ex = bx ? bx - 1075 : -1074;
        const int sh = ex + 7 * S - e;
        if (sh >= 0)
          v = (long long)(mant << sh);
        else if (sh > -64)
          v = (long long)((mant + (1ull << (-sh - 1))) >> (-sh));
        if (bits >> 63) v = -v;
      }
      V[h] = v;
    }
    const int kk = 2 * lane, c = kk >> 3, e8 = kk & 7;
    const int64_t off = (int64_t)rr * 64 + ((c ^ (rr & 7)) << 3) + e8;
    // balanced base-128 digits in closed form: with U = V + 64 (1 + 128 + ... + 128^(S-2)), digit k (least
    // significant first) is ((U >> 7 k) & 127) - 64 for k < S - 1 and the top digit is U >> 7 (S - 1) (|d| <= 64)
    constexpr long long C = 64ll * ((1ll << (7 * (S - 1))) - 1) / 127;
    const long long U0 = V[0] + C, U1 = V[1] + C;
    const int64_t plane = (int64_t)out.nsub * ntile * (TM * 64);  // elements between digit images
    uint32_t* img = reinterpret_cast<uint32_t*>(base + ((int64_t)s * ntile + t) * (TM * 64) + off);
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = S - 1 - k;  // digit index, 0 = most significant
      const int d0 = (k < S - 1) ? (int)((U0 >> (7 * k)) & 127) - 64 : (int)(U0 >> (7 * k));
      const int d1 = (k < S - 1) ? (int)((U1 >> (7 * k)) & 127) - 64 : (int)(U1 >> (7 * k));
      img[(i * plane) >> 1] = bf16_bits_of_small(d0) | (bf16_bits_of_small(d1) << 16);
    }
  }
  if (lane == 0) out.exps[b * out.exp_bstride + (int64_t)kb * out.rows_pad + r] = e;
}

// ---------------------------------------------------------------------------------------------------------------
struct Tile {
  int m0, n0, kb0, kb1;
};

template <int TN>
__device__ __forceinline__ bool tile_of(const Oz7Args& g, long long t, Tile& T) {
  constexpr long long CPB = TM / TN;  // column tiles per 128 columns
  if (g.lower || g.wtw) {  // lower tiles in row-major order: row block I holds the column tiles 0 .. CPB (I + 1) - 1
    // I = max { I : CPB I (I + 1) / 2 <= t } from an FP32 estimate and integer corrections (FP64 is scarce here)
    int I = (int)((sqrtf(8.0f * (float)t / (float)CPB + 1.0f) - 1.0f) * 0.5f);
    while (CPB * (I + 1) * (I + 2) / 2 <= t) ++I;
    while (I > 0 && CPB * I * (I + 1) / 2 > t) --I;
    T.m0 = I * TM;
    T.n0 = (int)(t - CPB * I * (I + 1) / 2) * TN;
  } else {
    const int tx = (g.M + TM - 1) / TM;
    T.m0 = (int)(t % tx) * TM;
    T.n0 = (int)(t / tx) * TN;
  }
  if (g.wtw) {
    T.kb0 = T.m0 / (OZ7_SUB * g.SA.sub_per_blk);  // W is lower triangular: rows above m0 contribute zeros
    T.kb1 = g.SA.nblk;
  } else {
    T.kb0 = g.kb0;
    T.kb1 = g.kb1;
  }
  if (T.m0 >= g.M || T.n0 >= g.N || T.kb1 <= T.kb0) return false;
  if ((g.lower || g.wtw) && T.m0 + TM - 1 < T.n0) return false;
  return true;
}

struct Bars {
  uint64_t a_full[NA_MAX], a_empty[NA_MAX], b_full[2], b_empty[2], acc_full[2], acc_empty[2], drain;
};

template <int S, int TN>
__global__ void __launch_bounds__(NTHREADS, 1) k_oz7_gemm(Oz7Args g, long long ntiles) {
  static_assert(S >= 5 && S <= 8, "digit count");
  static_assert(TN == 32 || TN == 64, "tile width");
  constexpr int NA = ring_depth<S, TN>();
  static_assert(NA >= 2 && NA <= NA_MAX, "A ring depth");
  constexpr uint32_t B_BYTES = b_bytes<TN>();
  constexpr uint32_t B_BUF = S * B_BYTES;
  constexpr int NSET = nsets<S, TN>();
  constexpr uint32_t TMEM_SET = S * TN;  // columns of one accumulator set
  extern __shared__ unsigned char oz7_raw[];
  __shared__ Bars bars;
  __shared__ uint32_t tslot;
  const uint32_t raw = su32(oz7_raw);
  const uint32_t sA = (raw + 1023u) & ~1023u;  // NA stages of one A digit
  const uint32_t sB = sA + NA * A_BYTES;        // 2 buffers of S B digits
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const int64_t bz = blockIdx.z;
  const __nv_bfloat16* pa = g.SA.planes + bz * g.SA.plane_bstride;
  const __nv_bfloat16* pb = g.SB.planes + bz * g.SB.plane_bstride;
  const int* ea = g.SA.exps + bz * g.SA.exp_bstride;
  const int* eb = g.SB.exps + bz * g.SB.exp_bstride;
  const int ntA = g.SA.rows_pad / TM, ntB = g.SB.rows_pad / TM;
  const int spb = g.SA.sub_per_blk;
  auto bar = [](const uint64_t& x) { return su32(&x); };

  if (t == 0) {
    for (int i = 0; i < NA; ++i) {
      mbar_init(bar(bars.a_full[i]), 1);
      mbar_init(bar(bars.a_empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar(bars.b_full[i]), 1);
      mbar_init(bar(bars.b_empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(bar(bars.acc_full[i]), 1);
      mbar_init(bar(bars.acc_empty[i]), 16);
    }
    mbar_init(bar(bars.drain), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (w == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(su32(&tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tslot;
  bool ok = true;

  if (w == 0) {
    // ------------------------------- producer -------------------------------
    if (lane == 0) {
      uint32_t ua = 0, ub = 0;
      int last_fill_a[NA], last_fill_b[2];
      for (int i = 0; i < NA; ++i) last_fill_a[i] = -1;
      last_fill_b[0] = last_fill_b[1] = -1;
      for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        Tile T;
        if (!tile_of<TN>(g, ti, T)) continue;
        const int tA = (T.m0 + g.a_row0) / TM, tB = (T.n0 + g.b_row0) / TM, hB = (T.n0 + g.b_row0) % TM;
        for (int kb = T.kb0; kb < T.kb1 && ok; ++kb) {
          const int s1 = min((kb + 1) * spb, g.SA.nsub);
          for (int s = kb * spb; s < s1 && ok; ++s) {
            const int bb = ub & 1;
            if (!mbar_wait(bar(bars.b_empty[bb]), ((ub >> 1) & 1) ^ 1)) {
              record_expiry(1, ti, kb, s, -1, ua, ub, 0);
              ok = false;
              break;
            }
            mbar_expect_tx(bar(bars.b_full[bb]), S * B_BYTES);
            for (int j = 0; j < S; ++j) {
              const __nv_bfloat16* src = pb + (((int64_t)j * g.SB.nsub + s) * ntB + tB) * (TM * 64) + (int64_t)hB * 64;
              bulk_g2s(sB + bb * B_BUF + j * B_BYTES, src, B_BYTES, bar(bars.b_full[bb]));
            }
            last_fill_b[bb] = (int)(ub >> 1);
            ++ub;
            for (int i = 0; i < S; ++i) {
              const int st = ua % NA;
              const uint32_t us = ua / NA;
              if (!mbar_wait(bar(bars.a_empty[st]), (us & 1) ^ 1)) {
                record_expiry(2, ti, kb, s, i, ua, ub, 0);
                ok = false;
                break;
              }
              mbar_expect_tx(bar(bars.a_full[st]), A_BYTES);
              const __nv_bfloat16* src = pa + (((int64_t)i * g.SA.nsub + s) * ntA + tA) * (TM * 64);
              bulk_g2s(sA + st * A_BYTES, src, A_BYTES, bar(bars.a_full[st]));
              last_fill_a[st] = (int)us;
              ++ua;
            }
          }
        }
      }
      // every copy issued has landed before the CTA may exit
      for (int i = 0; i < NA; ++i)
        if (last_fill_a[i] >= 0) (void)mbar_wait(bar(bars.a_full[i]), last_fill_a[i] & 1);
      for (int i = 0; i < 2; ++i)
        if (last_fill_b[i] >= 0) (void)mbar_wait(bar(bars.b_full[i]), last_fill_b[i] & 1);
      if (!ok) atomicExch(&g_oz7_error, 1);
    }
  } else if (w == 1) {
    // ------------------------------- MMA issue -------------------------------
    if (lane == 0) {
      uint32_t ua = 0, ub = 0, uacc = 0;
      bool issued = false;
      for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        Tile T;
        if (!tile_of<TN>(g, ti, T)) continue;
        for (int kb = T.kb0; kb < T.kb1 && ok; ++kb) {
          // accumulator set uacc % NSET: the epilogue releases a set after folding the block that used it (with two
          // sets the products of this block overlap the fold of the previous one)
          const int set = NSET == 2 ? (int)(uacc & 1) : 0;
          const uint32_t use = NSET == 2 ? (uacc >> 1) : uacc;  // uses of this set before this one
          if (!mbar_wait(bar(bars.acc_empty[set]), (use & 1) ^ 1)) {
            record_expiry(3, ti, kb, -1, -1, ua, ub, uacc);
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t tset = tmem + (uint32_t)set * TMEM_SET;
          const int s1 = min((kb + 1) * spb, g.SA.nsub);
          for (int s = kb * spb; s < s1 && ok; ++s) {
            const bool first_sub = (s == kb * spb);
            const int bb = ub & 1;
            if (!mbar_wait(bar(bars.b_full[bb]), (ub >> 1) & 1)) {
              record_expiry(4, ti, kb, s, -1, ua, ub, uacc);
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            // descriptors advance with the address: +2 per 32-byte (16-element) step along k, so each MMA costs one
            // add and one issue
            const uint64_t bdesc0 = sdesc(sB + bb * B_BUF);
#pragma unroll
            for (int i = 1; i <= S; ++i) {
              const int st = ua % NA;
              if (!mbar_wait(bar(bars.a_full[st]), (ua / NA) & 1)) {
                record_expiry(5, ti, kb, s, i, ua, ub, uacc);
                ok = false;
                break;
              }
              asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
              const uint64_t adesc0 = sdesc(sA + st * A_BYTES);
              // A digit i meets B digits 1 .. S + 1 - i: adjacent TN-row blocks of one K-major operand, whose
              // diagonals i + 1 .. S + 1 are adjacent TN-column blocks of TMEM -- MMAs of up to N = 256 (256 / TN
              // digits each: one MMA for TN = 32)
#pragma unroll
              for (int j0 = 1; j0 <= S + 1 - i; j0 += 256 / TN) {
                const int k = (S + 2 - i - j0) < 256 / TN ? (S + 2 - i - j0) : 256 / TN;
                const uint32_t d = tset + (uint32_t)((i + j0 - 2) * TN);
                const uint64_t bdesc = bdesc0 + (uint64_t)((j0 - 1) * (B_BYTES >> 4));
                const uint32_t idesc = idesc_n(TN * k);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                  mma_issue(d, adesc0 + (uint64_t)(2 * kk), bdesc + (uint64_t)(2 * kk), idesc,
                            (!first_sub || i > 1 || kk > 0) ? 1u : 0u);
              }
              mma_commit(bar(bars.a_empty[st]));
              issued = true;
              ++ua;
            }
            if (!ok) break;
            mma_commit(bar(bars.b_empty[bb]));
            ++ub;
          }
          if (!ok) break;
          mma_commit(bar(bars.acc_full[set]));
          ++uacc;
        }
      }
      if (issued) {  // all products retired before TMEM is released
        mma_commit(bar(bars.drain));
        (void)mbar_wait(bar(bars.drain), 0);
      }
      if (!ok) atomicExch(&g_oz7_error, 1);
    }
  } else {
    // ------------------------------- epilogue -------------------------------
    // 16 warps: warp w owns TMEM lanes 32 (w % 4) .. +31 (rows) and the 8 columns 8 cg .. +7, taken 4 at a time:
    // the S diagonals of 4 columns are loaded together, folded exactly, rounded once and added into C.
    constexpr int CPW = TN / 4;  // columns per epilogue warp
    const int quarter = w & 3, cg = (w - 2) >> 2;
    const uint32_t tl0 = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(cg * CPW);
    double* Cb = g.C + bz * g.c_batch;
    const bool tri = g.lower || g.wtw;
    uint32_t uacc = 0;
    for (long long ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
      Tile T;
      if (!tile_of<TN>(g, ti, T)) continue;
      const int row = T.m0 + 32 * quarter + lane, col0 = T.n0 + cg * CPW;
      for (int kb = T.kb0; kb < T.kb1 && ok; ++kb) {
        const int set = NSET == 2 ? (int)(uacc & 1) : 0;
        const uint32_t use = NSET == 2 ? (uacc >> 1) : uacc;
        const uint32_t tl = tl0 + (uint32_t)set * TMEM_SET;
        const bool first = (kb == T.kb0);
        const bool need_c = !(first && g.beta == 0.0);
        // operands of the update, loaded while the block's products run: the column exponents and the first four
        // C values (each group then prefetches the next group's C)
        const int er = ea[(int64_t)kb * g.SA.rows_pad + g.a_row0 + row];
        const int* ebk = eb + (int64_t)kb * g.SB.rows_pad + g.b_row0;
        double cnext[4];
        int enext[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int col = col0 + q;
          enext[q] = (col < g.N) ? ebk[col] : 0;
          cnext[q] = (need_c && row < g.M && col < g.N && (!tri || row >= col)) ? Cb[row + (int64_t)col * g.ldc] : 0.0;
        }
        // C = beta C + alpha P in one FP64 operation where the coefficients allow it
        const int upd = !need_c ? (g.alpha == 1.0 ? 0 : 1)
                                : ((!first || g.beta == 1.0) ? (g.alpha == -1.0 ? 2 : (g.alpha == 1.0 ? 3 : 4)) : 5);
        const bool got = mbar_wait(bar(bars.acc_full[set]), use & 1);
        if (!__all_sync(0xffffffffu, got)) {
          if (lane == 0) record_expiry(6 + 16 * w, ti, kb, -1, -1, 0, 0, uacc);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
        for (int q0 = 0; q0 < CPW; q0 += 4) {
          double cold[4];
          int ec[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            cold[q] = cnext[q];
            ec[q] = enext[q];
          }
          if (q0 + 4 < CPW) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int col = col0 + q0 + 4 + q;
              enext[q] = (col < g.N) ? ebk[col] : 0;
              cnext[q] = (need_c && row < g.M && col < g.N && (!tri || row >= col)) ? Cb[row + (int64_t)col * g.ldc]
                                                                                     : 0.0;
            }
          }
          uint32_t v[S][4];
#pragma unroll
          for (int dg = 2; dg <= S + 1; ++dg)
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
                         : "=r"(v[dg - 2][0]), "=r"(v[dg - 2][1]), "=r"(v[dg - 2][2]), "=r"(v[dg - 2][3])
                         : "r"(tl + (uint32_t)((dg - 2) * TN + q0)));
          asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int col = col0 + q0 + q;
            if (row < g.M && col < g.N && (!tri || row >= col)) {
              // the block's exact product, in units 2^(er + ec - 7 (S + 1)), rounded once
              const double val = fold_diagonals<S>(v, q, er + ec[q] - 7 * (S + 1));
              double out;
              switch (upd) {
                case 0: out = val; break;
                case 1: out = g.alpha * val; break;
                case 2: out = cold[q] - val; break;
                case 3: out = cold[q] + val; break;
                case 4: out = fma(g.alpha, val, cold[q]); break;
                default: out = fma(g.alpha, val, g.beta * cold[q]); break;
              }
              Cb[row + (int64_t)col * g.ldc] = out;
            }
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(bars.acc_empty[set]));
        ++uacc;
      }
    }
    if (!ok && lane == 0) atomicExch(&g_oz7_error, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (w == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
}

template <int S, int TN>
void launch_oz7(const Oz7Args& a, long long ntiles, int batch, int max_ctas, cudaStream_t st) {
  const size_t smem = (size_t)ring_depth<S, TN>() * A_BYTES + 2 * S * b_bytes<TN>() + 1024;
  static bool attr = false;
  if (!attr) {
    LKG_CUDA(cudaFuncSetAttribute(k_oz7_gemm<S, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    LKG_CUDA(cudaGetDevice(&dev));
    LKG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  long long gx = std::min<long long>(ntiles, std::max(1, nsm / std::max(1, batch)));
  if (max_ctas > 0) gx = std::min<long long>(gx, max_ctas);
  k_oz7_gemm<S, TN><<<dim3((unsigned)gx, 1, batch), NTHREADS, smem, st>>>(a, ntiles);
  LKG_LAUNCH("k_oz7_gemm");
}

int g_tile_n = 32;  // the tile width of the next launches (oz7_set_tile)

template <int TN>
void dispatch_tn(int S, const Oz7Args& a, long long ntiles, int batch, int max_ctas, cudaStream_t st) {
  switch (S) {
    case 5: launch_oz7<5, TN>(a, ntiles, batch, max_ctas, st); break;
    case 6: launch_oz7<6, TN>(a, ntiles, batch, max_ctas, st); break;
    case 7: launch_oz7<7, TN>(a, ntiles, batch, max_ctas, st); break;
    case 8: launch_oz7<8, TN>(a, ntiles, batch, max_ctas, st); break;
    default: throw std::invalid_argument("ozaki7: number of digits must be 5 .. 8");
  }
}

// number of tiles of a launch for the tile width tn: lower / W^T W products enumerate the tiles on or below the
// diagonal (row block I holds (128 / tn) (I + 1) column tiles)
long long tile_count(const Oz7Args& a, int tn) {
  const long long tx = ceil_div(a.M, TM), ty = ceil_div(a.N, tn);
  return (a.lower || a.wtw) ? (long long)(TM / tn) * tx * (tx + 1) / 2 : tx * ty;
}

void dispatch(int S, const Oz7Args& a, int batch, cudaStream_t st, int max_ctas = 0) {
  if (g_tile_n == 64)
    dispatch_tn<64>(S, a, tile_count(a, 64), batch, max_ctas, st);
  else
    dispatch_tn<32>(S, a, tile_count(a, 32), batch, max_ctas, st);
}

}  // namespace

size_t oz7_plane_elems(int rows, int K, int S) {
  return (size_t)S * ceil_div(K, OZ7_SUB) * (ceil_div(rows, TM) * TM) * OZ7_SUB;
}

size_t oz7_exp_elems(int rows, int K, int kb) {
  return (size_t)ceil_div(K, kb) * (ceil_div(rows, TM) * TM);
}

Split7 oz7_buffer(void* planes, int* exps, int S, int rows_cap, int K_cap, int kb) {
  Split7 s;
  s.planes = static_cast<__nv_bfloat16*>(planes);
  s.exps = exps;
  s.S = S;
  s.sub_per_blk = kb / OZ7_SUB;
  s.plane_bstride = (int64_t)oz7_plane_elems(rows_cap, K_cap, S);
  s.exp_bstride = (int64_t)oz7_exp_elems(rows_cap, K_cap, kb);
  return s;
}

namespace {

// fills the descriptor's extents for a rows x K operand and checks them against its buffer
void split_prepare(int rows, int K, Split7& out) {
  if (out.sub_per_blk < 1 || out.sub_per_blk > OZ7_MAX_SPB) throw std::invalid_argument("oz7_split: bad k block");
  if (out.S < 5 || out.S > 8) throw std::invalid_argument("oz7_split: digits must be 5 .. 8");
  out.rows_pad = ceil_div(rows, TM) * TM;
  out.nsub = ceil_div(K, OZ7_SUB);
  out.nblk = ceil_div(out.nsub, out.sub_per_blk);
  if ((size_t)out.S * out.nsub * out.rows_pad * OZ7_SUB > (size_t)out.plane_bstride ||
      (size_t)out.nblk * out.rows_pad > (size_t)out.exp_bstride)
    throw std::logic_error("oz7_split: operand larger than its buffer");
}

void split_launch(const SplitJob& j0, const SplitJob& j1, int batch, cudaStream_t st) {
  const int nx0 = j0.rows > 0 ? j0.out.rows_pad / 8 : 0, nx1 = j1.rows > 0 ? j1.out.rows_pad / 8 : 0;
  const int ny = std::max(j0.rows > 0 ? j0.out.nblk : 0, j1.rows > 0 ? j1.out.nblk : 0);
  if (nx0 + nx1 == 0) return;
  dim3 grid(nx0 + nx1, ny, batch);
  LaunchTimer lt("k_oz7_split", st, 0.0,
                 ((double)j0.rows * j0.K * (8.0 + 2.0 * j0.out.S) + (double)j1.rows * j1.K * (8.0 + 2.0 * j1.out.S)) *
                     batch);
  switch (j0.rows > 0 ? j0.out.S : j1.out.S) {
    case 5: k_oz7_split<5><<<grid, 256, 0, st>>>(j0, j1, nx0); break;
    case 6: k_oz7_split<6><<<grid, 256, 0, st>>>(j0, j1, nx0); break;
    case 7: k_oz7_split<7><<<grid, 256, 0, st>>>(j0, j1, nx0); break;
    default: k_oz7_split<8><<<grid, 256, 0, st>>>(j0, j1, nx0); break;
  }
  LKG_LAUNCH("k_oz7_split");
}

}  // namespace

void oz7_split(int rows, int K, const double* p, int64_t s_r, int64_t s_k, int64_t bstride, int batch, Split7& out,
               cudaStream_t st) {
  if (rows <= 0 || K <= 0) return;
  split_prepare(rows, K, out);
  const SplitJob j0{rows, K, p, s_r, s_k, bstride, out}, none{0, 0, nullptr, 0, 0, 0, Split7{}};
  split_launch(j0, none, batch, st);
}

void oz7_split2(int rows0, int K0, const double* p0, int64_t s_r0, int64_t s_k0, int64_t bstride0, Split7& out0,
                int rows1, int K1, const double* p1, int64_t s_r1, int64_t s_k1, int64_t bstride1, Split7& out1,
                int batch, cudaStream_t st) {
  const bool a = rows0 > 0 && K0 > 0, c = rows1 > 0 && K1 > 0;
  if (a) split_prepare(rows0, K0, out0);
  if (c) split_prepare(rows1, K1, out1);
  if (a && c && out0.S != out1.S) throw std::invalid_argument("oz7_split2: operands with different digit counts");
  const SplitJob none{0, 0, nullptr, 0, 0, 0, Split7{}};
  split_launch(a ? SplitJob{rows0, K0, p0, s_r0, s_k0, bstride0, out0} : none,
               c ? SplitJob{rows1, K1, p1, s_r1, s_k1, bstride1, out1} : none, batch, st);
}

void oz7_gemm(int M, int N, int kb0, int kb1, double alpha, const Split7& SA, const Split7& SB, double beta, double* C,
              int64_t ldc, int64_t c_batch, int batch, bool lower, cudaStream_t st) {
  oz7_gemm_ex(M, N, kb0, kb1, alpha, SA, 0, SB, 0, beta, C, ldc, c_batch, batch, lower, 0, st);
}

int oz7_sm_count() {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    LKG_CUDA(cudaGetDevice(&dev));
    LKG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  return nsm;
}

void oz7_gemm_ex(int M, int N, int kb0, int kb1, double alpha, const Split7& SA, int a_row0, const Split7& SB,
                 int b_row0, double beta, double* C, int64_t ldc, int64_t c_batch, int batch, bool lower, int max_ctas,
                 cudaStream_t st) {
  if (M <= 0 || N <= 0 || kb1 <= kb0) return;
  if (SA.S != SB.S || SA.sub_per_blk != SB.sub_per_blk || SA.nsub != SB.nsub)
    throw std::invalid_argument("oz7_gemm: operands split differently");
  if (a_row0 < 0 || b_row0 < 0 || a_row0 % TM || b_row0 % TM)
    throw std::invalid_argument("oz7_gemm: operand row offsets must be multiples of 128");
  // split operands are padded to whole 128-row images, which cover any 32- or 64-wide column tile
  if (SA.rows_pad < a_row0 + ceil_div(M, TM) * TM || SB.rows_pad < b_row0 + ceil_div(N, TM) * TM)
    throw std::logic_error("oz7_gemm: operand rows do not cover C");
  if (lower && M != N) throw std::invalid_argument("oz7_gemm: lower products are square");
  Oz7Args a{M, N, kb0, kb1, alpha, beta, SA, SB, C, ldc, c_batch, lower ? 1 : 0, 0, a_row0, b_row0};
  const double K = std::min<double>((double)(kb1 - kb0) * SA.sub_per_blk * OZ7_SUB,
                                    (double)(SA.nsub - kb0 * SA.sub_per_blk) * OZ7_SUB);
  const double fl = lower ? K * M * (M + 1.0) : 2.0 * M * N * K;
  LaunchTimer lt("k_oz7_gemm", st, fl * batch * SA.S * (SA.S + 1) / 2.0,
                 8.0 * ((beta == 0.0) ? 1.0 : 2.0) * M * N * batch);
  dispatch(SA.S, a, batch, st, max_ctas);
}

void oz7_wtw(int n, const Split7& SW, double* C, int64_t ldc, int64_t cstride, int batch, cudaStream_t st) {
  Oz7Args a{n, n, 0, SW.nblk, 1.0, 0.0, SW, SW, C, ldc, cstride, 0, 1, 0, 0};
  // executed work: tile (I, J) sums the k blocks from the one holding row 128 I
  LaunchTimer lt("k_oz7_wtw", st, (double)n * (n + 1.0) * (n + 2.0) / 3.0 * batch * SW.S * (SW.S + 1) / 2.0,
                 8.0 * n * (n + 1.0) * batch);
  dispatch(SW.S, a, batch, st);
}

void oz7_set_tile(int tn) {
  if (tn != 32 && tn != 64) throw std::invalid_argument("oz7_set_tile: tile width must be 32 or 64");
  g_tile_n = tn;
}

int oz7_tile() { return g_tile_n; }

int oz7_error_and_reset(int* where) {
  int e = 0, z = 0;
  LKG_CUDA(cudaMemcpyFromSymbol(&e, g_oz7_error, sizeof(int)));
  if (e) {
    if (where) LKG_CUDA(cudaMemcpyFromSymbol(where, g_oz7_where, 8 * sizeof(int)));
    LKG_CUDA(cudaMemcpyToSymbol(g_oz7_error, &z, sizeof(int)));
  }
  return e;
}

// Diagnostic entry: one product of each mode on host data (see the declaration in the C ABI header)
extern "C" int lkg_oz7_mode_check(int mode, int M, int N, int K, const double* A, const double* B, int S, double* C,
                                  int* where_out) {
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  void *pa = nullptr, *pb = nullptr;
  int *ea = nullptr, *eb = nullptr;
  int rc = -1;
  try {
    if (mode == 1 || mode == 2) N = M;
    const int ka = (mode == 2) ? M : K;  // W^T W: k runs over the rows of the n x n matrix W
    LKG_CUDA(cudaMalloc(&dA, sizeof(double) * (size_t)M * ka));
    LKG_CUDA(cudaMemcpy(dA, A, sizeof(double) * (size_t)M * ka, cudaMemcpyHostToDevice));
    if (mode == 0) {
      LKG_CUDA(cudaMalloc(&dB, sizeof(double) * (size_t)N * K));
      LKG_CUDA(cudaMemcpy(dB, B, sizeof(double) * (size_t)N * K, cudaMemcpyHostToDevice));
    }
    LKG_CUDA(cudaMalloc(&dC, sizeof(double) * (size_t)M * N));
    LKG_CUDA(cudaMemset(dC, 0, sizeof(double) * (size_t)M * N));
    LKG_CUDA(cudaMalloc(&pa, oz7_plane_elems(M, ka, S) * 2));
    LKG_CUDA(cudaMalloc(&ea, oz7_exp_elems(M, ka, OZ7_KB) * sizeof(int)));
    Split7 sa = oz7_buffer(pa, ea, S, M, ka, OZ7_KB);
    if (mode == 2) {
      oz7_split(M, M, dA, M, 1, 0, 1, sa, 0);  // rows of the split = columns of W
      oz7_wtw(M, sa, dC, M, 0, 1, 0);
    } else {
      oz7_split(M, K, dA, 1, M, 0, 1, sa, 0);
      Split7 sb = sa;
      if (mode == 0) {
        LKG_CUDA(cudaMalloc(&pb, oz7_plane_elems(N, K, S) * 2));
        LKG_CUDA(cudaMalloc(&eb, oz7_exp_elems(N, K, OZ7_KB) * sizeof(int)));
        sb = oz7_buffer(pb, eb, S, N, K, OZ7_KB);
        oz7_split(N, K, dB, 1, N, 0, 1, sb, 0);
      }
      oz7_gemm(M, N, 0, sa.nblk, 1.0, sa, sb, 0.0, dC, M, 0, 1, mode == 1, 0);
    }
    LKG_CUDA(cudaDeviceSynchronize());
    LKG_CUDA(cudaMemcpy(C, dC, sizeof(double) * (size_t)M * N, cudaMemcpyDeviceToHost));
    rc = oz7_error_and_reset(where_out) ? -2 : 0;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    rc = -1;
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(pa);
  cudaFree(pb);
  cudaFree(ea);
  cudaFree(eb);
  return rc;
}

}  // namespace lkg
