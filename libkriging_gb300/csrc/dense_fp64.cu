// dense_fp64.cu -- FP64 blocked Cholesky / triangular inverse / R^-1 / small-RHS solves (sm_103a).
//
// These replace the LAPACK calls of libKriging's populate_Model (src/lib/KrigingImpl.cpp:73-125):
//   arma::chol (dpotrf)                 -> potrf_blocked   (right-looking, NB = 64 blocks)
//   inv_sympd = solve(L', solve(L, I))  -> trtri_blocked + wtw_lower  (2n^3/3 flops instead of 2n^3)
//   solve(trimatl(L), B), solve(trimatu(L'), B) -> trsm_lower_left[_t] (blocked, uses the diagonal-block inverses)
#include "dense_fp64.cuh"

#include "stats.hpp"

namespace lkg {

namespace {

constexpr int TB = 64;   // tile edge
constexpr int KC = 16;   // k-chunk staged through shared memory
constexpr int NT = 256;  // threads per tile CTA (16 x 16, 4 x 4 accumulators each)

struct TileSmem {
  double a[KC][TB];
  double b[KC][TB];
};

// acc += A(m0.., k) * B(k, n0..) over k in [0, K); A/B element (r,c) at p[r*sr + c*sc].
__device__ __forceinline__ void tile_mma_fp64(int M, int N, int K, const double* __restrict__ Ap, int64_t asr,
                                              int64_t asc, const double* __restrict__ Bp, int64_t bsr, int64_t bsc,
                                              int m0, int n0, TileSmem& sm, double (&acc)[4][4]) {
  const int t = threadIdx.x;
  const int tm = t & 15, tn = t >> 4;
  const bool a_mfast = (asr == 1);
  const bool b_kfast = (bsr == 1);
  for (int k0 = 0; k0 < K; k0 += KC) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = t + NT * r;
      int m, k;
      if (a_mfast) {
        m = idx & 63;
        k = idx >> 6;
      } else {
        k = idx & 15;
        m = idx >> 4;
      }
      const int gm = m0 + m, gk = k0 + k;
      sm.a[k][m] = (gm < M && gk < K) ? Ap[(int64_t)gm * asr + (int64_t)gk * asc] : 0.0;
      int n;
      if (b_kfast) {
        k = idx & 15;
        n = idx >> 4;
      } else {
        n = idx & 63;
        k = idx >> 6;
      }
      const int gn = n0 + n;
      const int gk2 = k0 + k;
      sm.b[k][n] = (gn < N && gk2 < K) ? Bp[(int64_t)gk2 * bsr + (int64_t)gn * bsc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      double av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = sm.a[k][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = sm.b[k][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void tile_store(int M, int N, double alpha, double beta, double* C, int64_t ldc, int m0,
                                           int n0, bool lower_only, const double (&acc)[4][4]) {
  const int t = threadIdx.x;
  const int tm = t & 15, tn = t >> 4;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = m0 + tm + 16 * i, c = n0 + tn + 16 * j;
      if (r < M && c < N && (!lower_only || r >= c)) {
        double* cp = C + r + (int64_t)c * ldc;
        *cp = (beta == 0.0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *cp);
      }
    }
  }
}

__global__ void __launch_bounds__(NT) k_gemm_tiles(int M, int N, int K, double alpha, MatView A, MatView B,
                                                   double beta, double* C, int64_t ldc, int64_t c_batch,
                                                   bool lower_only) {
  const int m0 = blockIdx.x * TB, n0 = blockIdx.y * TB;
  if (lower_only && m0 + TB - 1 < n0) return;  // tile strictly above the diagonal
  const int64_t b = blockIdx.z;
  __shared__ TileSmem sm;
  double acc[4][4] = {};
  tile_mma_fp64(M, N, K, A.p + b * A.batch, A.sr, A.sc, B.p + b * B.batch, B.sr, B.sc, m0, n0, sm, acc);
  tile_store(M, N, alpha, beta, C + b * c_batch, ldc, m0, n0, lower_only, acc);
}

// ---- diagonal block: Cholesky + inverse in shared memory (one CTA per batch entry) ----
constexpr int DPAD = NB + 1;

constexpr int PB = 16;  // panel width inside a diagonal block

// Inverse of the 16 x 16 lower block of s at (jb, jb) into the same block of w, one warp, row by row: row i is scaled
// by 1 / L_ii, then subtracted from the rows below it, w(r, c) -= L(r, i) w(i, c) for c <= i < r, with the (r, c)
// pairs spread over the lanes.  Each entry accumulates its terms in ascending i from the identity and is scaled
// last: the same operations, in the same order, as forward substitution column by column.
__device__ __forceinline__ void diag16_inverse(const double* s, double* w, int jb, int lane) {
  const double rdl = (lane < PB) ? __drcp_rn(s[(jb + lane) * DPAD + jb + lane]) : 0.0;
  for (int e = lane; e < PB * PB; e += 32) {
    const int r = e / PB, c = e % PB;
    if (c <= r) w[(jb + r) * DPAD + jb + c] = (r == c) ? 1.0 : 0.0;
  }
  __syncwarp();
  for (int i = 0; i < PB; ++i) {
    const double rd = __shfl_sync(0xffffffffu, rdl, i);
    if (lane <= i) w[(jb + i) * DPAD + jb + lane] *= rd;
    __syncwarp();
    const int ncol = i + 1, nel = (PB - 1 - i) * ncol;
    for (int e = lane; e < nel; e += 32) {
      const int r = jb + i + 1 + e / ncol, c = jb + e % ncol;
      w[r * DPAD + c] = fma(-s[r * DPAD + jb + i], w[(jb + i) * DPAD + c], w[r * DPAD + c]);
    }
    __syncwarp();
  }
}

// (row, column) of entry e of a lower triangle enumerated row by row: e = r (r + 1) / 2 + c, c <= r
__device__ __forceinline__ void tri_index(int e, int& r, int& c) {
  r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
  if ((r + 1) * (r + 2) / 2 <= e) ++r;
  if (r * (r + 1) / 2 > e) --r;
  c = e - r * (r + 1) / 2;
}

// The off-diagonal 16 x 16 blocks of the inverse from the diagonal ones, by block diagonals:
// W_ij = -W_ii sum_{k=j}^{i-1} L_ik W_kj.  scratch: 3 x 16 x 16 doubles.  Ends with a barrier.
__device__ __forceinline__ void assemble_inverse(const double* s, double* w, double* scratch, int t) {
  constexpr int NPB = NB / PB;
  for (int dist = 1; dist < NPB; ++dist) {
    const int npair = NPB - dist;
    for (int it = t; it < npair * PB * PB; it += NT) {  // T = sum_k L_ik W_kj
      const int pr = it / (PB * PB), r = (it / PB) % PB, c = it % PB;
      const int bi = (pr + dist) * PB, bj = pr * PB;
      double acc = 0.0;
      for (int k = bj; k < bi; ++k) acc = fma(s[(bi + r) * DPAD + k], w[k * DPAD + bj + c], acc);
      scratch[it] = acc;
    }
    __syncthreads();
    for (int it = t; it < npair * PB * PB; it += NT) {  // W_ij = -W_ii T
      const int pr = it / (PB * PB), r = (it / PB) % PB, c = it % PB;
      const int bi = (pr + dist) * PB, bj = pr * PB;
      double acc = 0.0;
      for (int m = 0; m <= r; ++m) acc = fma(w[(bi + r) * DPAD + bi + m], scratch[pr * PB * PB + m * PB + c], acc);
      w[(bi + r) * DPAD + bj + c] = -acc;
    }
    __syncthreads();
  }
}

// Cholesky factor and inverse of one nb x nb diagonal block (nb <= 64) in shared memory.  16-column block steps:
// update the block column with the columns left of it, factor and invert its 16 x 16 diagonal block in one warp,
// then solve the rows below with that inverse; the full inverse is assembled from the diagonal inverses.  A ragged
// block is padded with the identity.
__global__ void __launch_bounds__(NT) k_potrf_diag(double* A, int64_t lda, int64_t mstride, int k0, int nb,
                                                   double* Dinv, int64_t dinv_bstride, int blk, int* info) {
  const int64_t b = blockIdx.z;
  if (info[b] != 0) return;  // an earlier block of this matrix already failed
  extern __shared__ double dsm[];
  double* s = dsm;                   // [NB][DPAD]  s[i*DPAD + j] = L(i, j)
  double* w = dsm + NB * DPAD;       // [NB][DPAD]  w[i*DPAD + j] = L^-1(i, j)
  double* scratch = w + NB * DPAD;   // [3][PB][PB]
  __shared__ int failed;
  double* Ab = A + b * mstride + k0 + (int64_t)k0 * lda;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) failed = 0;
  {  // all 16 loads of a thread in flight before the shared-memory stores
    double v[NB * NB / NT];
#pragma unroll
    for (int u = 0; u < NB * NB / NT; ++u) {
      const int idx = t + u * NT, i = idx & 63, j = idx >> 6;
      v[u] = (i < nb && j < nb) ? ((i >= j) ? Ab[i + (int64_t)j * lda] : 0.0) : (i == j ? 1.0 : 0.0);
    }
#pragma unroll
    for (int u = 0; u < NB * NB / NT; ++u) {
      const int idx = t + u * NT, i = idx & 63, j = idx >> 6;
      s[i * DPAD + j] = v[u];
      w[i * DPAD + j] = 0.0;
    }
  }
  __syncthreads();
  for (int jb = 0; jb < NB; jb += PB) {
    // (1) columns jb .. jb+15, rows i >= c: subtract the columns 0 .. jb-1
    if (jb > 0) {
      for (int it = t; it < (NB - jb) * PB; it += NT) {
        const int c = jb + (it % PB), i = jb + it / PB;
        if (i >= c) {
          double acc = s[i * DPAD + c];
          for (int k = 0; k < jb; ++k) acc = fma(-s[i * DPAD + k], s[c * DPAD + k], acc);
          s[i * DPAD + c] = acc;
        }
      }
      __syncthreads();
    }
    // (2) the 16 x 16 diagonal block: right-looking Cholesky (column scaling by the reciprocal of the pivot, as
    // LAPACK's dpotf2 does), then its inverse
    if (warp == 0) {
      const int r = jb + lane;
      bool bad = false;
      for (int j = 0; j < PB; ++j) {
        const int cj = jb + j;
        const double piv = s[cj * DPAD + cj];
        if (!(piv > 0.0)) {  // non-positive or NaN pivot
          bad = true;
          if (lane == 0) {
            failed = 1;
            info[b] = k0 + cj + 1;
          }
          break;
        }
        const double d = sqrt(piv), rd = __drcp_rn(d);
        __syncwarp();
        if (lane == 0) s[cj * DPAD + cj] = d;
        if (lane > j && lane < PB) s[r * DPAD + cj] *= rd;
        __syncwarp();
        // trailing update s(r, c) -= L(r, j) L(c, j), j < c <= r < 16, the (r, c) pairs spread over the lanes
        const int m = PB - 1 - j;
        for (int e = lane; e < m * (m + 1) / 2; e += 32) {
          int rr, cc;
          tri_index(e, rr, cc);
          const int ra = jb + j + 1 + rr, ca = jb + j + 1 + cc;
          s[ra * DPAD + ca] = fma(-s[ra * DPAD + cj], s[ca * DPAD + cj], s[ra * DPAD + ca]);
        }
        __syncwarp();
      }
      if (!bad) diag16_inverse(s, w, jb, lane);
    }
    __syncthreads();
    if (failed) return;
    // (3) rows below: L(i, jb..jb+15) = A(i, jb..jb+15) W_dd^T, computed into registers, then stored
    {
      const int nrow = NB - jb - PB;
      double out[3];
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int it = t + u * NT;
        out[u] = 0.0;
        if (it < nrow * PB) {
          const int i = jb + PB + it / PB, c = it % PB;
          double acc = 0.0;
          for (int k = 0; k <= c; ++k) acc = fma(s[i * DPAD + jb + k], w[(jb + c) * DPAD + jb + k], acc);
          out[u] = acc;
        }
      }
      __syncthreads();
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int it = t + u * NT;
        if (it < nrow * PB) s[(jb + PB + it / PB) * DPAD + jb + it % PB] = out[u];
      }
      __syncthreads();
    }
  }
  assemble_inverse(s, w, scratch, t);
  double* Db = Dinv + b * dinv_bstride + (int64_t)blk * NB * NB;
  for (int idx = t; idx < NB * NB; idx += NT) {
    const int i = idx & 63, j = idx >> 6;
    if (i < nb && j < nb && i >= j) Ab[i + (int64_t)j * lda] = s[i * DPAD + j];
    Db[i + j * NB] = (i >= j && i < nb && j < nb) ? w[i * DPAD + j] : 0.0;  // zero above the diagonal and padding
  }
}

// ---- R^-1 = W^T W lower tiles, each tile with its own k range ----
__global__ void __launch_bounds__(NT) k_wtw(const double* W, int64_t ldw, int64_t wstride, int n, double* C,
                                            int64_t ldc, int64_t cstride) {
  // linear lower-tile index -> (I, J), I >= J, ordered by I (heaviest tiles first)
  const int64_t x = blockIdx.x;
  int I = (int)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
  while ((int64_t)(I + 1) * (I + 2) / 2 <= x) ++I;
  while ((int64_t)I * (I + 1) / 2 > x) --I;
  const int J = (int)(x - (int64_t)I * (I + 1) / 2);
  const int64_t b = blockIdx.z;
  const double* Wb = W + b * wstride;
  const int r0 = I * TB, c0 = J * TB;
  const int K = n - r0;
  __shared__ TileSmem sm;
  double acc[4][4] = {};
  // A(m, kk) = W(r0 + kk, r0 + m) ; B(kk, c) = W(r0 + kk, c0 + c)
  tile_mma_fp64(n - r0, n - c0, K, Wb + r0 + (int64_t)r0 * ldw, ldw, 1, Wb + r0 + (int64_t)c0 * ldw, 1, ldw, 0, 0,
                sm, acc);
  // store into C(r0.., c0..), lower triangle only on diagonal tiles
  tile_store(n - r0, n - c0, 1.0, 0.0, C + b * cstride + r0 + (int64_t)c0 * ldc, ldc, 0, 0, I == J, acc);
}

// ---- small-RHS solves: one launch per diagonal block ----
// Step k of the blocked substitution with X_k = Dinv_k B_k (TRANS: Dinv_k^T B_k).  The update CTAs (blockIdx.x < nupd)
// each form X_k in shared memory from the untouched B_k and apply it to their own rows of B:
//   forward   B(k0+nb+i, :) -= L(k0+nb+i, k0:k0+nb) X_k     64 rows per CTA
//   TRANS     B(j, :)       -= L(k0:k0+nb, j)^T X_k          64 columns j < k0 per CTA
// The last CTA (blockIdx.x == nupd, when kw >= 0) overwrites block kw -- the block of the previous step, which no
// other CTA of this step reads or writes -- with X_kw = Dinv_kw B_kw.  A solve is nblk + 1 such launches.
constexpr int TS_THREADS = 128;
constexpr int TS_ROWS = 64;
constexpr int TS_LD = NB + 1;  // padded row of the staged L tile (TRANS)

// Dinv_k staged column-major with a padded leading dimension (conflict-free for both access orders)
// (loads batched in registers ahead of the shared-memory stores, so that a thread keeps 16 loads in flight)
__device__ __forceinline__ void ts_stage_dinv(const double* __restrict__ D, double* ds) {
#pragma unroll
  for (int h = 0; h < NB * NB / TS_THREADS; h += 16) {
    double v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) v[u] = D[threadIdx.x + (h + u) * TS_THREADS];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int idx = threadIdx.x + (h + u) * TS_THREADS;
      ds[(idx / NB) * TS_LD + idx % NB] = v[u];
    }
  }
}

// xs = Dinv_k bs (trans: Dinv_k^T bs) from the staged block
__device__ __forceinline__ void ts_block_apply(const double* ds, const double* bs, double* xs, int nb, int r,
                                               bool trans) {
  for (int idx = threadIdx.x; idx < nb * r; idx += blockDim.x) {
    const int i = idx % nb, c = idx / nb;
    double sum = 0.0;
    if (!trans) {
      for (int kk = 0; kk <= i; ++kk) sum = fma(ds[kk * TS_LD + i], bs[kk + c * nb], sum);
    } else {
      for (int kk = i; kk < nb; ++kk) sum = fma(ds[i * TS_LD + kk], bs[kk + c * nb], sum);
    }
    xs[idx] = sum;
  }
}

// RC: right-hand sides per pass of the update (1, 2, 4 or 8), so that no FP64 issue slot goes to a masked column
template <bool TRANS, int RC>
__global__ void __launch_bounds__(TS_THREADS) k_trsv_step(const double* L, int64_t lda, int64_t mstride,
                                                          const double* Dinv, int64_t dstride, double* B, int64_t ldb,
                                                          int64_t bstride, int n, int k, int kw, int r, int nupd) {
  extern __shared__ double tsm[];
  const int rs = max(r, 8);                     // B_k's slot also holds the [TS_ROWS][8] partial sums
  double* bs = tsm;                             // nb x r: B_k (or B_kw)
  double* xs = tsm + NB * rs;                   // nb x r: X_k
  double* ds = tsm + 2 * NB * rs;               // [NB][TS_LD]: Dinv_k, ds[c * TS_LD + r] = Dinv_k(r, c)
  double* ls = tsm + 2 * NB * rs + NB * TS_LD;  // TRANS: [TS_ROWS][TS_LD], ls[j * TS_LD + kk] = L(k0 + kk, j0 + j)
  const int64_t b = blockIdx.z;
  const int t = threadIdx.x;
  double* Bb = B + b * bstride;
  const double* Db = Dinv + b * dstride;
  if ((int)blockIdx.x == nupd) {  // writer: X_kw over B_kw
    const int w0 = kw * NB, nbw = min(NB, n - w0);
    for (int idx = t; idx < nbw * r; idx += TS_THREADS) bs[idx] = Bb[w0 + idx % nbw + (int64_t)(idx / nbw) * ldb];
    ts_stage_dinv(Db + (int64_t)kw * NB * NB, ds);
    __syncthreads();
    ts_block_apply(ds, bs, xs, nbw, r, TRANS);
    __syncthreads();
    for (int idx = t; idx < nbw * r; idx += TS_THREADS) Bb[w0 + idx % nbw + (int64_t)(idx / nbw) * ldb] = xs[idx];
    return;
  }
  const int k0 = k * NB, nb = min(NB, n - k0);
  for (int idx = t; idx < nb * r; idx += TS_THREADS) bs[idx] = Bb[k0 + idx % nb + (int64_t)(idx / nb) * ldb];
  ts_stage_dinv(Db + (int64_t)k * NB * NB, ds);
  const double* Lb = L + b * mstride;
  const int half = t >> 6, q = t & 63;  // two threads per row (column): kk halves
  const int kh0 = half * (NB / 2);
  if constexpr (TRANS) {
    // stage L(k0:k0+nb, j0:j0+64) with lanes along kk (contiguous in memory)
    const int j0 = blockIdx.x * TS_ROWS;
#pragma unroll
    for (int h = 0; h < TS_ROWS * NB / TS_THREADS; h += 16) {
      double v[16];
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int idx = t + (h + u) * TS_THREADS, kk = idx % NB, j = idx / NB;
        v[u] = (kk < nb && j0 + j < k0) ? Lb[(k0 + kk) + (int64_t)(j0 + j) * lda] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        const int idx = t + (h + u) * TS_THREADS;
        ls[(idx / NB) * TS_LD + idx % NB] = v[u];
      }
    }
  }
  __syncthreads();
  ts_block_apply(ds, bs, xs, nb, r, TRANS);
  __syncthreads();
  double* red = bs;  // B_k is no longer needed: partial sums of the upper kk half, [TS_ROWS][8]
  int row;
  if constexpr (TRANS) row = blockIdx.x * TS_ROWS + q;  // column j of L = row j of B
  else row = k0 + nb + blockIdx.x * TS_ROWS + q;
  const bool active = TRANS ? (row < k0) : (row < n);
  const double* Lrow = Lb + row + (int64_t)k0 * lda;
  for (int c0 = 0; c0 < r; c0 += RC) {
    const int rc = min(RC, r - c0);
    double acc[RC];
#pragma unroll
    for (int c = 0; c < RC; ++c) acc[c] = 0.0;
    if (active) {
#pragma unroll
      for (int u0 = 0; u0 < NB / 2; u0 += 16) {
        double lv[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int kk = kh0 + u0 + u;
          if constexpr (TRANS) lv[u] = ls[q * TS_LD + kk];
          else lv[u] = (kk < nb) ? Lrow[(int64_t)kk * lda] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int kk = kh0 + u0 + u;
          if (kk < nb) {
#pragma unroll
            for (int c = 0; c < RC; ++c)
              if (c < rc) acc[c] = fma(lv[u], xs[kk + (c0 + c) * nb], acc[c]);
          }
        }
      }
    }
    if (half == 1) {
#pragma unroll
      for (int c = 0; c < RC; ++c) red[q * RC + c] = acc[c];
    }
    __syncthreads();
    if (half == 0 && active) {
#pragma unroll
      for (int c = 0; c < RC; ++c)
        if (c < rc) Bb[row + (int64_t)(c0 + c) * ldb] -= acc[c] + red[q * RC + c];
    }
    __syncthreads();
  }
}

size_t trsv_smem(int r, bool trans) {
  return sizeof(double) * ((size_t)2 * NB * std::max(r, 8) + (size_t)NB * TS_LD + (trans ? (size_t)TS_ROWS * TS_LD : 0));
}

template <bool TRANS, int RC>
void trsv_launch_rc(const double* L, int64_t lda, int64_t mstride, const double* Dinv, int64_t dstride, double* B,
                    int64_t ldb, int64_t bstride, int n, int k, int kw, int r, int nupd, int batch, cudaStream_t st) {
  static bool attr_set = false;  // one flag per instantiation
  if (!attr_set) {
    LKG_CUDA(cudaFuncSetAttribute(k_trsv_step<TRANS, RC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)trsv_smem(16, TRANS)));
    attr_set = true;
  }
  const int grid = nupd + (kw >= 0 ? 1 : 0);
  const double rows = (double)nupd * TS_ROWS;
  const char* name = TRANS ? "k_trsv_step_t" : "k_trsv_step";
  LaunchTimer lt(name, st, 2.0 * rows * NB * r * batch, 8.0 * (rows * NB + 2.0 * rows * r) * batch);
  k_trsv_step<TRANS, RC><<<dim3(grid, 1, batch), TS_THREADS, trsv_smem(r, TRANS), st>>>(
      L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, kw, r, nupd);
  LKG_LAUNCH(name);
}

template <bool TRANS>
void trsv_launch(const double* L, int64_t lda, int64_t mstride, const double* Dinv, int64_t dstride, double* B,
                 int64_t ldb, int64_t bstride, int n, int k, int kw, int r, int nupd, int batch, cudaStream_t st) {
  if (nupd + (kw >= 0 ? 1 : 0) == 0) return;
  if (r == 1)
    trsv_launch_rc<TRANS, 1>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, kw, r, nupd, batch, st);
  else if (r == 2)
    trsv_launch_rc<TRANS, 2>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, kw, r, nupd, batch, st);
  else if (r <= 4)
    trsv_launch_rc<TRANS, 4>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, kw, r, nupd, batch, st);
  else
    trsv_launch_rc<TRANS, 8>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, kw, r, nupd, batch, st);
}

__global__ void __launch_bounds__(256) k_copy_dinv_block(const double* __restrict__ Dinv, int64_t dinv_bstride,
                                                         int blk, double* W, int64_t ldw, int64_t wstride, int k0,
                                                         int nb) {
  const int64_t b = blockIdx.z;
  const double* D = Dinv + b * dinv_bstride + (int64_t)blk * NB * NB;
  double* Wb = W + b * wstride + k0 + (int64_t)k0 * ldw;
  double v[NB * NB / 256];
#pragma unroll
  for (int u = 0; u < NB * NB / 256; ++u) v[u] = D[threadIdx.x + u * 256];
#pragma unroll
  for (int u = 0; u < NB * NB / 256; ++u) {
    const int idx = threadIdx.x + u * 256, i = idx % NB, j = idx / NB;
    if (i < nb && j < nb) Wb[i + (int64_t)j * ldw] = v[u];
  }
}

// Inverses of the NB x NB diagonal blocks of an existing lower factor (one CTA per block): the same row wavefront as
// k_potrf_diag, so a block inverted here equals the one the factorisation itself stored.
__global__ void __launch_bounds__(NT) k_trtri_diag(const double* L, int64_t lda, int64_t mstride, int n, double* Dinv,
                                                   int64_t dinv_bstride) {
  extern __shared__ double tsm[];
  double* s = tsm;
  double* w = tsm + NB * DPAD;
  double* scratch = w + NB * DPAD;
  const int64_t b = blockIdx.z;
  const int blk = blockIdx.x, k0 = blk * NB, nb = min(NB, n - k0);
  const double* Lb = L + b * mstride + k0 + (int64_t)k0 * lda;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  {  // all 16 loads of a thread in flight before the shared-memory stores
    double v[NB * NB / NT];
#pragma unroll
    for (int u = 0; u < NB * NB / NT; ++u) {
      const int idx = t + u * NT, i = idx & 63, j = idx >> 6;
      v[u] = (i < nb && j < nb) ? ((i >= j) ? Lb[i + (int64_t)j * lda] : 0.0) : (i == j ? 1.0 : 0.0);
    }
#pragma unroll
    for (int u = 0; u < NB * NB / NT; ++u) {
      const int idx = t + u * NT, i = idx & 63, j = idx >> 6;
      s[i * DPAD + j] = v[u];
      w[i * DPAD + j] = 0.0;
    }
  }
  __syncthreads();
  if (warp < NB / PB) diag16_inverse(s, w, warp * PB, lane);
  __syncthreads();
  assemble_inverse(s, w, scratch, t);
  double* Db = Dinv + b * dinv_bstride + (int64_t)blk * NB * NB;
  for (int idx = t; idx < NB * NB; idx += NT) {
    const int i = idx & 63, j = idx >> 6;
    Db[i + j * NB] = (i >= j && i < nb && j < nb) ? w[i * DPAD + j] : 0.0;
  }
}

// D(c, r) = S(r, c) for an rows x cols block; 32 x 32 tiles through shared memory
__global__ void k_transpose_copy(const double* __restrict__ S, int64_t lds, double* __restrict__ D, int64_t ldd,
                                 int rows, int cols) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  for (int k = ty; k < 32; k += 8) {
    const int r = r0 + tx, c = c0 + k;
    tile[k][tx] = (r < rows && c < cols) ? S[r + (int64_t)c * lds] : 0.0;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + tx, r = r0 + k;  // D(c, r) with c contiguous
    if (r < rows && c < cols) D[c + (int64_t)r * ldd] = tile[tx][k];
  }
}

__global__ void k_add_diag(double* A, int64_t lda, int n, double v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) A[i + (int64_t)i * lda] += v;
}

// zero the strictly upper part of an n x n block (column j: rows 0 .. j-1)
__global__ void k_zero_upper(double* A, int64_t lda, int64_t mstride, int n) {
  const int64_t b = blockIdx.z;
  const int j = blockIdx.x;
  double* col = A + b * mstride + (int64_t)j * lda;
  for (int i = threadIdx.x; i < j && i < n; i += blockDim.x) col[i] = 0.0;
}

bool g_diag_attr_set = false;
bool g_trtri_diag_attr_set = false;

}  // namespace

void trtri_diag_blocks(const double* L, int64_t lda, int64_t mstride, int n, double* Dinv, int batch,
                       cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const size_t smem = (2 * NB * DPAD + 3 * PB * PB) * sizeof(double);
  if (!g_trtri_diag_attr_set) {
    LKG_CUDA(cudaFuncSetAttribute(k_trtri_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    g_trtri_diag_attr_set = true;
  }
  LaunchTimer lt("k_trtri_diag", st, (double)nblk * NB * NB * NB / 3.0 * batch, 16.0 * nblk * NB * NB * batch);
  k_trtri_diag<<<dim3(nblk, 1, batch), NT, smem, st>>>(L, lda, mstride, n, Dinv, (int64_t)nblk * NB * NB);
  LKG_LAUNCH("k_trtri_diag");
}

void transpose_copy(const double* S, int64_t lds, double* D, int64_t ldd, int rows, int cols, cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return;
  LaunchTimer lt("k_transpose_copy", st, 0.0, 16.0 * rows * cols);
  k_transpose_copy<<<dim3(ceil_div(rows, 32), ceil_div(cols, 32)), 256, 0, st>>>(S, lds, D, ldd, rows, cols);
  LKG_LAUNCH("k_transpose_copy");
}

void add_diag(double* A, int64_t lda, int n, double v, cudaStream_t st) {
  if (n <= 0) return;
  k_add_diag<<<ceil_div(n, 256), 256, 0, st>>>(A, lda, n, v);
  LKG_LAUNCH("k_add_diag");
}

void zero_upper(double* A, int64_t lda, int64_t mstride, int n, int batch, cudaStream_t st) {
  if (n <= 1) return;
  k_zero_upper<<<dim3(n, 1, batch), 128, 0, st>>>(A, lda, mstride, n);
  LKG_LAUNCH("k_zero_upper");
}

void gemm_tiles(int M, int N, int K, double alpha, MatView A, MatView B, double beta, double* C, int64_t ldc,
                int64_t c_batch, int batch, bool lower_only, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  dim3 grid(ceil_div(M, TB), ceil_div(N, TB), batch);
  const double fl = (lower_only && M == N) ? (double)K * M * (M + 1.0) : 2.0 * M * N * K;
  const double by = 8.0 * ((double)M * K + (double)K * N + (beta == 0.0 ? 1.0 : 2.0) * M * N);
  LaunchTimer lt("k_gemm_tiles", st, fl * batch, by * batch);
  k_gemm_tiles<<<grid, NT, 0, st>>>(M, N, K, alpha, A, B, beta, C, ldc, c_batch, lower_only);
  LKG_LAUNCH("k_gemm_tiles");
}

void potrf_diag(double* A, int64_t lda, int64_t mstride, int k0, int nb, double* Dinv, int64_t dinv_bstride, int blk,
                int* info, int batch, cudaStream_t st) {
  const size_t smem = (2 * NB * DPAD + 3 * PB * PB) * sizeof(double);
  if (!g_diag_attr_set) {
    LKG_CUDA(cudaFuncSetAttribute(k_potrf_diag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    g_diag_attr_set = true;
  }
  LaunchTimer lt("k_potrf_diag", st, 2.0 * nb * nb * nb / 3.0 * batch, 16.0 * nb * nb * batch);
  k_potrf_diag<<<dim3(1, 1, batch), NT, smem, st>>>(A, lda, mstride, k0, nb, Dinv, dinv_bstride, blk, info);
  LKG_LAUNCH("k_potrf_diag");
}

void potrf_blocked(double* A, int64_t lda, int64_t mstride, int n, double* Dinv, int* info, int batch,
                   cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  LKG_CUDA(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
  for (int k = 0; k < nblk; ++k) {
    const int k0 = k * NB, nb = std::min(NB, n - k0);
    potrf_diag(A, lda, mstride, k0, nb, Dinv, dstride, k, info, batch, st);
    const int M = n - k0 - nb;
    if (M <= 0) continue;
    double* A21 = A + (k0 + nb) + (int64_t)k0 * lda;
    // L21 = A21 * Dinv_k^T   (in place: each CTA reads its whole row block before writing)
    MatView a{A21, 1, lda, mstride};
    MatView bt{Dinv + (int64_t)k * NB * NB, NB, 1, dstride};  // B(kk, c) = Dinv(c, kk)
    gemm_tiles(M, nb, nb, 1.0, a, bt, 0.0, A21, lda, mstride, batch, false, st);
    // A22 -= L21 L21^T (lower tiles)
    MatView l21t{A21, lda, 1, mstride};  // B(kk, c) = L21(c, kk)
    gemm_tiles(M, M, nb, -1.0, a, l21t, 1.0, A21 + (int64_t)nb * lda, lda, mstride, batch, true, st);
  }
}

void copy_dinv_block(const double* Dinv, int64_t dinv_bstride, int blk, double* W, int64_t ldw, int64_t wstride,
                     int k0, int nb, int batch, cudaStream_t st) {
  LaunchTimer lt("k_copy_dinv_block", st, 0.0, 16.0 * nb * nb * batch);
  k_copy_dinv_block<<<dim3(1, 1, batch), 256, 0, st>>>(Dinv, dinv_bstride, blk, W, ldw, wstride, k0, nb);
  LKG_LAUNCH("k_copy_dinv_block");
}

void trtri_blocked(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* W, int64_t ldw,
                   int64_t wstride, int batch, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  for (int b = 0; b < batch; ++b)
    LKG_CUDA(cudaMemset2DAsync(W + b * wstride, ldw * sizeof(double), 0, n * sizeof(double), n, st));
  for (int k = 0; k < nblk; ++k) {
    const int k0 = k * NB, nb = std::min(NB, n - k0);
    copy_dinv_block(Dinv, dstride, k, W, ldw, wstride, k0, nb, batch, st);
    if (k0 > 0) {
      // W(k0:k0+nb, 0:k0) = -Dinv_k * Acc(k0:k0+nb, 0:k0)   (in place per column tile)
      MatView d{Dinv + (int64_t)k * NB * NB, 1, NB, dstride};
      MatView acc{W + k0, 1, ldw, wstride};
      gemm_tiles(nb, k0, nb, -1.0, d, acc, 0.0, W + k0, ldw, wstride, batch, false, st);
    }
    const int M2 = n - k0 - nb;
    if (M2 > 0) {
      // Acc(k0+nb:, 0:k0+nb) += L(k0+nb:, k0:k0+nb) * W(k0:k0+nb, 0:k0+nb)
      MatView a{L + (k0 + nb) + (int64_t)k0 * lda, 1, lda, mstride};
      MatView bw{W + k0, 1, ldw, wstride};
      gemm_tiles(M2, k0 + nb, nb, 1.0, a, bw, 1.0, W + k0 + nb, ldw, wstride, batch, false, st);
    }
  }
}

void wtw_lower(const double* W, int64_t ldw, int64_t wstride, int n, double* C, int64_t ldc, int64_t cstride,
               int batch, cudaStream_t st) {
  const int nblk = ceil_div(n, TB);
  const int64_t ntiles = (int64_t)nblk * (nblk + 1) / 2;
  // sum over the lower triangle of 2 (n - i) flops per entry = n (n + 1) (n + 2) / 3
  LaunchTimer lt("k_wtw", st, (double)n * (n + 1.0) * (n + 2.0) / 3.0 * batch, 8.0 * n * (n + 1.0) * batch);
  k_wtw<<<dim3((unsigned)ntiles, 1, batch), NT, 0, st>>>(W, ldw, wstride, n, C, ldc, cstride);
  LKG_LAUNCH("k_wtw");
}

void trsm_lower_left(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* B,
                     int64_t ldb, int64_t bstride, int r, int batch, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  if (r > 16 && batch != 1 && mstride == 0)
    throw std::invalid_argument("trsm_lower_left: shared factor with many right-hand sides is not supported");
  if (r > 16) {  // many right-hand sides: tile GEMMs (X_k = Dinv_k B_k in place per column tile, then update)
    for (int k = 0; k < nblk; ++k) {
      const int k0 = k * NB, nb = std::min(NB, n - k0);
      const int M = n - k0 - nb;
      MatView d{Dinv + (int64_t)k * NB * NB, 1, NB, dstride};
      MatView bk{B + k0, 1, ldb, bstride};
      gemm_tiles(nb, r, nb, 1.0, d, bk, 0.0, B + k0, ldb, bstride, batch, false, st);
      if (M > 0) {
        MatView a{L + (k0 + nb) + (int64_t)k0 * lda, 1, lda, mstride};
        gemm_tiles(M, r, nb, -1.0, a, bk, 1.0, B + k0 + nb, ldb, bstride, batch, false, st);
      }
    }
    return;
  }
  // step k updates the rows below block k and writes X_{k-1}; the extra step writes the last block
  for (int k = 0; k <= nblk; ++k) {
    const int k0 = k * NB;
    const int M = (k < nblk) ? n - k0 - std::min(NB, n - k0) : 0;
    trsv_launch<false>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, k - 1, r, ceil_div(M, TS_ROWS), batch,
                       st);
  }
}

void trsm_lower_left_t(const double* L, int64_t lda, int64_t mstride, int n, const double* Dinv, double* B,
                       int64_t ldb, int64_t bstride, int r, int batch, cudaStream_t st) {
  const int nblk = ceil_div(n, NB);
  const int64_t dstride = (int64_t)nblk * NB * NB;
  if (r > 16 && batch != 1 && mstride == 0)
    throw std::invalid_argument("trsm_lower_left_t: shared factor with many right-hand sides is not supported");
  if (r > 16) {  // many right-hand sides: X_k = Dinv_k^T B_k in place, then B_0:k0 -= L(k0:k0+nb, 0:k0)^T X_k
    for (int k = nblk - 1; k >= 0; --k) {
      const int k0 = k * NB, nb = std::min(NB, n - k0);
      MatView dt{Dinv + (int64_t)k * NB * NB, NB, 1, dstride};  // (i, kk) = Dinv_k(kk, i)
      MatView bk{B + k0, 1, ldb, bstride};
      gemm_tiles(nb, r, nb, 1.0, dt, bk, 0.0, B + k0, ldb, bstride, batch, false, st);
      if (k0 > 0) {
        MatView lt{L + k0, lda, 1, mstride};  // (i, kk) = L(k0 + kk, i)
        gemm_tiles(k0, r, nb, -1.0, lt, bk, 1.0, B, ldb, bstride, batch, false, st);
      }
    }
    return;
  }
  // step k (descending) updates the rows above block k and writes X_{k+1}; the extra step writes block 0
  for (int k = nblk - 1; k >= -1; --k) {
    const int nupd = (k >= 0) ? ceil_div(k * NB, TS_ROWS) : 0;
    trsv_launch<true>(L, lda, mstride, Dinv, dstride, B, ldb, bstride, n, k, (k + 1 < nblk) ? k + 1 : -1, r, nupd,
                      batch, st);
  }
}

}  // namespace lkg
