// nested_kernels.cu -- k-means assignment and the NK aggregation's per-chunk kernels (nested_kernels.cuh).
#include "common.cuh"
#include "nested_kernels.cuh"
#include "stats.hpp"

namespace lkg {

namespace {

constexpr int KT = 256;  // centroids per shared-memory tile of the assignment kernel

template <int DM>
__global__ void __launch_bounds__(256) k_kmeans_assign(int N, int d, const double* __restrict__ X, int k,
                                                       const double* __restrict__ C, int* __restrict__ assign) {
  __shared__ double sc[KT * DM];
  const int i = blockIdx.x * 256 + threadIdx.x;
  double x[DM];
#pragma unroll
  for (int q = 0; q < DM; ++q) x[q] = (q < d && i < N) ? X[i + (int64_t)q * N] : 0.0;
  double best = INFINITY;
  int bi = 0;
  for (int c0 = 0; c0 < k; c0 += KT) {
    const int nc = min(KT, k - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nc * d; idx += 256) sc[(idx / d) * DM + idx % d] = C[(int64_t)c0 * d + idx];
    __syncthreads();
    for (int c = 0; c < nc; ++c) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < DM; ++q)
        if (q < d) {
          const double dq = __dsub_rn(x[q], sc[c * DM + q]);
          s = __dadd_rn(s, __dmul_rn(dq, dq));
        }
      if (s < best) {
        best = s;
        bi = c0 + c;
      }
    }
  }
  if (i < N) assign[i] = bi;
}

template <int K, int DM>
__global__ void __launch_bounds__(128) k_nk_corr(int n, int d, const double* __restrict__ X, int64_t xs,
                                                 const int* __restrict__ nvalid, const double* __restrict__ theta,
                                                 const double* __restrict__ Xc, int qc, double* __restrict__ out,
                                                 int64_t os) {
  const int e = blockIdx.z, t = blockIdx.y;
  const int a = blockIdx.x * 128 + threadIdx.x;
  if (a >= n) return;
  double v = 0.0;
  if (a < nvalid[e]) {
    const double* Xe = X + (int64_t)e * xs;
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < DM; ++q)
      if (q < d) s += cov_term<K>(Xe[a + (int64_t)q * n] - Xc[t + (int64_t)q * qc], theta[q]);
    v = cov_from_sum<K>(s);
  }
  out[(int64_t)e * os + a + (int64_t)t * n] = v;
}

// one warp per (entry, chunk point)
__global__ void __launch_bounds__(256) k_nk_moments(int n, int qc, const double* __restrict__ U, int64_t us,
                                                    const double* __restrict__ z, int64_t zs, double beta0,
                                                    double* __restrict__ M, double* __restrict__ Kd, int64_t ms) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * 8 + w, e = blockIdx.y;
  if (t >= qc) return;
  const double* u = U + (int64_t)e * us + (int64_t)t * n;
  const double* ze = z + (int64_t)e * zs;
  double m = 0.0, kk = 0.0;
  for (int a = lane; a < n; a += 32) {
    const double ua = u[a];
    m += ua * ze[a];
    kk += ua * ua;
  }
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    kk += __shfl_xor_sync(0xffffffffu, kk, o);
  }
  if (lane == 0) {
    M[(int64_t)e * ms + t] = beta0 + m;
    Kd[(int64_t)e * ms + t] = kk;
  }
}

// block = (pair of groups, up to NKP chunk points); thread (ty, tx): rows a0 + ty + 8m of group i and chunk points
// t0 + tx + 32u.  Each 32 x 32 tile of R_ij is formed once (division- and log1p-free covariance form) and applied to
// every chunk point of the block: T(a, t) = sum_b R_ij(a, b) W_j(b, t), then cross(t) = sum_a W_i(a, t) T(a, t).
constexpr int NKP = 128;
template <int K, int DM>
__global__ void __launch_bounds__(256) k_nk_cross(int p, int d, const NkGroup* __restrict__ G,
                                                  const double* __restrict__ theta, int qc,
                                                  double* __restrict__ cross) {
  __shared__ double sxi[32][DM], sxj[32][DM], sR[32][33], sW[32][NKP + 1];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  long long k = blockIdx.x;
  int i = 0;
  while (k >= p - 1 - i) {
    k -= p - 1 - i;
    ++i;
  }
  const int j = i + 1 + (int)k;
  const NkGroup gi = G[i], gj = G[j];
  const int t0 = blockIdx.y * NKP, nt = min(NKP, qc - t0);
  double ck[DM];
#pragma unroll
  for (int q = 0; q < DM; ++q) ck[q] = cov_scale<K>() / ((q < d) ? theta[q] : 1.0);
  double cacc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int a0 = 0; a0 < gi.n; a0 += 32) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < 32 * DM; idx += 256) {
      const int a = idx % 32, q = idx / 32;
      sxi[a][q] = (q < d && a0 + a < gi.n) ? gi.X[(a0 + a) + (int64_t)q * gi.ldx] : 0.0;
    }
    double T[4][4] = {};
    for (int b0 = 0; b0 < gj.n; b0 += 32) {
      __syncthreads();
      for (int idx = threadIdx.x; idx < 32 * DM; idx += 256) {
        const int b = idx % 32, q = idx / 32;
        sxj[b][q] = (q < d && b0 + b < gj.n) ? gj.X[(b0 + b) + (int64_t)q * gj.ldx] : 0.0;
      }
      for (int idx = threadIdx.x; idx < 32 * NKP; idx += 256) {  // coalesced over b: sW[b][tt] = W_j(b0 + b, t0 + tt)
        const int b = idx % 32, tt = idx / 32;
        sW[b][tt] = (b0 + b < gj.n && tt < nt) ? gj.W[(b0 + b) + (int64_t)(t0 + tt) * gj.ldw] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int a = ty + 8 * m;
        double v = 0.0;
        if (a0 + a < gi.n && b0 + tx < gj.n) {
          double sum = 0.0, prod = 1.0;
#pragma unroll
          for (int q = 0; q < DM; ++q)
            if (q < d) cov_fast_term<K>(sxi[a][q] - sxj[tx][q], ck[q], sum, prod);
          v = cov_fast_finish<K>(sum, prod);
        }
        sR[a][tx] = v;
      }
      __syncthreads();
#pragma unroll 4
      for (int bb = 0; bb < 32; ++bb) {
        double w[4], r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) w[u] = sW[bb][tx + 32 * u];
#pragma unroll
        for (int m = 0; m < 4; ++m) r[m] = sR[ty + 8 * m][bb];
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
          for (int u = 0; u < 4; ++u) T[m][u] = fma(r[m], w[u], T[m][u]);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int tt = tx + 32 * u;
      if (tt >= nt) continue;
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int a = a0 + ty + 8 * m;
        if (a < gi.n) cacc[u] = fma(gi.W[a + (int64_t)(t0 + tt) * gi.ldw], T[m][u], cacc[u]);
      }
    }
  }
  // fixed-order sum over the 8 row groups (sR reused: 8 x NKP partials)
  __syncthreads();
  double* red = &sR[0][0];
#pragma unroll
  for (int u = 0; u < 4; ++u) red[ty * NKP + tx + 32 * u] = cacc[u];
  __syncthreads();
  if (ty < 4) {
    const int tt = tx + 32 * ty;
    if (tt < nt) {
      double s = red[tt];
      for (int r = 1; r < 8; ++r) s += red[r * NKP + tt];
      cross[(int64_t)blockIdx.x * qc + t0 + tt] = s;
    }
  }
}

template <int K, int DM>
struct NkCorrLaunch {
  static void run(int n, int d, const double* X, int64_t xs, const int* nvalid, int ne, const double* theta,
                  const double* Xc, int qc, double* out, int64_t os, cudaStream_t st) {
    LaunchTimer lt("k_nk_corr", st, (double)n * qc * ne, 8.0 * n * qc * ne);
    k_nk_corr<K, DM><<<dim3(ceil_div(n, 128), qc, ne), 128, 0, st>>>(n, d, X, xs, nvalid, theta, Xc, qc, out, os);
    LKG_LAUNCH("k_nk_corr");
  }
};

template <int K, int DM>
struct NkCrossLaunch {
  static void run(int d, int p, const NkGroup* groups, const double* theta, int qc, double* cross, cudaStream_t st) {
    const long long npairs = (long long)p * (p - 1) / 2;
    if (npairs <= 0) return;
    if (npairs > 0x7fffffffLL) throw std::invalid_argument("NK aggregation: too many groups");
    LaunchTimer lt("k_nk_cross", st, 0.0, 0.0);
    k_nk_cross<K, DM><<<dim3((unsigned)npairs, ceil_div(qc, NKP), 1), 256, 0, st>>>(p, d, groups, theta, qc, cross);
    LKG_LAUNCH("k_nk_cross");
  }
};

}  // namespace

void kmeans_assign(int N, int d, const double* X, int k, const double* C, int* assign, cudaStream_t st) {
  if (N <= 0) return;
  if (k < 1) throw std::invalid_argument("kmeans_assign: k < 1");
  LaunchTimer lt("k_kmeans_assign", st, 3.0 * N * (double)k * d, 8.0 * N * d);
  if (d <= 4)
    k_kmeans_assign<4><<<ceil_div(N, 256), 256, 0, st>>>(N, d, X, k, C, assign);
  else if (d <= 8)
    k_kmeans_assign<8><<<ceil_div(N, 256), 256, 0, st>>>(N, d, X, k, C, assign);
  else
    throw std::invalid_argument("k-means partition on the GPU supports d <= 8");
  LKG_LAUNCH("k_kmeans_assign");
}

void nk_corr_entries(int kernel, int n, int d, const double* X, int64_t x_estride, const int* nvalid, int ne,
                     const double* theta, const double* Xc, int qc, double* out, int64_t o_estride, cudaStream_t st) {
  if (n <= 0 || qc <= 0 || ne <= 0) return;
  dispatch_kd<NkCorrLaunch>(kernel, d, n, d, X, x_estride, nvalid, ne, theta, Xc, qc, out, o_estride, st);
}

void nk_moments(int n, int qc, const double* U, int64_t u_estride, const double* z, int64_t z_estride, double beta0,
                int ne, double* M, double* K, int64_t mk_estride, cudaStream_t st) {
  if (n <= 0 || qc <= 0 || ne <= 0) return;
  k_nk_moments<<<dim3(ceil_div(qc, 8), ne, 1), 256, 0, st>>>(n, qc, U, u_estride, z, z_estride, beta0, M, K,
                                                             mk_estride);
  LKG_LAUNCH("k_nk_moments");
}

void nk_cross(int kernel, int d, int p, const NkGroup* groups, const double* theta, int qc, double* cross,
              cudaStream_t st) {
  if (p < 2 || qc <= 0) return;
  if (d > 8) throw std::invalid_argument("NK aggregation on the GPU supports d <= 8");
  auto go = [&](auto kc) {
    constexpr int KK = decltype(kc)::value;
    if (d <= 4)
      NkCrossLaunch<KK, 4>::run(d, p, groups, theta, qc, cross, st);
    else
      NkCrossLaunch<KK, 8>::run(d, p, groups, theta, qc, cross, st);
  };
  switch (kernel) {
    case KGAUSS: go(std::integral_constant<int, KGAUSS>{}); break;
    case KEXP: go(std::integral_constant<int, KEXP>{}); break;
    case KMATERN32: go(std::integral_constant<int, KMATERN32>{}); break;
    case KMATERN52: go(std::integral_constant<int, KMATERN52>{}); break;
    default: throw std::invalid_argument("Unsupported covariance kernel id");
  }
}

}  // namespace lkg
