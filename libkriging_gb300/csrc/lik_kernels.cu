// lik_kernels.cu -- covariance build, adjoint gradient and likelihood reductions (sm_103a).
//
// Reference routines these kernels replace (libKriging source tree):
//   cov_build_lower   LinearAlgebra::cholCov pair loop + "R *= factor" + diag  (src/lib/LinearAlgebra.cpp:142-181)
//                     with dX recomputed from X instead of the n^2 x d cube of compute_dX (:440-485)
//   adjoint_sums      KrigingImpl::compute_ll_grad_theta_vecs (src/lib/KrigingImpl.cpp:855-885) and the Nugget
//                     alpha-gradient dot products of Kriging::_logLikelihood (src/lib/Kriging.cpp:307-326)
//   gram/gls/residual KrigingImpl::populate_Model GLS block (src/lib/KrigingImpl.cpp:101-124)
//   cov_cross         KrigingImpl::predict_impl R_on loop (src/lib/KrigingImpl.cpp:194-221)
//   dcov_cross        KrigingImpl::predict_impl DR_on_i loop of the derivatives (src/lib/KrigingImpl.cpp:255-261)
#include "lik_kernels.cuh"

#include "stats.hpp"

namespace lkg {

namespace {

constexpr int T = 64;  // tile edge

__device__ __forceinline__ void lower_tile_of(int64_t x, int& I, int& J) {
  I = (int)((sqrt(8.0 * (double)x + 1.0) - 1.0) * 0.5);
  while ((int64_t)(I + 1) * (I + 2) / 2 <= x) ++I;
  while ((int64_t)I * (I + 1) / 2 > x) --I;
  J = (int)(x - (int64_t)I * (I + 1) / 2);
}

// deterministic block sum (fixed shuffle tree, then warps in order); every thread gets the result
template <int NTH>
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < NTH / 32; ++i) s += red[i];
  return s;
}

template <int K, int DM, bool FAST>
__global__ void __launch_bounds__(256) k_cov_lower(int n, int d, const double* __restrict__ X, int64_t xb,
                                                   const double* __restrict__ theta, const double* __restrict__ factor,
                                                   const double* __restrict__ diag, double* __restrict__ A,
                                                   int64_t lda, int64_t mstride, const int* __restrict__ nvalid) {
  int I, J;
  lower_tile_of(blockIdx.x, I, J);
  const int64_t b = blockIdx.z;
  __shared__ double xi[DM][T], xj[DM][T], th[DM];
  const int r0 = I * T, c0 = J * T, t = threadIdx.x;
  const double* Xb = X + b * xb;
  for (int idx = t; idx < DM * T; idx += 256) {
    const int k = idx / T, q = idx % T;
    xi[k][q] = (k < d && r0 + q < n) ? Xb[(r0 + q) + (int64_t)k * n] : 0.0;
    xj[k][q] = (k < d && c0 + q < n) ? Xb[(c0 + q) + (int64_t)k * n] : 0.0;
  }
  if (t < DM) th[t] = (t < d) ? theta[b * d + t] : 1.0;
  __syncthreads();
  const double f = factor[b], dv = diag[b];
  const int nv = nvalid ? nvalid[b] : n;  // rows/columns >= nv are padding: identity
  const int ri = t & 63, i = r0 + ri;
  if (i >= n) return;
  double* Ab = A + b * mstride;
  double xr[DM], ck[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) {
    xr[k] = xi[k][ri];
    ck[k] = FAST ? cov_scale<K>() / th[k] : 0.0;
  }
  for (int s = 0; s < 16; ++s) {
    const int cj = (t >> 6) + 4 * s, j = c0 + cj;
    if (j >= n || j > i) continue;
    double v;
    if (i >= nv) {
      v = (j == i) ? 1.0 : 0.0;
    } else if (j == i) {
      v = dv;
    } else if (FAST) {
      double sum = 0.0, prod = 1.0;
#pragma unroll
      for (int k = 0; k < DM; ++k)
        if (k < d) cov_fast_term<K>(xj[k][cj] - xr[k], ck[k], sum, prod);
      v = cov_fast_finish<K>(sum, prod) * f;
    } else {
      double sum = 0.0;
#pragma unroll
      for (int k = 0; k < DM; ++k)
        if (k < d) sum += cov_term<K>(xj[k][cj] - xr[k], th[k]);
      v = cov_from_sum<K>(sum) * f;
    }
    Ab[i + (int64_t)j * lda] = v;
  }
}

template <int K, int DM>
__global__ void __launch_bounds__(256) k_cov_cross(int n_o, int q, int d, const double* __restrict__ Xo,
                                                   const double* __restrict__ Xn, const double* __restrict__ theta,
                                                   double factor, double* __restrict__ R, bool snap) {
  __shared__ double xo[DM][T], xn[DM][T], th[DM];
  const int r0 = blockIdx.x * T, c0 = blockIdx.y * T, t = threadIdx.x;
  for (int idx = t; idx < DM * T; idx += 256) {
    const int k = idx / T, qq = idx % T;
    xo[k][qq] = (k < d && r0 + qq < n_o) ? Xo[(r0 + qq) + (int64_t)k * n_o] : 0.0;
    xn[k][qq] = (k < d && c0 + qq < q) ? Xn[(c0 + qq) + (int64_t)k * q] : 0.0;
  }
  if (t < DM) th[t] = (t < d) ? theta[t] : 1.0;
  __syncthreads();
  const int ri = t & 63, i = r0 + ri;
  if (i >= n_o) return;
  for (int s = 0; s < 16; ++s) {
    const int cj = (t >> 6) + 4 * s, j = c0 + cj;
    if (j >= q) continue;
    double sum = 0.0;
    bool coincident = true;
#pragma unroll
    for (int k = 0; k < DM; ++k) {
      if (k < d) {
        const double dx = xo[k][ri] - xn[k][cj];
        coincident = coincident && (fabs(dx) <= 2.220446049250313e-16);
        sum += cov_term<K>(dx, th[k]);
      }
    }
    R[i + (int64_t)j * n_o] = (snap && coincident) ? 1.0 : cov_from_sum<K>(sum) * factor;
  }
}

// d ln C / d x_k at dx = x_new - x_obs (Covariance.cpp:52-63, 90-100, 132-145, 181-196), the reference's operation
// order: gauss -dx / theta^2; exp -sign(dx) / theta; matern3_2 -sqrt3 sign t / (1 + t) / theta;
// matern5_2 -sqrt5 sign (a b) / (a + t b) / theta with t = s |dx / theta|, a = 1 + t, b = t / 3.
template <int K>
__device__ __forceinline__ double dlncov_dx(double dx, double th) {
  const double sg = dx > 0.0 ? 1.0 : (dx < 0.0 ? -1.0 : 0.0);
  if constexpr (K == KGAUSS) {
    return -dx / (th * th);
  } else if constexpr (K == KEXP) {
    return -sg / th;
  } else if constexpr (K == KMATERN32) {
    const double t = sqrt(3.0) * fabs(dx / th);
    return -sqrt(3.0) * sg * t / (1.0 + t) / th;
  } else {
    const double t = sqrt(5.0) * fabs(dx / th);
    const double a = 1.0 + t, b = t / 3.0;
    return -sqrt(5.0) * sg * (a * b) / (a + t * b) / th;
  }
}

// DR(j, c * d + k) = R_on(j, c) d ln C / d x_k (Xn_c - Xo_j) for the q new points c (KrigingImpl.cpp:256-261), with
// R_on(j, c) formed exactly as k_cov_cross forms it (coincident points give 1).  n_o x (q d), ld n_o.
template <int K, int DM>
__global__ void __launch_bounds__(256) k_dcov_cross(int n_o, int q, int d, const double* __restrict__ Xo,
                                                    const double* __restrict__ Xn, const double* __restrict__ theta,
                                                    double factor, double* __restrict__ DR) {
  __shared__ double xo[DM][T], xn[DM][T], th[DM];
  const int r0 = blockIdx.x * T, c0 = blockIdx.y * T, t = threadIdx.x;
  for (int idx = t; idx < DM * T; idx += 256) {
    const int k = idx / T, qq = idx % T;
    xo[k][qq] = (k < d && r0 + qq < n_o) ? Xo[(r0 + qq) + (int64_t)k * n_o] : 0.0;
    xn[k][qq] = (k < d && c0 + qq < q) ? Xn[(c0 + qq) + (int64_t)k * q] : 0.0;
  }
  if (t < DM) th[t] = (t < d) ? theta[t] : 1.0;
  __syncthreads();
  const int ri = t & 63, i = r0 + ri;
  if (i >= n_o) return;
  for (int s = 0; s < 16; ++s) {
    const int cj = (t >> 6) + 4 * s, j = c0 + cj;
    if (j >= q) continue;
    double sum = 0.0;
    bool coincident = true;
#pragma unroll
    for (int k = 0; k < DM; ++k) {
      if (k < d) {
        const double dx = xo[k][ri] - xn[k][cj];
        coincident = coincident && (fabs(dx) <= 2.220446049250313e-16);
        sum += cov_term<K>(dx, th[k]);
      }
    }
    const double r = coincident ? 1.0 : cov_from_sum<K>(sum) * factor;
    double* out = DR + i + (int64_t)j * d * n_o;
#pragma unroll
    for (int k = 0; k < DM; ++k)
      if (k < d) out[(int64_t)k * n_o] = r * dlncov_dx<K>(xn[k][cj] - xo[k][ri], th[k]);
  }
}

template <int K, int DM>
__global__ void __launch_bounds__(256) k_adjoint(int n, int d, const double* __restrict__ X, int64_t xb,
                                                 const double* __restrict__ theta, const double* __restrict__ factor,
                                                 const double* __restrict__ xv, int64_t xvb,
                                                 const double* __restrict__ Rinv, int64_t ldr, int64_t rstride,
                                                 double* __restrict__ partials, int64_t ntiles) {
  int I, J;
  lower_tile_of(blockIdx.x, I, J);
  const int64_t b = blockIdx.z;
  constexpr int NA = 2 * DM + 4;
  __shared__ double xi[DM][T], xj[DM][T], th[DM], cks[DM], vi[T], vj[T];
  __shared__ double red[NA][8];
  const int r0 = I * T, c0 = J * T, t = threadIdx.x;
  const double* Xb = X + b * xb;
  for (int idx = t; idx < DM * T; idx += 256) {
    const int k = idx / T, q = idx % T;
    xi[k][q] = (k < d && r0 + q < n) ? Xb[(r0 + q) + (int64_t)k * n] : 0.0;
    xj[k][q] = (k < d && c0 + q < n) ? Xb[(c0 + q) + (int64_t)k * n] : 0.0;
  }
  if (t < T) {
    vi[t] = (r0 + t < n) ? xv[b * xvb + r0 + t] : 0.0;
    vj[t] = (c0 + t < n) ? xv[b * xvb + c0 + t] : 0.0;
  }
  if (t < DM) {
    th[t] = (t < d) ? theta[b * d + t] : 1.0;
    cks[t] = cov_scale<K>() / th[t];
  }
  __syncthreads();
  const double f = factor[b];
  double t1[DM], t2[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) t1[k] = t2[k] = 0.0;
  double u1 = 0.0, u2 = 0.0, d1 = 0.0, d2 = 0.0;
  const int ri = t & 63, i = r0 + ri;
  const double* Rb = Rinv + b * rstride;
  if (i < n) {
    // Division-free gradient sums.  With t_m = s |dx_m| / theta_m (s = 1, sqrt 3, sqrt 5), p_m the Matern polynomial
    // factor and E = factor exp(-sum_m t_m):
    //   gauss      r dlnC/dtheta_k = r v_k^2           / theta_k,  v_k = dx_k / theta_k
    //   exp        r dlnC/dtheta_k = r t_k             / theta_k
    //   matern3_2  r dlnC/dtheta_k = E t_k^2           prod_{m != k} p_m / theta_k
    //   matern5_2  r dlnC/dtheta_k = E t_k^2 (1 + t_k) prod_{m != k} p_m / (3 theta_k)
    // The Matern products over m != k come from prefix products and a running suffix product, so no term needs a
    // division; the 1 / theta_k (and 1/3) factor is applied once per accumulator after the pair loop.  The row's
    // coordinates and the scales stay in shared memory (the loop is bound by the FP64 pipe, not by its loads).
    const double x_i = vi[ri];
    for (int s = 0; s < 16; ++s) {
      const int cj = (t >> 6) + 4 * s, j = c0 + cj;
      if (j >= n || j > i) continue;
      const double rinv = Rb[i + (int64_t)j * ldr];
      if (j == i) {
        d1 += x_i * x_i;
        d2 += rinv;
        continue;
      }
      const double wx = x_i * vj[cj];
      double tk[DM], sum = 0.0;
#pragma unroll
      for (int k = 0; k < DM; ++k) {
        tk[k] = 0.0;
        if (k < d) {
          const double dx = xj[k][cj] - xi[k][ri];
          if constexpr (K == KGAUSS) {
            tk[k] = dx * cks[k];
            sum = fma(tk[k], tk[k], sum);
          } else {
            tk[k] = fabs(dx) * cks[k];
            sum += tk[k];
          }
        }
      }
      if constexpr (K == KGAUSS || K == KEXP) {
        const double c = exp(K == KGAUSS ? -0.5 * sum : -sum);
        const double rij = c * f;
        u1 = fma(wx, c, u1);
        u2 = fma(rinv, c, u2);
#pragma unroll
        for (int k = 0; k < DM; ++k) {
          if (k < d) {
            const double g = rij * (K == KGAUSS ? tk[k] * tk[k] : tk[k]);
            t1[k] = fma(wx, g, t1[k]);
            t2[k] = fma(rinv, g, t2[k]);
          }
        }
      } else {
        auto poly = [](double tt) { return (K == KMATERN32) ? 1.0 + tt : fma(tt, fma(tt, 1.0 / 3.0, 1.0), 1.0); };
        if constexpr (DM <= 16) {
          // prefix products pre[k] = prod_{m <= k} p_m and a running suffix product
          double pk[DM], pre[DM];
#pragma unroll
          for (int k = 0; k < DM; ++k) {
            pk[k] = poly(tk[k]);
            pre[k] = (k == 0) ? pk[0] : ((k < d) ? pre[k - 1] * pk[k] : pre[k - 1]);
          }
          const double ex = exp(-sum);
          const double c = pre[DM - 1] * ex;
          u1 = fma(wx, c, u1);
          u2 = fma(rinv, c, u2);
          double suf = ex * f;  // E prod_{m > k} p_m
#pragma unroll
          for (int k = DM - 1; k >= 0; --k) {
            if (k < d) {
              const double t2k = tk[k] * tk[k];
              const double q = (K == KMATERN32) ? t2k : fma(t2k, tk[k], t2k);
              const double g = (k > 0) ? q * (pre[k - 1] * suf) : q * suf;
              t1[k] = fma(wx, g, t1[k]);
              t2[k] = fma(rinv, g, t2[k]);
              suf *= pk[k];
            }
          }
        } else {
          // d > 16: the prefix array would not fit in registers; divide by p_k instead
          double prod = 1.0;
#pragma unroll
          for (int k = 0; k < DM; ++k)
            if (k < d) prod *= poly(tk[k]);
          const double ex = exp(-sum);
          const double c = prod * ex;
          const double rij = c * f;
          u1 = fma(wx, c, u1);
          u2 = fma(rinv, c, u2);
#pragma unroll
          for (int k = 0; k < DM; ++k) {
            if (k < d) {
              const double t2k = tk[k] * tk[k];
              const double q = (K == KMATERN32) ? t2k : fma(t2k, tk[k], t2k);
              const double g = rij * q / poly(tk[k]);
              t1[k] = fma(wx, g, t1[k]);
              t2[k] = fma(rinv, g, t2[k]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < DM; ++k) {
      const double sc = (K == KMATERN52 ? 1.0 / 3.0 : 1.0) / th[k];
      t1[k] *= sc;
      t2[k] *= sc;
    }
  }
  // deterministic block reduction of the NA accumulators
  const int w = t >> 5, l = t & 31;
  auto wred = [&](double v, int a) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) red[a][w] = v;
  };
#pragma unroll
  for (int k = 0; k < DM; ++k) {
    wred(t1[k], k);
    wred(t2[k], DM + k);
  }
  wred(u1, 2 * DM);
  wred(u2, 2 * DM + 1);
  wred(d1, 2 * DM + 2);
  wred(d2, 2 * DM + 3);
  __syncthreads();
  // compact layout: [T1(d), T2(d), U1, U2, D1, D2]
  const int nacc = 2 * d + 4;
  if (t < nacc) {
    int a;
    if (t < d) a = t;
    else if (t < 2 * d) a = DM + (t - d);
    else a = 2 * DM + (t - 2 * d);
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += red[a][q];
    partials[(b * ntiles + blockIdx.x) * nacc + t] = s;
  }
}

// out[b*nacc + a] = sum over tiles (fixed order)
__global__ void k_reduce_partials(const double* __restrict__ partials, int64_t ntiles, int nacc,
                                  double* __restrict__ out) {
  const int64_t b = blockIdx.z;
  const int a = blockIdx.x;
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t tt = threadIdx.x; tt < ntiles; tt += blockDim.x) s += partials[(b * ntiles + tt) * nacc + a];
  s = block_sum<1024>(s, red);
  if (threadIdx.x == 0) out[b * nacc + a] = s;
}

__global__ void k_gram_logdet(int n, int ncols, const double* __restrict__ M, int64_t ldm, int64_t mstride,
                              const double* __restrict__ L, int64_t ldl, int64_t lstride, double* __restrict__ out,
                              int64_t out_bstride) {
  const int64_t b = blockIdx.z;
  const int npairs = ncols * (ncols + 1) / 2;
  __shared__ double red[32];
  double s = 0.0;
  if ((int)blockIdx.x < npairs) {
    int q1, q2;
    lower_tile_of(blockIdx.x, q1, q2);
    const double* a = M + b * mstride + (int64_t)q1 * ldm;
    const double* c = M + b * mstride + (int64_t)q2 * ldm;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(a[i], c[i], s);
    s = block_sum<256>(s, red);
    if (threadIdx.x == 0) out[b * out_bstride + q1 * ncols + q2] = s;
  } else {
    const double* Lb = L + b * lstride;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += log(Lb[i + (int64_t)i * ldl]);
    s = block_sum<256>(s, red);
    if (threadIdx.x == 0) out[b * out_bstride + ncols * ncols] = s;
  }
}

constexpr int PMAX = 64;

__global__ void k_gls_solve(int p, const double* __restrict__ gram, int64_t gram_bstride, double* __restrict__ beta,
                            int64_t beta_bstride, double* __restrict__ rstar, int64_t rstar_bstride,
                            int* __restrict__ info) {
  const int64_t b = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int nc = p + 1;
  const double* g = gram + b * gram_bstride;
  double* U = rstar + b * rstar_bstride;  // p x p column-major, upper
  double h[PMAX], z[PMAX];
  for (int i = 0; i < p; ++i) h[i] = g[p * nc + i];  // row p (y*), col i (F*_i)
  // upper Cholesky U'U = G
  for (int j = 0; j < p; ++j) {
    for (int i = 0; i <= j; ++i) {
      double s = g[j * nc + i];  // G(i, j) = G(j, i), stored at row j col i (j >= i)
      for (int k = 0; k < i; ++k) s -= U[k + i * p] * U[k + j * p];
      if (i == j) {
        if (!(s > 0.0)) {
          info[b] = j + 1;
          return;
        }
        U[j + j * p] = sqrt(s);
      } else {
        U[i + j * p] = s / U[i + i * p];
      }
    }
    for (int i = j + 1; i < p; ++i) U[i + j * p] = 0.0;
  }
  // U' z = h ; U beta = z
  for (int i = 0; i < p; ++i) {
    double s = h[i];
    for (int k = 0; k < i; ++k) s -= U[k + i * p] * z[k];
    z[i] = s / U[i + i * p];
  }
  double* bt = beta + b * beta_bstride;
  for (int i = p - 1; i >= 0; --i) {
    double s = z[i];
    for (int k = i + 1; k < p; ++k) s -= U[i + k * p] * bt[k];
    bt[i] = s / U[i + i * p];
  }
  info[b] = 0;
}

__global__ void k_residual_sse(int n, int p, const double* __restrict__ FY, int64_t ldfy, int64_t fystride,
                               const double* __restrict__ beta, int64_t beta_bstride, double* __restrict__ Estar,
                               int64_t estride, double* __restrict__ sse, int64_t sse_bstride) {
  const int64_t b = blockIdx.x;
  __shared__ double red[32];
  __shared__ double bt[PMAX];
  if (threadIdx.x < p) bt[threadIdx.x] = beta[b * beta_bstride + threadIdx.x];
  __syncthreads();
  const double* M = FY + b * fystride;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double fb = 0.0;
    for (int q = 0; q < p; ++q) fb = fma(M[i + (int64_t)q * ldfy], bt[q], fb);
    const double e = M[i + (int64_t)p * ldfy] - fb;
    Estar[b * estride + i] = e;
    s = fma(e, e, s);
  }
  s = block_sum<1024>(s, red);
  if (threadIdx.x == 0) sse[b * sse_bstride] = s;
}

__global__ void k_lower_colsum_abs(int n, const double* __restrict__ L, int64_t ldl, int64_t lstride,
                                   double* __restrict__ colsum) {
  const int64_t b = blockIdx.z;
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= n) return;
  const double* c = L + b * lstride + (int64_t)j * ldl;
  double s = 0.0;
  for (int i = j + lane; i < n; i += 32) s += fabs(c[i]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) colsum[b * n + j] = s;
}

// ---- leave-one-out building blocks ----
template <int K, int DM>
__global__ void __launch_bounds__(256) k_loo_gradR(int n, int d, const double* __restrict__ X,
                                                   const double* __restrict__ theta, double factor, int kdim,
                                                   double* __restrict__ G, int64_t ldg) {
  __shared__ double xi[DM][T], xj[DM][T], th[DM];
  const int r0 = blockIdx.x * T, c0 = blockIdx.y * T, t = threadIdx.x;
  for (int idx = t; idx < DM * T; idx += 256) {
    const int k = idx / T, q = idx % T;
    xi[k][q] = (k < d && r0 + q < n) ? X[(r0 + q) + (int64_t)k * n] : 0.0;
    xj[k][q] = (k < d && c0 + q < n) ? X[(c0 + q) + (int64_t)k * n] : 0.0;
  }
  if (t < DM) th[t] = (t < d) ? theta[t] : 1.0;
  __syncthreads();
  const int ri = t & 63, i = r0 + ri;
  if (i >= n) return;
  for (int s = 0; s < 16; ++s) {
    const int cj = (t >> 6) + 4 * s, j = c0 + cj;
    if (j >= n) continue;
    double v = 0.0;
    if (j != i) {
      double sum = 0.0, dk = 0.0;
#pragma unroll
      for (int k = 0; k < DM; ++k) {
        if (k < d) {
          const double dx = xj[k][cj] - xi[k][ri];
          sum += cov_term<K>(dx, th[k]);
          if (k == kdim) dk = dlncov_term<K>(dx, th[k]);
        }
      }
      v = (cov_from_sum<K>(sum) * factor) * dk;
    }
    G[i + (int64_t)j * ldg] = v;
  }
}

__global__ void k_loo_B(int n, int p, const double* __restrict__ Rinv, int64_t ldr, const double* __restrict__ At,
                        double* __restrict__ B, int64_t ldb) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= n || j >= n) return;
  double v = (i >= j) ? Rinv[i + (int64_t)j * ldr] : Rinv[j + (int64_t)i * ldr];
  for (int k = 0; k < p; ++k) v -= At[i + (int64_t)k * n] * At[j + (int64_t)k * n];
  B[i + (int64_t)j * ldb] = v;
}

__global__ void k_right_solve_upper(int n, int p, double* __restrict__ H, int64_t hstride,
                                    const double* __restrict__ R) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  H += blockIdx.y * hstride;
  R += (int64_t)blockIdx.y * p * p;
  for (int j = 0; j < p; ++j) {
    double v = H[i + (int64_t)j * n];
    for (int l = 0; l < j; ++l) v -= H[i + (int64_t)l * n] * R[l + j * p];
    H[i + (int64_t)j * n] = v / R[j + j * p];
  }
}

__global__ void k_sub_aat_lower(int n, int p, const double* __restrict__ At, int64_t atstride, double* __restrict__ C,
                                int64_t ldc, int64_t cstride) {
  const int i = blockIdx.x * 32 + (threadIdx.x & 31);
  const int j = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (i >= n || j > i) return;
  const double* a = At + blockIdx.z * atstride;
  double* c = C + blockIdx.z * cstride;
  double v = c[i + (int64_t)j * ldc];
  for (int k = 0; k < p; ++k) v -= a[i + (int64_t)k * n] * a[j + (int64_t)k * n];
  c[i + (int64_t)j * ldc] = v;
}

__global__ void k_col_dot(int n, const double* __restrict__ B, int64_t ldb, const double* __restrict__ M,
                          int64_t ldm, double* __restrict__ out) {
  const int col = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (col >= n) return;
  const double* b = B + (int64_t)col * ldb;
  const double* m = M + (int64_t)col * ldm;
  double s = 0.0;
  for (int r = lane; r < n; r += 32) s = fma(b[r], m[r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[col] = s;
}

template <int K, int DM>
struct LooGradRLaunch {
  static void run(int n, int d, const double* X, const double* theta, double factor, int kdim, double* G,
                  int64_t ldg, cudaStream_t st) {
    LaunchTimer lt("k_loo_gradR", st, (double)n * n, 8.0 * n * n);
    k_loo_gradR<K, DM><<<dim3(ceil_div(n, T), ceil_div(n, T), 1), 256, 0, st>>>(n, d, X, theta, factor, kdim, G,
                                                                                           ldg);
    LKG_LAUNCH("k_loo_gradR");
  }
};

template <int K, int DM>
struct CovLowerLaunch {
  static void run(int n, int d, const double* X, int64_t xb, const double* theta, const double* factor,
                  const double* diag, double* A, int64_t lda, int64_t mstride, int batch, bool fast, const int* nvalid,
                  cudaStream_t st) {
    const int nb = ceil_div(n, T);
    const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
    LaunchTimer lt("k_cov_lower", st, 0.5 * n * (n - 1.0) * batch, 4.0 * n * (n + 1.0) * batch);
    if (fast)
      k_cov_lower<K, DM, true><<<dim3((unsigned)ntiles, 1, batch), 256, 0, st>>>(n, d, X, xb, theta, factor, diag, A,
                                                                                  lda, mstride, nvalid);
    else
      k_cov_lower<K, DM, false><<<dim3((unsigned)ntiles, 1, batch), 256, 0, st>>>(n, d, X, xb, theta, factor, diag,
                                                                                   A, lda, mstride, nvalid);
    LKG_LAUNCH("k_cov_lower");
  }
};

template <int K, int DM>
struct CovCrossLaunch {
  static void run(int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta, double factor,
                  double* R, bool snap, cudaStream_t st) {
    LaunchTimer lt("k_cov_cross", st, (double)n_o * q, 8.0 * n_o * q);
    k_cov_cross<K, DM><<<dim3(ceil_div(n_o, T), ceil_div(q, T), 1), 256, 0, st>>>(n_o, q, d, Xo, Xn, theta, factor,
                                                                                   R, snap);
    LKG_LAUNCH("k_cov_cross");
  }
};

template <int K, int DM>
struct DCovCrossLaunch {
  static void run(int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta, double factor,
                  double* DR, cudaStream_t st) {
    LaunchTimer lt("k_dcov_cross", st, (double)n_o * q * (1.0 + d), 8.0 * n_o * q * d);
    k_dcov_cross<K, DM><<<dim3(ceil_div(n_o, T), ceil_div(q, T), 1), 256, 0, st>>>(n_o, q, d, Xo, Xn, theta, factor,
                                                                                    DR);
    LKG_LAUNCH("k_dcov_cross");
  }
};

template <int K, int DM>
struct AdjointLaunch {
  static void run(int n, int d, const double* X, int64_t xb, const double* theta, const double* factor,
                  const double* xv, int64_t xvb, const double* Rinv, int64_t ldr, int64_t rstride, double* partials,
                  int64_t ntiles, int batch, cudaStream_t st) {
    LaunchTimer lt("k_adjoint", st, 0.5 * n * (n - 1.0) * batch, 4.0 * n * (n + 1.0) * batch);
    k_adjoint<K, DM><<<dim3((unsigned)ntiles, 1, batch), 256, 0, st>>>(n, d, X, xb, theta, factor, xv, xvb, Rinv, ldr,
                                                                        rstride, partials, ntiles);
    LKG_LAUNCH("k_adjoint");
  }
};

}  // namespace

void cov_build_lower(int kernel, int n, int d, const double* X, int64_t x_bstride, const double* theta,
                     const double* factor, const double* diag, double* A, int64_t lda, int64_t mstride, int batch,
                     cudaStream_t st, bool fast, const int* nvalid) {
  if (n <= 0) return;
  dispatch_kd<CovLowerLaunch>(kernel, d, n, d, X, x_bstride, theta, factor, diag, A, lda, mstride, batch, fast, nvalid,
                              st);
}

void cov_cross(int kernel, int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta,
               double factor, double* R, cudaStream_t st, bool snap_coincident) {
  if (n_o <= 0 || q <= 0) return;
  dispatch_kd<CovCrossLaunch>(kernel, d, n_o, q, d, Xo, Xn, theta, factor, R, snap_coincident, st);
}

void dcov_cross(int kernel, int n_o, int q, int d, const double* Xo, const double* Xn, const double* theta,
                double factor, double* DR, cudaStream_t st) {
  if (n_o <= 0 || q <= 0) return;
  dispatch_kd<DCovCrossLaunch>(kernel, d, n_o, q, d, Xo, Xn, theta, factor, DR, st);
}

size_t adjoint_partials_size(int n, int d, int batch) {
  const int nb = ceil_div(n, T);
  return (size_t)nb * (nb + 1) / 2 * adjoint_nacc(d) * batch;
}

void adjoint_sums(int kernel, int n, int d, const double* X, int64_t x_bstride, const double* theta,
                  const double* factor, const double* xv, int64_t xv_bstride, const double* Rinv, int64_t ldr,
                  int64_t rstride, double* partials, double* out, int batch, cudaStream_t st) {
  const int nb = ceil_div(n, T);
  const int64_t ntiles = (int64_t)nb * (nb + 1) / 2;
  dispatch_kd<AdjointLaunch>(kernel, d, n, d, X, x_bstride, theta, factor, xv, xv_bstride, Rinv, ldr, rstride,
                             partials, ntiles, batch, st);
  const int nacc = adjoint_nacc(d);
  LaunchTimer lt("k_reduce_partials", st, 0.0, 8.0 * ntiles * nacc * batch);
  k_reduce_partials<<<dim3(nacc, 1, batch), 1024, 0, st>>>(partials, ntiles, nacc, out);
  LKG_LAUNCH("k_reduce_partials");
}

void gram_and_logdet(int n, int ncols, const double* Mat, int64_t ldm, int64_t mstride, const double* L, int64_t ldl,
                     int64_t lstride, double* out, int64_t out_bstride, int batch, cudaStream_t st) {
  const int npairs = ncols * (ncols + 1) / 2;
  LaunchTimer lt("k_gram_logdet", st, 2.0 * n * npairs * batch, 8.0 * n * ncols * batch);
  k_gram_logdet<<<dim3(npairs + 1, 1, batch), 256, 0, st>>>(n, ncols, Mat, ldm, mstride, L, ldl, lstride, out,
                                                             out_bstride);
  LKG_LAUNCH("k_gram_logdet");
}

void gls_solve(int p, const double* gram, int64_t gram_bstride, double* beta, int64_t beta_bstride, double* rstar,
               int64_t rstar_bstride, int* gls_info, int batch, cudaStream_t st) {
  if (p > PMAX) throw std::invalid_argument("trend with more than 64 columns is not supported");
  LaunchTimer lt("k_gls_solve", st, 0.0, 0.0);
  k_gls_solve<<<batch, 32, 0, st>>>(p, gram, gram_bstride, beta, beta_bstride, rstar, rstar_bstride, gls_info);
  LKG_LAUNCH("k_gls_solve");
}

void residual_sse(int n, int p, const double* FY, int64_t ldfy, int64_t fystride, const double* beta,
                  int64_t beta_bstride, double* Estar, int64_t estride, double* sse, int64_t sse_bstride, int batch,
                  cudaStream_t st) {
  LaunchTimer lt("k_residual_sse", st, 2.0 * n * (p + 1.0) * batch, 8.0 * n * (p + 2.0) * batch);
  k_residual_sse<<<batch, 1024, 0, st>>>(n, p, FY, ldfy, fystride, beta, beta_bstride, Estar, estride, sse,
                                         sse_bstride);
  LKG_LAUNCH("k_residual_sse");
}

void lower_colsum_abs(int n, const double* L, int64_t ldl, int64_t lstride, double* colsum, int batch,
                      cudaStream_t st) {
  LaunchTimer lt("k_lower_colsum_abs", st, 0.5 * n * (n + 1.0) * batch, 4.0 * n * (n + 1.0) * batch);
  k_lower_colsum_abs<<<dim3(ceil_div(n, 8), 1, batch), 256, 0, st>>>(n, L, ldl, lstride, colsum);
  LKG_LAUNCH("k_lower_colsum_abs");
}

void loo_gradR(int kernel, int n, int d, const double* X, const double* theta, double factor, int k, double* G,
               int64_t ldg, cudaStream_t st) {
  if (n <= 0) return;
  dispatch_kd<LooGradRLaunch>(kernel, d, n, d, X, theta, factor, k, G, ldg, st);
}

void loo_build_B(int n, int p, const double* Rinv, int64_t ldr, const double* At, double* B, int64_t ldb,
                 cudaStream_t st) {
  if (n <= 0) return;
  LaunchTimer lt("k_loo_B", st, 2.0 * n * n * p, 8.0 * n * n * 1.5);
  k_loo_B<<<dim3(ceil_div(n, 32), ceil_div(n, 8), 1), 256, 0, st>>>(n, p, Rinv, ldr, At, B, ldb);
  LKG_LAUNCH("k_loo_B");
}

void right_solve_upper(int n, int p, double* H, int64_t hstride, const double* Rstar, int batch, cudaStream_t st) {
  if (n <= 0 || p <= 0) return;
  LaunchTimer lt("k_right_solve_upper", st, (double)n * p * p * batch, 16.0 * n * p * batch);
  k_right_solve_upper<<<dim3(ceil_div(n, 128), batch), 128, 0, st>>>(n, p, H, hstride, Rstar);
  LKG_LAUNCH("k_right_solve_upper");
}

void sub_aat_lower(int n, int p, const double* At, int64_t atstride, double* C, int64_t ldc, int64_t cstride,
                   int batch, cudaStream_t st) {
  if (n <= 0 || p <= 0) return;
  LaunchTimer lt("k_sub_aat_lower", st, (double)n * (n + 1.0) * p * batch, 8.0 * n * (n + 1.0) * batch);
  k_sub_aat_lower<<<dim3(ceil_div(n, 32), ceil_div(n, 8), batch), 256, 0, st>>>(n, p, At, atstride, C, ldc, cstride);
  LKG_LAUNCH("k_sub_aat_lower");
}

void col_dot(int n, const double* B, int64_t ldb, const double* M, int64_t ldm, double* out, cudaStream_t st) {
  if (n <= 0) return;
  LaunchTimer lt("k_col_dot", st, 2.0 * n * n, 16.0 * n * n);
  k_col_dot<<<ceil_div(n, 8), 256, 0, st>>>(n, B, ldb, M, ldm, out);
  LKG_LAUNCH("k_col_dot");
}

}  // namespace lkg
