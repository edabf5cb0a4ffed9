// vecchia.cu -- Vecchia log-likelihood and conditioning sets on the GPU (see vecchia.hpp).
//
// Per ordered point t (Kriging.cpp:829-889): RN = C(N_t, N_t) + num_nugget I, r = C(N_t, x_t), LN = chol(RN) with
// the safe_chol_lower rules (LinearAlgebra.cpp:68-115: cumulative 1e-10 * 10^k increments, rcond(LN)^2 check),
// a = RN^-1 r, v = max(1 - r'a, 1e-15), u = y_t - a'y_N, W = f_t - F_N' a.  The theta-derivatives use
//   da_k = RN^-1 g_k with g_k = dr_k - dRN_k a, and RN symmetric:
//   dv_k = -(dr_k'a + r'da_k) = -(2 a'dr_k - a'dRN_k a),  du_k = -g_k' (RN^-1 y_N),  dW_k = -(RN^-1 F_N)' g_k,
// which is the reference's algebra rearranged so that no per-k solve is needed (2 + p solves per point in total).
#include "vecchia.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "config.hpp"
#include "stats.hpp"

namespace lkg {

namespace {

constexpr int WPB = 4;    // warps per block of the point kernel
constexpr int LDP = 33;   // shared-memory row pitch of the m x m blocks
constexpr int VPMAX = 16; // trend columns supported by the Vecchia kernels
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double wsum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}
__device__ __forceinline__ double wmax(double x) {
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(FULL, x, o));
  return x;
}
// first index of the maximum of v over lanes < mi
__device__ __forceinline__ int wargmax(double v, int lane, int mi) {
  double val = (lane < mi) ? v : -1.0;
  int idx = lane;
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_xor_sync(FULL, val, o);
    const int oi = __shfl_xor_sync(FULL, idx, o);
    if (ov > val || (ov == val && oi < idx)) {
      val = ov;
      idx = oi;
    }
  }
  return idx;
}

// The factor keeps 1 / L_jj in the spare last column of row j (index RCP = LDP - 1 = 32, never a matrix column since
// m <= 32 fills 0 .. 31), and the unit lower factor U = L D^-1 (D = diag L) transposed in the strict upper part:
// L[j][i] = L_ij / L_jj for i > j.  The solves then take one fused multiply-add per step and scale by 1 / L_jj once
// (FP64 issue bounds these kernels: GB300 runs FP64 at 1/64 of the FP32 rate).
constexpr int RCP = LDP - 1;

// solve L z = b (lane i holds b_i): U w = b by forward substitution, then z = D^-1 w; lanes >= mi return 0
__device__ double wsolve_lower(const double* L, double b, int mi, int lane) {
  double val = (lane < mi) ? b : 0.0;
  for (int j = 0; j < mi; ++j) {
    const double wj = __shfl_sync(FULL, val, j);
    if (lane > j && lane < mi) val -= L[j * LDP + lane] * wj;
  }
  return (lane < mi) ? val * L[lane * LDP + RCP] : 0.0;
}
// solve L' x = z: U' x = D^-1 z by back substitution
__device__ double wsolve_upper_t(const double* L, double z, int mi, int lane) {
  double val = (lane < mi) ? z * L[lane * LDP + RCP] : 0.0;
  for (int j = mi - 1; j >= 0; --j) {
    const double xj = __shfl_sync(FULL, val, j);
    if (lane < j) val -= L[lane * LDP + j] * xj;
  }
  return (lane < mi) ? val : 0.0;
}

// (row, column) of entry e of a lower triangle enumerated row by row: e = r (r + 1) / 2 + c, c <= r
__device__ __forceinline__ void tri_rc(int e, int& r, int& c) {
  r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
  if ((r + 1) * (r + 2) / 2 <= e) ++r;
  if (r * (r + 1) / 2 > e) --r;
  c = e - r * (r + 1) / 2;
}

// in-place lower Cholesky, right-looking: column j scaled by 1 / L_jj, then the trailing lower triangle updated with
// its (row, column) pairs spread over the lanes; returns false on a non-positive / NaN pivot (uniform over the warp)
__device__ bool wchol(double* L, int mi, int lane) {
  for (int j = 0; j < mi; ++j) {
    __syncwarp();
    const double piv = L[j * LDP + j];
    if (!(piv > 0.0)) return false;
    double ljj, rj;
    pivot_root(piv, ljj, rj);
    __syncwarp();
    if (lane == j) {
      L[j * LDP + j] = ljj;
      L[j * LDP + RCP] = rj;
    }
    if (lane > j && lane < mi) L[lane * LDP + j] *= rj;
    __syncwarp();
    const int m1 = mi - 1 - j, ne = m1 * (m1 + 1) / 2;
    for (int e = lane; e < ne; e += 32) {
      int rr, cc;
      tri_rc(e, rr, cc);
      const int r = j + 1 + rr, c = j + 1 + cc;
      L[r * LDP + c] -= L[r * LDP + j] * L[c * LDP + j];
    }
  }
  __syncwarp();
  // the unit lower factor, transposed into the strict upper part: L[j][i] = L_ij / L_jj
  const int np = mi * (mi - 1) / 2;
  for (int e = lane; e < np; e += 32) {
    int rr, cc;
    tri_rc(e, rr, cc);
    const int i = rr + 1;
    L[cc * LDP + i] = L[i * LDP + cc] * L[cc * LDP + RCP];
  }
  __syncwarp();
  return true;
}

// rcond(L)^2 of dtrcon('1', 'L', 'N'): |L|_1 and the dlacn2 estimate of |L^-1|_1 with warp solves
__device__ double wrcond2(const double* L, int mi, int lane) {
  double cs = 0.0;
  if (lane < mi)
    for (int i = lane; i < mi; ++i) cs += fabs(L[i * LDP + lane]);
  const double anorm = wmax(cs);
  if (!(anorm > 0.0)) return 0.0;
  double y = wsolve_lower(L, 1.0 / mi, mi, lane);
  double est;
  if (mi == 1) {
    est = fabs(__shfl_sync(FULL, y, 0));
  } else {
    est = wsum(fabs(y));
    double xi = (y >= 0.0) ? 1.0 : -1.0;
    double z = wsolve_upper_t(L, xi, mi, lane);
    int j = wargmax(fabs(z), lane, mi);
    int iter = 2;
    for (;;) {
      y = wsolve_lower(L, (lane == j) ? 1.0 : 0.0, mi, lane);
      const double estold = est;
      est = wsum(fabs(y));
      const double sg = (y >= 0.0) ? 1.0 : -1.0;
      const bool same = __all_sync(FULL, lane >= mi || sg == xi);
      if (same || est <= estold) break;
      xi = sg;
      z = wsolve_upper_t(L, xi, mi, lane);
      const int jlast = j;
      j = wargmax(fabs(z), lane, mi);
      const double zl = __shfl_sync(FULL, z, jlast), zj = __shfl_sync(FULL, z, j);
      if (zl != fabs(zj) && iter < 5) {
        iter++;
        continue;
      }
      break;
    }
    const double alt = ((lane & 1) ? -1.0 : 1.0) * (1.0 + (double)lane / (double)(mi - 1));
    y = wsolve_lower(L, alt, mi, lane);
    const double temp = 2.0 * wsum(fabs(y)) / (3.0 * mi);
    if (temp > est) est = temp;
  }
  const double rc = (1.0 / anorm) / est;
  return rc * rc;
}

struct VPointArgs {
  int n, d, p, m;
  int t0, t1;  // ordered positions evaluated: [t0, t1)
  const double *X, *y, *F, *theta;
  const int32_t *order, *nbr;
  double num_nugget, min_rcond;
  int rcond_check, max_inc, with_grad;
  double *u, *v, *W, *du, *dv, *dW;
  int* status;
};

template <int K, int DM>
__global__ void __launch_bounds__(WPB * 32) k_vecchia_points(VPointArgs a) {
  extern __shared__ double vsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* RN = vsm + (size_t)w * (2 * 32 * LDP + 32 * DM + 32);
  double* LN = RN + 32 * LDP;
  double* xs = LN + 32 * LDP;  // [32][DM]
  double* sa = xs + 32 * DM;   // [32]
  const int t = a.t0 + blockIdx.x * WPB + w;
  if (t >= a.t1) return;
  const int n = a.n, d = a.d, p = a.p;
  const int oi = a.order[t];
  const int nbv = (lane < a.m) ? a.nbr[(int64_t)t * a.m + lane] : -1;
  const int mi = __popc(__ballot_sync(FULL, nbv >= 0));
  if (mi == 0) {
    if (lane == 0) {
      a.u[t] = a.y[oi];
      a.v[t] = 1.0;
      for (int q = 0; q < p; ++q) a.W[(int64_t)t * p + q] = a.F[oi + (int64_t)q * n];
      if (a.with_grad)
        for (int k = 0; k < d; ++k) {
          a.du[(int64_t)t * d + k] = 0.0;
          a.dv[(int64_t)t * d + k] = 0.0;
          for (int q = 0; q < p; ++q) a.dW[((int64_t)t * d + k) * p + q] = 0.0;
        }
      a.status[t] = 0;
    }
    return;
  }
  // division- and log1p-free covariance forms (common.cuh), equal to the reference's to a few ulps
  double inv[DM], ck[DM], xo[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) {
    const double th = (k < d) ? a.theta[k] : 1.0;
    inv[k] = 1.0 / th;
    ck[k] = cov_scale<K>() * inv[k];
    xo[k] = (k < d) ? a.X[oi + (int64_t)k * n] : 0.0;
  }
  if (lane < mi)
#pragma unroll
    for (int k = 0; k < DM; ++k) xs[lane * DM + k] = (k < d) ? a.X[nbv + (int64_t)k * n] : 0.0;
  __syncwarp();
  double r = 0.0;
  {  // RN: the strict lower triangle's pairs spread over the lanes and mirrored (C depends on |dx| or dx^2 only, so
     // both orders give the same value)
    const int np = mi * (mi - 1) / 2;
    for (int e = lane; e < np; e += 32) {
      int rr, cc;
      tri_rc(e, rr, cc);
      const int ra = rr + 1;
      double s = 0.0, pr = 1.0;
#pragma unroll
      for (int k = 0; k < DM; ++k)
        if (k < d) cov_fast_term<K>(xs[ra * DM + k] - xs[cc * DM + k], ck[k], s, pr);
      const double c = cov_fast_finish<K>(s, pr);
      RN[ra * LDP + cc] = c;
      RN[cc * LDP + ra] = c;
    }
  }
  if (lane < mi) {
    RN[lane * LDP + lane] = 1.0 + a.num_nugget;
    double s = 0.0, pr = 1.0;
#pragma unroll
    for (int k = 0; k < DM; ++k)
      if (k < d) cov_fast_term<K>(xs[lane * DM + k] - xo[k], ck[k], s, pr);
    r = cov_fast_finish<K>(s, pr);
  }
  __syncwarp();
  // ---- factor with the numerical-nugget retry / rcond rules ----
  int inc = 0;
  for (;;) {
    if (lane < mi)
      for (int b = 0; b < mi; ++b) LN[lane * LDP + b] = RN[lane * LDP + b];
    __syncwarp();
    const bool ok = wchol(LN, mi, lane);
    bool wrong = false;
    if (ok && a.rcond_check) wrong = wrcond2(LN, mi, lane) < a.min_rcond;
    if (ok && !wrong) break;
    if (inc > a.max_inc || !(a.num_nugget > 0.0)) {
      if (lane == 0) a.status[t] = -1;
      return;
    }
    __syncwarp();
    if (lane < mi) RN[lane * LDP + lane] += a.num_nugget * pow(10.0, (double)inc);
    inc++;
    __syncwarp();
  }
  // ---- a, v, u, W ----
  const double av = wsolve_upper_t(LN, wsolve_lower(LN, r, mi, lane), mi, lane);
  const double yN = (lane < mi) ? a.y[nbv] : 0.0;
  const double ra = wsum(r * av), ay = wsum(av * yN);
  double fN[VPMAX];
  for (int q = 0; q < p; ++q) fN[q] = (lane < mi) ? a.F[nbv + (int64_t)q * n] : 0.0;
  if (lane == 0) {
    a.v[t] = fmax(1.0 - ra, 1e-15);
    a.u[t] = a.y[oi] - ay;
    a.status[t] = inc;
  }
  for (int q = 0; q < p; ++q) {
    const double s = wsum(fN[q] * av);
    if (lane == 0) a.W[(int64_t)t * p + q] = a.F[oi + (int64_t)q * n] - s;
  }
  if (!a.with_grad) return;
  // ---- theta-derivatives ----
  const double by = wsolve_upper_t(LN, wsolve_lower(LN, yN, mi, lane), mi, lane);
  double cq[VPMAX];
  for (int q = 0; q < p; ++q) cq[q] = wsolve_upper_t(LN, wsolve_lower(LN, fN[q], mi, lane), mi, lane);
  if (lane < 32) sa[lane] = av;
  __syncwarp();
  // the factor is no longer needed: its buffer holds M_k(a, b) = RN(a, b) dlnC/dtheta_k(x_a - x_b) (a != b), formed
  // once per pair (symmetric: |dx| or dx^2 only) with the pairs spread over the lanes, then s_a = sum_b M_k(a, b) a_b
  const int npair = mi * (mi - 1) / 2;
  for (int k = 0; k < d; ++k) {
    __syncwarp();
    for (int e = lane; e < npair; e += 32) {
      int rr, cc;
      tri_rc(e, rr, cc);
      const int ra = rr + 1;
      const double mk = RN[ra * LDP + cc] * dlncov_fast<K>(xs[ra * DM + k] - xs[cc * DM + k], inv[k], ck[k]);
      LN[ra * LDP + cc] = mk;
      LN[cc * LDP + ra] = mk;
    }
    __syncwarp();
    double drk = 0.0, s = 0.0;
    if (lane < mi) {
      drk = r * dlncov_fast<K>(xs[lane * DM + k] - xo[k], inv[k], ck[k]);
      for (int b = 0; b < mi; ++b)
        if (b != lane) s += LN[lane * LDP + b] * sa[b];
    }
    const double g = drk - s;
    const double adr = wsum(av * drk), as = wsum(av * s), gb = wsum(g * by);
    if (lane == 0) {
      a.dv[(int64_t)t * d + k] = -(2.0 * adr - as);
      a.du[(int64_t)t * d + k] = -gb;
    }
    for (int q = 0; q < p; ++q) {
      const double gc = wsum(g * cq[q]);
      if (lane == 0) a.dW[((int64_t)t * d + k) * p + q] = -gc;
    }
  }
}

// ---- deterministic reductions over the points ----
constexpr int RED_BLOCKS = 304;

template <int NTH>
__device__ double bsum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < NTH / 32; ++i) s += red[i];
  return s;
}

// stage 1: [A (p x p, row a col b), b (p), sum log v] partials per block
__global__ void k_vsum1(int t0, int t1, int p, const double* __restrict__ u, const double* __restrict__ v,
                        const double* __restrict__ W, double* __restrict__ part) {
  __shared__ double red[8];
  const int P = p * p + p + 1;
  const int64_t cnt = t1 - t0;
  const int64_t lo = t0 + cnt * blockIdx.x / gridDim.x, hi = t0 + cnt * (blockIdx.x + 1) / gridDim.x;
  for (int e = 0; e < P; ++e) {
    double s = 0.0;
    for (int64_t t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      if (e < p * p) {
        const int qa = e / p, qb = e % p;
        s += W[t * p + qa] * W[t * p + qb] / v[t];
      } else if (e < p * p + p) {
        s += W[t * p + (e - p * p)] * u[t] / v[t];
      } else {
        s += log(v[t]);
      }
    }
    s = bsum<256>(s, red);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * P + e] = s;
  }
}

// stage 2: [Q, dQ_k (d), sum dv_k / v (d)] partials per block, given beta
__global__ void k_vsum2(int t0, int t1, int p, int d, const double* __restrict__ u, const double* __restrict__ v,
                        const double* __restrict__ W, const double* __restrict__ du, const double* __restrict__ dv,
                        const double* __restrict__ dW, const double* __restrict__ beta, int with_grad,
                        double* __restrict__ part) {
  __shared__ double red[8];
  const int P = 1 + 2 * d;
  const int64_t cnt = t1 - t0;
  const int64_t lo = t0 + cnt * blockIdx.x / gridDim.x, hi = t0 + cnt * (blockIdx.x + 1) / gridDim.x;
  for (int e = 0; e < (with_grad ? P : 1); ++e) {
    double s = 0.0;
    for (int64_t t = lo + threadIdx.x; t < hi; t += blockDim.x) {
      double wb = 0.0;
      for (int q = 0; q < p; ++q) wb += W[t * p + q] * beta[q];
      const double et = u[t] - wb, vt = v[t];
      if (e == 0) {
        s += et * et / vt;
      } else if (e <= d) {
        const int k = e - 1;
        double dwb = 0.0;
        for (int q = 0; q < p; ++q) dwb += dW[(t * d + k) * p + q] * beta[q];
        const double de = du[t * d + k] - dwb;
        s += 2.0 * et * de / vt - (et * et / (vt * vt)) * dv[t * d + k];
      } else {
        s += dv[t * d + (e - d - 1)] / vt;
      }
    }
    s = bsum<256>(s, red);
    if (threadIdx.x == 0) part[(int64_t)blockIdx.x * P + e] = s;
  }
}

// out[e] = sum over blocks of part[b * stride + e], e < count (fixed order)
__global__ void k_vsum_final(int nblocks, int stride, int count, const double* __restrict__ part,
                             double* __restrict__ out) {
  __shared__ double red[8];
  for (int e = 0; e < count; ++e) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += part[(int64_t)b * stride + e];
    s = bsum<256>(s, red);
    if (threadIdx.x == 0) out[e] = s;
  }
}

__global__ void k_count_status(int t0, int t1, const int* __restrict__ status, int* __restrict__ out) {
  // out[0] = number of failed points, out[1] = number of points that needed nugget increments
  int f = 0, c = 0;
  for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
    f += status[t] < 0;
    c += status[t] > 0;
  }
  for (int o = 16; o > 0; o >>= 1) {
    f += __shfl_xor_sync(FULL, f, o);
    c += __shfl_xor_sync(FULL, c, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, f);  // integer counts: order-independent
    atomicAdd(out + 1, c);
  }
}

template <int K, int DM>
struct VPointLaunch {
  static void run(const VPointArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)WPB * (2 * 32 * LDP + 32 * DM + 32) * sizeof(double);
    static bool attr = false;
    if (!attr) {
      LKG_CUDA(cudaFuncSetAttribute(k_vecchia_points<K, DM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      attr = true;
    }
    k_vecchia_points<K, DM><<<ceil_div(a.t1 - a.t0, WPB), WPB * 32, smem, st>>>(a);
    LKG_LAUNCH("k_vecchia_points");
  }
};

void launch_points(int kernel, const VPointArgs& a, cudaStream_t st) {
  auto go = [&](auto kc) {
    constexpr int KK = decltype(kc)::value;
    if (a.d <= 4) VPointLaunch<KK, 4>::run(a, st);
    else if (a.d <= 8) VPointLaunch<KK, 8>::run(a, st);
    else throw std::invalid_argument("LLVecchia on the GPU supports d <= 8");
  };
  switch (kernel) {
    case KGAUSS: go(std::integral_constant<int, KGAUSS>{}); break;
    case KEXP: go(std::integral_constant<int, KEXP>{}); break;
    case KMATERN32: go(std::integral_constant<int, KMATERN32>{}); break;
    case KMATERN52: go(std::integral_constant<int, KMATERN52>{}); break;
    default: throw std::invalid_argument("Unsupported covariance kernel id");
  }
}

// ---- predictVecchia (Kriging.cpp:950-1022): one warp per prediction point ----
constexpr int PTILE = 256;  // observations per shared-memory tile of the neighbour scan

struct VPredArgs {
  int n, d, m, q;
  const double *X, *resid, *theta, *Xq;
  double num_nugget, min_rcond;
  int rcond_check, max_inc;
  double *ar, *ra;
  int* status;
};

// m nearest observations by (squared distance, index) from a scan of all n in shared-memory tiles, then local
// kriging: RN = C(N, N) + num_nugget I factored with the safe_chol_lower rules, a = RN^-1 r,
// ar = a . (y_N - F_N beta), ra = r . a
template <int K, int DM>
__global__ void __launch_bounds__(WPB * 32) k_vecchia_predict(VPredArgs a) {
  extern __shared__ double psm[];
  double* tile = psm;  // [PTILE][DM]
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* RN = psm + PTILE * DM + (size_t)w * (2 * 32 * LDP + 32 * DM + 64);
  double* LN = RN + 32 * LDP;
  double* xs = LN + 32 * LDP;  // [32][DM]
  double* kd = xs + 32 * DM;   // [32] distances of the current m best
  int* ki = reinterpret_cast<int*>(kd + 32);  // [32] their indices
  const int t = blockIdx.x * WPB + w;
  const bool active = t < a.q;
  const int n = a.n, d = a.d, m = a.m;
  double xq[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) xq[k] = (active && k < d) ? a.Xq[t + (int64_t)k * a.q] : 0.0;
  int cnt = 0;
  double thr = INFINITY;
  int thri = 0x7fffffff;
  for (int j0 = 0; j0 < n; j0 += PTILE) {
    __syncthreads();
    for (int idx = threadIdx.x; idx < PTILE * DM; idx += WPB * 32) {
      const int jj = idx % PTILE, k = idx / PTILE;
      tile[jj * DM + k] = (k < d && j0 + jj < n) ? a.X[(j0 + jj) + (int64_t)k * n] : 0.0;
    }
    __syncthreads();
    if (!active) continue;
    for (int s0 = 0; s0 < PTILE; s0 += 32) {
      const int j = j0 + s0 + lane;
      double dj = INFINITY;
      int ij = 0x7fffffff;
      if (j < n) {
        double ss = 0.0;
#pragma unroll
        for (int k = 0; k < DM; ++k)
          if (k < d) {
            const double dk = xq[k] - tile[(s0 + lane) * DM + k];
            ss += dk * dk;
          }
        dj = ss;
        ij = j;
      }
      const bool qual = (j < n) && (cnt < m || dj < thr || (dj == thr && ij < thri));
      unsigned mask = __ballot_sync(FULL, qual);
      while (mask) {
        const int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const double cd = __shfl_sync(FULL, dj, src);
        const int ci = __shfl_sync(FULL, ij, src);
        if (lane == 0) {
          const bool full = cnt >= m;
          if (!full || cd < kd[m - 1] || (cd == kd[m - 1] && ci < ki[m - 1])) {
            int pos = full ? m - 1 : cnt;
            while (pos > 0 && (kd[pos - 1] > cd || (kd[pos - 1] == cd && ki[pos - 1] > ci))) {
              kd[pos] = kd[pos - 1];
              ki[pos] = ki[pos - 1];
              --pos;
            }
            kd[pos] = cd;
            ki[pos] = ci;
          }
        }
        cnt = cnt < m ? cnt + 1 : m;
        __syncwarp();
      }
      __syncwarp();
      if (cnt >= m) {
        thr = kd[m - 1];
        thri = ki[m - 1];
      }
    }
  }
  if (!active) return;
  __syncwarp();
  const int mi = m;
  const int nbv = (lane < mi) ? ki[lane] : -1;
  double ck[DM];
#pragma unroll
  for (int k = 0; k < DM; ++k) ck[k] = cov_scale<K>() / ((k < d) ? a.theta[k] : 1.0);
  if (lane < mi)
#pragma unroll
    for (int k = 0; k < DM; ++k) xs[lane * DM + k] = (k < d) ? a.X[nbv + (int64_t)k * n] : 0.0;
  __syncwarp();
  double r = 0.0;
  if (lane < mi) {  // division- and log1p-free covariance forms (common.cuh)
    for (int b = 0; b < mi; ++b) {
      double c;
      if (b == lane) {
        c = 1.0 + a.num_nugget;
      } else {
        double s = 0.0, pr = 1.0;
#pragma unroll
        for (int k = 0; k < DM; ++k)
          if (k < d) cov_fast_term<K>(xs[lane * DM + k] - xs[b * DM + k], ck[k], s, pr);
        c = cov_fast_finish<K>(s, pr);
      }
      RN[lane * LDP + b] = c;
    }
    double s = 0.0, pr = 1.0;
#pragma unroll
    for (int k = 0; k < DM; ++k)
      if (k < d) cov_fast_term<K>(xs[lane * DM + k] - xq[k], ck[k], s, pr);
    r = cov_fast_finish<K>(s, pr);
  }
  __syncwarp();
  int inc = 0;
  for (;;) {
    if (lane < mi)
      for (int b = 0; b < mi; ++b) LN[lane * LDP + b] = RN[lane * LDP + b];
    __syncwarp();
    const bool ok = wchol(LN, mi, lane);
    bool wrong = false;
    if (ok && a.rcond_check) wrong = wrcond2(LN, mi, lane) < a.min_rcond;
    if (ok && !wrong) break;
    if (inc > a.max_inc || !(a.num_nugget > 0.0)) {
      if (lane == 0) a.status[t] = -1;
      return;
    }
    __syncwarp();
    if (lane < mi) RN[lane * LDP + lane] += a.num_nugget * pow(10.0, (double)inc);
    inc++;
    __syncwarp();
  }
  const double av = wsolve_upper_t(LN, wsolve_lower(LN, r, mi, lane), mi, lane);
  const double rs = (lane < mi) ? a.resid[nbv] : 0.0;
  const double ar = wsum(av * rs), ra = wsum(r * av);
  if (lane == 0) {
    a.ar[t] = ar;
    a.ra[t] = ra;
    a.status[t] = inc;
  }
}

template <int K, int DM>
struct VPredLaunch {
  static void run(const VPredArgs& a, cudaStream_t st) {
    const size_t smem = ((size_t)PTILE * DM + (size_t)WPB * (2 * 32 * LDP + 32 * DM + 64)) * sizeof(double);
    LKG_CUDA(cudaFuncSetAttribute(k_vecchia_predict<K, DM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    LaunchTimer lt("k_vecchia_predict", st, 3.0 * a.q * (double)a.n * a.d, 8.0 * a.n * a.d);
    k_vecchia_predict<K, DM><<<ceil_div(a.q, WPB), WPB * 32, smem, st>>>(a);
    LKG_LAUNCH("k_vecchia_predict");
  }
};

template <typename P>
void valloc(P** p, size_t count) {
  LKG_CUDA(cudaMalloc((void**)p, sizeof(P) * std::max<size_t>(count, 1)));
}

// host Cholesky solve of the small GLS system (arma::solve with likely_sympd)
bool small_spd_solve(int p, std::vector<double> A, std::vector<double> b, std::vector<double>& x) {
  for (int j = 0; j < p; ++j) {
    double s = A[j * p + j];
    for (int k = 0; k < j; ++k) s -= A[j * p + k] * A[j * p + k];
    if (!(s > 0.0)) return false;
    A[j * p + j] = std::sqrt(s);
    for (int i = j + 1; i < p; ++i) {
      double t = A[i * p + j];
      for (int k = 0; k < j; ++k) t -= A[i * p + k] * A[j * p + k];
      A[i * p + j] = t / A[j * p + j];
    }
  }
  for (int i = 0; i < p; ++i) {
    for (int k = 0; k < i; ++k) b[i] -= A[i * p + k] * b[k];
    b[i] /= A[i * p + i];
  }
  for (int i = p - 1; i >= 0; --i) {
    for (int k = i + 1; k < p; ++k) b[i] -= A[k * p + i] * b[k];
    b[i] /= A[i * p + i];
  }
  x = b;
  return true;
}

}  // namespace

VecchiaEngine::VecchiaEngine(int kernel, int n, int d, int p, const double* X, const double* y, const double* F,
                             const int32_t* order, const int32_t* nbr, int m)
    : kernel_(kernel), n_(n), d_(d), p_(p), m_(m) {
  if (m < 0 || m > VECCHIA_MAX_M) throw std::invalid_argument("LLVecchia on the GPU supports m <= 32");
  if (p > VPMAX) throw std::invalid_argument("LLVecchia on the GPU supports at most 16 trend columns");
  if (d < 1 || d > 8) throw std::invalid_argument("LLVecchia on the GPU supports d <= 8");
  LKG_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
  valloc(&dX_, (size_t)n * d);
  valloc(&dY_, n);
  valloc(&dF_, (size_t)n * std::max(p, 1));
  valloc(&dth_, d);
  valloc(&dorder_, n);
  valloc(&dnbr_, (size_t)n * std::max(m, 1));
  LKG_CUDA(cudaMemcpyAsync(dX_, X, sizeof(double) * n * d, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dY_, y, sizeof(double) * n, cudaMemcpyHostToDevice, st_));
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(dF_, F, sizeof(double) * n * p, cudaMemcpyHostToDevice, st_));
  LKG_CUDA(cudaMemcpyAsync(dorder_, order, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st_));
  if (m > 0) LKG_CUDA(cudaMemcpyAsync(dnbr_, nbr, sizeof(int32_t) * n * m, cudaMemcpyHostToDevice, st_));
  valloc(&du_, n);
  valloc(&dv_, n);
  valloc(&dW_, (size_t)n * std::max(p, 1));
  valloc(&ddu_, (size_t)n * d);
  valloc(&ddv_, (size_t)n * d);
  valloc(&ddW_, (size_t)n * d * std::max(p, 1));
  valloc(&dstatus_, n + 2);
  nblk_red_ = RED_BLOCKS;
  valloc(&dpart_, (size_t)nblk_red_ * (VPMAX * VPMAX + VPMAX + 1 + 2 * 8 + 1) + 512);
  valloc(&dbeta_, VPMAX);
  t0_ = 0;
  t1_ = n;
  LKG_CUDA(cudaStreamSynchronize(st_));
}

VecchiaEngine::~VecchiaEngine() {
  for (double* p : {dX_, dY_, dF_, dth_, du_, dv_, dW_, ddu_, ddv_, ddW_, dpart_, dbeta_})
    if (p) cudaFree(p);
  if (dorder_) cudaFree(dorder_);
  if (dnbr_) cudaFree(dnbr_);
  if (dstatus_) cudaFree(dstatus_);
  if (st_) cudaStreamDestroy(st_);
}

void VecchiaEngine::set_range(int t0, int t1) {
  if (t0 < 0 || t1 > n_ || t0 > t1) throw std::invalid_argument("VecchiaEngine::set_range: need 0 <= t0 <= t1 <= n");
  t0_ = t0;
  t1_ = t1;
}

int VecchiaEngine::partial_sums1(const double* theta, bool with_grad, std::vector<double>& s1,
                                 long long* nugget_points) {
  const Config& cfg = config();
  const int n = n_, d = d_, p = p_;
  const int P1 = p * p + p + 1;
  s1.assign(P1, 0.0);
  if (t1_ <= t0_) return 0;
  LKG_CUDA(cudaMemcpyAsync(dth_, theta, sizeof(double) * d, cudaMemcpyHostToDevice, st_));
  VPointArgs a{n, d, p, m_, t0_, t1_, dX_, dY_, dF_, dth_, dorder_, dnbr_, cfg.num_nugget, cfg.min_rcond,
               cfg.chol_rcond_check ? 1 : 0, cfg.max_inc_choldiag, with_grad ? 1 : 0, du_, dv_, dW_, ddu_, ddv_,
               ddW_, dstatus_};
  const double cnt = t1_ - t0_;
  {
    // per point: the (m + 1)^3 / 3 Cholesky-and-solve work of the conditional and the d (4 m^2) derivative terms
    const double mm = m_;
    LaunchTimer lt("k_vecchia_points", st_,
                   cnt * ((mm + 1) * (mm + 1) * (mm + 1) / 3.0 + (with_grad ? d * 4.0 * mm * mm : 0.0)),
                   8.0 * cnt * (1.0 + d) * m_);
    launch_points(kernel_, a, st_);
  }
  int* dcount = dstatus_ + n;
  LKG_CUDA(cudaMemsetAsync(dcount, 0, 2 * sizeof(int), st_));
  {
    LaunchTimer lt("k_count_status", st_, 0.0, 4.0 * cnt);
    k_count_status<<<152, 256, 0, st_>>>(t0_, t1_, dstatus_, dcount);
    LKG_LAUNCH("k_count_status");
  }
  double* fin = dpart_ + (size_t)nblk_red_ * (VPMAX * VPMAX + VPMAX + 1 + 2 * 8 + 1);
  {
    LaunchTimer lt("k_vsum1", st_, 0.0, 8.0 * cnt * (2.0 + p));
    k_vsum1<<<nblk_red_, 256, 0, st_>>>(t0_, t1_, p, du_, dv_, dW_, dpart_);
    LKG_LAUNCH("k_vsum1");
    k_vsum_final<<<1, 256, 0, st_>>>(nblk_red_, P1, P1, dpart_, fin);
    LKG_LAUNCH("k_vsum_final");
  }
  int counts[2];
  LKG_CUDA(cudaMemcpyAsync(s1.data(), fin, sizeof(double) * P1, cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaMemcpyAsync(counts, dcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaStreamSynchronize(st_));
  if (nugget_points) *nugget_points += counts[1];
  return counts[0];
}

void VecchiaEngine::partial_sums2(const double* beta, bool with_grad, std::vector<double>& s2) {
  const int d = d_, p = p_;
  const int P2 = 1 + 2 * d;
  s2.assign(P2, 0.0);
  if (t1_ <= t0_) return;
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(dbeta_, beta, sizeof(double) * p, cudaMemcpyHostToDevice, st_));
  double* fin = dpart_ + (size_t)nblk_red_ * (VPMAX * VPMAX + VPMAX + 1 + 2 * 8 + 1);
  const double cnt = t1_ - t0_;
  {
    LaunchTimer lt("k_vsum2", st_, 0.0, 8.0 * cnt * (2.0 + p) * (with_grad ? 1.0 + d : 1.0));
    k_vsum2<<<nblk_red_, 256, 0, st_>>>(t0_, t1_, p, d, du_, dv_, dW_, ddu_, ddv_, ddW_, dbeta_, with_grad ? 1 : 0,
                                        dpart_);
    LKG_LAUNCH("k_vsum2");
    k_vsum_final<<<1, 256, 0, st_>>>(nblk_red_, P2, with_grad ? P2 : 1, dpart_, fin);
    LKG_LAUNCH("k_vsum_final");
  }
  LKG_CUDA(cudaMemcpyAsync(s2.data(), fin, sizeof(double) * (with_grad ? P2 : 1), cudaMemcpyDeviceToHost, st_));
  LKG_CUDA(cudaStreamSynchronize(st_));
}

std::string vecchia_failure_message() {
  const Config& cfg = config();
  return "[ERROR] Exceed max numerical nugget (" + std::to_string(cfg.max_inc_choldiag + 1) + " x 1e" +
         std::to_string(std::log10(cfg.num_nugget)) + ") added to force chol matrix";
}

int vecchia_gls_beta(int p, const std::vector<double>& s1, std::vector<double>& beta) {
  const Config& cfg = config();
  std::vector<double> A(s1.begin(), s1.begin() + p * p), b(s1.begin() + p * p, s1.begin() + p * p + p);
  for (int q = 0; q < p; ++q) A[q * p + q] += cfg.num_nugget;  // Kriging.cpp:898
  beta.assign(p, 0.0);
  return (p == 0 || small_spd_solve(p, A, b, beta)) ? 0 : -1;
}

void vecchia_finish(int n, int d, double slogv, const std::vector<double>& s2, bool with_grad, VecchiaOut& out) {
  const double Q = s2[0];
  const double sigma2 = Q / n;
  out.sigma2 = sigma2;
  out.vll = -0.5 * n * std::log(2 * M_PI * sigma2) - 0.5 * slogv - 0.5 * n;
  if (with_grad) {
    out.grad.resize(d);
    for (int k = 0; k < d; ++k) out.grad[k] = -0.5 * n * s2[1 + k] / Q - 0.5 * s2[1 + d + k];
  }
}

VecchiaOut VecchiaEngine::evaluate(const double* theta, bool with_grad, bool est_beta, const double* beta_fixed) {
  const int n = n_, d = d_, p = p_;
  VecchiaOut out;
  std::vector<double> s1, s2;
  const int failed = partial_sums1(theta, with_grad, s1, &out.nugget_points);
  if (failed > 0) {
    out.status = 1;
    out.message = vecchia_failure_message();
    return out;
  }
  std::vector<double> beta(p, 0.0);
  if (est_beta || beta_fixed == nullptr) {
    if (vecchia_gls_beta(p, s1, beta) != 0) {
      out.status = 2;
      out.message = "solve(): GLS system of the Vecchia likelihood is not positive definite";
      return out;
    }
  } else {
    beta.assign(beta_fixed, beta_fixed + p);
  }
  partial_sums2(beta.data(), with_grad, s2);
  out.beta = beta;
  vecchia_finish(n, d, s1[p * p + p], s2, with_grad, out);
  return out;
}

// ---------------------------------------------------------------------------------------------------------------
// conditioning sets
namespace {

// one launch per ordering step t: every block reduces the previous step's block maxima (identically), block 0
// records order[t], then each block updates its range of min squared distances and writes its new (max, index)
__global__ void k_maxmin_step(int n, int d, const double* __restrict__ Xp, double* __restrict__ mind2,
                              const double* __restrict__ pin_v, const int* __restrict__ pin_i, double* __restrict__ pout_v,
                              int* __restrict__ pout_i, int* __restrict__ order, int t) {
  __shared__ double sv[256];
  __shared__ int si[256];
  __shared__ int next_s;
  const int nb = gridDim.x;
  // reduce the previous partials (nb <= 256 entries)
  double bv = -INFINITY;
  int bi = 0x7fffffff;
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    const double v = pin_v[q];
    const int i = pin_i[q];
    if (v > bv || (v == bv && i < bi)) {
      bv = v;
      bi = i;
    }
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double ov = sv[threadIdx.x + s];
      const int oi = si[threadIdx.x + s];
      if (ov > sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = ov;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) next_s = si[0];
  __syncthreads();
  const int next = next_s;
  if (blockIdx.x == 0 && threadIdx.x == 0) order[t] = next;
  double nx[8];
  for (int k = 0; k < d; ++k) nx[k] = Xp[(int64_t)next * d + k];
  const int64_t lo = (int64_t)n * blockIdx.x / nb, hi = (int64_t)n * (blockIdx.x + 1) / nb;
  bv = -INFINITY;
  bi = 0x7fffffff;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double m = mind2[i];
    if (m != -INFINITY) {
      if (i == next) {
        m = -INFINITY;
      } else {
        double s = 0.0;
        for (int k = 0; k < d; ++k) {
          const double dk = Xp[i * d + k] - nx[k];
          s = __dadd_rn(s, __dmul_rn(dk, dk));  // no fused multiply-add, as the reference's loop
        }
        if (s < m) m = s;
      }
      mind2[i] = m;
    }
    if (m > bv || (m == bv && (int)i < bi)) {
      bv = m;
      bi = (int)i;
    }
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double ov = sv[threadIdx.x + s];
      const int oi = si[threadIdx.x + s];
      if (ov > sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = ov;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    pout_v[blockIdx.x] = sv[0];
    pout_i[blockIdx.x] = si[0];
  }
}

// m nearest earlier-ordered points of ordered point t, one warp per t: brute force over positions [0, t) with a
// sorted per-warp list of the m best (squared distance, global index) keys
__global__ void __launch_bounds__(256) k_knn_earlier(int n, int d, int m, const double* __restrict__ Xo,
                                                     const int32_t* __restrict__ order, int32_t* __restrict__ nbr) {
  __shared__ double kd[8][VECCHIA_MAX_M];
  __shared__ int ki[8][VECCHIA_MAX_M];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * 8 + w;
  if (t >= n) return;
  const int k = t < m ? t : m;
  double xt[8];
  for (int q = 0; q < d; ++q) xt[q] = Xo[(int64_t)t * d + q];
  int cnt = 0;  // entries in the list (uniform over the warp)
  double thr = INFINITY;
  int thri = 0x7fffffff;
  for (int j0 = 0; j0 < t; j0 += 32) {
    const int j = j0 + lane;
    double dj = INFINITY;
    int ij = 0x7fffffff;
    if (j < t) {
      double s = 0.0;
      for (int q = 0; q < d; ++q) {
        const double dq = xt[q] - Xo[(int64_t)j * d + q];
        s = __dadd_rn(s, __dmul_rn(dq, dq));
      }
      dj = s;
      ij = order[j];
    }
    bool qual = (j < t) && (cnt < k || dj < thr || (dj == thr && ij < thri));
    unsigned mask = __ballot_sync(FULL, qual);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const double cd = __shfl_sync(FULL, dj, src);
      const int ci = __shfl_sync(FULL, ij, src);
      if (lane == 0) {
        const bool full = cnt >= k;
        if (!full || cd < kd[w][k - 1] || (cd == kd[w][k - 1] && ci < ki[w][k - 1])) {
          int pos = full ? k - 1 : cnt;
          while (pos > 0 && (kd[w][pos - 1] > cd || (kd[w][pos - 1] == cd && ki[w][pos - 1] > ci))) {
            kd[w][pos] = kd[w][pos - 1];
            ki[w][pos] = ki[w][pos - 1];
            --pos;
          }
          kd[w][pos] = cd;
          ki[w][pos] = ci;
        }
      }
      cnt = cnt < k ? cnt + 1 : k;
      __syncwarp();
    }
    __syncwarp();
    if (cnt >= k && k > 0) {
      thr = kd[w][k - 1];
      thri = ki[w][k - 1];
    }
  }
  __syncwarp();
  for (int a = lane; a < m; a += 32) nbr[(int64_t)t * m + a] = (a < k) ? ki[w][a] : -1;
}

__global__ void k_gather_points(int n, int d, const double* __restrict__ X, const int32_t* __restrict__ order,
                                double* __restrict__ Xo, double* __restrict__ Xp) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int q = 0; q < d; ++q) {
    Xp[i * d + q] = X[i + (int64_t)q * n];  // point-major copy of X
    if (order) Xo[i * d + q] = X[order[i] + (int64_t)q * n];
  }
}

}  // namespace

void vecchia_sets_gpu(int n, int d, const double* X, int m, int32_t* order, int32_t* nbr) {
  if (d > 8) throw std::invalid_argument("Vecchia sets on the GPU support d <= 8");
  if (m > VECCHIA_MAX_M) throw std::invalid_argument("Vecchia sets on the GPU support m <= 32");
  const int mm = std::min(m, n - 1);
  cudaStream_t st;
  LKG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double* dX;
  int32_t *dorder, *dnbr;
  valloc(&dX, (size_t)n * d);
  valloc(&dorder, n);
  valloc(&dnbr, (size_t)n * std::max(m, 1));
  LKG_CUDA(cudaMemcpyAsync(dX, X, sizeof(double) * n * d, cudaMemcpyHostToDevice, st));
  // first point: closest to the centroid (index_min: first minimum), computed on the host in FP64 with the
  // reference's sequential sums (the host code is built without floating-point contraction)
  std::vector<double> cen(d, 0.0);
  for (int q = 0; q < d; ++q) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += X[i + (size_t)q * n];
    cen[q] = s / n;
  }
  int first = 0;
  double best = INFINITY;
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int q = 0; q < d; ++q) {
      const double dk = X[i + (size_t)q * n] - cen[q];
      s += dk * dk;
    }
    if (s < best) {
      best = s;
      first = i;
    }
  }
  vecchia_sets_grid(n, d, X, dX, first, m, dorder, dnbr, st);
  LKG_CUDA(cudaMemcpyAsync(order, dorder, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  std::vector<int32_t> tmp((size_t)n * std::max(mm, 1));
  if (mm > 0)
    LKG_CUDA(cudaMemcpyAsync(tmp.data(), dnbr, sizeof(int32_t) * n * mm, cudaMemcpyDeviceToHost, st));
  LKG_CUDA(cudaStreamSynchronize(st));
  for (int t = 0; t < n; ++t)
    for (int a = 0; a < m; ++a) nbr[(size_t)t * m + a] = (a < mm) ? tmp[(size_t)t * mm + a] : -1;
  cudaFree(dX);
  cudaFree(dorder);
  cudaFree(dnbr);
  cudaStreamDestroy(st);
}

void vecchia_predict_gpu(int kernel, int n, int d, const double* X, const double* resid, const double* theta, int q,
                         const double* Xq, int m, std::vector<double>& ar, std::vector<double>& ra) {
  if (d < 1 || d > 8) throw std::invalid_argument("predictVecchia on the GPU supports d <= 8");
  if (m < 1 || m > VECCHIA_MAX_M || m > n) throw std::invalid_argument("predictVecchia on the GPU supports m <= 32");
  ar.assign(q, 0.0);
  ra.assign(q, 0.0);
  if (q <= 0) return;
  const Config& cfg = config();
  cudaStream_t st;
  LKG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  double *dX = nullptr, *dR = nullptr, *dth = nullptr, *dXq = nullptr, *dar = nullptr, *dra = nullptr;
  int* dst = nullptr;
  auto cleanup = [&]() {
    for (double* p : {dX, dR, dth, dXq, dar, dra})
      if (p) cudaFree(p);
    if (dst) cudaFree(dst);
    cudaStreamDestroy(st);
  };
  std::vector<int> status(q);
  try {
    valloc(&dX, (size_t)n * d);
    valloc(&dR, n);
    valloc(&dth, d);
    valloc(&dXq, (size_t)q * d);
    valloc(&dar, q);
    valloc(&dra, q);
    valloc(&dst, q);
    LKG_CUDA(cudaMemcpyAsync(dX, X, sizeof(double) * (size_t)n * d, cudaMemcpyHostToDevice, st));
    LKG_CUDA(cudaMemcpyAsync(dR, resid, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    LKG_CUDA(cudaMemcpyAsync(dth, theta, sizeof(double) * d, cudaMemcpyHostToDevice, st));
    LKG_CUDA(cudaMemcpyAsync(dXq, Xq, sizeof(double) * (size_t)q * d, cudaMemcpyHostToDevice, st));
    VPredArgs a{n, d, m, q, dX, dR, dth, dXq, cfg.num_nugget, cfg.min_rcond, cfg.chol_rcond_check ? 1 : 0,
                cfg.max_inc_choldiag, dar, dra, dst};
    auto go = [&](auto kc) {
      constexpr int KK = decltype(kc)::value;
      if (d <= 4) VPredLaunch<KK, 4>::run(a, st);
      else VPredLaunch<KK, 8>::run(a, st);
    };
    switch (kernel) {
      case KGAUSS: go(std::integral_constant<int, KGAUSS>{}); break;
      case KEXP: go(std::integral_constant<int, KEXP>{}); break;
      case KMATERN32: go(std::integral_constant<int, KMATERN32>{}); break;
      case KMATERN52: go(std::integral_constant<int, KMATERN52>{}); break;
      default: throw std::invalid_argument("Unsupported covariance kernel id");
    }
    LKG_CUDA(cudaMemcpyAsync(ar.data(), dar, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
    LKG_CUDA(cudaMemcpyAsync(ra.data(), dra, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
    LKG_CUDA(cudaMemcpyAsync(status.data(), dst, sizeof(int) * q, cudaMemcpyDeviceToHost, st));
    LKG_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    cleanup();
    throw;
  }
  cleanup();
  for (int t = 0; t < q; ++t)
    if (status[t] < 0)
      throw std::runtime_error("[ERROR] Exceed max numerical nugget (" + std::to_string(cfg.max_inc_choldiag + 1) +
                               " x 1e" + std::to_string(std::log10(cfg.num_nugget)) + ") added to force chol matrix");
}

// ---------------------------------------------------------------------------------------------------------------
// conditioning sets with no allocation: the intermediates of vecchia_sets_gpu (point-major X, ordered X, running
// minimum distances, block maxima) live in one fixed device array.  Layout in doubles, for n points in d dims:
//   [0, nd) point-major X | [nd, 2nd) X in maxmin order | [2nd, 2nd + n) min squared distances |
//   512 doubles of block maxima (two buffers of <= 256) | 256 doubles holding their 2 x 256 int indices
// Every word is written before it is read within one call, so nothing has to start at zero and nothing is carried
// from one call to the next.
static __device__ __align__(256) double g_sets_scratch[SETS_SCRATCH_DOUBLES];

namespace {

constexpr int SETS_MAX_DEVICES = 64;
constexpr long long SETS_FIXED_DOUBLES = 768;  // block maxima and their indices
std::mutex g_sets_mu;
// g_sets_scratch's address on each device, with the ID of the context it was resolved in.  A context reset
// (cudaDeviceReset, a primary-context reset by another library) reloads the module and may move the array, so
// the address is resolved again whenever the current context's ID differs from the recorded one.
struct SetsSlot {
  unsigned long long ctx_id;
  double* addr;
};
SetsSlot g_sets_slot[SETS_MAX_DEVICES];
thread_local char g_sets_msg[320];

// driver entry points for the current context's ID, looked up through the runtime (the library does not link
// libcuda directly); the types mirror cuCtxGetCurrent / cuCtxGetId with opaque handles
using CtxGetCurrentFn = int (*)(void** ctx);
using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

const char* sets_msg_cuda(const char* what, cudaError_t e) {
  std::snprintf(g_sets_msg, sizeof g_sets_msg, "lkg_vecchia_sets_noalloc: %s failed: %s", what,
                cudaGetErrorString(e));
  return g_sets_msg;
}

// device (or managed) memory usable from device `dev`
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}

// first point of the maxmin order (closest to the centroid, lowest index on ties -- the host computation of
// vecchia_sets_gpu moved to one block), min squared distances set to +inf, and step-0 block maxima that all name
// that point, so that k_maxmin_step at t = 0 records it and computes the distances to that point
__global__ void __launch_bounds__(1024) k_sets_prepare(int n, int d, const double* __restrict__ X, int nb,
                                                       double* __restrict__ mind2, double* __restrict__ pv,
                                                       int* __restrict__ pi) {
  __shared__ double cen[8];
  __shared__ double sv[1024];
  __shared__ int si[1024];
  if (threadIdx.x < d) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += X[i + (int64_t)threadIdx.x * n];  // same order as the host sum
    cen[threadIdx.x] = s / n;
  }
  __syncthreads();
  double bv = INFINITY;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int q = 0; q < d; ++q) {
      const double dk = X[i + (int64_t)q * n] - cen[q];
      s = __dadd_rn(s, __dmul_rn(dk, dk));  // no fused multiply-add, as in the host loop
    }
    if (s < bv) {
      bv = s;
      bi = i;
    }
    mind2[i] = INFINITY;
  }
  sv[threadIdx.x] = bv;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = 512; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      const double ov = sv[threadIdx.x + s];
      const int oi = si[threadIdx.x + s];
      if (ov < sv[threadIdx.x] || (ov == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = ov;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int first = si[0] == 0x7fffffff ? 0 : si[0];
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    pv[q] = 0.0;
    pi[q] = first;
  }
}

}  // namespace

const char* vecchia_sets_noalloc(int n, int d, const double* X, int m, int32_t* order, int32_t* nbr,
                                 cudaStream_t st) {
  if (n < 1 || d < 1 || d > 8 || m < 0 || m > VECCHIA_MAX_M)
    return "lkg_vecchia_sets_noalloc: needs n >= 1, 1 <= d <= 8 and 0 <= m <= 32";
  const long long need = (long long)n * (2 * d + 1) + SETS_FIXED_DOUBLES;
  if (need > SETS_SCRATCH_DOUBLES) {
    std::snprintf(g_sets_msg, sizeof g_sets_msg,
                  "lkg_vecchia_sets_noalloc: n = %d points in d = %d dims need %lld doubles of scratch, more than the "
                  "fixed %lld (n * (2 d + 1) + %lld <= %lld; at d = %d, n <= %lld); use lkg_vecchia_sets",
                  n, d, need, SETS_SCRATCH_DOUBLES, SETS_FIXED_DOUBLES, SETS_SCRATCH_DOUBLES, d,
                  (SETS_SCRATCH_DOUBLES - SETS_FIXED_DOUBLES) / (2 * d + 1));
    return g_sets_msg;
  }
  if (!X || !order || (m > 0 && !nbr)) return "lkg_vecchia_sets_noalloc: null buffer";
  if ((uintptr_t)X % alignof(double) || (uintptr_t)order % alignof(int32_t) ||
      (m > 0 && (uintptr_t)nbr % alignof(int32_t)))
    return "lkg_vecchia_sets_noalloc: misaligned buffer";
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return sets_msg_cuda("cudaGetDevice", e);
  if (dev < 0 || dev >= SETS_MAX_DEVICES) return "lkg_vecchia_sets_noalloc: device ordinal >= 64";
  if (!on_device(X, dev) || !on_device(order, dev) || (m > 0 && !on_device(nbr, dev)))
    return "lkg_vecchia_sets_noalloc: X, order and nbr must be device (or managed) memory of the current device";
  double* base;
  {
    std::lock_guard<std::mutex> lock(g_sets_mu);
    if (!g_ctx_get_current || !g_ctx_get_id) {
      void* f1 = nullptr;
      void* f2 = nullptr;
      cudaDriverEntryPointQueryResult q1, q2;
      e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
      if (e != cudaSuccess || q1 != cudaDriverEntryPointSuccess || !f1)
        return e != cudaSuccess ? sets_msg_cuda("cudaGetDriverEntryPointByVersion", e)
                                : "lkg_vecchia_sets_noalloc: the driver has no cuCtxGetCurrent";
      e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
      if (e != cudaSuccess || q2 != cudaDriverEntryPointSuccess || !f2)
        return e != cudaSuccess ? sets_msg_cuda("cudaGetDriverEntryPointByVersion", e)
                                : "lkg_vecchia_sets_noalloc: the driver has no cuCtxGetId";
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    void* ctx = nullptr;
    unsigned long long ctx_id = 0;
    if (g_ctx_get_current(&ctx) == 0 && !ctx) {
      // the caller's buffers live in this device's primary context; make it current on this thread
      e = cudaSetDevice(dev);
      if (e != cudaSuccess) return sets_msg_cuda("cudaSetDevice", e);
      g_ctx_get_current(&ctx);
    }
    if (!ctx || g_ctx_get_id(ctx, &ctx_id) != 0)
      return "lkg_vecchia_sets_noalloc: no current CUDA context on this thread";
    SetsSlot& slot = g_sets_slot[dev];
    if (!slot.addr || slot.ctx_id != ctx_id) {
      // first call in this context: resolve the array and load every kernel the call may launch, so that later
      // calls load nothing (with lazy module loading a kernel is otherwise loaded at its first launch)
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_sets_scratch);
      if (e != cudaSuccess) return sets_msg_cuda("cudaGetSymbolAddress", e);
      cudaFuncAttributes fa;
      const void* kernels[] = {(const void*)k_gather_points, (const void*)k_sets_prepare,
                               (const void*)k_maxmin_step, (const void*)k_knn_earlier};
      for (const void* k : kernels) {
        e = cudaFuncGetAttributes(&fa, k);
        if (e != cudaSuccess) return sets_msg_cuda("cudaFuncGetAttributes", e);
      }
      slot.addr = static_cast<double*>(p);
      slot.ctx_id = ctx_id;
    }
    base = slot.addr;
  }
  // an error left by an earlier, unrelated runtime call on this thread must not be reported as this call's
  (void)cudaGetLastError();
  double* Xp = base;
  double* Xo = Xp + (int64_t)n * d;
  double* mind2 = Xo + (int64_t)n * d;
  double* pv = mind2 + n;
  int* pi = reinterpret_cast<int*>(pv + 512);
  const int nb = std::min(256, std::max(1, ceil_div(n, 1024)));
  k_gather_points<<<ceil_div(n, 256), 256, 0, st>>>(n, d, X, nullptr, nullptr, Xp);
  // step t reads the maxima buffer (t + 1) & 1 and writes t & 1; step 0 reads the prepared buffer 1
  k_sets_prepare<<<1, 1024, 0, st>>>(n, d, X, nb, mind2, pv + nb, pi + nb);
  e = cudaGetLastError();
  if (e != cudaSuccess) return sets_msg_cuda("kernel launch", e);
  for (int t = 0; t < n; ++t) {
    const int in = (t + 1) & 1, outb = t & 1;
    k_maxmin_step<<<nb, 256, 0, st>>>(n, d, Xp, mind2, pv + in * nb, pi + in * nb, pv + outb * nb, pi + outb * nb,
                                      order, t);
  }
  k_gather_points<<<ceil_div(n, 256), 256, 0, st>>>(n, d, X, order, Xo, Xp);
  if (m > 0) k_knn_earlier<<<ceil_div(n, 8), 256, 0, st>>>(n, d, m, Xo, order, nbr);
  e = cudaGetLastError();
  if (e != cudaSuccess) return sets_msg_cuda("kernel launch", e);
  return nullptr;
}

}  // namespace lkg
