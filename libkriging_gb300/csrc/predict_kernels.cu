// predict_kernels.cu -- GPU part of Kriging::predict.
//
// KrigingImpl::predict_impl (src/lib/KrigingImpl.cpp:145-251): R_on (:194-221), Rstar_on = L \ R_on (:223),
// yhat = F_n beta + Rstar_on' z (:226), Fhat_n = Rstar_on' M (:232), sd2 = 1 - colsum(Rstar_on^2) + ... (:238),
// Sigma_n = R_nn - Rstar_on' Rstar_on + Ecirc Ecirc' (:248).  The p-column trend algebra stays on the host.
#include "predict_kernels.cuh"

#include "stats.hpp"

#include "common.cuh"
#include "dense_fp64.cuh"
#include "lik_kernels.cuh"

namespace lkg {

namespace {

template <int NTH>
__device__ double bsum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < NTH / 32; ++i) s += red[i];
  return s;
}

// per column j of Rs (n x q): rz[j] = Rs(:,j)'z, rr[j] = Rs(:,j)'Rs(:,j), rm[j*p + k] = Rs(:,j)'M(:,k)
__global__ void k_predict_reduce(int n, int q, int p, const double* __restrict__ Rs, const double* __restrict__ z,
                                 const double* __restrict__ M, double* __restrict__ rz, double* __restrict__ rr,
                                 double* __restrict__ rm) {
  const int j = blockIdx.x;
  const int k = (int)blockIdx.y - 2;  // -2: rz, -1: rr, >= 0: rm column k
  __shared__ double red[32];
  const double* c = Rs + (size_t)j * n;
  double s = 0.0;
  if (k == -2) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(c[i], z[i], s);
  } else if (k == -1) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(c[i], c[i], s);
  } else {
    const double* m = M + (size_t)k * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(c[i], m[i], s);
  }
  s = bsum<256>(s, red);
  if (threadIdx.x == 0) {
    if (k == -2) rz[j] = s;
    else if (k == -1) rr[j] = s;
    else rm[(size_t)j * p + k] = s;
  }
}

struct DevBuf {
  double* p = nullptr;
  explicit DevBuf(size_t n) { LKG_CUDA(cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1))); }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

PredictOut predict_gpu(const Engine& model, const double* Xn, int q, const double* theta, double factor,
                       const double* z, bool need_rr, bool need_cov, double nn_factor, bool nugget) {
  (void)nugget;
  const int n = model.n(), d = model.d(), p = model.p();
  cudaStream_t st = model.stream();
  PredictOut o;
  if (q <= 0) return o;
  DevBuf dXn((size_t)q * d), dth(d), dz(n), dRs((size_t)n * q), drz(q), drr(q), drm((size_t)q * std::max(p, 1));
  LKG_CUDA(cudaMemcpyAsync(dXn.p, Xn, sizeof(double) * q * d, cudaMemcpyHostToDevice, st));
  LKG_CUDA(cudaMemcpyAsync(dth.p, theta, sizeof(double) * d, cudaMemcpyHostToDevice, st));
  LKG_CUDA(cudaMemcpyAsync(dz.p, z, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  cov_cross(model.kernel(), n, q, d, model.dX(), dXn.p, dth.p, factor, dRs.p, st);
  model.solve_lower_inplace(0, dRs.p, n, q);
  LaunchTimer lt("k_predict_reduce", st, 2.0 * n * q * (p + 2.0), 8.0 * n * q);
  k_predict_reduce<<<dim3(q, 2 + p), 256, 0, st>>>(n, q, p, dRs.p, dz.p, model.dFY(0), drz.p, drr.p, drm.p);
  LKG_LAUNCH("k_predict_reduce");
  o.rz.resize(q);
  o.rr.resize(q);
  o.rm.resize((size_t)q * p);
  LKG_CUDA(cudaMemcpyAsync(o.rz.data(), drz.p, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
  if (need_rr) LKG_CUDA(cudaMemcpyAsync(o.rr.data(), drr.p, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(o.rm.data(), drm.p, sizeof(double) * q * p, cudaMemcpyDeviceToHost, st));
  if (need_cov) {
    // R_nn (lower, diag 1) then Sigma = R_nn - Rs' Rs (lower), mirrored on the host
    DevBuf dRnn((size_t)q * q), dfac(1), ddiag(1);
    LKG_CUDA(cudaMemcpyAsync(dfac.p, &nn_factor, sizeof(double), cudaMemcpyHostToDevice, st));
    const double one = 1.0;
    LKG_CUDA(cudaMemcpyAsync(ddiag.p, &one, sizeof(double), cudaMemcpyHostToDevice, st));
    cov_build_lower(model.kernel(), q, d, dXn.p, 0, dth.p, dfac.p, ddiag.p, dRnn.p, q, 0, 1, st);
    MatView a{dRs.p, n, 1, 0};   // A(m, k) = Rs(k, m)
    MatView b{dRs.p, 1, n, 0};   // B(k, c) = Rs(k, c)
    gemm_tiles(q, q, n, -1.0, a, b, 1.0, dRnn.p, q, 0, 1, true, st);
    o.sigma.resize((size_t)q * q);
    LKG_CUDA(cudaMemcpyAsync(o.sigma.data(), dRnn.p, sizeof(double) * q * q, cudaMemcpyDeviceToHost, st));
    LKG_CUDA(cudaStreamSynchronize(st));
    for (int j = 0; j < q; ++j)
      for (int i = 0; i < j; ++i) o.sigma[i + (size_t)j * q] = o.sigma[j + (size_t)i * q];
  }
  LKG_CUDA(cudaStreamSynchronize(st));
  return o;
}

}  // namespace lkg
