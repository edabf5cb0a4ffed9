// predict_kernels.cu -- GPU part of Kriging::predict.
//
// KrigingImpl::predict_impl (src/lib/KrigingImpl.cpp:145-300): R_on (:194-221), Rstar_on = L \ R_on (:223),
// yhat = F_n beta + Rstar_on' z (:226), Fhat_n = Rstar_on' M (:232), sd2 = 1 - colsum(Rstar_on^2) + ... (:238),
// Sigma_n = R_nn - Rstar_on' Rstar_on + Ecirc Ecirc' (:248); the derivatives' W_i = L \ DR_on_i and its products
// with z, Rstar_on and M (:254-281).  The p-column trend algebra stays on the host.
#include "predict_kernels.cuh"

#include <cstdint>
#include <mutex>

#include "stats.hpp"

#include "common.cuh"
#include "dense_fp64.cuh"
#include "lik_kernels.cuh"
#include "ozaki7.cuh"

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

// per column c of W (n x ncols, ld n): oz[c] = W(:,c)'z, orr[c] = W(:,c)'R(:, c / rdiv) (ld n),
// om[c * p + k] = W(:,c)'M(:,k); one CTA per (column, product), fixed-order sums
__global__ void k_predict_reduce(int n, int ncols, int p, const double* __restrict__ W, const double* __restrict__ z,
                                 const double* __restrict__ R, int rdiv, const double* __restrict__ M,
                                 double* __restrict__ oz, double* __restrict__ orr, double* __restrict__ om) {
  const int j = blockIdx.x;
  const int k = (int)blockIdx.y - 2;  // -2: z, -1: R, >= 0: M column k
  __shared__ double red[32];
  const double* c = W + (size_t)j * n;
  const double* v = (k == -2) ? z : (k == -1) ? R + (size_t)(j / rdiv) * n : M + (size_t)k * n;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(c[i], v[i], s);
  s = bsum<256>(s, red);
  if (threadIdx.x == 0) {
    if (k == -2) oz[j] = s;
    else if (k == -1) orr[j] = s;
    else om[(size_t)j * p + k] = s;
  }
}

void predict_reduce(int n, int ncols, int p, const double* W, const double* z, const double* R, int rdiv,
                    const double* M, double* oz, double* orr, double* om, cudaStream_t st) {
  LaunchTimer lt("k_predict_reduce", st, 2.0 * n * ncols * (p + 2.0), 8.0 * n * ncols);
  k_predict_reduce<<<dim3(ncols, 2 + p), 256, 0, st>>>(n, ncols, p, W, z, R, rdiv, M, oz, orr, om);
  LKG_LAUNCH("k_predict_reduce");
}

// Device scratch from the stream-ordered pool: allocation and release are queued on the stream (no device-wide
// synchronisation when many submodels predict concurrently), and the device's default pool keeps up to 8 GiB of
// released memory for reuse (raised from its default of none, never lowered).
void keep_pool_memory() {
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    LKG_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    LKG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t keep = 0;
    LKG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    const uint64_t want = (uint64_t)8 << 30;
    if (keep < want) LKG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, (void*)&want));
  });
}

struct DevBuf {
  double* p = nullptr;
  cudaStream_t st;
  DevBuf(size_t n, cudaStream_t s) : st(s) {
    keep_pool_memory();
    LKG_CUDA(cudaMallocAsync((void**)&p, sizeof(double) * std::max<size_t>(n, 1), st));
  }
  ~DevBuf() {
    if (p) cudaFreeAsync(p, st);
  }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

}  // namespace

PredictOut predict_gpu(Engine& model, const double* Xn, int q, const double* theta, double factor, const double* z,
                       bool need_rr, bool need_cov, double nn_factor, bool need_deriv, bool digits) {
  const int n = model.n(), d = model.d(), p = model.p();
  cudaStream_t st = model.stream();
  PredictOut o;
  if (q <= 0) return o;
  // the covariance and the derivatives need Rstar_on for all points at once; otherwise the points go in chunks of
  // at most 2^25 / n (Rstar_on of a chunk below 256 MB)
  const bool whole = need_cov || need_deriv;
  const int qc = whole ? q : (int)std::max<int64_t>(1, std::min<int64_t>(q, ((int64_t)1 << 25) / n));
  DevBuf dXn((size_t)q * d, st), dth(d, st), dz(n, st), dRs((size_t)n * qc, st), drz(q, st), drr(q, st),
      drm((size_t)q * std::max(p, 1), st);
  LKG_CUDA(cudaMemcpyAsync(dXn.p, Xn, sizeof(double) * q * d, cudaMemcpyHostToDevice, st));
  LKG_CUDA(cudaMemcpyAsync(dth.p, theta, sizeof(double) * d, cudaMemcpyHostToDevice, st));
  LKG_CUDA(cudaMemcpyAsync(dz.p, z, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  if (whole) {
    cov_cross(model.kernel(), n, q, d, model.dX(), dXn.p, dth.p, factor, dRs.p, st);
    model.solve_lower_inplace(0, dRs.p, n, q);
    predict_reduce(n, q, p, dRs.p, dz.p, dRs.p, 1, model.dFY(0), drz.p, drr.p, drm.p, st);
  } else {
    // the chunk's points as their own q x d column-major block
    DevBuf dXc((size_t)qc * d, st);
    // digit products: L^-1 split once (rows of W, k = its columns), each chunk's R_on split by points (rows = points,
    // k = observations), Rstar_on = W R_on written over R_on (the product reads the split copies)
    constexpr int S = 8;
    const double* W = digits ? model.factor_inverse() : nullptr;
    DevBuf dWs(digits ? oz7_plane_elems(n, n, S) / 4 + 1 : 1, st), dRsp(digits ? oz7_plane_elems(qc, n, S) / 4 + 1 : 1, st);
    DevBuf dWe(digits ? oz7_exp_elems(n, n, OZ7_KB) / 2 + 1 : 1, st), dRse(digits ? oz7_exp_elems(qc, n, OZ7_KB) / 2 + 1 : 1, st);
    Split7 SW, SR;
    if (digits) {
      SW = oz7_buffer(dWs.p, reinterpret_cast<int*>(dWe.p), S, n, n, OZ7_KB);
      SR = oz7_buffer(dRsp.p, reinterpret_cast<int*>(dRse.p), S, qc, n, OZ7_KB);
      oz7_split(n, n, W, 1, model.lda(), 0, 1, SW, st);
    }
    for (int c0 = 0; c0 < q; c0 += qc) {
      const int nc = std::min(qc, q - c0);
      for (int k = 0; k < d; ++k)
        LKG_CUDA(cudaMemcpyAsync(dXc.p + (size_t)k * nc, dXn.p + (size_t)k * q + c0, sizeof(double) * nc,
                                 cudaMemcpyDeviceToDevice, st));
      cov_cross(model.kernel(), n, nc, d, model.dX(), dXc.p, dth.p, factor, dRs.p, st);
      if (digits) {
        oz7_split(nc, n, dRs.p, n, 1, 0, 1, SR, st);
        oz7_gemm(n, nc, 0, SW.nblk, 1.0, SW, SR, 0.0, dRs.p, n, 0, 1, false, st);
      } else {
        model.solve_lower_inplace(0, dRs.p, n, nc);
      }
      predict_reduce(n, nc, p, dRs.p, dz.p, dRs.p, 1, model.dFY(0), drz.p + c0, drr.p + c0,
                     drm.p + (size_t)c0 * p, st);
    }
    if (digits && oz7_error_and_reset())
      throw std::runtime_error("predict: a tensor-core digit product did not complete (timed out)");
  }
  o.rz.resize(q);
  o.rr.resize(q);
  o.rm.resize((size_t)q * p);
  LKG_CUDA(cudaMemcpyAsync(o.rz.data(), drz.p, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
  if (need_rr) LKG_CUDA(cudaMemcpyAsync(o.rr.data(), drr.p, sizeof(double) * q, cudaMemcpyDeviceToHost, st));
  if (p > 0) LKG_CUDA(cudaMemcpyAsync(o.rm.data(), drm.p, sizeof(double) * q * p, cudaMemcpyDeviceToHost, st));
  if (need_cov) {
    // R_nn (lower, diag 1) then Sigma = R_nn - Rs' Rs (lower), mirrored on the host
    DevBuf dRnn((size_t)q * q, st), dfac(1, st), ddiag(1, st);
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
  if (need_deriv) {
    // W = L \ DR_on in chunks of points (n x qd d doubles at most 2^26), then its column products with z,
    // Rstar_on(:, c) and M (KrigingImpl.cpp:254-281)
    const int qd = (int)std::max<int64_t>(1, std::min<int64_t>(q, ((int64_t)1 << 26) / ((int64_t)n * d)));
    DevBuf dW((size_t)n * qd * d, st), dwz((size_t)qd * d, st), dwr((size_t)qd * d, st),
        dwm((size_t)qd * d * std::max(p, 1), st);
    o.wz.resize((size_t)q * d);
    o.wr.resize((size_t)q * d);
    o.wm.resize((size_t)q * d * p);
    for (int c0 = 0; c0 < q; c0 += qd) {
      const int nc = std::min(qd, q - c0), ncol = nc * d;
      // the chunk's points are columns c0.. of the q x d column-major Xn: pass them with their own leading dimension
      std::vector<double> xc((size_t)nc * d);
      for (int k = 0; k < d; ++k)
        for (int c = 0; c < nc; ++c) xc[c + (size_t)k * nc] = Xn[(c0 + c) + (size_t)k * q];
      DevBuf dxc((size_t)nc * d, st);
      LKG_CUDA(cudaMemcpyAsync(dxc.p, xc.data(), sizeof(double) * nc * d, cudaMemcpyHostToDevice, st));
      dcov_cross(model.kernel(), n, nc, d, model.dX(), dxc.p, dth.p, factor, dW.p, st);
      model.solve_lower_inplace(0, dW.p, n, ncol);
      predict_reduce(n, ncol, p, dW.p, dz.p, dRs.p + (size_t)c0 * n, d, model.dFY(0), dwz.p, dwr.p, dwm.p, st);
      LKG_CUDA(cudaMemcpyAsync(o.wz.data() + (size_t)c0 * d, dwz.p, sizeof(double) * ncol, cudaMemcpyDeviceToHost,
                               st));
      LKG_CUDA(cudaMemcpyAsync(o.wr.data() + (size_t)c0 * d, dwr.p, sizeof(double) * ncol, cudaMemcpyDeviceToHost,
                               st));
      if (p > 0)
        LKG_CUDA(cudaMemcpyAsync(o.wm.data() + (size_t)c0 * d * p, dwm.p, sizeof(double) * ncol * p,
                                 cudaMemcpyDeviceToHost, st));
      LKG_CUDA(cudaStreamSynchronize(st));  // xc and dxc are released at the end of the iteration
    }
  }
  LKG_CUDA(cudaStreamSynchronize(st));
  return o;
}

}  // namespace lkg
