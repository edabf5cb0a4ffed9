// common.cuh -- shared definitions for the GB300 likelihood kernels (sm_103a).
//
// Covariance functions restate libKriging src/lib/Covariance.cpp (same formulas, same operation order):
//   gauss      Cov :24-36   DlnCovDtheta :38-50
//   exp        Cov :65-75   DlnCovDtheta :77-88
//   matern3_2  Cov :104-116 DlnCovDtheta :118-130
//   matern5_2  Cov :149-161 DlnCovDtheta :163-179
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>

namespace lkg {

enum Kernel : int { KGAUSS = 0, KEXP = 1, KMATERN32 = 2, KMATERN52 = 3 };

constexpr int MAX_D = 32;  // largest input dimension the fused kernels accept

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

inline void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess)
    throw CudaError(std::string("CUDA error in ") + what + " (" + file + ":" + std::to_string(line) +
                    "): " + cudaGetErrorString(e));
}
#define LKG_CUDA(x) ::lkg::check_cuda((x), #x, __FILE__, __LINE__)
#define LKG_LAUNCH(what) ::lkg::check_cuda(cudaGetLastError(), what, __FILE__, __LINE__)

// 1 / sqrt(piv) by Newton's iteration y <- y (3 - piv y^2) / 2 from a single-precision seed: two steps take the
// seed's 2^-23 relative error below FP64 rounding; outside the range where the seed is a normal float the square
// root and the reciprocal are taken directly
__device__ __forceinline__ void pivot_root(double piv, double& root, double& rroot) {
  if (piv >= 1e-30 && piv <= 1e30) {
    double y = (double)rsqrtf((float)piv);
    const double h = -0.5 * piv;
    y = y * fma(h, y * y, 1.5);
    y = y * fma(h, y * y, 1.5);
    rroot = y;
    root = piv * y;
  } else {
    root = sqrt(piv);
    rroot = 1.0 / root;
  }
}

// ---------------------------------------------------------------------------------------------------------------
// device covariance functions.  dx is X_j - X_i (sign irrelevant for Cov and DlnCovDtheta), inv_theta = 1/theta is
// NOT used for the value so that the rounding matches the reference's dx/theta division.
// ---------------------------------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ double cov_term(double dx, double th) {
  if constexpr (K == KGAUSS) {
    double v = dx / th;
    return v * v;
  } else if constexpr (K == KEXP) {
    return fabs(dx / th);
  } else if constexpr (K == KMATERN32) {
    double t = sqrt(3.0) * fabs(dx / th);
    return t - log1p(t);
  } else {
    double t = sqrt(5.0) * fabs(dx / th);
    return t - log1p(t + (t * t) / 3.0);
  }
}

template <int K>
__device__ __forceinline__ double cov_from_sum(double s) {
  if constexpr (K == KGAUSS)
    return exp(-0.5 * s);
  else
    return exp(-s);
}

template <int K>
__device__ __forceinline__ double dlncov_term(double dx, double th) {
  if constexpr (K == KGAUSS) {
    return (dx * dx) / (th * th * th);
  } else if constexpr (K == KEXP) {
    return fabs(dx) / (th * th);
  } else if constexpr (K == KMATERN32) {
    double t = sqrt(3.0) * fabs(dx / th);
    return (t * t) / (1.0 + t) / th;
  } else {
    double t = sqrt(5.0) * fabs(dx / th);
    double a = 1.0 + t;
    double b = (t * t) / 3.0;
    return (a * b) / (a + b) / th;
  }
}

// Fast forms (no per-dimension division or log1p): with c_k = s / theta_k (s = 1, sqrt(3), sqrt(5)) and
// t_k = c_k |dx_k|,
//   gauss     exp(-0.5 sum (dx_k / theta_k)^2)
//   exp       exp(-sum t_k)
//   matern3_2 prod (1 + t_k) exp(-sum t_k)              = exp(-sum (t_k - log1p t_k))
//   matern5_2 prod (1 + t_k + t_k^2 / 3) exp(-sum t_k)  = exp(-sum (t_k - log1p(t_k + t_k^2 / 3)))
// Equal to the reference forms up to a few ulps; used where the reference's rounding is not the contract (the
// gradient sums and the mixed-precision covariance build).
template <int K>
__device__ __forceinline__ double cov_scale() {
  if constexpr (K == KMATERN32) return sqrt(3.0);
  else if constexpr (K == KMATERN52) return sqrt(5.0);
  else return 1.0;
}

// accumulate one dimension: sum_state (the exponent argument) and prod_state (the polynomial product)
template <int K>
__device__ __forceinline__ void cov_fast_term(double dx, double ck, double& sum_state, double& prod_state) {
  if constexpr (K == KGAUSS) {
    const double v = dx * ck;
    sum_state = fma(v, v, sum_state);
  } else {
    const double t = fabs(dx) * ck;
    sum_state += t;
    if constexpr (K == KMATERN32) prod_state *= (1.0 + t);
    if constexpr (K == KMATERN52) prod_state *= fma(t, t * (1.0 / 3.0), 1.0 + t);
  }
}

template <int K>
__device__ __forceinline__ double cov_fast_finish(double sum_state, double prod_state) {
  if constexpr (K == KGAUSS) return exp(-0.5 * sum_state);
  else if constexpr (K == KEXP) return exp(-sum_state);
  else return prod_state * exp(-sum_state);
}

// dlnC/dtheta_k with inv = 1 / theta_k and ck = s / theta_k
template <int K>
__device__ __forceinline__ double dlncov_fast(double dx, double inv, double ck) {
  if constexpr (K == KGAUSS) {
    const double v = dx * inv;
    return v * v * inv;
  } else if constexpr (K == KEXP) {
    return fabs(dx) * inv * inv;
  } else if constexpr (K == KMATERN32) {
    const double t = fabs(dx) * ck;
    return (t * t) / (1.0 + t) * inv;
  } else {
    const double t = fabs(dx) * ck;
    const double a = 1.0 + t, b = t * t * (1.0 / 3.0);
    return (a * b) / (a + b) * inv;
  }
}

// dispatch a runtime kernel id to a template functor call
template <typename F>
inline void dispatch_kernel(int k, F&& f) {
  switch (k) {
    case KGAUSS: f.template operator()<KGAUSS>(); break;
    case KEXP: f.template operator()<KEXP>(); break;
    case KMATERN32: f.template operator()<KMATERN32>(); break;
    case KMATERN52: f.template operator()<KMATERN52>(); break;
    default: throw std::invalid_argument("Unsupported covariance kernel id " + std::to_string(k));
  }
}

inline int kernel_from_name(const std::string& s) {
  if (s == "gauss") return KGAUSS;
  if (s == "exp") return KEXP;
  if (s == "matern3_2") return KMATERN32;
  if (s == "matern5_2") return KMATERN52;
  throw std::invalid_argument("Unsupported covariance kernel: " + s);
}

inline const char* kernel_name(int k) {
  switch (k) {
    case KGAUSS: return "gauss";
    case KEXP: return "exp";
    case KMATERN32: return "matern3_2";
    case KMATERN52: return "matern5_2";
  }
  return "?";
}

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Launch<kernel, DM>::run(args...) for the runtime kernel id and the smallest DM in {4, 8, 16, 32} holding d
template <template <int, int> class Launch, typename... Args>
void dispatch_kd(int kernel, int d, Args&&... args) {
  auto go = [&](auto kc) {
    constexpr int KK = decltype(kc)::value;
    if (d <= 4) Launch<KK, 4>::run(args...);
    else if (d <= 8) Launch<KK, 8>::run(args...);
    else if (d <= 16) Launch<KK, 16>::run(args...);
    else if (d <= 32) Launch<KK, 32>::run(args...);
    else throw std::invalid_argument("input dimension d > 32 is not supported by the GPU kernels");
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
