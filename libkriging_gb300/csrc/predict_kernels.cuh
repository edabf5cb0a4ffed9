// predict_kernels.cuh -- GPU part of Kriging::predict (KrigingImpl::predict_impl, src/lib/KrigingImpl.cpp:145-300).
#pragma once
#include <vector>

#include "engine.hpp"

namespace lkg {

struct PredictOut {
  std::vector<double> rz;     // q:     Rstar_on' z
  std::vector<double> rr;     // q:     colsum(Rstar_on % Rstar_on)
  std::vector<double> rm;     // q x p (row-major per point): Rstar_on' M
  std::vector<double> sigma;  // q x q column-major: R_nn - Rstar_on' Rstar_on (when need_cov)
  // derivatives (when need_deriv), W = L \ DR_on with column c d + k for point c and input dimension k:
  std::vector<double> wz;     // q d: W(:, c d + k)' z
  std::vector<double> wr;     // q d: W(:, c d + k)' Rstar_on(:, c)
  std::vector<double> wm;     // q d x p (row-major per column): W(:, c d + k)' M
};

// Xn: q x d column-major, already normalised.  R_on = factor * C(X_o - X_n) (coincident points -> 1),
// Rstar_on = L \ R_on with the committed factor of `model`.  digits: Rstar_on as the product L^-1 R_on on the
// tensor cores (8 seven-bit digits, FP64-level products; L^-1 formed once per factor) instead of the FP64
// triangular solve -- used for the mean and stdev of large predictions on a mixed-precision model.
PredictOut predict_gpu(Engine& model, const double* Xn, int q, const double* theta, double factor, const double* z,
                       bool need_rr, bool need_cov, double nn_factor, bool need_deriv = false, bool digits = false);

}  // namespace lkg
