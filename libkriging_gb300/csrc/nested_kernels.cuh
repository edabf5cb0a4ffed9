// nested_kernels.cuh -- device parts of NestedKriging (src/lib/NestedKriging.cpp of libKriging): k-means
// assignment for the partition, and the per-chunk quantities of the NK aggregation.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace lkg {

// a[i] = argmin_c |x_i - C_c|^2 over k centroids (lowest index on ties).  X: N x d column-major, C: k x d row-major.
// The squared distance sums the dimensions in order without fused multiply-adds (the host restatement's rounding).
void kmeans_assign(int N, int d, const double* X, int k, const double* C, int* assign, cudaStream_t st);

// Correlation of each design's points with the chunk points under the common prior (NestedKriging::corrMat:
// plain Cov of x_a - xc_t, no coincidence rule).  Entry e: X_e = X + e * x_estride (n x d column-major, ld n,
// first nvalid[e] rows used), out_e = out + e * o_estride (n x qc column-major, ld n; rows >= nvalid[e] zero).
void nk_corr_entries(int kernel, int n, int d, const double* X, int64_t x_estride, const int* nvalid, int ne,
                     const double* theta, const double* Xc, int qc, double* out, int64_t o_estride, cudaStream_t st);

// Per entry e and chunk point t: M[e*s+t] = beta0 + sum_a U_e(a,t) z_e(a) and K[e*s+t] = sum_a U_e(a,t)^2 (s =
// mk_estride), with U_e = L_e \ C_e (n x qc, ld n) and z_e = L_e \ (y_e - beta0) (n).
void nk_moments(int n, int qc, const double* U, int64_t u_estride, const double* z, int64_t z_estride, double beta0,
                int ne, double* M, double* K, int64_t mk_estride, cudaStream_t st);

// One group of the NK cross step: its points (n x d column-major, ld ldx) and W = R_g^-1 C_g (n x qc, ld ldw).
struct NkGroup {
  const double* X;
  int64_t ldx;
  const double* W;
  int64_t ldw;
  int n;
};

// cross[k * qc + t] = sum_{a,b} W_i(a,t) R_ij(a,b) W_j(b,t) for every pair k = (i < j) of the p groups, pairs
// ranked i-major (k = 0 is (0,1), then (0,2), ...), R_ij recomputed from the points with the common theta (the
// covariance's product form, equal to the reference's to a few ulps).  groups: device array of p NkGroup.  One block
// per (pair, 128 chunk points), each tile of R_ij formed once per block; deterministic.
void nk_cross(int kernel, int d, int p, const NkGroup* groups, const double* theta, int qc, double* cross,
              cudaStream_t st);

}  // namespace lkg
