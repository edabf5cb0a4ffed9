// diag.cu -- device diagnostics exported through the C ABI: device name and the FP64 FMA throughput probe that
// serves as the roofline denominator of the FP64 kernels (the published HBM and bf16 peaks do not cover the FP64 pipe).
#include <algorithm>
#include <string>

#include "../../include/libkriging_gb300.h"
#include "common.cuh"

namespace {

constexpr int kProbeIters = 4096;

// every thread runs 8 independent FMA chains and writes exactly one element of out (grid * block elements)
__global__ void k_dfma_probe(double* out, double s) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  const double b = s, c = 1.0 - s;
  for (int i = 0; i < kProbeIters; ++i) {
    a0 = fma(a0, b, c);
    a1 = fma(a1, b, c);
    a2 = fma(a2, b, c);
    a3 = fma(a3, b, c);
    a4 = fma(a4, b, c);
    a5 = fma(a5, b, c);
    a6 = fma(a6, b, c);
    a7 = fma(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// FP64 tensor-core (DMMA) throughput: every warp runs 8 independent accumulator chains of
// mma.sync.m8n8k4.f64 (512 flops each); every thread writes exactly one element of out
__global__ void k_dmma_probe(double* out, double s) {
  const double a = 1.0 + threadIdx.x * 1e-6, b = s;
  double c[8][2];
#pragma unroll
  for (int q = 0; q < 8; ++q) c[q][0] = c[q][1] = q * 1e-3;
  for (int i = 0; i < kProbeIters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                   : "+d"(c[q][0]), "+d"(c[q][1])
                   : "d"(a), "d"(b));
  }
  double sum = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) sum += c[q][0] + c[q][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

// best of 4 timed launches (after one untimed) of kernel k over sms * 8 blocks of 256 threads; ms per launch
template <class K>
int time_probe(K k, double* ms_out) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return -1;
  const int blocks = sms * 8, threads = 256;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    k<<<blocks, threads>>>(out, 0.999);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return -1;
  *ms_out = best;
  return blocks * threads;
}

thread_local std::string g_name;

}  // namespace

extern "C" {

const char* lkg_device_name(void) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) return nullptr;
  g_name = prop.name;
  return g_name.c_str();
}

int lkg_probe_fp64_peak(double* tflops_out) {
  double ms = 0.0;
  const int threads = time_probe(k_dfma_probe, &ms);
  if (threads < 0) return -1;
  const double flops = (double)threads * kProbeIters * 8 * 2;
  if (tflops_out) *tflops_out = flops / (ms * 1e-3) / 1e12;
  return 0;
}

int lkg_probe_dmma_peak(double* tflops_out) {
  double ms = 0.0;
  const int threads = time_probe(k_dmma_probe, &ms);
  if (threads < 0) return -1;
  const double flops = (double)(threads / 32) * kProbeIters * 8 * 512.0;  // per warp: 8 m8n8k4 MMAs per iteration
  if (tflops_out) *tflops_out = flops / (ms * 1e-3) / 1e12;
  return 0;
}

}  // extern "C"

// ---- emulated-GEMM check entry point (host buffers) ----
#include "engine.hpp"
#include "ozaki7.cuh"

namespace lkg {
void set_last_error(const char* msg);
}

// the digit products run on one kernel family: tcgen05 on 7-bit digits (tensor path 3)
extern "C" int lkg_set_tensor_path(int tc) {
  if (tc != 3) {
    lkg::set_last_error("lkg_set_tensor_path: the only tensor path is 3 (tcgen05, 7-bit digits)");
    return -1;
  }
  return 3;
}

extern "C" int lkg_get_tensor_path(void) { return 3; }

extern "C" int lkg_set_digit_tile(int tn) {
  try {
    lkg::oz7_set_tile(tn);
  } catch (const std::exception& e) {
    lkg::set_last_error(e.what());
    return -1;
  }
  return tn;
}

extern "C" int lkg_get_digit_tile(void) { return lkg::oz7_tile(); }

extern "C" int lkg_set_lookahead(int ctas) {
  try {
    lkg::set_lookahead_ctas(ctas);
  } catch (const std::exception& e) {
    lkg::set_last_error(e.what());
    return -2;
  }
  return ctas;
}

extern "C" int lkg_get_lookahead(void) { return lkg::lookahead_ctas_setting(); }

extern "C" int lkg_set_graphs(int on) {
  const int old = lkg::graphs_enabled() ? 1 : 0;
  lkg::set_graphs_enabled(on != 0);
  return old;
}

extern "C" int lkg_ozaki_gemm_check(int M, int N, int K, const double* A, const double* B, int slices, double* C) {
  // C = A * B^T with A (M x K) and B (N x K) column-major, computed by the split-bf16 tensor-core path
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  void *pa = nullptr, *pb = nullptr;
  int *ea = nullptr, *eb = nullptr;
  int rc = -1;
  lkg::set_last_error("");
  try {
    LKG_CUDA(cudaMalloc(&dA, sizeof(double) * M * K));
    LKG_CUDA(cudaMalloc(&dB, sizeof(double) * N * K));
    LKG_CUDA(cudaMalloc(&dC, sizeof(double) * M * N));
    LKG_CUDA(cudaMemcpy(dA, A, sizeof(double) * M * K, cudaMemcpyHostToDevice));
    LKG_CUDA(cudaMemcpy(dB, B, sizeof(double) * N * K, cudaMemcpyHostToDevice));
    // 7-bit digits, one more than the slices (5..8), 256-wide k blocks
    const int kb = lkg::OZ7_KB;
    slices = std::min(8, std::max(5, slices + 1));
    LKG_CUDA(cudaMalloc(&pa, lkg::oz7_plane_elems(M, K, slices) * 2));
    LKG_CUDA(cudaMalloc(&pb, lkg::oz7_plane_elems(N, K, slices) * 2));
    LKG_CUDA(cudaMalloc(&ea, lkg::oz7_exp_elems(M, K, kb) * sizeof(int)));
    LKG_CUDA(cudaMalloc(&eb, lkg::oz7_exp_elems(N, K, kb) * sizeof(int)));
    lkg::Split7 sa = lkg::oz7_buffer(pa, ea, slices, M, K, kb), sb = lkg::oz7_buffer(pb, eb, slices, N, K, kb);
    lkg::oz7_split(M, K, dA, 1, M, 0, 1, sa, 0);
    lkg::oz7_split(N, K, dB, 1, N, 0, 1, sb, 0);
    lkg::oz7_gemm(M, N, 0, sa.nblk, 1.0, sa, sb, 0.0, dC, M, 0, 1, false, 0);
    LKG_CUDA(cudaDeviceSynchronize());
    LKG_CUDA(cudaMemcpy(C, dC, sizeof(double) * M * N, cudaMemcpyDeviceToHost));
    rc = lkg::oz7_error_and_reset() ? -1 : 0;
  } catch (const std::exception& e) {
    lkg::set_last_error(e.what());
    rc = -1;
  }
  if (rc != 0 && std::string(lkg_get_last_error()).empty()) lkg::set_last_error("tensor-core digit product timed out");
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(pa);
  cudaFree(pb);
  cudaFree(ea);
  cudaFree(eb);
  return rc;
}
