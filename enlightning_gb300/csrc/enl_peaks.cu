// Arithmetic ceilings of the GPU the library runs on, measured live.
//
// The FP64 right-hand side is bound by the FP64 pipe, not by HBM: this file
// times long independent chains of FP64 fused multiply-adds, correctly rounded
// FP64 divisions and FP32 fused multiply-adds over every SM, so that a
// benchmark can state its FP64 kernels' fraction of the measured FP64 rate
// beside their fraction of the HBM bandwidth.
#include <cstdio>

#include "enl_common.cuh"

namespace enl {

constexpr int kChains = 8;  // independent dependency chains per thread

template <typename T>
__global__ void fma_chain_kernel(T* out, int iters, T a, T b) {
  T x[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) x[q] = (T)(threadIdx.x + q) * (T)1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = fma(x[q], a, b);
  }
  T s = 0;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void div_chain_kernel(double* out, int iters, double a) {
  double x[kChains];
#pragma unroll
  for (int q = 0; q < kChains; ++q) x[q] = 1.0 + (double)(threadIdx.x + q) * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = a / x[q];  // x alternates between two values: no overflow
  }
  double s = 0;
#pragma unroll
  for (int q = 0; q < kChains; ++q) s += x[q];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Best-of-3 time (ms) of one launch, after one warm-up launch.
template <typename F>
static float time_best(cudaStream_t s, F launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace enl

using namespace enl;

extern "C" {

int enl_measure_fp_peaks(double* out, int n) {
  if (!out || n < 3) {
    set_error(ENL_ERR_ARG);
    return ENL_ERR_ARG;
  }
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  const int threads = 256, blocks = sms * 8;
  const long nthreads = (long)threads * blocks;
  void* buf = nullptr;
  if (cudaMalloc(&buf, nthreads * sizeof(double)) != cudaSuccess) {
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(buf);
    set_error(ENL_ERR_CUDA);
    return ENL_ERR_CUDA;
  }
  double* d = static_cast<double*>(buf);
  float* f = static_cast<float*>(buf);
  const int it64 = 2048, itdiv = 256, it32 = 32768;
  const float t64 = time_best(s, [&] { fma_chain_kernel<double><<<blocks, threads, 0, s>>>(d, it64, 0.9999999, 1e-7); });
  const float tdiv = time_best(s, [&] { div_chain_kernel<<<blocks, threads, 0, s>>>(d, itdiv, 1.0000001); });
  const float t32 = time_best(s, [&] { fma_chain_kernel<float><<<blocks, threads, 0, s>>>(f, it32, 0.9999f, 1e-4f); });
  int rc = check_launch("measure_fp_peaks");
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  cudaFree(buf);
  if (rc != ENL_OK) return rc;
  const double ops = (double)nthreads * kChains;
  out[0] = 2.0 * ops * it64 / (t64 * 1e-3) / 1e12;  // FP64 FMA, TFLOP/s (2 flops per FMA)
  out[1] = ops * itdiv / (tdiv * 1e-3) / 1e9;       // FP64 divisions, G/s
  out[2] = 2.0 * ops * it32 / (t32 * 1e-3) / 1e12;  // FP32 FMA, TFLOP/s
  return ENL_OK;
}

}  // extern "C"
