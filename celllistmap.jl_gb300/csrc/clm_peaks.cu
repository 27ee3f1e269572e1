// FP32 / FP64 FMA-pipe throughput probes (libclm_peaks.so).
//
// The pair kernels are bound by the FP32 (or FP64) CUDA-core pipes, not by
// HBM or tensor cores, so their roofline needs a measured FMA peak of the same
// GPU at the same clocks.  Each thread runs independent FMA chains on registers
// (no memory traffic); the result is written once so the work is not removed.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kChains = 8;

template <class T>
__global__ void __launch_bounds__(256) k_fma(T* out, int iters, T a, T b) {
  T v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = fma(v[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == (T)-1.2345) out[blockIdx.x] = s;  // practically never true; keeps the chains alive
}

template <class T> double measure(int iters) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc(&out, sizeof(T) * blocks) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma<T><<<blocks, threads>>>(out, iters / 10, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fma<T><<<blocks, threads>>>(out, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0) return -1.0;
  double flops = 2.0 * kChains * (double)iters * blocks * threads;
  return flops / (ms * 1e-3) / 1e9;
}

}  // namespace

extern "C" {
// GFLOP/s (FMA = 2 flops) of the FP32 and FP64 pipes; negative on error.
double clm_peak_fp32_gflops(int iters) { return measure<float>(iters > 0 ? iters : 1 << 16); }
double clm_peak_fp64_gflops(int iters) { return measure<double>(iters > 0 ? iters : 1 << 12); }
}
