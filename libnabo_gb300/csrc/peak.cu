// peak.cu -- FMA throughput of this GPU, the denominator of the brute-force
// roofline (the brute force is bound by the FP32 / FP64 pipes, not by HBM).
//
// Every thread runs 8 independent chains of fused multiply-adds (enough to
// cover the pipe latency) for `iters` steps; a grid of 8 blocks of 256
// threads per SM keeps every scheduler busy. Two flops per FMA.
#include <cuda_runtime.h>

#include "internal.cuh"
#include "nabo_gb300.h"

using namespace nabo_gb300;

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T* sink, int iters, T b, T c) {
  T a[kChains];
#pragma unroll
  for (int j = 0; j < kChains; ++j) a[j] = (T)(threadIdx.x + j) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], b, c);
  }
  T s = a[0];
#pragma unroll
  for (int j = 1; j < kChains; ++j) s += a[j];
  if (s == (T)-1.2345) sink[blockIdx.x] = s;  // never true; keeps the chains alive
}

template <typename T>
int measure(double* flops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_error(e, "device query");
  const int grid = sms * 8, block = 256;
  const int iters = sizeof(T) == 4 ? 16384 : 1024;
  T* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaMalloc((void**)&sink, (size_t)grid * sizeof(T));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.0f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // first run warms up
    cudaEventRecord(e0);
    k_fma_chains<T><<<grid, block>>>(sink, iters, (T)0.999999, (T)1e-6);
    cudaEventRecord(e1);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) return cuda_error(e, "FMA peak kernel");
  *flops = 2.0 * kChains * (double)iters * grid * block / (best * 1e-3);
  return kOk;
}

}  // namespace

extern "C" int nabo_cuda_measure_fma_peak(int dtype, double* flops) {
  if (!flops) return set_error(kErrArgument, "NULL argument");
  if (dtype == NABO_CUDA_FLOAT32) return measure<float>(flops);
  if (dtype == NABO_CUDA_FLOAT64) return measure<double>(flops);
  return set_error(kErrArgument, "unknown scalar type");
}
