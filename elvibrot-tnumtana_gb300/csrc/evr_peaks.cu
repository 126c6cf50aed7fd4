// evr_peaks.cu -- FMA issue-rate micro-benchmark: the compute denominator of the roofline
// for the CUDA-core FP64 / FP32 contractions (no figure for these pipes is published for
// this part, and a cuBLAS GEMM may run on a different pipe).
#include <cuda_runtime.h>

#include "evr_internal.h"

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * T(1e-7), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-1234.5)) out[blockIdx.x] = s;  // keeps the chains alive
}

template <typename T>
int measure(int device, double* tflops) {
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess) return EVR_EDEVICE;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return EVR_EDEVICE;
  T* out = nullptr;
  const int blocks = sms * 8, threads = 256, iters = sizeof(T) == 8 ? 256 : 4096;
  if (cudaMalloc(&out, blocks * sizeof(T)) != cudaSuccess) return EVR_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, threads>>>(out, iters / 8, T(0.999999), T(1e-9));  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-9));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return EVR_EDEVICE;
  const double flop = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flop / (best * 1e-3) / 1e12;
  return EVR_OK;
}

}  // namespace

extern "C" int evr_fma_peak(int device, int prec, double* tflops) {
  if (!tflops) return EVR_EINVAL;
  return prec == EVR_PREC_FP32 ? measure<float>(device, tflops) : measure<double>(device, tflops);
}
