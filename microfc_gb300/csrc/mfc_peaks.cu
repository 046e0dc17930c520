// Measured arithmetic peaks of the device, the denominators of the compute
// roofline of the stage kernels (which are bound by the FP64 pipe on GB300).
//
// Each thread runs K independent fused multiply-add chains (no memory
// traffic in the loop); the grid fills every SM many times over.  Flops are
// counted as 2 per FMA.  Timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mfc_gpu.h"

namespace {

constexpr int kChains = 8;

template <class T>
__global__ void fma_chains(T* __restrict__ out, int iters, T a, T b) {
  T acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) acc[k] = T(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) acc[k] = fma(acc[k], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += acc[k];
  if (s == T(-1.2345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

template <class T>
double time_fma(int sms, int iters, cudaError_t* err) {
  const int threads = 256, blocks = sms * 16;
  T* out = nullptr;
  cudaEvent_t e0, e1;
  *err = cudaMalloc(&out, sizeof(T) * threads * blocks);
  if (*err != cudaSuccess) return 0.0;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, threads>>>(out, iters / 8, T(0.999999), T(1e-7));
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(e1);
  *err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (*err == cudaSuccess) *err = cudaGetLastError();
  const double flops = 2.0 * kChains * double(iters) * threads * blocks;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int mfc_gpu_measure_peaks(int device, double* fp64_tflops, double* fp32_tflops) {
  if (!fp64_tflops || !fp32_tflops) return MFC_ERR_INVALID;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return MFC_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  *fp64_tflops = time_fma<double>(sms, 1 << 12, &e);
  if (e != cudaSuccess) return MFC_ERR_CUDA;
  *fp32_tflops = time_fma<float>(sms, 1 << 16, &e);
  if (e != cudaSuccess) return MFC_ERR_CUDA;
  return MFC_OK;
}
