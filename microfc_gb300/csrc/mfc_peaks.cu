// Measured arithmetic peaks of the device, the denominators of the compute
// roofline of the stage kernels (which are bound by the FP64 pipe on GB300).
//
// Each thread runs K independent fused multiply-add chains (no memory
// traffic in the loop); the grid fills every SM many times over.  Flops are
// counted as 2 per FMA.  Timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mfc_gpu.h"
#include "mfc_device.cuh"

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

// div_rn (the plain path's shared-divisor division) beside the IEEE
// division, element by element.
__global__ void div_check_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                 double* __restrict__ q_fast, double* __restrict__ q_ieee, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    q_fast[i] = mfc::div_rn(a[i], mfc::divisor(b[i]));
    q_ieee[i] = mfc::div_ieee(a[i], b[i]);
  }
}

}  // namespace

extern "C" int mfc_gpu_selftest_div(const double* a, const double* b, double* q_fast, double* q_ieee, long long n,
                                    void* stream) {
  if (n < 0 || (n > 0 && (!a || !b || !q_fast || !q_ieee))) return MFC_ERR_INVALID;
  if (n == 0) return MFC_OK;
  const long long blocks = (n + 255) / 256 < 152 * 64 ? (n + 255) / 256 : 152 * 64;
  div_check_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(a, b, q_fast, q_ieee, n);
  return cudaGetLastError() == cudaSuccess ? MFC_OK : MFC_ERR_CUDA;
}

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
