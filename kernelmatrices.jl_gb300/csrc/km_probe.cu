// Device FP64 FMA throughput probe (the roofline denominator of FP64-ALU-bound kernels: the
// measured peaks file of the GPU pool carries only HBM copy and bf16 tensor rates).
#include <map>
#include <mutex>
#include <utility>

#include "km_kernels.h"

namespace km {

__global__ void k_dfma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ffma_loop(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace km

extern "C" int km_probe_fp32_tflops(int device, double* out) {
  if (!out) return KM_ERR_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return KM_ERR_CUDA;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return KM_ERR_CUDA;
  const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 100000;
  float* d = nullptr;
  if (cudaMalloc(&d, sizeof(float) * blocks * threads) != cudaSuccess) return KM_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  km::k_ffma_loop<<<blocks, threads>>>(d, 100, 0.999f, 0.001f);
  cudaEventRecord(e0);
  km::k_ffma_loop<<<blocks, threads>>>(d, iters, 0.999f, 0.001f);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || ms <= 0.f) return KM_ERR_CUDA;
  *out = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return KM_OK;
}

extern "C" int km_probe_fp64_tflops(int device, double* out) {
  if (!out) return KM_ERR_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return KM_ERR_CUDA;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return KM_ERR_CUDA;
  const int blocks = p.multiProcessorCount * 4, threads = 256, iters = 4000;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return KM_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  km::k_dfma_loop<<<blocks, threads>>>(d, 100, 0.999, 0.001);
  cudaEventRecord(e0);
  km::k_dfma_loop<<<blocks, threads>>>(d, iters, 0.999, 0.001);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || ms <= 0.f) return KM_ERR_CUDA;
  *out = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return KM_OK;
}

// ---- dynamic shared-memory limits (declared in km_kernels.h) ---------------------------------

namespace km {

void smem_limit(const void* func, size_t bytes) {
  if (bytes <= 48 * 1024) return;  // within the default limit
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, bool> raised;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  bool& done = raised[{func, dev}];
  if (done) return;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, func);
  const int cap = optin - (int)fa.sharedSizeBytes;
  if (cap > 0 && cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, cap) == cudaSuccess)
    done = true;
  else
    cudaGetLastError();  // the launch then reports the size error itself
}

}  // namespace km
