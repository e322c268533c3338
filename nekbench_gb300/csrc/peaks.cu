// Microbenchmarks of the device roofs the kernels are measured against:
// FMA throughput (FP64 or FP32, CUDA cores) and device-to-device copy bandwidth.
#include "internal.h"

namespace nekb {
namespace {

template <typename T>
__global__ void k_fma(T* out, int iters, T a, T b)
{
  // 8 independent chains per thread keep the FMA pipe busy
  T v0 = threadIdx.x, v1 = v0 + 1, v2 = v0 + 2, v3 = v0 + 3, v4 = v0 + 4, v5 = v0 + 5, v6 = v0 + 6,
    v7 = v0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      v0 = v0 * a + b; v1 = v1 * a + b; v2 = v2 * a + b; v3 = v3 * a + b;
      v4 = v4 * a + b; v5 = v5 * a + b; v6 = v6 * a + b; v7 = v7 * a + b;
    }
  }
  const T s = v0 + v1 + v2 + v3 + v4 + v5 + v6 + v7;
  if (s == T(12345.678)) out[blockIdx.x] = s;  // keep the chains alive
}

__global__ void k_copy(const float4* __restrict__ a, float4* __restrict__ b, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

}  // namespace

int peak_fma(int fp64, double* tflops)
{
  int dev = 0, sms = 0;
  NEKB_CUDA(cudaGetDevice(&dev));
  NEKB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  const int iters = fp64 ? 64 : 2048;
  void* out = nullptr;
  NEKB_CUDA(cudaMalloc(&out, sizeof(double) * blocks));
  cudaEvent_t e0, e1;
  NEKB_CUDA(cudaEventCreate(&e0));
  NEKB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (fp64)
      k_fma<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
    else
      k_fma<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    NEKB_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  NEKB_CUDA(cudaGetLastError());
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return NEKB_OK;
}

int peak_copy(double* gbs)
{
  const int64_t bytes = (int64_t)1 << 30;
  void *a = nullptr, *b = nullptr;
  NEKB_CUDA(cudaMalloc(&a, bytes));
  if (cudaMalloc(&b, bytes) != cudaSuccess) {
    cudaFree(a);
    return fail(NEKB_ERR_ALLOC, "peak copy: allocation failed");
  }
  cudaMemset(a, 0, bytes);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 6; ++rep) {
    cudaEventRecord(e0);
    k_copy<<<sms * 8, 256>>>((const float4*)a, (float4*)b, bytes / 16);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(b);
  NEKB_CUDA(cudaGetLastError());
  *gbs = 2.0 * bytes / (best * 1e-3) / 1e9;
  return NEKB_OK;
}

}  // namespace nekb
