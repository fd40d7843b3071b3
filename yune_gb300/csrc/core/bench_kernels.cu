// bench_kernels.cu -- L2 read-bandwidth probe used as the roofline denominator of the
// traversal kernels (their node and triangle working set stays resident in L2).
//
// Every CTA streams over a buffer of `bytes` (sized below L2) with 128-bit loads, `iters`
// times; the buffer is warmed once so the timed sweeps hit L2. The sum is written out so
// the loads cannot be removed.
#include <cuda_runtime.h>

#include "yc_internal.h"

namespace yc {

__global__ void k_l2_read(const float4* __restrict__ buf, size_t n, int iters, float* out) {
  float acc = 0.0f;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int it = 0; it < iters; ++it) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      const float4 v = __ldcg(buf + i);
      acc += (v.x + v.y) + (v.z + v.w);
    }
  }
  if (acc == 12345.678f) out[0] = acc;
}

int l2_read_gbs(size_t bytes, int iters, cudaStream_t s, double* gbs) {
  float4* buf = nullptr;
  float* out = nullptr;
  const size_t n = bytes / sizeof(float4);
  if (cudaMalloc(&buf, n * sizeof(float4)) != cudaSuccess) return -1;
  if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) { cudaFree(buf); return -1; }
  cudaMemsetAsync(buf, 0, n * sizeof(float4), s);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = sms * 8, tb = 256;
  k_l2_read<<<grid, tb, 0, s>>>(buf, n, 2, out);   // warm
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  k_l2_read<<<grid, tb, 0, s>>>(buf, n, iters, out);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.0f) return -1;
  *gbs = (double)n * sizeof(float4) * iters / (ms * 1e-3) / 1e9;
  return 0;
}

}  // namespace yc
