// probe.cu -- measured arithmetic peaks used as roofline denominators for
// the FP64 kernels (MEASURED_PEAKS-style figures exist only for HBM and
// bf16 GEMM).  Independent FMA chains, 8 per thread, no memory traffic.
#include <cuda_runtime.h>

#include "../../include/qgw_gpu.h"

namespace {
// explicit fused multiply-adds: the library is compiled without implicit
// contraction (-fmad=false), which would otherwise split them in two
__device__ __forceinline__ double fma_t(double x, double a, double b) { return __fma_rn(x, a, b); }
__device__ __forceinline__ float fma_t(float x, float a, float b) { return __fmaf_rn(x, a, b); }

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma_t(x0, a, b); x1 = fma_t(x1, a, b); x2 = fma_t(x2, a, b); x3 = fma_t(x3, a, b);
    x4 = fma_t(x4, a, b); x5 = fma_t(x5, a, b); x6 = fma_t(x6, a, b); x7 = fma_t(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
double rate(int nsm, int iters, T a, T b) {
  T* out = nullptr;
  const int blocks = nsm * 4, threads = 256;
  if (cudaMalloc(&out, sizeof(T) * blocks * threads) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, threads>>>(out, iters, a, b);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  // 8 FMA per iteration per thread, 2 flops each
  return 2.0 * 8.0 * (double)blocks * threads * iters / (best * 1e-3) / 1e12;
}
}  // namespace

extern "C" int qgw_probe_fp_rates(double* fp64_tflops, double* fp32_tflops) {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QGW_ERR_CUDA;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return QGW_ERR_CUDA;
  if (fp64_tflops) *fp64_tflops = rate<double>(nsm, 4000, 1.0000001, 1e-9);
  if (fp32_tflops) *fp32_tflops = rate<float>(nsm, 100000, 1.0000001f, 1e-9f);
  return cudaGetLastError() == cudaSuccess ? QGW_OK : QGW_ERR_CUDA;
}
