// FMA-throughput microbenchmark: the FP64 / FP32 pipe peaks of this GPU, the
// roofline denominators of the batched step (the step is not a dense
// contraction, so neither the HBM copy rate nor the tensor-core rate bounds
// it).  Each thread runs 8 independent dependency chains of fused multiply-adds
// in registers; nothing is read or written but one result per thread.

#include <cuda_runtime.h>

#include "gpb.h"

namespace {

template <typename T>
__global__ void fma_chains(T* out, int iters, T a, T b, int active_lanes) {
  T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  if ((int)(threadIdx.x & 31) < active_lanes) {
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int u = 0; u < 16; ++u) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
      }
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// FP32 -> FP64 conversions, each result consumed by an integer xor (so no
// round trip can be folded away), 8 independent chains per thread.
__global__ void cvt_chains(long long* out, int iters) {
  float f[8];
  long long acc = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) f[j] = threadIdx.x * 1e-3f + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      f[j] = f[j] * 1.0001f + 1e-3f;
      acc ^= __double_as_longlong((double)f[j]);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace

// FP32 -> FP64 conversion throughput in G conversions/s (all lanes active).
extern "C" int gpb_cvt_peak(int device, double* gops) {
  if (!gops) return GPB_E_INVAL;
  if (cudaSetDevice(device) != cudaSuccess) return GPB_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int threads = 256, blocks = sms * 8, iters = 256;
  void* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * 8) != cudaSuccess) return GPB_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    cvt_chains<<<blocks, threads>>>((long long*)out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GPB_E_CUDA;
  *gops = 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
  return GPB_OK;
}

// TFLOP/s (2 per FMA, counted for active lanes only) of `precision`
// (GPB_FP64 / GPB_MIXED = FP32) with `active_lanes` of every warp issuing.
extern "C" int gpb_fma_peak(int device, int precision, int active_lanes, double* tflops) {
  if (!tflops || active_lanes < 1 || active_lanes > 32) return GPB_E_INVAL;
  if (cudaSetDevice(device) != cudaSuccess) return GPB_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int threads = 256, blocks = sms * 8;
  const int iters = precision == GPB_FP64 ? 64 : 2048;
  void* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * 8) != cudaSuccess) return GPB_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    if (precision == GPB_FP64)
      fma_chains<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7, active_lanes);
    else
      fma_chains<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f, active_lanes);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GPB_E_CUDA;
  double flops = 2.0 * 8 * 16 * (double)iters * blocks * (threads / 32) * active_lanes;
  *tflops = flops / (best * 1e-3) / 1e12;
  return GPB_OK;
}
