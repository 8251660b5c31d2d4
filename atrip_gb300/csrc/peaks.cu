// Short on-device timing loops that give the FP64 throughput (the larger of a
// DFMA loop and a DMMA m8n8k4 loop) and the FP32 (FFMA) throughput, used as
// roofline denominators for the FP64 form.
#include <cuda_runtime.h>

#include "atrip_gb300.h"
#include "engine.cuh"

namespace {

constexpr int kChains = 16;

// Independent FMA chains with all operands in registers.
template <typename T>
__global__ void fma_chains(T *out, int iters, T s) {
  T acc[kChains];
  const T add = (T)(1e-9 * (threadIdx.x + 1));
  const T mul = s + (T)(threadIdx.x * 1e-12);
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = (T)(threadIdx.x * 1e-3 + c);
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma(acc[c], mul, add);
  T r = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) r += acc[c];
  if (r == (T)12345.678) out[0] = r;  // keeps the chains live
}

constexpr int kMmaChains = 16;  // as many independent chains as the DFMA loop

__global__ void dmma_chains(double *out, int iters) {
  const double a = threadIdx.x * 1e-3, b = 0.999;
  double d[kMmaChains][2];
#pragma unroll
  for (int c = 0; c < kMmaChains; ++c) {
    d[c][0] = c;
    d[c][1] = c + 1;
  }
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int c = 0; c < kMmaChains; ++c)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(d[c][0]), "+d"(d[c][1])
                   : "d"(a), "d"(b));
  double r = 0;
#pragma unroll
  for (int c = 0; c < kMmaChains; ++c) r += d[c][0] + d[c][1];
  if (r == 12345.678) out[0] = r;
}

double time_dmma(int sms, int iters) {
  double *d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 4, threads = 256;
  dmma_chains<<<blocks, threads>>>(d, 16);
  cudaDeviceSynchronize();
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dmma_chains<<<blocks, threads>>>(d, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  const double flops = 2.0 * 256 * kMmaChains * (double)iters * blocks * (threads / 32);
  return flops / (best * 1e-3) / 1e12;
}

template <typename T>
double time_fma(int sms, int iters) {
  T *d = nullptr;
  if (cudaMalloc(&d, 64) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 4, threads = 256;
  fma_chains<T><<<blocks, threads>>>(d, 16, (T)1.0000001);
  cudaDeviceSynchronize();
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fma_chains<T><<<blocks, threads>>>(d, iters, (T)1.0000001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  const double flops = 2.0 * kChains * (double)iters * blocks * threads;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace

extern "C" int atrip_gpu_measure_peaks(int32_t device, double *fp64_tflops, double *fp32_tflops) {
  atrip_gb300::clear_error();
  if (!fp64_tflops || !fp32_tflops) {
    atrip_gb300::set_error("null argument");
    return ATRIP_ERR_ARGUMENT;
  }
  ATRIP_CUDA_TRY(cudaSetDevice(device));
  int sms = 0;
  ATRIP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const double dfma = time_fma<double>(sms, 2048), dmma = time_dmma(sms, 512);
  *fp64_tflops = dfma > dmma ? dfma : dmma;
  *fp32_tflops = time_fma<float>(sms, 8192);
  ATRIP_CUDA_TRY(cudaGetLastError());
  return ATRIP_OK;
}
