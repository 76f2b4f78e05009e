// fb_probe.cu -- FP64 FMA throughput probe (the FP64 roofline denominator).
#include "fb_common.cuh"

namespace fb {

// Each thread runs 16 independent DFMA chains, unrolled four iterations
// deep, so neither the chains' latency nor the loop's own instructions hold
// the FP64 pipe back; the result is written only if it is impossible
// (never), so the chains are not removed.
constexpr int PROBE_CHAINS = 16;
__global__ void __launch_bounds__(256) k_probe_dfma(int iters, double seed, double *sink) {
  double a[PROBE_CHAINS];
#pragma unroll
  for (int k = 0; k < PROBE_CHAINS; k++) a[k] = seed + 1e-3 * (threadIdx.x + k);
  const double m = 0.999999, c = 1e-7;
#pragma unroll 4
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; k++) a[k] = fma(a[k], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < PROBE_CHAINS; k++) s += a[k];
  if (s == -1.2345678e300) sink[0] = s;
}

int probe_dfma(cudaStream_t s, double *ms, double *flops) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int blocks = nsm * 8, threads = 256, iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_probe_dfma<<<blocks, threads, 0, s>>>(iters / 8, 1.0, nullptr);
  cudaEventRecord(a, s);
  k_probe_dfma<<<blocks, threads, 0, s>>>(iters, 1.0, nullptr);
  cudaEventRecord(b, s);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.0f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return (int)e;
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  *ms = t;
  *flops = 2.0 * PROBE_CHAINS * (double)iters * (double)blocks * threads;
  return 0;
}

// FP32 FMA throughput probe: 8 independent FFMA chains per thread
__global__ void __launch_bounds__(256) k_probe_ffma(int iters, float seed, float *sink) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = seed + 1e-3f * (threadIdx.x + k);
  const float m = 0.9999f, c = 1e-4f;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fmaf(a[k], m, c);
  }
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  if (s == -1.2345e30f) sink[0] = s;
}

int probe_ffma(cudaStream_t s, double *ms, double *flops) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int blocks = nsm * 8, threads = 256, iters = 65536;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_probe_ffma<<<blocks, threads, 0, s>>>(iters / 8, 1.0f, nullptr);
  cudaEventRecord(a, s);
  k_probe_ffma<<<blocks, threads, 0, s>>>(iters, 1.0f, nullptr);
  cudaEventRecord(b, s);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.0f;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (e != cudaSuccess) return (int)e;
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  *ms = t;
  *flops = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
  return 0;
}

}  // namespace fb
