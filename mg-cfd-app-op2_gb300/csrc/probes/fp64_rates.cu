// Issue-rate probe for the arithmetic the hot path is built from: FP64 FMA,
// FP32 FMA, FP64 reciprocal, square root and rsqrt, float<->double
// conversions (hardware and the integer-pipe f2d_bits/d2f_bits), FP64
// atomics to an HBM-resident array, and a device-to-device copy.  Each rate
// is reported per second and in FP64-FMA equivalents, the unit the kernels'
// cost model counts in.  Prints one JSON object.  Not part of the library;
// built and run by `python bench.py --mode rates`.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "device_math.cuh"

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) {                                                           \
      fprintf(stderr, "CUDA error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
      return 1;                                                                        \
    }                                                                                  \
  } while (0)

namespace {

constexpr int kBlocks = 152 * 8, kThreads = 256, kN = kBlocks * kThreads;

// Eight independent chains per thread keep the pipe full; each chain does
// `iters` operations.
__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x[8];
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  double s = 0;
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_ffma(float* out, int iters, float a, float b) {
  float x[8];
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, b);
  float s = 0;
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
// op: 0 = 1/x, 1 = sqrt, 2 = rsqrt, 3 = hardware d->f->d, 4 = integer-pipe d->f->d
template <int OP>
__global__ void k_unary(double* out, int iters) {
  double x[8];
  for (int k = 0; k < 8; k++) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (OP == 0) x[k] = 1.0 / x[k] + 0.5;
      if (OP == 1) x[k] = sqrt(x[k]) + 0.5;
      if (OP == 2) x[k] = rsqrt(x[k]) + 0.5;
      if (OP == 3) x[k] = (double)(float)x[k] + 0.5;
      if (OP == 4) x[k] = mgcfd::f2d_bits(mgcfd::d2f_bits(x[k])) + 0.5;
    }
  double s = 0;
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_red(double* arr, uint32_t n, int per_thread) {
  uint32_t h = (blockIdx.x * blockDim.x + threadIdx.x) * 2654435761u;
  for (int i = 0; i < per_thread; i++) {
    h = h * 1664525u + 1013904223u;
    atomicAdd(&arr[h % n], 1.0);
  }
}

template <class F>
float timed(F launch) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch();  // warm-up
  cudaEventRecord(a);
  launch();
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

}  // namespace

int main() {
  double* od;
  float* of;
  CK(cudaMalloc(&od, sizeof(double) * kN));
  CK(cudaMalloc(&of, sizeof(float) * kN));
  const int it = 2000;
  const double ops = 8.0 * it * kN;
  const float t_dfma = timed([&] { k_dfma<<<kBlocks, kThreads>>>(od, it, 0.999, 0.001); });
  const float t_ffma = timed([&] { k_ffma<<<kBlocks, kThreads>>>(of, 8 * it, 0.999f, 0.001f); });
  const int iu = it / 4;
  const double uops = 8.0 * iu * kN;
  const float t_rcp = timed([&] { k_unary<0><<<kBlocks, kThreads>>>(od, iu); });
  const float t_sqrt = timed([&] { k_unary<1><<<kBlocks, kThreads>>>(od, iu); });
  const float t_rsqrt = timed([&] { k_unary<2><<<kBlocks, kThreads>>>(od, iu); });
  const float t_cvt = timed([&] { k_unary<3><<<kBlocks, kThreads>>>(od, iu); });
  const float t_cvti = timed([&] { k_unary<4><<<kBlocks, kThreads>>>(od, iu); });
  CK(cudaGetLastError());
  const uint32_t an = 64u << 20;  // 512 MB of doubles: atomics go to HBM
  double* arr;
  CK(cudaMalloc(&arr, sizeof(double) * an));
  CK(cudaMemset(arr, 0, sizeof(double) * an));
  const int per = 64;
  const float t_red = timed([&] { k_red<<<kBlocks, kThreads>>>(arr, an, per); });
  const size_t big = (size_t)1 << 28;
  double *src, *dst;
  CK(cudaMalloc(&src, big * 8));
  CK(cudaMalloc(&dst, big * 8));
  CK(cudaMemset(src, 0, big * 8));
  const float t_copy = timed([&] { cudaMemcpyAsync(dst, src, big * 8, cudaMemcpyDeviceToDevice); });
  CK(cudaDeviceSynchronize());
  const double dfma_per_s = ops / (t_dfma * 1e-3);
  auto eq = [&](float t, double n) { return (t * 1e-3) * dfma_per_s / n; };  // DFMA-equivalents per op
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, 0));
  printf("{\"device\": \"%s\", \"sms\": %d, \"dfma_g_per_s\": %.1f, \"fp64_tflops\": %.3f, \"fp32_tflops\": %.2f, "
         "\"rcp_g_per_s\": %.1f, \"rcp_dfma_eq\": %.2f, \"sqrt_g_per_s\": %.1f, \"sqrt_dfma_eq\": %.2f, "
         "\"rsqrt_g_per_s\": %.1f, \"rsqrt_dfma_eq\": %.2f, \"cvt_d2f2d_dfma_eq\": %.2f, "
         "\"intpipe_d2f2d_dfma_eq\": %.2f, \"red_f64_hbm_g_per_s\": %.1f, \"d2d_copy_gb_per_s\": %.1f}\n",
         p.name, p.multiProcessorCount, dfma_per_s / 1e9, 2 * dfma_per_s / 1e12,
         2 * 8.0 * ops / (t_ffma * 1e-3) / 1e12, uops / (t_rcp * 1e-3) / 1e9, eq(t_rcp, uops),
         uops / (t_sqrt * 1e-3) / 1e9, eq(t_sqrt, uops), uops / (t_rsqrt * 1e-3) / 1e9, eq(t_rsqrt, uops),
         eq(t_cvt, uops), eq(t_cvti, uops), (double)per * kN / (t_red * 1e-3) / 1e9,
         2.0 * big * 8 / (t_copy * 1e-3) / 1e9);
  cudaFree(od); cudaFree(of); cudaFree(arr); cudaFree(src); cudaFree(dst);
  return 0;
}
