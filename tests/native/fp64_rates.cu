// Issue-rate probe for the arithmetic the hot path is built from: FP64 FMA,
// FP32 FMA, FP64 reciprocal, square root and rsqrt, float<->double
// conversions (hardware and the integer-pipe f2d_bits/d2f_bits), FP64
// atomics to an HBM-resident array, and a device-to-device copy.  Each rate
// is reported per second and in FP64-FMA equivalents, the unit the kernels'
// cost model counts in.  Prints one JSON object.  Not part of the library;
// built and run by `python bench.py --mode rates` and by
// tests/test_gpu_rates.py, which checks the FP64 FMA rate the roofline uses.
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
// Widening and accumulating FP32 values into FP64, as the mixed-precision
// node sums do: op 0 = acc += 1.0 (the FP64 add alone), 1 = acc += (double)x
// (hardware cvt), 2 = acc += f2d_bits(x) (integer pipe).  The FP32 chain that
// makes x runs on the FP32 pipe in all three.
template <int OP>
__global__ void k_widen(double* out, int iters) {
  float x[8];
  double acc[8];
  for (int k = 0; k < 8; k++) { x[k] = 1.0f + 1e-3f * (threadIdx.x + k); acc[k] = 0.0; }
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) {
      x[k] = fmaf(x[k], 1.0001f, 1e-3f);
      if (OP == 0) acc[k] += 1.0;
      if (OP == 1) acc[k] += (double)x[k];
      if (OP == 2) acc[k] += mgcfd::f2d_bits(x[k]);
    }
  double s = 0;
  for (int k = 0; k < 8; k++) s += acc[k] + x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Widening forms for the node-sum probe (finite normal inputs only).
__device__ __forceinline__ double widen_hilo(float f) {  // __hiloint2double packing
  const uint32_t u = __float_as_uint(f), a = u & 0x7fffffffu;
  return __hiloint2double((int)((u & 0x80000000u) | ((a >> 3) + (896u << 20))), (int)(u << 29));
}
__device__ __forceinline__ double widen_i64(float f) {  // one 64-bit integer expression
  const unsigned long long u = __float_as_uint(f);
  const unsigned long long b = ((u & 0x80000000ull) << 32) | (((u & 0x7fffffffull) << 29) + (896ull << 52));
  return __longlong_as_double((long long)b);
}
__device__ __forceinline__ double widen_asm(float f) {  // asm packing, no special cases
  const uint32_t u = __float_as_uint(f), a = u & 0x7fffffffu;
  return mgcfd::pack_words((u & 0x80000000u) | ((a >> 3) + (896u << 20)), u << 29);
}

// The node-sum pattern of the mixed-precision update: each thread widens 30
// FP32 values read from memory (6 edges x 5 variables) and adds them into 5
// FP64 sums.  op 0 = hardware cvt, 1 = f2d_bits, 2 = FP32 sums widened once,
// 3..5 = other packings of the widened bits, 6 = the same sums of doubles read
// from memory (no widening at all).  The arrays (256 K threads x 30 values)
// stay in L2, so the arithmetic shows.
template <int OP>
__global__ void k_node_sums(int n, const float* __restrict__ fe, const double* __restrict__ fd,
                            double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double F[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  float G[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  const float* p = fe + 30 * (int64_t)i;
  const double* q = fd + 30 * (int64_t)i;
  for (int e = 0; e < 6; e++)
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const float x = OP == 6 ? 0.f : p[5 * e + k];
      if (OP == 6) F[k] += q[5 * e + k];
      if (OP == 0) F[k] += (double)x;
      if (OP == 1) F[k] += mgcfd::f2d_bits(x);
      if (OP == 2) G[k] += x;
      if (OP == 3) F[k] += widen_hilo(x);
      if (OP == 4) F[k] += widen_i64(x);
      if (OP == 5) F[k] += widen_asm(x);
    }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 5; k++) s += OP == 2 ? mgcfd::f2d_bits(G[k]) : F[k];
  out[i] = s;
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
  const float t_w0 = timed([&] { k_widen<0><<<kBlocks, kThreads>>>(od, iu); });
  const float t_w1 = timed([&] { k_widen<1><<<kBlocks, kThreads>>>(od, iu); });
  const float t_w2 = timed([&] { k_widen<2><<<kBlocks, kThreads>>>(od, iu); });
  const int nsum = 256 * 1024;
  float* fe;
  CK(cudaMalloc(&fe, sizeof(float) * 30 * (size_t)nsum));
  CK(cudaMemset(fe, 0x3f, sizeof(float) * 30 * (size_t)nsum));  // every float 0x3f3f3f3f = 0.747: normal
  double* fd;
  CK(cudaMalloc(&fd, sizeof(double) * 30 * (size_t)nsum));
  CK(cudaMemset(fd, 0x3f, sizeof(double) * 30 * (size_t)nsum));  // 0x3f3f...3f: a normal double
  auto sums = [&](auto kernel) {
    return timed([&] {
      for (int r = 0; r < 20; r++) kernel<<<(nsum + 255) / 256, 256>>>(nsum, fe, fd, od);
    });
  };
  const float t_s0 = sums(k_node_sums<0>), t_s1 = sums(k_node_sums<1>), t_s2 = sums(k_node_sums<2>);
  const float t_s3 = sums(k_node_sums<3>), t_s4 = sums(k_node_sums<4>), t_s5 = sums(k_node_sums<5>);
  const float t_s6 = sums(k_node_sums<6>);
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
         "\"intpipe_d2f2d_dfma_eq\": %.2f, \"widen_add_dfma_eq\": {\"add_only\": %.2f, \"hw_cvt\": %.2f, "
         "\"f2d_bits\": %.2f}, \"node_sums_us\": {\"hw_cvt\": %.1f, \"f2d_bits\": %.1f, \"fp32_then_once\": %.1f, \"hilo\": %.1f, "
         "\"i64\": %.1f, \"asm_normal_only\": %.1f, \"doubles_from_memory\": %.1f}, "
         "\"red_f64_hbm_g_per_s\": %.1f, \"d2d_copy_gb_per_s\": %.1f}\n",
         p.name, p.multiProcessorCount, dfma_per_s / 1e9, 2 * dfma_per_s / 1e12,
         2 * 8.0 * ops / (t_ffma * 1e-3) / 1e12, uops / (t_rcp * 1e-3) / 1e9, eq(t_rcp, uops),
         uops / (t_sqrt * 1e-3) / 1e9, eq(t_sqrt, uops), uops / (t_rsqrt * 1e-3) / 1e9, eq(t_rsqrt, uops),
         eq(t_cvt, uops), eq(t_cvti, uops), eq(t_w0, uops), eq(t_w1, uops), eq(t_w2, uops),
         1e3 * t_s0 / 20, 1e3 * t_s1 / 20, 1e3 * t_s2 / 20, 1e3 * t_s3 / 20, 1e3 * t_s4 / 20, 1e3 * t_s5 / 20,
         1e3 * t_s6 / 20,
         (double)per * kN / (t_red * 1e-3) / 1e9,
         2.0 * big * 8 / (t_copy * 1e-3) / 1e9);
  cudaFree(od); cudaFree(of); cudaFree(arr); cudaFree(src); cudaFree(dst); cudaFree(fe); cudaFree(fd);
  return 0;
}
