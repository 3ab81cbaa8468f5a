// Test harness (not part of the library): runs the integer-pipe format
// conversions of device_math.cuh and the hardware conversions side by side.
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_math.cuh"

namespace {

__global__ void k_conv(int64_t nd, const double* __restrict__ d, float* __restrict__ d2f_hw,
                       float* __restrict__ d2f_int, int64_t nf, const float* __restrict__ f,
                       double* __restrict__ f2d_hw, double* __restrict__ f2d_int) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nd) {
    d2f_hw[i] = __double2float_rn(d[i]);
    d2f_int[i] = mgcfd::d2f_bits(d[i]);
  }
  if (i < nf) {
    f2d_hw[i] = (double)f[i];
    f2d_int[i] = mgcfd::f2d_bits(f[i]);
  }
}

}  // namespace

// Host buffers in, host buffers out; returns a cudaError_t value.
extern "C" int conv_check(int64_t nd, const double* d, float* d2f_hw, float* d2f_int, int64_t nf, const float* f,
                          double* f2d_hw, double* f2d_int) {
  double *dd = nullptr, *o3 = nullptr, *o4 = nullptr;
  float *ff = nullptr, *o1 = nullptr, *o2 = nullptr;
  cudaError_t e = cudaSuccess;
  const int64_t n = nd > nf ? nd : nf;
  if ((e = cudaMalloc(&dd, 8 * (nd + 1))) || (e = cudaMalloc(&o1, 4 * (nd + 1))) || (e = cudaMalloc(&o2, 4 * (nd + 1))) ||
      (e = cudaMalloc(&ff, 4 * (nf + 1))) || (e = cudaMalloc(&o3, 8 * (nf + 1))) || (e = cudaMalloc(&o4, 8 * (nf + 1))))
    goto done;
  if ((e = cudaMemcpy(dd, d, 8 * nd, cudaMemcpyHostToDevice)) || (e = cudaMemcpy(ff, f, 4 * nf, cudaMemcpyHostToDevice)))
    goto done;
  k_conv<<<(unsigned)((n + 255) / 256), 256>>>(nd, dd, o1, o2, nf, ff, o3, o4);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) goto done;
  if ((e = cudaMemcpy(d2f_hw, o1, 4 * nd, cudaMemcpyDeviceToHost)) || (e = cudaMemcpy(d2f_int, o2, 4 * nd, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(f2d_hw, o3, 8 * nf, cudaMemcpyDeviceToHost)) || (e = cudaMemcpy(f2d_int, o4, 8 * nf, cudaMemcpyDeviceToHost)))
    goto done;
done:
  cudaFree(dd); cudaFree(o1); cudaFree(o2); cudaFree(ff); cudaFree(o3); cudaFree(o4);
  return (int)e;
}
