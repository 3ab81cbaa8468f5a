// Multigrid restriction (mg.h:29-64, euler3d.cpp:581-592) for callers that
// cannot allocate device memory.
//
// The reference's restriction needs a per-coarse-node child count
// (p_up_scratch, euler3d.cpp:405).  mgcfd_op_up_pre/up/up_post take that
// buffer from the caller.  Some callers cannot provide it: a host framework
// that owns every byte of device memory through its own allocator (OP2 keeps
// all dats in its own pool), or code that must not call cudaMalloc between
// time steps.  mgcfd_op_restrict_noalloc keeps the counts in a fixed
// file-scope device array instead, so the call allocates nothing.
//
//   * Capacity: kMaxCoarse = 1,048,576 coarse nodes (4 MiB of int32).  Every
//     GPU that loads this library holds the array until the process exits.
//     Larger coarse levels are rejected with MGCFD_ERR_INVALID.
//   * All calls share the one array, and it keeps the last call's counts, so
//     each call first clears the entries it uses.  Calls whose work overlaps
//     on the GPU (different streams, or the same stream from several host
//     threads without ordering) race on the counts and give wrong results.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and remembers it.
//     Make that first call before any stream capture begins.  Later calls
//     made while their stream is not capturing look the address up again
//     and replace the remembered one if it moved -- it does after a
//     cudaDeviceReset, or in another context on the same device, where the
//     library's module is loaded anew -- so a stale address is never passed
//     to a kernel.  Calls made while capturing use the remembered address.
//   * A fine node whose map entry is outside [0, ncoarse) is skipped and
//     counted; mgcfd_op_map_errors reports these skips together with those
//     of the other mapped entry points.
#include <mutex>

#include "common.h"

namespace {

constexpr int32_t kMaxCoarse = 1 << 20;
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

static __device__ __align__(256) int32_t g_restrict_counts[kMaxCoarse];

// Fine nodes skipped because their map entry was out of range.
__device__ unsigned long long g_restrict_map_errors;

std::mutex g_mu;
int32_t* g_counts_ptr[kMaxDevices] = {nullptr};

// Host-side name g_restrict_counts is only a stand-in: kernels get the
// device address found here.  The lookup runs on the first call on each
// device and again on every call whose stream is not capturing (a CUDA
// graph capture must not load modules, and reuses the remembered address).
int counts_address(cudaStream_t stream, int32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return mgcfd::set_error(MGCFD_ERR_INVALID, "device ordinal out of range");
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess)
    return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("cudaStreamIsCapturing: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(g_mu);
  if (cap == cudaStreamCaptureStatusNone || !g_counts_ptr[dev]) {
    if (cap != cudaStreamCaptureStatusNone)
      return mgcfd::set_error(MGCFD_ERR_INVALID,
                              "mgcfd_op_restrict_noalloc: the first call on a device must not be inside a stream capture");
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_restrict_counts);
    if (e != cudaSuccess)
      return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_counts_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_counts_ptr[dev];
  return MGCFD_OK;
}

int grid(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

#define GRID_STRIDE(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_clear_counts(int32_t nc, int32_t* __restrict__ cnt) {
  GRID_STRIDE(i, nc) cnt[i] = 0;
}

// up_pre_kernel (mg.h:29-39): coarse nodes with children start from zero.
__global__ void k_zero_mapped(int32_t nf, int32_t nc, const int32_t* __restrict__ map, double* __restrict__ cv) {
  GRID_STRIDE(i, nf) {
    const int32_t c = map[i];
    if ((uint32_t)c >= (uint32_t)nc) continue;
#pragma unroll
    for (int k = 0; k < 5; k++) cv[5 * (int64_t)c + k] = 0.0;
  }
}

// up_kernel (mg.h:41-52).  The skipped entries are counted here only
// (k_zero_mapped skips the same ones).
__global__ void k_accumulate(int32_t nf, int32_t nc, const int32_t* __restrict__ map, const double* __restrict__ fv,
                             double* __restrict__ cv, int32_t* __restrict__ cnt) {
  GRID_STRIDE(i, nf) {
    const int32_t c = map[i];
    if ((uint32_t)c >= (uint32_t)nc) {
      atomicAdd(&g_restrict_map_errors, 1ull);
      continue;
    }
#pragma unroll
    for (int k = 0; k < 5; k++) atomicAdd(cv + 5 * (int64_t)c + k, fv[5 * i + k]);
    atomicAdd(cnt + c, 1);
  }
}

// up_post_kernel (mg.h:54-64).
__global__ void k_average(int32_t nc, double* __restrict__ cv, const int32_t* __restrict__ cnt) {
  GRID_STRIDE(i, nc) {
    const int32_t s = cnt[i];
    const double avg = s == 0 ? 1.0 : 1.0 / (double)s;
#pragma unroll
    for (int k = 0; k < 5; k++) cv[5 * i + k] *= avg;
  }
}

}  // namespace

extern "C" int mgcfd_op_restrict_noalloc(int32_t nfine, int32_t ncoarse, const int32_t* node_to_mg,
                                         const double* fine_variables, double* coarse_variables, void* stream) {
  if (nfine < 0 || ncoarse < 0) return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_op_restrict_noalloc: negative size");
  if (ncoarse > kMaxCoarse)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_op_restrict_noalloc: " + std::to_string(ncoarse) +
                                                   " coarse nodes exceed the fixed capacity of " +
                                                   std::to_string(kMaxCoarse));
  if ((nfine > 0 && (!node_to_mg || !fine_variables)) || (ncoarse > 0 && !coarse_variables))
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_op_restrict_noalloc: null pointer");
  if (ncoarse == 0) return MGCFD_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int32_t* cnt = nullptr;
  int r = counts_address(s, &cnt);
  if (r) return r;
  k_clear_counts<<<grid(ncoarse), kThreads, 0, s>>>(ncoarse, cnt);
  if (nfine > 0) {
    k_zero_mapped<<<grid(nfine), kThreads, 0, s>>>(nfine, ncoarse, node_to_mg, coarse_variables);
    k_accumulate<<<grid(nfine), kThreads, 0, s>>>(nfine, ncoarse, node_to_mg, fine_variables, coarse_variables, cnt);
  }
  k_average<<<grid(ncoarse), kThreads, 0, s>>>(ncoarse, coarse_variables, cnt);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("mgcfd_op_restrict_noalloc: ") + cudaGetErrorString(e));
  return MGCFD_OK;
}

// The skip counter of this entry point, for mgcfd_op_map_errors.
int mgcfd::restrict_noalloc_map_errors(unsigned long long* count, bool reset) {
  cudaError_t e = cudaMemcpyFromSymbol(count, g_restrict_map_errors, sizeof(*count));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero = 0;
    e = cudaMemcpyToSymbol(g_restrict_map_errors, &zero, sizeof(zero));
  }
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("map error counter: ") + cudaGetErrorString(e));
  return MGCFD_OK;
}
