// Test harness (not part of the library): runs the double-word helpers of
// dw_math.cuh -- the binary64 -> pair split and the DW edge flux beside the
// FP64 edge flux -- on host arrays.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dw_math.cuh"

namespace {

__global__ void k_split(int64_t n, const double* __restrict__ d, float* __restrict__ h, float* __restrict__ l) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const mgcfd::dwf x = mgcfd::dw_split(d[i]);
  h[i] = x.h;
  l[i] = x.l;
}

// a, b: [n][8] NodePrim fields (rho, mx, my, mz, rhoE, p, s, rinv); w: [n][4]
// (hx, hy, hz, wfac).  f64, fdw: [n][5] increments of node a.
__global__ void k_flux(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                       const double* __restrict__ w, double* __restrict__ f64, double* __restrict__ fdw) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* pa = a + 8 * i;
  const double* pb = b + 8 * i;
  const double* pw = w + 4 * i;
  const mgcfd::NodePrim A{pa[0], pa[1], pa[2], pa[3], pa[4], pa[5], pa[6], pa[7]};
  const mgcfd::NodePrim B{pb[0], pb[1], pb[2], pb[3], pb[4], pb[5], pb[6], pb[7]};
  double f[5];
  mgcfd::edge_flux(A, B, pw[0], pw[1], pw[2], pw[3], f);
  for (int k = 0; k < 5; k++) f64[5 * i + k] = f[k];
  using mgcfd::dw_split;
  const mgcfd::NodePrimDW AD{dw_split(pa[0]), dw_split(pa[1]), dw_split(pa[2]), dw_split(pa[3]),
                             dw_split(pa[4]), dw_split(pa[5]), dw_split(pa[6]), dw_split(pa[7])};
  const mgcfd::NodePrimDW BD{dw_split(pb[0]), dw_split(pb[1]), dw_split(pb[2]), dw_split(pb[3]),
                             dw_split(pb[4]), dw_split(pb[5]), dw_split(pb[6]), dw_split(pb[7])};
  mgcfd::edge_flux_dw(AD, BD, dw_split(pw[0]), dw_split(pw[1]), dw_split(pw[2]), dw_split(pw[3]), f);
  for (int k = 0; k < 5; k++) fdw[5 * i + k] = f[k];
}

// One node per thread: its state me[5] (conserved variables) and K
// neighbours' states nb[K][5] with weights w[K][4] (h, wfac, h already
// oriented from the node); out[5] = node_flux_dw over the K edges, with the
// pair primitives of every state from node_prim_dw.  prims_dw / prims_64:
// [8] node_prim_dw (as binary64) and node_prim of the node's own state.
__global__ void k_node(int64_t n, int K, const double* __restrict__ me, const double* __restrict__ nb,
                       const double* __restrict__ w, double* __restrict__ out, double* __restrict__ prims_dw,
                       double* __restrict__ prims_64) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* x = me + 5 * i;
  const mgcfd::NodePrimDW q = mgcfd::node_prim_dw(x[0], x[1], x[2], x[3], x[4]);
  const mgcfd::NodePrim p = mgcfd::node_prim(x[0], x[1], x[2], x[3], x[4]);
  const mgcfd::dwf qf[8] = {q.rho, q.mx, q.my, q.mz, q.rhoE, q.p, q.s, q.rinv};
  const double pf[8] = {p.rho, p.mx, p.my, p.mz, p.rhoE, p.p, p.s, p.rinv};
  for (int k = 0; k < 8; k++) {
    prims_dw[8 * i + k] = mgcfd::dw_to_double(qf[k]);
    prims_64[8 * i + k] = pf[k];
  }
  mgcfd::NodeFluxDW acc;
  mgcfd::node_flux_dw_init(acc);
  for (int j = 0; j < K; j++) {
    const double* y = nb + 5 * (K * i + j);
    const double* ww = w + 4 * (K * i + j);
    const mgcfd::NodePrimDW o = mgcfd::node_prim_dw(y[0], y[1], y[2], y[3], y[4]);
    mgcfd::node_flux_dw_edge(acc, q.s, o, mgcfd::dw_split(ww[0]), mgcfd::dw_split(ww[1]), mgcfd::dw_split(ww[2]),
                             mgcfd::dw_split(ww[3]));
  }
  mgcfd::node_flux_dw_finish(acc, q, out + 5 * i);
}

template <class T>
cudaError_t to_device(T** p, const T* src, int64_t count) {
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * (size_t)(count + 1));
  if (e == cudaSuccess && src) e = cudaMemcpy(*p, src, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice);
  return e;
}

}  // namespace

// Host buffers in, host buffers out; each returns a cudaError_t value.
extern "C" int dw_check_split(int64_t n, const double* d, float* h, float* l) {
  double* dd = nullptr;
  float *hh = nullptr, *ll = nullptr;
  cudaError_t e;
  if ((e = to_device(&dd, d, n)) || (e = to_device<float>(&hh, nullptr, n)) || (e = to_device<float>(&ll, nullptr, n)))
    goto done;
  k_split<<<(unsigned)((n + 255) / 256), 256>>>(n, dd, hh, ll);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) goto done;
  if ((e = cudaMemcpy(h, hh, 4 * (size_t)n, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(l, ll, 4 * (size_t)n, cudaMemcpyDeviceToHost)))
    goto done;
done:
  cudaFree(dd); cudaFree(hh); cudaFree(ll);
  return (int)e;
}

extern "C" int dw_check_flux(int64_t n, const double* a, const double* b, const double* w, double* f64, double* fdw) {
  double *da = nullptr, *db = nullptr, *dw = nullptr, *o1 = nullptr, *o2 = nullptr;
  cudaError_t e;
  if ((e = to_device(&da, a, 8 * n)) || (e = to_device(&db, b, 8 * n)) || (e = to_device(&dw, w, 4 * n)) ||
      (e = to_device<double>(&o1, nullptr, 5 * n)) || (e = to_device<double>(&o2, nullptr, 5 * n)))
    goto done;
  k_flux<<<(unsigned)((n + 127) / 128), 128>>>(n, da, db, dw, o1, o2);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) goto done;
  if ((e = cudaMemcpy(f64, o1, 40 * (size_t)n, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(fdw, o2, 40 * (size_t)n, cudaMemcpyDeviceToHost)))
    goto done;
done:
  cudaFree(da); cudaFree(db); cudaFree(dw); cudaFree(o1); cudaFree(o2);
  return (int)e;
}

extern "C" int dw_check_node(int64_t n, int32_t K, const double* me, const double* nb, const double* w, double* out,
                             double* prims_dw, double* prims_64) {
  double *dm = nullptr, *dn = nullptr, *dw = nullptr, *o1 = nullptr, *o2 = nullptr, *o3 = nullptr;
  cudaError_t e;
  if ((e = to_device(&dm, me, 5 * n)) || (e = to_device(&dn, nb, 5 * n * K)) || (e = to_device(&dw, w, 4 * n * K)) ||
      (e = to_device<double>(&o1, nullptr, 5 * n)) || (e = to_device<double>(&o2, nullptr, 8 * n)) ||
      (e = to_device<double>(&o3, nullptr, 8 * n)))
    goto done;
  k_node<<<(unsigned)((n + 127) / 128), 128>>>(n, K, dm, dn, dw, o1, o2, o3);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize())) goto done;
  if ((e = cudaMemcpy(out, o1, 40 * (size_t)n, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(prims_dw, o2, 64 * (size_t)n, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(prims_64, o3, 64 * (size_t)n, cudaMemcpyDeviceToHost)))
    goto done;
done:
  cudaFree(dm); cudaFree(dn); cudaFree(dw); cudaFree(o1); cudaFree(o2); cudaFree(o3);
  return (int)e;
}
