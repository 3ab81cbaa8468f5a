// Per-loop drop-in entry points: one CUDA kernel per op_par_loop of the
// reference V-cycle, over device arrays in OP2's dat layout (AoS,
// [set size][dim], 0-based int32 maps).  Indirect OP_INC arguments use FP64
// atomics (native red.global.add.f64); OP_MIN/OP_INC globals are reduced per
// block and combined with one atomic per block.  Map entries are
// range-checked against the target set size: an element with an
// out-of-range entry is skipped and counted in g_map_errors (read by
// mgcfd_op_map_errors), never dereferenced.
//
// The edge flux and the restriction's up_pre/up loops run through an
// execution plan cached per map (plans.cu), as OP2's CUDA backend caches one
// per indirect loop: the plan-free kernels below remain for calls made while
// plans are switched off, or while a stream captures a graph before the
// map's plan exists.
#include <cfloat>
#include <cstdio>

#include "common.h"
#include "device_math.cuh"
#include "plans.h"

using namespace mgcfd;

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  const int64_t cap = 152 * 32;  // grid-stride loops beyond 32 blocks per SM
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MGCFD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return MGCFD_OK;
}

__device__ unsigned long long g_map_errors;

__device__ __forceinline__ bool in_range(int32_t i, int32_t n) { return (uint32_t)i < (uint32_t)n; }

__device__ __forceinline__ void map_error() { atomicAdd(&g_map_errors, 1ull); }

// Elements a plan left out, counted once per call as the plan-free kernels
// count them.
__global__ void k_add_map_errors(unsigned long long n) { atomicAdd(&g_map_errors, n); }

int count_skipped(int64_t n, cudaStream_t s) {
  if (n > 0) k_add_map_errors<<<1, 1, 0, s>>>((unsigned long long)n);
  return MGCFD_OK;
}

#define MGCFD_GRID_STRIDE(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_initialize_variables(int32_t n, double v0, double v1, double v2, double v3, double v4,
                                       double* __restrict__ var) {
  MGCFD_GRID_STRIDE(i, n) {
    double* x = var + 5 * i;
    x[0] = v0; x[1] = v1; x[2] = v2; x[3] = v3; x[4] = v4;
  }
}

__global__ void k_zero(int64_t n, double* __restrict__ a) {
  MGCFD_GRID_STRIDE(i, n) a[i] = 0.0;
}

// misc.h:40-76 for one edge.
__global__ void k_cell_volumes(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n,
                               const double* __restrict__ xyz, double* __restrict__ ewt, double* __restrict__ vol) {
  MGCFD_GRID_STRIDE(e, ne) {
    const int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
    if (!in_range(a, nn) || !in_range(b, nn)) { map_error(); continue; }
    double d[3], dist = 0.0, area = 0.0;
    for (int i = 0; i < 3; i++) {
      d[i] = xyz[3 * (int64_t)b + i] - xyz[3 * (int64_t)a + i];
      dist += d[i] * d[i];
    }
    dist = sqrt(dist);
    double* w = ewt + 3 * e;
    for (int i = 0; i < 3; i++) area += w[i] * w[i];
    area = sqrt(area);
    const double tv = (1.0 / 3.0) * 0.5 * dist * area;
    atomicAdd(vol + a, tv);
    atomicAdd(vol + b, tv);
    for (int i = 0; i < 3; i++) w[i] = ((d[i] / dist) * area) / dist;
  }
}

__global__ void k_scale(int64_t n, double s, double* __restrict__ a) {
  MGCFD_GRID_STRIDE(i, n) a[i] *= s;
}

__global__ void k_copy(int64_t n, const double* __restrict__ src, double* __restrict__ dst) {
  MGCFD_GRID_STRIDE(i, n) dst[i] = src[i];
}

// time_stepping_kernels.h:13-32
__global__ void k_calculate_dt(int32_t n, const double* __restrict__ var, const double* __restrict__ vol,
                               double* __restrict__ dt) {
  MGCFD_GRID_STRIDE(i, n) {
    const double* x = var + 5 * i;
    NodePrim p = node_prim(x[0], x[1], x[2], x[3], x[4]);
    dt[i] = 0.5 * (cbrt(vol[i]) / p.s);
  }
}

__global__ void k_set_scalar(double* p, double v) { *p = v; }

// Block minimum, then one compare-and-swap loop per block on the double.
__device__ void atomic_min_double(double* addr, double v) {
  unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
  unsigned long long old = *a;
  while (v < __longlong_as_double((long long)old)) {
    unsigned long long assumed = old;
    old = atomicCAS(a, assumed, (unsigned long long)__double_as_longlong(v));
    if (old == assumed) break;
  }
}

__global__ void k_min_dt(int32_t n, const double* __restrict__ dt, double* __restrict__ out) {
  __shared__ double sm[kThreads / 32];
  double m = DBL_MAX;
  MGCFD_GRID_STRIDE(i, n) {
    const double v = dt[i];
    if (v < m) m = v;  // NaN never replaces, as in get_min_dt_kernel
  }
  m = warp_min(m);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : DBL_MAX;
    m = warp_min(m);
    if (threadIdx.x == 0 && m < DBL_MAX) atomic_min_double(out, m);
  }
}

// time_stepping_kernels.h:43-64 (only the final division matters).
__global__ void k_step_factor(int32_t n, const double* __restrict__ vol, const double* __restrict__ min_dt,
                              double* __restrict__ sf) {
  const double m = *min_dt;
  MGCFD_GRID_STRIDE(i, n) sf[i] = m / vol[i];
}

// flux.h:41-208 over edges with atomic increments at both ends.
__global__ void k_flux_edge(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, const double* __restrict__ var,
                            const double* __restrict__ ewt, double sc, double* __restrict__ flux) {
  MGCFD_GRID_STRIDE(e, ne) {
    const int32_t ia = e2n[2 * e], ib = e2n[2 * e + 1];
    if (!in_range(ia, nn) || !in_range(ib, nn)) { map_error(); continue; }
    const double* va = var + 5 * (int64_t)ia;
    const double* vb = var + 5 * (int64_t)ib;
    const NodePrim a = node_prim(va[0], va[1], va[2], va[3], va[4]);
    const NodePrim b = node_prim(vb[0], vb[1], vb[2], vb[3], vb[4]);
    const double wx = ewt[3 * e], wy = ewt[3 * e + 1], wz = ewt[3 * e + 2];
    const double wfac = -sqrt(wx * wx + wy * wy + wz * wz) * sc * 0.5;
    double f[5];
    edge_flux(a, b, -0.5 * wx, -0.5 * wy, -0.5 * wz, wfac, f);
    double* fa = flux + 5 * (int64_t)ia;
    double* fb = flux + 5 * (int64_t)ib;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      atomicAdd(fa + k, f[k]);
      atomicAdd(fb + k, negate(f[k]));
    }
  }
}

// flux.h:14-39 over boundary entries.
__global__ void k_bnd_flux(int32_t nb, int32_t nn, const int32_t* __restrict__ b2n, const int32_t* __restrict__ grp,
                           const double* __restrict__ bw, const double* __restrict__ var, mgcfd_freestream ff,
                           double* __restrict__ flux) {
  MGCFD_GRID_STRIDE(i, nb) {
    const int g = grp[i];
    if (g > 7) continue;
    const int32_t n = b2n[i];
    if (!in_range(n, nn)) { map_error(); continue; }
    const double* x = var + 5 * (int64_t)n;
    const NodePrim b = node_prim(x[0], x[1], x[2], x[3], x[4]);
    const double wx = bw[3 * i], wy = bw[3 * i + 1], wz = bw[3 * i + 2];
    double* fb = flux + 5 * (int64_t)n;
    if (g <= 2) {
      atomicAdd(fb + 1, wx * b.p);
      atomicAdd(fb + 2, wy * b.p);
      atomicAdd(fb + 3, wz * b.p);
    } else {
      double ffw[5];
      ffw[0] = wx * ff.ff_variable[1] + wy * ff.ff_variable[2] + wz * ff.ff_variable[3];
      ffw[1] = wx * ff.ff_flux_contribution_momentum_x[0] + wy * ff.ff_flux_contribution_momentum_x[1] +
               wz * ff.ff_flux_contribution_momentum_x[2];
      ffw[2] = wx * ff.ff_flux_contribution_momentum_y[0] + wy * ff.ff_flux_contribution_momentum_y[1] +
               wz * ff.ff_flux_contribution_momentum_y[2];
      ffw[3] = wx * ff.ff_flux_contribution_momentum_z[0] + wy * ff.ff_flux_contribution_momentum_z[1] +
               wz * ff.ff_flux_contribution_momentum_z[2];
      ffw[4] = wx * ff.ff_flux_contribution_density_energy[0] + wy * ff.ff_flux_contribution_density_energy[1] +
               wz * ff.ff_flux_contribution_density_energy[2];
      double f[5];
      farfield_flux(b, wx, wy, wz, ffw, f);
#pragma unroll
      for (int k = 0; k < 5; k++) atomicAdd(fb + k, f[k]);
    }
  }
}

// time_stepping_kernels.h:66-86, one thread per (node, variable) so every
// access of the [N][5] dats is coalesced (a thread per node reads rows 40 B
// apart, five times per array: measured 1.06 ms at 8M nodes against the
// 0.2 ms its bytes need).
__global__ void k_time_step(int64_t n5, double inv_div, const double* __restrict__ sf, double* __restrict__ flux,
                            const double* __restrict__ old, double* __restrict__ var) {
  MGCFD_GRID_STRIDE(j, n5) {
    const double factor = sf[j / 5] * inv_div;
    var[j] = old[j] + factor * flux[j];
    flux[j] = 0.0;
  }
}

// unstructured_stream.h:7-57
__global__ void k_stream(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, const double* __restrict__ var,
                         const double* __restrict__ ewt, double* __restrict__ flux) {
  MGCFD_GRID_STRIDE(e, ne) {
    const int32_t ia = e2n[2 * e], ib = e2n[2 * e + 1];
    if (!in_range(ia, nn) || !in_range(ib, nn)) { map_error(); continue; }
    const double* va = var + 5 * (int64_t)ia;
    const double* vb = var + 5 * (int64_t)ib;
    const double ex = ewt[3 * e], ey = ewt[3 * e + 1], ez = ewt[3 * e + 2];
    double* fa = flux + 5 * (int64_t)ia;
    double* fb = flux + 5 * (int64_t)ib;
    atomicAdd(fa + 0, vb[0] + ex);
    atomicAdd(fa + 1, vb[1] + ez);
    atomicAdd(fa + 2, vb[2]);
    atomicAdd(fa + 3, vb[3]);
    atomicAdd(fa + 4, vb[4] + ey);
    atomicAdd(fb + 0, va[0]);
    atomicAdd(fb + 1, va[1]);
    atomicAdd(fb + 2, va[2]);
    atomicAdd(fb + 3, va[3]);
    atomicAdd(fb + 4, va[4]);
  }
}

__global__ void k_residual(int64_t n, const double* __restrict__ old, const double* __restrict__ var,
                           double* __restrict__ res) {
  MGCFD_GRID_STRIDE(i, n) res[i] = var[i] - old[i];
}

__global__ void k_sum_squares(int64_t n, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double sm[kThreads / 32];
  double s = 0.0;
  MGCFD_GRID_STRIDE(i, n) s += x[i] * x[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0.0;
    s = warp_sum(s);
    if (threadIdx.x == 0) atomicAdd(out, s);
  }
}

__device__ __forceinline__ void block_add_int(int c, int32_t* out) {
  __shared__ int sm[kThreads / 32];
  c = warp_sum_int(c);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    c = threadIdx.x < kThreads / 32 ? sm[threadIdx.x] : 0;
    c = warp_sum_int(c);
    if (threadIdx.x == 0 && c) atomicAdd(out, c);
  }
}

__global__ void k_count_bad(int64_t n, const double* __restrict__ x, int32_t* __restrict__ out) {
  int c = 0;
  MGCFD_GRID_STRIDE(i, n) {
    const double v = x[i];
    if (isnan(v) || isinf(v)) c++;
  }
  block_add_int(c, out);
}

// validation.h:46-100: count of values outside the reference's tolerance.
__global__ void k_count_diff(int64_t n, const double* __restrict__ test, const double* __restrict__ master,
                             int32_t* __restrict__ out) {
  int c = 0;
  MGCFD_GRID_STRIDE(i, n) {
    double acc = master[i] * 10.0e-8;
    if (acc < 0.0) acc = -acc;
    if (acc < 3.0e-19) acc = 3.0e-19;
    double d = test[i] - master[i];
    if (d < 0.0) d = -d;
    if (d > acc) c++;
  }
  block_add_int(c, out);
}

// mg.h:29-64
__global__ void k_up_pre(int32_t nf, int32_t nc, const int32_t* __restrict__ map, double* __restrict__ cv,
                         int32_t* __restrict__ scratch) {
  MGCFD_GRID_STRIDE(i, nf) {
    const int32_t c = map[i];
    if (!in_range(c, nc)) { map_error(); continue; }
#pragma unroll
    for (int k = 0; k < 5; k++) cv[5 * (int64_t)c + k] = 0.0;
    scratch[c] = 0;
  }
}
__global__ void k_up(int32_t nf, int32_t nc, const int32_t* __restrict__ map, const double* __restrict__ fv,
                     double* __restrict__ cv, int32_t* __restrict__ scratch) {
  MGCFD_GRID_STRIDE(i, nf) {
    const int32_t c = map[i];
    if (!in_range(c, nc)) { map_error(); continue; }
#pragma unroll
    for (int k = 0; k < 5; k++) atomicAdd(cv + 5 * (int64_t)c + k, fv[5 * i + k]);
    atomicAdd(scratch + c, 1);
  }
}
__global__ void k_up_post(int32_t nc, double* __restrict__ cv, const int32_t* __restrict__ scratch) {
  MGCFD_GRID_STRIDE(i, nc) {
    const int32_t s = scratch[i];
    const double avg = s == 0 ? 1.0 : 1.0 / (double)s;
#pragma unroll
    for (int k = 0; k < 5; k++) cv[5 * i + k] *= avg;
  }
}

// mg.h:66-88.  (Staging the fine rows through shared memory for coalesced
// access measured slower here, 0.78 against 0.39 ms at 8M nodes: the gathers
// of the coarse rows are latency-bound and the staging barriers expose them.)
__global__ void k_down(int32_t nf, int32_t nc, const int32_t* __restrict__ map, double* __restrict__ fv,
                       const double* __restrict__ fres, const double* __restrict__ fx,
                       const double* __restrict__ cres, const double* __restrict__ cx) {
  MGCFD_GRID_STRIDE(i, nf) {
    const int32_t ci = map[i];
    if (!in_range(ci, nc)) { map_error(); continue; }
    const int64_t c = ci;
    const double dx = fabs(fx[3 * i] - cx[3 * c]);
    const double dy = fabs(fx[3 * i + 1] - cx[3 * c + 1]);
    const double dz = fabs(fx[3 * i + 2] - cx[3 * c + 2]);
    const double dm = sqrt(dx * dx + dy * dy + dz * dz);
    const double d[5] = {dm, dx, dy, dz, dm};
#pragma unroll
    for (int k = 0; k < 5; k++) fv[5 * i + k] -= d[k] * (cres[5 * c + k] - fres[5 * i + k]);
  }
}

bool bad_size(int64_t n) { return n < 0; }

}  // namespace

#define CHECK_N(n, name) \
  if (bad_size(n)) return set_error(MGCFD_ERR_INVALID, std::string(name) + ": negative size")
#define CHECK_PTR(p, n, name) \
  if ((n) > 0 && !(p)) return set_error(MGCFD_ERR_INVALID, std::string(name) + ": null pointer")
#define STREAM(s) (static_cast<cudaStream_t>(s))

extern "C" int mgcfd_op_initialize_variables(int32_t n, const mgcfd_freestream* ff, double* var, void* s) {
  CHECK_N(n, "mgcfd_op_initialize_variables");
  CHECK_PTR(var, n, "mgcfd_op_initialize_variables");
  if (!ff) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_initialize_variables: null freestream");
  if (n == 0) return MGCFD_OK;
  const double* v = ff->ff_variable;
  k_initialize_variables<<<grid_for(n), kThreads, 0, STREAM(s)>>>(n, v[0], v[1], v[2], v[3], v[4], var);
  return launch_status("initialize_variables");
}

extern "C" int mgcfd_op_zero(int32_t n, int32_t dim, double* a, void* s) {
  CHECK_N(n, "mgcfd_op_zero");
  if (dim < 1) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_zero: dim must be >= 1");
  CHECK_PTR(a, n, "mgcfd_op_zero");
  if (n == 0) return MGCFD_OK;
  k_zero<<<grid_for((int64_t)n * dim), kThreads, 0, STREAM(s)>>>((int64_t)n * dim, a);
  return launch_status("zero");
}

extern "C" int mgcfd_op_calculate_cell_volumes(int32_t ne, int32_t nn, const int32_t* e2n, const double* xyz,
                                               double* ewt, double* vol, void* s) {
  CHECK_N(ne, "mgcfd_op_calculate_cell_volumes");
  CHECK_N(nn, "mgcfd_op_calculate_cell_volumes");
  CHECK_PTR(e2n, ne, "calculate_cell_volumes"); CHECK_PTR(xyz, ne, "calculate_cell_volumes");
  CHECK_PTR(ewt, ne, "calculate_cell_volumes"); CHECK_PTR(vol, ne, "calculate_cell_volumes");
  if (ne == 0) return MGCFD_OK;
  k_cell_volumes<<<grid_for(ne), kThreads, 0, STREAM(s)>>>(ne, nn, e2n, xyz, ewt, vol);
  return launch_status("calculate_cell_volumes");
}

extern "C" int mgcfd_op_dampen_ewt(int32_t n, double* w, void* s) {
  CHECK_N(n, "mgcfd_op_dampen_ewt");
  CHECK_PTR(w, n, "mgcfd_op_dampen_ewt");
  if (n == 0) return MGCFD_OK;
  k_scale<<<grid_for(3 * (int64_t)n), kThreads, 0, STREAM(s)>>>(3 * (int64_t)n, 1e-7, w);
  return launch_status("dampen_ewt");
}

extern "C" int mgcfd_op_copy_double(int32_t n, const double* v, double* old, void* s) {
  CHECK_N(n, "mgcfd_op_copy_double");
  CHECK_PTR(v, n, "copy_double"); CHECK_PTR(old, n, "copy_double");
  if (n == 0) return MGCFD_OK;
  k_copy<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, v, old);
  return launch_status("copy_double");
}

extern "C" int mgcfd_op_calculate_dt(int32_t n, const double* v, const double* vol, double* dt, void* s) {
  CHECK_N(n, "mgcfd_op_calculate_dt");
  CHECK_PTR(v, n, "calculate_dt"); CHECK_PTR(vol, n, "calculate_dt"); CHECK_PTR(dt, n, "calculate_dt");
  if (n == 0) return MGCFD_OK;
  VolPlan* plan = nullptr;
  int r = vol_plan_get(vol, n, STREAM(s), &plan);
  if (r) return r;
  if (plan) return vol_plan_calculate_dt(plan, v, vol, dt, STREAM(s));
  k_calculate_dt<<<grid_for(n), kThreads, 0, STREAM(s)>>>(n, v, vol, dt);
  return launch_status("calculate_dt");
}

extern "C" int mgcfd_op_get_min_dt(int32_t n, const double* dt, double* min_dt, void* s) {
  CHECK_N(n, "mgcfd_op_get_min_dt");
  CHECK_PTR(dt, n, "get_min_dt");
  if (!min_dt) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_get_min_dt: null output");
  k_set_scalar<<<1, 1, 0, STREAM(s)>>>(min_dt, DBL_MAX);
  if (n > 0) k_min_dt<<<grid_for(n), kThreads, 0, STREAM(s)>>>(n, dt, min_dt);
  return launch_status("get_min_dt");
}

extern "C" int mgcfd_op_compute_step_factor(int32_t n, const double* v, const double* vol, const double* min_dt,
                                            double* sf, void* s) {
  (void)v;
  CHECK_N(n, "mgcfd_op_compute_step_factor");
  CHECK_PTR(vol, n, "compute_step_factor"); CHECK_PTR(sf, n, "compute_step_factor");
  if (!min_dt) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_compute_step_factor: null min_dt");
  if (n == 0) return MGCFD_OK;
  k_step_factor<<<grid_for(n), kThreads, 0, STREAM(s)>>>(n, vol, min_dt, sf);
  return launch_status("compute_step_factor");
}

extern "C" int mgcfd_op_compute_flux_edge(int32_t ne, int32_t nn, const int32_t* e2n, const double* v,
                                          const double* ewt, double sc, double* flux, void* s) {
  CHECK_N(ne, "mgcfd_op_compute_flux_edge");
  CHECK_N(nn, "mgcfd_op_compute_flux_edge");
  CHECK_PTR(e2n, ne, "compute_flux_edge"); CHECK_PTR(v, ne, "compute_flux_edge");
  CHECK_PTR(ewt, ne, "compute_flux_edge"); CHECK_PTR(flux, ne, "compute_flux_edge");
  if (ne == 0) return MGCFD_OK;
  EdgePlan* plan = nullptr;
  int r = edge_plan_get(e2n, ne, nn, STREAM(s), &plan);
  if (r) return r;
  if (plan) {
    int64_t skipped = 0;
    if ((r = edge_plan_flux(plan, v, ewt, sc, flux, STREAM(s), &skipped))) return r;
    count_skipped(skipped, STREAM(s));
  } else {
    k_flux_edge<<<grid_for(ne), kThreads, 0, STREAM(s)>>>(ne, nn, e2n, v, ewt, sc, flux);
  }
  return launch_status("compute_flux_edge");
}

extern "C" int mgcfd_op_compute_bnd_node_flux(int32_t nb, int32_t nn, const int32_t* b2n, const int32_t* grp,
                                              const double* bw, const double* v, const mgcfd_freestream* ff,
                                              double* flux, void* s) {
  CHECK_N(nb, "mgcfd_op_compute_bnd_node_flux");
  CHECK_N(nn, "mgcfd_op_compute_bnd_node_flux");
  CHECK_PTR(b2n, nb, "compute_bnd_node_flux"); CHECK_PTR(grp, nb, "compute_bnd_node_flux");
  CHECK_PTR(bw, nb, "compute_bnd_node_flux"); CHECK_PTR(v, nb, "compute_bnd_node_flux");
  CHECK_PTR(flux, nb, "compute_bnd_node_flux");
  if (!ff) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_compute_bnd_node_flux: null freestream");
  if (nb == 0) return MGCFD_OK;
  k_bnd_flux<<<grid_for(nb), kThreads, 0, STREAM(s)>>>(nb, nn, b2n, grp, bw, v, *ff, flux);
  return launch_status("compute_bnd_node_flux");
}

extern "C" int mgcfd_op_time_step(int32_t n, int32_t rk, const double* sf, double* flux, const double* old,
                                  double* v, void* s) {
  CHECK_N(n, "mgcfd_op_time_step");
  if (rk < 0 || rk >= kRK) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_time_step: rk_cycle must be 0, 1 or 2");
  CHECK_PTR(sf, n, "time_step"); CHECK_PTR(flux, n, "time_step"); CHECK_PTR(old, n, "time_step");
  CHECK_PTR(v, n, "time_step");
  if (n == 0) return MGCFD_OK;
  // factor = sf / (RK + 1 - rk): divisors 4, 3, 2 become multiplications.
  const double inv_div = 1.0 / (double)(kRK + 1 - rk);
  k_time_step<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, inv_div, sf, flux, old, v);
  return launch_status("time_step");
}

extern "C" int mgcfd_op_unstructured_stream(int32_t ne, int32_t nn, const int32_t* e2n, const double* v,
                                            const double* ewt, double* flux, void* s) {
  CHECK_N(ne, "mgcfd_op_unstructured_stream");
  CHECK_N(nn, "mgcfd_op_unstructured_stream");
  CHECK_PTR(e2n, ne, "unstructured_stream"); CHECK_PTR(v, ne, "unstructured_stream");
  CHECK_PTR(ewt, ne, "unstructured_stream"); CHECK_PTR(flux, ne, "unstructured_stream");
  if (ne == 0) return MGCFD_OK;
  k_stream<<<grid_for(ne), kThreads, 0, STREAM(s)>>>(ne, nn, e2n, v, ewt, flux);
  return launch_status("unstructured_stream");
}

extern "C" int mgcfd_op_residual(int32_t n, const double* old, const double* v, double* res, void* s) {
  CHECK_N(n, "mgcfd_op_residual");
  CHECK_PTR(old, n, "residual"); CHECK_PTR(v, n, "residual"); CHECK_PTR(res, n, "residual");
  if (n == 0) return MGCFD_OK;
  k_residual<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, old, v, res);
  return launch_status("residual");
}

extern "C" int mgcfd_op_calc_rms(int32_t n, const double* res, double* rms, void* s) {
  CHECK_N(n, "mgcfd_op_calc_rms");
  CHECK_PTR(res, n, "calc_rms");
  if (!rms) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_calc_rms: null output");
  if (n == 0) return MGCFD_OK;
  k_sum_squares<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, res, rms);
  return launch_status("calc_rms");
}

extern "C" int mgcfd_op_count_bad_vals(int32_t n, const double* v, int32_t* count, void* s) {
  CHECK_N(n, "mgcfd_op_count_bad_vals");
  CHECK_PTR(v, n, "count_bad_vals");
  if (!count) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_count_bad_vals: null output");
  if (n == 0) return MGCFD_OK;
  k_count_bad<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, v, count);
  return launch_status("count_bad_vals");
}

extern "C" int mgcfd_op_count_differences(int32_t n, const double* test, const double* master, int32_t* count,
                                          void* s) {
  CHECK_N(n, "mgcfd_op_count_differences");
  CHECK_PTR(test, n, "count_differences"); CHECK_PTR(master, n, "count_differences");
  if (!count) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_count_differences: null output");
  if (n == 0) return MGCFD_OK;
  k_count_diff<<<grid_for(5 * (int64_t)n), kThreads, 0, STREAM(s)>>>(5 * (int64_t)n, test, master, count);
  return launch_status("count_differences");
}

extern "C" int mgcfd_op_up_pre(int32_t nf, int32_t nc, const int32_t* map, double* cv, int32_t* scratch,
                               void* s) {
  CHECK_N(nf, "mgcfd_op_up_pre");
  CHECK_N(nc, "mgcfd_op_up_pre");
  CHECK_PTR(map, nf, "up_pre"); CHECK_PTR(cv, nf, "up_pre"); CHECK_PTR(scratch, nf, "up_pre");
  if (nf == 0) return MGCFD_OK;
  ChildPlan* plan = nullptr;
  int r = child_plan_get(map, nf, nc, STREAM(s), &plan);
  if (r) return r;
  if (plan) {
    int64_t skipped = 0;
    if ((r = child_plan_up_pre(plan, cv, scratch, STREAM(s), &skipped))) return r;
    count_skipped(skipped, STREAM(s));
  } else {
    k_up_pre<<<grid_for(nf), kThreads, 0, STREAM(s)>>>(nf, nc, map, cv, scratch);
  }
  return launch_status("up_pre");
}

extern "C" int mgcfd_op_up(int32_t nf, int32_t nc, const int32_t* map, const double* fv, double* cv,
                           int32_t* scratch, void* s) {
  CHECK_N(nf, "mgcfd_op_up");
  CHECK_N(nc, "mgcfd_op_up");
  CHECK_PTR(map, nf, "up"); CHECK_PTR(fv, nf, "up"); CHECK_PTR(cv, nf, "up"); CHECK_PTR(scratch, nf, "up");
  if (nf == 0) return MGCFD_OK;
  ChildPlan* plan = nullptr;
  int r = child_plan_get(map, nf, nc, STREAM(s), &plan);
  if (r) return r;
  if (plan) {
    int64_t skipped = 0;
    if ((r = child_plan_up(plan, fv, cv, scratch, STREAM(s), &skipped))) return r;
    count_skipped(skipped, STREAM(s));
  } else {
    k_up<<<grid_for(nf), kThreads, 0, STREAM(s)>>>(nf, nc, map, fv, cv, scratch);
  }
  return launch_status("up");
}

extern "C" int mgcfd_op_up_post(int32_t nc, double* cv, const int32_t* scratch, void* s) {
  CHECK_N(nc, "mgcfd_op_up_post");
  CHECK_PTR(cv, nc, "up_post"); CHECK_PTR(scratch, nc, "up_post");
  if (nc == 0) return MGCFD_OK;
  k_up_post<<<grid_for(nc), kThreads, 0, STREAM(s)>>>(nc, cv, scratch);
  return launch_status("up_post");
}

extern "C" int mgcfd_op_down(int32_t nf, int32_t nc, const int32_t* map, double* fv, const double* fres,
                             const double* fx, const double* cres, const double* cx, void* s) {
  CHECK_N(nf, "mgcfd_op_down");
  CHECK_N(nc, "mgcfd_op_down");
  CHECK_PTR(map, nf, "down"); CHECK_PTR(fv, nf, "down"); CHECK_PTR(fres, nf, "down"); CHECK_PTR(fx, nf, "down");
  CHECK_PTR(cres, nf, "down"); CHECK_PTR(cx, nf, "down");
  if (nf == 0) return MGCFD_OK;
  k_down<<<grid_for(nf), kThreads, 0, STREAM(s)>>>(nf, nc, map, fv, fres, fx, cres, cx);
  return launch_status("down");
}

extern "C" int mgcfd_op_map_errors(int64_t* count, int32_t reset) {
  if (!count) return set_error(MGCFD_ERR_INVALID, "mgcfd_op_map_errors: null output");
  unsigned long long v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_map_errors, sizeof(v));
  if (e == cudaSuccess && reset) {
    const unsigned long long zero = 0;
    e = cudaMemcpyToSymbol(g_map_errors, &zero, sizeof(zero));
  }
  if (e != cudaSuccess) return set_error(MGCFD_ERR_CUDA, std::string("mgcfd_op_map_errors: ") + cudaGetErrorString(e));
  unsigned long long w = 0;
  const int r = restrict_noalloc_map_errors(&w, reset != 0);
  if (r) return r;
  *count = (int64_t)(v + w);
  return MGCFD_OK;
}
