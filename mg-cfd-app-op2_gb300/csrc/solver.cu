// Device-resident multigrid solver: the whole V-cycle of euler3d.cpp:452-641
// on one GPU with no host synchronisation inside a cycle.
//
// Layout in HBM (per level, nodes in renumbered order, see setup.h):
//   rec    [N][8]  f64  rho, rho*u, rho*v, rho*w, rho*E, p, |u|+c, 1/rho
//                       (the conserved state plus the primitives the edge
//                       kernel needs; 64 B rows read with two 256-bit loads)
//   rec32  [N][8]  f32  the same in FP32 (mixed precision only; the fused
//                       strategy alternates it with rec32b between stages)
//   old, res, flux [N][5] f64; inv_vol, cbrt_vol, vol [N] f64
//   e2n    [E]     int2 (a < b, sorted by a then b); w4 [E] double4
//                       (-wx/2, -wy/2, -wz/2, -|w|*smoothing*0.5) or float4 (mixed)
//   fe     [E][5]  f64  per-edge fluxes (gather increment strategy only;
//                       f32 fe32 in mixed precision)
//   a_off/b_off/b_list  CSR of each node's edges as end a and as end b
//                       (gather and fused); b_nbr/b_w4f: the b-side edge data
//                       in b_list order (fused)
//   bidx [N] int32 and bdata [NB][12] f64: boundary entries folded per node
//   n2mg [N], dvec [N] double4: prolongation parent and |dx|,|dy|,|dz|,dist
//   ch_off/ch_list: restriction children of each coarse node
//
// Kernels per smoothing step (euler3d.cpp:467-550):
//   memset(min_dt key)                      get_min_dt's DBL_MAX start
//   k_step_begin   nodes  old = var, primitives, dt, block min -> atomicMin
//                         (a step that a prolongation precedes -- every
//                         level-0 step after the first -- begins inside
//                         k_prolong instead, on the state it just wrote)
//   3 x { k_flux   edges  edge flux, +f to a and -f to b (FP64 atomics) or
//                         f stored per edge (gather strategy)
//         k_update nodes  gathered flux + boundary flux, time step, flux = 0,
//                         primitives for the next stage; in the last stage
//                         residual, and at level 0 the rms and NaN/Inf count }
//   (fused strategy, mixed precision: no k_flux; k_update computes each of
//   its node's edge fluxes itself from the stage's input primitives, and a
//   plain multi-level solver takes the level-0 rms and NaN/Inf count in the
//   restriction that follows instead of the last stage)
// then k_restrict (coarse nodes, children mean, mg.h:29-64) or k_prolong
// (fine nodes, mg.h:66-88), and under a stop rule k_cycle_end after each
// V-cycle.
//
// Failure handling: min_dt < 0 and NaN/Inf at level 0 set a sticky device
// status word; every later kernel sees it and returns, so the run stops at the
// same point the reference aborts (with the fused stage, one restriction
// later).  The host reads the status on synchronize.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <vector>

#include "common.h"
#include "device_math.cuh"
#include "dw_math.cuh"
#include "setup.h"
#include "solver_internal.h"

using namespace mgcfd;

namespace {

constexpr int kNodeThreads = 128;

// Keep freed solver and setup memory in the device's default pool, so that
// repeated solves (batches, serving) do not map fresh memory from the
// driver for every allocation.
void keep_freed_memory(int dev) {
  static std::once_flag once[kMaxDevices];
  if (dev < 0 || dev >= kMaxDevices) return;
  std::call_once(once[dev], [dev] {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
}

// ---------------------------------------------------------------------------
// Kernels.

__device__ __forceinline__ void store_rec(double* rec, int64_t i, const NodePrim& p) {
  double4_32a* r = reinterpret_cast<double4_32a*>(rec + 8 * i);
  r[0] = make_double4_32a(p.rho, p.mx, p.my, p.mz);
  r[1] = make_double4_32a(p.rhoE, p.p, p.s, p.rinv);
}

__device__ __forceinline__ NodePrim load_rec(const double* rec, int64_t i) {
  const double4_32a* r = reinterpret_cast<const double4_32a*>(rec + 8 * i);
  const double4_32a x = r[0], y = r[1];
  NodePrim p;
  p.rho = x.x; p.mx = x.y; p.my = x.z; p.mz = x.w;
  p.rhoE = y.x; p.p = y.y; p.s = y.z; p.rinv = y.w;
  return p;
}

struct NodePrimF {
  float rho, mx, my, mz, rhoE, p, s, rinv;
};

// Mixed precision: FP32 primitives of an FP32 state.
__device__ __forceinline__ NodePrimF prim32(float r, float x, float y, float z, float e) {
  const float rinv = 1.0f / r;
  const float ux = x * rinv, uy = y * rinv, uz = z * rinv;
  const float q2 = ux * ux + uy * uy + uz * uz;
  const float p = 0.4f * (e - 0.5f * r * q2);
  const float sp = sqrtf(q2) + sqrtf(1.4f * p * rinv);
  return NodePrimF{r, x, y, z, e, p, sp, rinv};
}

__device__ __forceinline__ void store_prim32(float* rec32, int64_t i, const NodePrimF& q) {
  float4* o = reinterpret_cast<float4*>(rec32 + 8 * i);
  o[0] = make_float4(q.rho, q.mx, q.my, q.mz);
  o[1] = make_float4(q.rhoE, q.p, q.s, q.rinv);
}

// FP32 primitives straight from the FP64 state; the narrowing runs on the
// integer pipe (d2f_bits), so this issues no FP64 instruction.
__device__ __forceinline__ NodePrimF store_rec32_from_var(float* rec32, int64_t i, double rho, double mx, double my,
                                                          double mz, double rhoE) {
  const NodePrimF q = prim32(d2f_bits(rho), d2f_bits(mx), d2f_bits(my), d2f_bits(mz), d2f_bits(rhoE));
  store_prim32(rec32, i, q);
  return q;
}

__device__ __forceinline__ NodePrimF load_rec32(const float* rec32, int64_t i) {
  const float4* r = reinterpret_cast<const float4*>(rec32 + 8 * i);
  const float4 x = r[0], y = r[1];
  return NodePrimF{x.x, x.y, x.z, x.w, y.x, y.y, y.z, y.w};
}

// The FP32 edge flux, spelled with explicit IEEE intrinsics (never contracted
// or reordered by the compiler), so every kernel that inlines it -- the edge
// kernel and the fused node-centric stage -- computes the same bits from the
// same inputs.
__device__ __forceinline__ void edge_flux_f32(const NodePrimF& a, const NodePrimF& b, float4 w, float f[5]) {
  // w = (-wx/2, -wy/2, -wz/2, wfac), as edge_flux in device_math.cuh.
  const float mha = __fmaf_rn(a.mz, w.z, __fmaf_rn(a.my, w.y, __fmul_rn(a.mx, w.x)));
  const float mhb = __fmaf_rn(b.mz, w.z, __fmaf_rn(b.my, w.y, __fmul_rn(b.mx, w.x)));
  const float uha = __fmul_rn(mha, a.rinv), uhb = __fmul_rn(mhb, b.rinv);
  const float fac = __fmul_rn(w.w, __fadd_rn(a.s, b.s));
  const float pp = __fadd_rn(a.p, b.p);
  f[0] = __fmaf_rn(fac, __fsub_rn(a.rho, b.rho), __fadd_rn(mha, mhb));
  f[1] = __fmaf_rn(fac, __fsub_rn(a.mx, b.mx), __fmaf_rn(pp, w.x, __fmaf_rn(b.mx, uhb, __fmul_rn(a.mx, uha))));
  f[2] = __fmaf_rn(fac, __fsub_rn(a.my, b.my), __fmaf_rn(pp, w.y, __fmaf_rn(b.my, uhb, __fmul_rn(a.my, uha))));
  f[3] = __fmaf_rn(fac, __fsub_rn(a.mz, b.mz), __fmaf_rn(pp, w.z, __fmaf_rn(b.mz, uhb, __fmul_rn(a.mz, uha))));
  f[4] = __fmaf_rn(fac, __fsub_rn(a.rhoE, b.rhoE),
                   __fmaf_rn(__fadd_rn(b.rhoE, b.p), uhb, __fmul_rn(__fadd_rn(a.rhoE, a.p), uha)));
}

// 1/vol and cbrt(vol) on the device for both setup paths, so the solver's
// constants do not depend on the host's libm.
__global__ void k_vol_constants(int32_t n, const double* __restrict__ vol, double* __restrict__ inv_vol,
                                double* __restrict__ cbrt_vol) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  inv_vol[i] = __ddiv_rn(1.0, vol[i]);
  cbrt_vol[i] = cbrt(vol[i]);
}

// Freestream state of each node's own mesh (batched solvers).
__global__ void k_init_state_seg(int32_t n, double* __restrict__ rec, const int32_t* __restrict__ mesh_id,
                                 const double* __restrict__ ffvar) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* v = ffvar + 5 * (int64_t)mesh_id[i];
  store_rec(rec, i, node_prim(v[0], v[1], v[2], v[3], v[4]));
}

// Freestream state into rec (initialize_variables_kernel, misc.h:10-16).
__global__ void k_init_state(int32_t n, double* __restrict__ rec, double v0, double v1, double v2, double v3,
                             double v4) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  store_rec(rec, i, node_prim(v0, v1, v2, v3, v4));
}

// Per-mesh block reductions for batched solvers (SEG): the nodes of a block
// are contiguous, so their mesh ids are nondecreasing and differ from the
// first node's id by less than the block size; each mesh of the block gets
// one shared slot and one global atomic.

// copy_double_kernel + calculate_dt_kernel + get_min_dt_kernel (block part)
// for node i of a block of kNodeThreads threads whose state x is in hand:
// old = x, the primitives for the first RK stage, and dt's candidate key into
// the block's minimum and one atomic per block (per mesh of the block when
// batched).  Every thread of the block calls it (it synchronises); `live`
// is false for threads past the end and for stopped meshes.  DW: the
// primitives go to rec2 as pairs (the edge flux's inputs); rec keeps the
// state only.
template <bool MIXED, bool SEG, bool DW>
__device__ __forceinline__ void step_begin_core(int64_t i, bool live, const double x[5], double* __restrict__ rec,
                                                double* __restrict__ rec2, float* __restrict__ rec32,
                                                double* __restrict__ old, const double* __restrict__ cbrt_vol,
                                                unsigned long long* __restrict__ dt_key,
                                                const int32_t* __restrict__ mesh_id) {
  __shared__ unsigned long long smin[kNodeThreads / 32];
  __shared__ unsigned int sest[kNodeThreads / 32];
  __shared__ unsigned long long s_key[SEG ? kNodeThreads : 1];
  if (SEG) {
    s_key[threadIdx.x] = ~0ull;
    __syncthreads();
  }
  // The minimum is taken over order-preserving integer keys of dt, so the
  // reduction issues no FP64 compare; ~0 = no candidate.
  unsigned long long key = ~0ull;
  double cv = 0.0, sp = 1.0;  // FP64: cbrt(vol) and |u| + c of this node
  float est = 0.0f;
  if (live) {
    double* o = old + 5 * i;
    o[0] = x[0]; o[1] = x[1]; o[2] = x[2]; o[3] = x[3]; o[4] = x[4];
    if (MIXED) {
      // The spectral radius is edge-flux arithmetic (FP32); min_dt itself
      // is exact in FP64 and the step factor and update stay FP64.
      const NodePrimF q = store_rec32_from_var(rec32, i, x[0], x[1], x[2], x[3], x[4]);
      key = dt_candidate_key(f2d_bits(0.5f * (d2f_bits(cbrt_vol[i]) / q.s)));  // time_stepping_kernels.h:31
    } else {
      if (DW) {  // the primitives in double-word arithmetic, no FP64 instruction
        const NodePrimDW q = node_prim_dw(x[0], x[1], x[2], x[3], x[4]);
        store_prim_dw(rec2, i, q);
        sp = dw_to_double(q.s);
      } else {
        const NodePrim p = node_prim(x[0], x[1], x[2], x[3], x[4]);
        store_rec(rec, i, p);
        sp = p.s;
      }
      cv = cbrt_vol[i];
      if (SEG) key = dt_candidate_key(0.5 * (cv / sp));  // time_stepping_kernels.h:31
      else est = 0.5f * __fdividef(d2f_bits(cv), d2f_bits(sp));
    }
  }
  if (!MIXED && !SEG) {
    // Only the minimum of dt is needed.  An FP32 estimate (relative error
    // below 4e-7: two narrowings and __fdividef's 2 ulp) picks the nodes
    // that can hold the minimum -- those within 4e-6 of the block's smallest
    // estimate -- and only they divide in FP64.  Estimates that are not
    // finite normal numbers always take the exact path.
    const uint32_t eb = __float_as_uint(est) & 0x7fffffffu;
    const bool normal = live && eb - 0x00800000u < 0x7f000000u;
    unsigned int ek = normal ? fkey(est) : 0xffffffffu;
    ek = __reduce_min_sync(0xffffffffu, ek);
    if ((threadIdx.x & 31) == 0) sest[threadIdx.x >> 5] = ek;
    __syncthreads();
    unsigned int bk = sest[0];
#pragma unroll
    for (int w = 1; w < kNodeThreads / 32; w++) bk = min(bk, sest[w]);
    const float m32 = bk == 0xffffffffu ? INFINITY : fkey_inv(bk);
    if (live && (!normal || est <= m32 + fabsf(m32) * 4e-6f))
      key = dt_candidate_key(0.5 * (cv / sp));  // time_stepping_kernels.h:31
  }
  if (SEG) {
    const int32_t m0 = mesh_id[(int64_t)blockIdx.x * blockDim.x];
    if (key != ~0ull) atomicMin(&s_key[mesh_id[i] - m0], key);
    __syncthreads();
    if (s_key[threadIdx.x] != ~0ull) atomicMin(dt_key + m0 + threadIdx.x, s_key[threadIdx.x]);
    return;
  }
  key = warp_min_u64(key);
  if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = key;
  __syncthreads();
  if (threadIdx.x < 32) {
    key = threadIdx.x < kNodeThreads / 32 ? smin[threadIdx.x] : ~0ull;
    key = warp_min_u64(key);
    // Keys only decrease, so a block whose minimum is not below the current
    // value skips its atomic: most of the grid's same-address atomics go away.
    if (threadIdx.x == 0 && key != ~0ull && key < *reinterpret_cast<volatile unsigned long long*>(dt_key))
      atomicMin(dt_key, key);
  }
}

// The step begin on its own (a step that no prolongation precedes).
template <bool MIXED, bool SEG, bool DW = false>
__global__ void __launch_bounds__(kNodeThreads) k_step_begin(int32_t n, double* __restrict__ rec,
                                                             double* __restrict__ rec2,
                                                             float* __restrict__ rec32, double* __restrict__ old,
                                                             const double* __restrict__ cbrt_vol,
                                                             unsigned long long* __restrict__ dt_key,
                                                             const DevStatus* __restrict__ st,
                                                             const int32_t* __restrict__ mesh_id,
                                                             const SegStop* __restrict__ seg_stop) {
  __shared__ int s_halt;
  if (threadIdx.x == 0) s_halt = st->halt;
  __syncthreads();
  if (s_halt) return;  // block-uniform: the reduction below synchronises
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // Batched solvers under a stop rule: a stopped mesh's nodes change no more.
  const bool live = i < n && !(SEG && seg_stop && seg_stop[mesh_id[i]].halt);
  double x[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (live) {
    const double4_32a* r = reinterpret_cast<const double4_32a*>(rec + 8 * i);
    const double4_32a v = r[0];
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w; x[4] = r[1].x;
  }
  step_begin_core<MIXED, SEG, DW>(i, live, x, rec, rec2, rec32, old, cbrt_vol, dt_key, mesh_id);
}

// compute_flux_edge_kernel (flux.h:41-208), FP64, both ends by FP64 atomics
// (GATHER=false) or stored per edge for the node-side gather (GATHER=true).
template <bool GATHER>
__global__ void k_flux_f64(int32_t ne, const int2* __restrict__ e2n, const double4_32a* __restrict__ w4,
                           const double* __restrict__ rec, double* __restrict__ flux, double* __restrict__ fe,
                           const DevStatus* __restrict__ st) {
  if (st->halt) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const double4_32a w = w4[e];
  const NodePrim a = load_rec(rec, ab.x);
  const NodePrim b = load_rec(rec, ab.y);
  double f[5];
  edge_flux(a, b, w.x, w.y, w.z, w.w, f);
  if (GATHER) {
    double* o = fe + 5 * e;
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = f[k];
  } else {
    double* fa = flux + 5 * (int64_t)ab.x;
    double* fb = flux + 5 * (int64_t)ab.y;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      atomicAdd(fa + k, f[k]);
      atomicAdd(fb + k, negate(f[k]));
    }
  }
}

// compute_flux_edge_kernel (flux.h:41-208) in double-word arithmetic on the
// FP32 pipes (dw_math.cuh): the primitives and weights as pairs, the
// increments in binary64, by FP64 atomics or stored per edge as k_flux_f64.
template <bool GATHER>
__global__ void k_flux_dw(int32_t ne, const int2* __restrict__ e2n, const double4_32a* __restrict__ w2,
                          const double* __restrict__ rec2, double* __restrict__ flux, double* __restrict__ fe,
                          const DevStatus* __restrict__ st) {
  if (st->halt) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const double4_32a w = w2[e];
  const NodePrimDW a = load_prim_dw(rec2, ab.x);
  const NodePrimDW b = load_prim_dw(rec2, ab.y);
  double f[5];
  edge_flux_dw(a, b, dw_unpack(w.x), dw_unpack(w.y), dw_unpack(w.z), dw_unpack(w.w), f);
  if (GATHER) {
    double* o = fe + 5 * e;
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = f[k];
  } else {
    double* fa = flux + 5 * (int64_t)ab.x;
    double* fb = flux + 5 * (int64_t)ab.y;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      atomicAdd(fa + k, f[k]);
      atomicAdd(fb + k, negate(f[k]));
    }
  }
}

// The per-node neighbour table of the fused DW stage: node i's entries start
// at a_off[i] + b_off[i] (its a-side edges, then its b-side edges).
__global__ void k_dw_offsets(int32_t n, const int32_t* __restrict__ a_off, const int32_t* __restrict__ b_off,
                             int32_t* __restrict__ off2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) off2[i] = a_off[i] + b_off[i];
}

__global__ void k_dw_table_a(int32_t ne, const int2* __restrict__ e2n, const int32_t* __restrict__ a_off,
                             const int32_t* __restrict__ off2, int2* __restrict__ ent2) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  ent2[off2[ab.x] + (e - a_off[ab.x])] = make_int2(ab.y, (int32_t)e);
}

// b side: the edge seen from its end b (bit 31 of the edge index set: the
// stage evaluates it with its own node as end a and h negated).
__global__ void k_dw_table_b(int32_t ne, const int2* __restrict__ e2n, const int32_t* __restrict__ b_list,
                             const int32_t* __restrict__ a_off, const int32_t* __restrict__ b_off,
                             const int32_t* __restrict__ off2, int2* __restrict__ ent2) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ne) return;
  const int32_t e = b_list[j];
  const int32_t a = e2n[e].x, b = e2n[e].y;
  ent2[off2[b] + (a_off[b + 1] - a_off[b]) + (j - b_off[b])] = make_int2(a, (int32_t)((uint32_t)e | 0x80000000u));
}

// The edge weights as pair words (DW precision), once at set-up, counting
// the finite non-zero weights outside [2^-70, 2^70): their products with the
// flow state would leave the pairs' binary32 exponent range.
__global__ void k_split_weights(int64_t n, const double* __restrict__ w, double* __restrict__ w2,
                                unsigned int* __restrict__ out_of_range) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double v = w[k];
  w2[k] = dw_pack(dw_split(v));
  const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  const int e = (int)(b >> 52) - 1023;
  if (b != 0 && b < 0x7ff0000000000000ull && (e < -70 || e >= 70)) atomicAdd(out_of_range, 1u);
}

// compute_flux_edge_kernel over one colour class: no two of these edges share
// a node, so each adds +f / -f to its end nodes with plain loads and stores.
// (A loop edge a == b is one thread's two updates of one row, in order.)
__global__ void k_flux_f64_coloured(int32_t ne, const int2* __restrict__ e2n, const double4_32a* __restrict__ w4,
                                    const double* __restrict__ rec, double* flux, const DevStatus* __restrict__ st) {
  if (st->halt) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const double4_32a w = w4[e];
  const NodePrim a = load_rec(rec, ab.x);
  const NodePrim b = load_rec(rec, ab.y);
  double f[5];
  edge_flux(a, b, w.x, w.y, w.z, w.w, f);
  double* fa = flux + 5 * (int64_t)ab.x;
#pragma unroll
  for (int k = 0; k < 5; k++) fa[k] += f[k];
  double* fb = flux + 5 * (int64_t)ab.y;
#pragma unroll
  for (int k = 0; k < 5; k++) fb[k] += negate(f[k]);
}

// Edges of a level into colour order (idx[k] = old position of edge k).
__global__ void k_gather_edges(int32_t ne, const int32_t* __restrict__ idx, const int2* __restrict__ e2n_in,
                               const double4_32a* __restrict__ w4_in, int2* __restrict__ e2n_out,
                               double4_32a* __restrict__ w4_out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ne) return;
  const int32_t e = idx[k];
  e2n_out[k] = e2n_in[e];
  w4_out[k] = w4_in[e];
}

// Mixed precision edge flux: FP32 arithmetic, FP64 accumulation.  The
// gather strategy stores the FP32 fluxes (widened exactly, on the integer
// pipe, where the node sums them in FP64); the atomic strategy widens them
// here and adds them with FP64 atomics.
template <bool GATHER>
__global__ void k_flux_mixed(int32_t ne, const int2* __restrict__ e2n, const float4* __restrict__ w4f,
                             const float* __restrict__ rec32, double* __restrict__ flux, float* __restrict__ fe32,
                             const DevStatus* __restrict__ st) {
  if (st->halt) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const float4 w = w4f[e];
  const NodePrimF a = load_rec32(rec32, ab.x);
  const NodePrimF b = load_rec32(rec32, ab.y);
  float f[5];
  edge_flux_f32(a, b, w, f);
  if (GATHER) {
    float* o = fe32 + 5 * e;
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = f[k];
  } else {
    double* fa = flux + 5 * (int64_t)ab.x;
    double* fb = flux + 5 * (int64_t)ab.y;
#pragma unroll
    for (int k = 0; k < 5; k++) {
      const double d = f2d_bits(f[k]);
      atomicAdd(fa + k, d);
      atomicAdd(fb + k, negate(d));
    }
  }
}

// unstructured_stream_kernel (unstructured_stream.h:7-57): the flux kernel's
// data movement with trivial arithmetic (the reference's -b probe).
__global__ void k_stream(int32_t ne, const int2* __restrict__ e2n, const double4_32a* __restrict__ w4,
                         const double* __restrict__ rec, double* __restrict__ dummy,
                         const DevStatus* __restrict__ st) {
  if (st->halt) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const double4_32a w = w4[e];
  const NodePrim a = load_rec(rec, ab.x);
  const NodePrim b = load_rec(rec, ab.y);
  double* fa = dummy + 5 * (int64_t)ab.x;
  double* fb = dummy + 5 * (int64_t)ab.y;
  // w4 holds -w/2; -2*(-w/2) recovers the weight exactly.
  atomicAdd(fa + 0, b.rho + -2.0 * w.x);
  atomicAdd(fa + 1, b.mx + -2.0 * w.z);
  atomicAdd(fa + 2, b.my);
  atomicAdd(fa + 3, b.mz);
  atomicAdd(fa + 4, b.rhoE + -2.0 * w.y);
  atomicAdd(fb + 0, a.rho);
  atomicAdd(fb + 1, a.mx);
  atomicAdd(fb + 2, a.my);
  atomicAdd(fb + 3, a.mz);
  atomicAdd(fb + 4, a.rhoE);
}

struct UpdateArgs {
  int32_t n;
  int32_t level0;
  double inv_div;  // 1 / (RK + 1 - rk)
  double* rec;
  double* rec2;            // DW: the next stage's primitives as pairs
  const double* rec2_in;   // DW fused: the stage's input primitives
  const int32_t* off2;     // DW fused: per-node neighbour table
  const int2* ent2;
  const double4_32a* w4dw;
  float* rec32;
  const double* old;
  double* flux;
  const double* fe;
  const float* fe32;
  const float* rec32_in;   // fused: the stage's input primitives (rec32 is the output)
  const int2* e2n;
  const float4* w4f;
  const int32_t* b_nbr;
  const float4* b_w4f;
  const int32_t* a_off;
  const int32_t* b_off;
  const int32_t* b_list;
  const double* inv_vol;
  const int32_t* bidx;
  const double* bdata;
  double* res;
  const unsigned long long* dt_key;  // plain: the level's key; batched: the level's per-mesh keys
  DevStatus* st;
  const int32_t* mesh_id;            // batched only
  int* seg_neg;
  int* seg_bad;
  double* seg_rms;
  double* seg_rho;
  const SegStop* seg_stop;           // batched solvers under a stop rule, else null
};

// Boundary flux of one node (flux.h:14-39 summed over the node's entries).
__device__ __forceinline__ void add_boundary(const NodePrim& p, const double* __restrict__ b, double F[5]) {
  double ffw[5] = {b[6], b[7], b[8], b[9], b[10]};
  double f[5];
  farfield_flux(p, b[0], b[1], b[2], ffw, f);
#pragma unroll
  for (int k = 0; k < 5; k++) F[k] += f[k];
  F[1] += b[3] * p.p;
  F[2] += b[4] * p.p;
  F[3] += b[5] * p.p;
}

// A node's edges in the gather order: those where it is end a (a contiguous
// range of the edge list), then those where it is end b (through b_list).  The
// node kernels walk both in one loop of deg iterations, so every lane of a
// warp runs as many iterations as its own node has edges.  With one loop per
// end, a warp ran each loop for its lane with the most edges of that end (the
// a/b split of a node's edges varies with the numbering) and issued the FP64
// adds for the idle lanes too.
struct EdgeRange {
  int32_t a0, na, b0, deg;
};

template <class Args>
__device__ __forceinline__ EdgeRange edge_range(const Args& A, int64_t i) {
  EdgeRange r;
  r.a0 = A.a_off[i];
  r.na = A.a_off[i + 1] - r.a0;
  r.b0 = A.b_off[i];
  r.deg = r.na + (A.b_off[i + 1] - r.b0);
  return r;
}

// Level-0 norms of one block of kNodeThreads threads (every thread arrives):
// sums through shared memory, halving the active threads each step down to
// one warp, so every FP64 add is a useful one (a shuffle tree in each warp
// would issue five per thread); then one atomic per sum.  A NaN or infinity
// stops the solver (euler3d.cpp:539-548).
__device__ __forceinline__ void block_norms(double* srms, double* srho, int* sbad, double r2, double rr, int bad,
                                            DevStatus* st) {
  const int t = threadIdx.x;
  srms[t] = r2;
  srho[t] = rr;
  sbad[t] = bad;
  __syncthreads();
#pragma unroll
  for (int w = kNodeThreads / 2; w >= 32; w >>= 1) {
    if (t < w) { srms[t] += srms[t + w]; srho[t] += srho[t + w]; sbad[t] += sbad[t + w]; }
    __syncthreads();
  }
  if (t < 32) {
    r2 = warp_sum(srms[t]);
    rr = warp_sum(srho[t]);
    bad = warp_sum_int(sbad[t]);
    if (t == 0) {
      atomicAdd(&st->rms_acc, r2);
      atomicAdd(&st->rho_acc, rr);
      if (bad) { atomicAdd(&st->bad_count, bad); atomicOr(&st->halt, 1); }
    }
  }
}

// compute_bnd_node_flux_kernel + time_step_kernel (+ residual_kernel,
// calc_rms_kernel and count_bad_vals in the last stage).  Plain solvers stop
// everything on min_dt < 0 or NaN/Inf (the reference aborts); batched
// solvers mark the failing mesh and leave the others running.  The fused
// stage with pair sums is latency-bound: capped at 48 registers (10 blocks
// per SM, a few bytes spilled) it runs 2% faster; the DW stage capped at 64
// (8 blocks, no spill) 1.5% faster than at its own 72, and slower at 56
// (spills).  Every other form keeps the
// compiler's own register choice: a minimum of 0 blocks is no constraint,
// whereas a minimum of 1 lets it grow to 70-80 registers and lose occupancy.
// Fused stage, STAGE (option stage_neighbour_ids): the block's neighbour ids
// (its contiguous ranges of the a-side and b-side edge lists, up to
// kStageIds each) are copied into shared memory with cp.async at the start,
// while the node's own data loads, so the edge loop's dependent chain is a
// shared-memory id load and one gather.  Measured slower on GB300 (8M nodes:
// 0.689 -> 0.713 ms with FP64 sums, 0.530 -> 0.577 ms with pair sums): the
// long-scoreboard stalls fall (10.3 -> 9.4 per issue) but the L1 hit rate of
// the neighbour gathers falls with the shared-memory carve-out (61% -> 53%)
// and the copies add instructions.  Off by default.
constexpr int kStageIds = 1024;

__device__ __forceinline__ void cp_async4(int32_t* smem_dst, const int32_t* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Fused stage, edge-parallel (option edge_parallel_stage): the block's edge
// ends -- each node's a-side edges then its b-side edges, nodes in order --
// are processed in chunks of kEpChunk by all threads at once (each end's
// flux depends on two loads, not on the node's previous edges), the signed
// FP32 fluxes go to shared memory, and each thread then sums its own node's
// ends in the gather order: the same operations on the same inputs in the
// same order as the per-node loop, so the same bits.  Measured slower on
// GB300 (8M nodes: 0.690 -> 0.876 ms with FP64 sums, 0.530 -> 0.785 ms with
// pair sums): a warp of consecutive nodes in the per-node loop gathers
// overlapping neighbour records together and hits in L1 (61%); spread over
// the block's threads the ends lose that reuse (47%) and add barrier and
// shared-memory stalls.  Off by default.
constexpr int kEpChunk = 768;

// DW: the state goes to rec and the next stage's primitives to rec2 as pairs.
template <bool GATHER, bool LAST, bool MIXED, bool SEG, bool PAIR = false, bool FUSED = false, int FV = 0,
          bool DW = false>
__global__ void __launch_bounds__(kNodeThreads, (FUSED && PAIR) ? 10 : (FUSED && DW) ? 8 : 0) k_update(UpdateArgs A) {
  constexpr bool STAGE = FV == 1;  // neighbour ids staged by cp.async
  constexpr bool EP = FV == 2;     // edge-parallel ends through shared memory
  __shared__ int32_t s_aid[STAGE ? kStageIds : 1], s_bid[STAGE ? kStageIds : 1];
  __shared__ float s_x[EP ? 5 * kEpChunk : 1];
  __shared__ float4 s_me[EP ? 2 * kNodeThreads : 1];
  __shared__ int32_t s_ao[EP ? kNodeThreads + 1 : 1], s_bo[EP ? kNodeThreads + 1 : 1], s_na[EP ? kNodeThreads : 1];
  __shared__ uint8_t s_owner[EP ? kEpChunk : 1];
  __shared__ double srms[LAST ? kNodeThreads : 1];
  __shared__ double srho[LAST ? kNodeThreads : 1];
  __shared__ int sbad[LAST ? kNodeThreads : 1];
  __shared__ int s_halt;
  __shared__ double s_sum[SEG && LAST ? kNodeThreads : 1];
  __shared__ double s_rho[SEG && LAST ? kNodeThreads : 1];
  __shared__ int s_bad[SEG && LAST ? kNodeThreads : 1];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int32_t a_base = 0, b_base = 0, a_cnt = 0, b_cnt = 0;
  if (STAGE) {
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x;
    const int64_t i1 = i0 + blockDim.x < A.n ? i0 + blockDim.x : A.n;
    a_base = A.a_off[i0];
    b_base = A.b_off[i0];
    a_cnt = min(A.a_off[i1] - a_base, kStageIds);
    b_cnt = min(A.b_off[i1] - b_base, kStageIds);
    for (int t = threadIdx.x; t < a_cnt; t += blockDim.x) cp_async4(s_aid + t, &A.e2n[a_base + t].y);
    for (int t = threadIdx.x; t < b_cnt; t += blockDim.x) cp_async4(s_bid + t, A.b_nbr + b_base + t);
  }
  // The node's own data is loaded before the block-uniform halt and min_dt
  // checks so that its latency overlaps them; nothing is written before.
  double o[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, Fa[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, ivol = 0.0;
  int32_t bi = -1;
  if (!GATHER && i < A.n) {  // (the gather forms load them after their edge loop)
#pragma unroll
    for (int k = 0; k < 5; k++) o[k] = A.old[5 * i + k];
    ivol = A.inv_vol[i];
    bi = A.bidx[i];
#pragma unroll
    for (int k = 0; k < 5; k++) Fa[k] = A.flux[5 * i + k];
  }
  if (threadIdx.x == 0) s_halt = A.st->halt;
  if (SEG && LAST) { s_sum[threadIdx.x] = 0.0; s_rho[threadIdx.x] = 0.0; s_bad[threadIdx.x] = 0; }
  if (STAGE) cp_async_wait_all();
  __syncthreads();
  if (s_halt) return;  // block-uniform: the reduction below synchronises
  int32_t mid = 0;
  double min_dt;
  if (SEG) {
    mid = i < A.n ? A.mesh_id[i] : 0;
    min_dt = dkey_inv(A.dt_key[mid]);
  } else {
    min_dt = dkey_inv(*A.dt_key);
    if (min_dt < 0.0) {  // euler3d.cpp:480: abort before the step factor is used
      if (threadIdx.x == 0) { A.st->neg_dt = 1; atomicOr(&A.st->halt, 1); }
      return;
    }
  }
  // Edge-parallel fused stage: every thread of the block takes part (the
  // barriers are block-wide), whatever its own node's state.
  float ep_hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, ep_lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  double ep_F[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (FUSED && EP) {
    const int t = threadIdx.x;
    const int64_t i0 = (int64_t)blockIdx.x * blockDim.x;
    const int nloc = (int)(A.n - i0 < (int64_t)blockDim.x ? A.n - i0 : (int64_t)blockDim.x);
    const int32_t A0 = A.a_off[i0], B0 = A.b_off[i0];
    if (t < nloc) {
      const int32_t ao = A.a_off[i] - A0, bo = A.b_off[i] - B0;
      s_ao[t] = ao;
      s_bo[t] = bo;
      s_na[t] = A.a_off[i + 1] - A.a_off[i];
      const float4* r = reinterpret_cast<const float4*>(A.rec32_in + 8 * i);
      s_me[2 * t] = r[0];
      s_me[2 * t + 1] = r[1];
    }
    if (t == 0) {
      s_ao[nloc] = A.a_off[i0 + nloc] - A0;
      s_bo[nloc] = A.b_off[i0 + nloc] - B0;
    }
    __syncthreads();
    const int32_t total = s_ao[nloc] + s_bo[nloc];
    const int32_t my0 = t < nloc ? s_ao[t] + s_bo[t] : 0, my1 = t < nloc ? s_ao[t + 1] + s_bo[t + 1] : 0;
    for (int32_t c0 = 0; c0 < total; c0 += kEpChunk) {
      const int32_t c1 = c0 + kEpChunk < total ? c0 + kEpChunk : total;
      for (int32_t k = (my0 > c0 ? my0 : c0); k < (my1 < c1 ? my1 : c1); k++) s_owner[k - c0] = (uint8_t)t;
      __syncthreads();
#pragma unroll 2
      for (int32_t k = c0 + t; k < c1; k += blockDim.x) {
        const int u = s_owner[k - c0];
        const int32_t j = k - (s_ao[u] + s_bo[u]);
        const bool end_a = j < s_na[u];
        const int32_t ja = end_a ? A0 + s_ao[u] + j : 0, jb = end_a ? 0 : B0 + s_bo[u] + (j - s_na[u]);
        const NodePrimF o = load_rec32(A.rec32_in, end_a ? A.e2n[ja].y : A.b_nbr[jb]);
        const float4 w = end_a ? A.w4f[ja] : A.b_w4f[jb];
        const float4 m0 = s_me[2 * u], m1 = s_me[2 * u + 1];
        const NodePrimF me{m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
        NodePrimF ea = me, eb = o;
        if (!end_a) { ea = o; eb = me; }
        float f[5];
        edge_flux_f32(ea, eb, w, f);
#pragma unroll
        for (int v = 0; v < 5; v++) s_x[5 * (k - c0) + v] = end_a ? f[v] : -f[v];
      }
      __syncthreads();
      for (int32_t k = (my0 > c0 ? my0 : c0); k < (my1 < c1 ? my1 : c1); k++) {
#pragma unroll
        for (int v = 0; v < 5; v++) {
          const float x = s_x[5 * (k - c0) + v];
          if (PAIR) two_sum_acc(ep_hi[v], ep_lo[v], x);
          else ep_F[v] += f2d_bits(x);
        }
      }
      __syncthreads();
    }
  }
  double r2 = 0.0, rr = 0.0;
  int bad = 0;
  bool active = i < A.n;
  if (SEG && active && A.seg_stop && A.seg_stop[mid].halt) active = false;  // a stopped mesh
  if (SEG && active && min_dt < 0.0) {
    atomicOr(A.seg_neg + mid, 1);
    active = false;
  }
  if (active) {
    double F[5];
    if (FUSED && EP) {
#pragma unroll
      for (int k = 0; k < 5; k++) F[k] = PAIR ? f2d_bits(ep_hi[k]) + f2d_bits(ep_lo[k]) : ep_F[k];
    } else if (FUSED && DW) {
      // Node-centric stage in double-word arithmetic: the sum of the fluxes
      // of this node's edges with the node as end a (f(b, a; -h) = -f(a, b; h):
      // on the b side h changes sign), in node_flux_dw's factored form, and
      // one FP64 addition per variable at the end.  Each edge's weights are
      // read from the edge list from both ends; the second read mostly hits L2.
      // Only |u|+c of the node is needed in the loop; its other primitives
      // are loaded for the finish (fewer registers live across the loop).
      const dwf s_me = dw_unpack(A.rec2_in[8 * i + 6]);
      NodeFluxDW acc;
      node_flux_dw_init(acc);
      const int32_t k0 = A.off2[i], k1 = A.off2[i + 1];
      int2 next = k0 < k1 ? A.ent2[k0] : make_int2(0, 0);
      for (int32_t j = k0; j < k1; j++) {
        const int2 en = next;  // the following entry loads during this edge's arithmetic
        if (j + 1 < k1) next = A.ent2[j + 1];
        const NodePrimDW o = load_prim_dw(A.rec2_in, en.x);
        const double4_32a w = A.w4dw[en.y & 0x7fffffff];
        const uint32_t sg = (uint32_t)en.y & 0x80000000u;  // b side: -h
        dwf hx = dw_unpack(w.x), hy = dw_unpack(w.y), hz = dw_unpack(w.z);
        hx = dwf{__uint_as_float(__float_as_uint(hx.h) ^ sg), __uint_as_float(__float_as_uint(hx.l) ^ sg)};
        hy = dwf{__uint_as_float(__float_as_uint(hy.h) ^ sg), __uint_as_float(__float_as_uint(hy.l) ^ sg)};
        hz = dwf{__uint_as_float(__float_as_uint(hz.h) ^ sg), __uint_as_float(__float_as_uint(hz.l) ^ sg)};
        node_flux_dw_edge(acc, s_me, o, hx, hy, hz, dw_unpack(w.w));
      }
      node_flux_dw_finish(acc, load_prim_dw(A.rec2_in, i), F);
    } else if (FUSED) {
      // Node-centric stage: the flux of each edge of this node, computed from
      // the stage's input primitives exactly as k_flux_mixed computes it
      // (end a first), summed in k_update's gather order.
      const NodePrimF me = load_rec32(A.rec32_in, i);
      float hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < 5; k++) F[k] = 0.0;
      float f[5];
      const EdgeRange er = edge_range(A, i);
      for (int32_t j = 0; j < er.deg; j++) {
        const bool end_a = j < er.na;
        const int32_t ja = end_a ? er.a0 + j : 0, jb = end_a ? 0 : er.b0 + j - er.na;  // both in range
        int32_t nb;
        if (STAGE) {
          const int32_t ka = ja - a_base, kb = jb - b_base;
          nb = end_a ? (ka < a_cnt ? s_aid[ka] : A.e2n[ja].y) : (kb < b_cnt ? s_bid[kb] : A.b_nbr[jb]);
        } else {
          nb = end_a ? A.e2n[ja].y : A.b_nbr[jb];
        }
        const NodePrimF o = load_rec32(A.rec32_in, nb);
        const float4 w = end_a ? A.w4f[ja] : A.b_w4f[jb];
        NodePrimF ea = me, eb = o;  // the edge's end a and end b
        if (!end_a) { ea = o; eb = me; }
        edge_flux_f32(ea, eb, w, f);
#pragma unroll
        for (int k = 0; k < 5; k++) {
          const float x = end_a ? f[k] : -f[k];  // node b receives -f
          if (PAIR) two_sum_acc(hi[k], lo[k], x);
          else F[k] += f2d_bits(x);
        }
      }
      if (PAIR) {
#pragma unroll
        for (int k = 0; k < 5; k++) F[k] = f2d_bits(hi[k]) + f2d_bits(lo[k]);
      }
    } else if (GATHER && MIXED && PAIR) {
      // Unevaluated FP32 pairs (hi, lo) fed by error-free TwoSum steps;
      // one FP64 add per variable at the end.
      float hi[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, lo[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      const EdgeRange er = edge_range(A, i);
      for (int32_t j = 0; j < er.deg; j++) {
        const bool end_a = j < er.na;
        const int64_t e = end_a ? er.a0 + j : A.b_list[end_a ? 0 : er.b0 + j - er.na];
#pragma unroll
        for (int k = 0; k < 5; k++) {
          const float x = A.fe32[5 * e + k];
          two_sum_acc(hi[k], lo[k], end_a ? x : -x);
        }
      }
#pragma unroll
      for (int k = 0; k < 5; k++) F[k] = f2d_bits(hi[k]) + f2d_bits(lo[k]);
    } else if (GATHER) {
#pragma unroll
      for (int k = 0; k < 5; k++) F[k] = 0.0;
      const EdgeRange er = edge_range(A, i);
      for (int32_t j = 0; j < er.deg; j++) {
        const bool end_a = j < er.na;
        const int64_t e = end_a ? er.a0 + j : A.b_list[end_a ? 0 : er.b0 + j - er.na];
#pragma unroll
        for (int k = 0; k < 5; k++) {  // F - x as F + (-x): the same bits, one add instruction for both ends
          if (MIXED) {
            const float x = A.fe32[5 * e + k];
            F[k] += f2d_bits(end_a ? x : -x);
          } else {
            const double x = A.fe[5 * e + k];
            F[k] += end_a ? x : negate(x);
          }
        }
      }
    } else {
      double* fl = A.flux + 5 * i;
#pragma unroll
      for (int k = 0; k < 5; k++) { F[k] = Fa[k]; fl[k] = 0.0; }
    }
    if (GATHER) {
#pragma unroll
      for (int k = 0; k < 5; k++) o[k] = A.old[5 * i + k];
      ivol = A.inv_vol[i];
      bi = A.bidx[i];
    }
    if (bi >= 0) {
      NodePrim p;
      if (MIXED || DW) {
        const double4_32a* r = reinterpret_cast<const double4_32a*>(A.rec + 8 * i);
        const double4_32a x = r[0];
        p = node_prim(x.x, x.y, x.z, x.w, r[1].x);
      } else {
        p = load_rec(A.rec, i);
      }
      add_boundary(p, A.bdata + 12 * (int64_t)bi, F);
    }
    const double factor = (min_dt * ivol) * A.inv_div;  // step_factor / (RK+1-rk)
    double v[5];
#pragma unroll
    for (int k = 0; k < 5; k++) v[k] = o[k] + factor * F[k];
    if (LAST) {
      double4_32a* r = reinterpret_cast<double4_32a*>(A.rec + 8 * i);
      r[0] = make_double4_32a(v[0], v[1], v[2], v[3]);
      A.rec[8 * i + 4] = v[4];
      double* rs = A.res + 5 * i;
      double d[5];
#pragma unroll
      for (int k = 0; k < 5; k++) {
        d[k] = v[k] - o[k];
        rs[k] = d[k];
      }
      if (A.level0) {  // calc_rms_kernel and count_bad_vals run on level 0 only
#pragma unroll
        for (int k = 0; k < 5; k++) {
          r2 += d[k] * d[k];
          bad += not_finite(v[k]) ? 1 : 0;
        }
        rr = d[0] * d[0];
      }
    } else if (MIXED) {
      // The fused stages read the next stage's state through its FP32
      // primitives; only a boundary node's FP64 state is read (for its
      // boundary flux) before the last stage writes every node's.
      if (!FUSED || bi >= 0) {
        double4_32a* r = reinterpret_cast<double4_32a*>(A.rec + 8 * i);
        r[0] = make_double4_32a(v[0], v[1], v[2], v[3]);
        A.rec[8 * i + 4] = v[4];
      }
      store_rec32_from_var(A.rec32, i, v[0], v[1], v[2], v[3], v[4]);
    } else if (DW) {
      // As for MIXED: the fused stages write the FP64 state of boundary
      // nodes only; the last stage writes every node's.
      if (!FUSED || bi >= 0) {
        double4_32a* r = reinterpret_cast<double4_32a*>(A.rec + 8 * i);
        r[0] = make_double4_32a(v[0], v[1], v[2], v[3]);
        A.rec[8 * i + 4] = v[4];
      }
      store_prim_dw(A.rec2, i, node_prim_dw(v[0], v[1], v[2], v[3], v[4]));
    } else {
      store_rec(A.rec, i, node_prim(v[0], v[1], v[2], v[3], v[4]));
    }
  } else if (SEG && LAST && i < A.n) {
    bad = 0;  // a mesh stopped by min_dt < 0 keeps its state
  }
  if (!LAST || !A.level0) return;
  if (SEG) {
    const int32_t m0 = A.mesh_id[(int64_t)blockIdx.x * blockDim.x];
    if (i < A.n) {
      if (r2 != 0.0) atomicAdd(&s_sum[mid - m0], r2);
      if (rr != 0.0) atomicAdd(&s_rho[mid - m0], rr);
      if (bad) atomicAdd(&s_bad[mid - m0], bad);
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (s_sum[t] != 0.0) atomicAdd(A.seg_rms + m0 + t, s_sum[t]);
    if (s_rho[t] != 0.0) atomicAdd(A.seg_rho + m0 + t, s_rho[t]);
    if (s_bad[t]) atomicAdd(A.seg_bad + m0 + t, s_bad[t]);
    return;
  }
  block_norms(srms, srho, sbad, r2, rr, bad, A.st);
}

// up_pre/up/up_post (mg.h:29-64) as a gather over each coarse node's children.
// NORMS (restriction from level 0 of a plain solver): the same pass also
// takes calc_rms_kernel and count_bad_vals (validation.h:37-44, 102-115) of
// the level-0 step just finished, since it reads every fine node's state once
// and the residuals sit beside it.  Its blocks cover about eight fine nodes
// per thread, so the block reductions are an eighth of those a fine-node
// kernel would run.
template <bool NORMS>
__global__ void __launch_bounds__(kNodeThreads) k_restrict(int32_t nc, const int32_t* __restrict__ ch_off,
                                                           const int32_t* __restrict__ ch_list,
                                                           const double* __restrict__ frec, double* __restrict__ crec,
                                                           const double* __restrict__ fres, DevStatus* st,
                                                           const int32_t* __restrict__ mesh_id,
                                                           const SegStop* __restrict__ seg_stop) {
  __shared__ double srms[NORMS ? kNodeThreads : 1], srho[NORMS ? kNodeThreads : 1];
  __shared__ int sbad[NORMS ? kNodeThreads : 1];
  __shared__ int s_halt;
  if (NORMS) {
    if (threadIdx.x == 0) s_halt = st->halt;
    __syncthreads();
    if (s_halt) return;  // block-uniform: the reduction below synchronises
  } else if (st->halt) {
    return;
  }
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double q[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // sums of squared residuals, one chain per variable
  int bad = 0;
  const int32_t lo = c < nc ? ch_off[c] : 0, hi = c < nc ? ch_off[c + 1] : 0;
  const bool halted = c < nc && seg_stop && seg_stop[mesh_id[c]].halt;  // a stopped mesh of a batch
  if (hi > lo && !halted) {  // no children: state unchanged (avg = 1 on untouched values)
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int32_t j = lo; j < hi; j++) {
      const int64_t f = ch_list[j];
      const double4_32a x = *reinterpret_cast<const double4_32a*>(frec + 8 * f);  // one 32-byte access
      const double r[5] = {x.x, x.y, x.z, x.w, frec[8 * f + 4]};
#pragma unroll
      for (int k = 0; k < 5; k++) s[k] += r[k];
      if (NORMS) {
        const double* d = fres + 5 * f;
#pragma unroll
        for (int k = 0; k < 5; k++) {
          q[k] += d[k] * d[k];
          bad += not_finite(r[k]) ? 1 : 0;
        }
      }
    }
    const double avg = 1.0 / (double)(hi - lo);
    double* r = crec + 8 * c;
#pragma unroll
    for (int k = 0; k < 5; k++) r[k] = s[k] * avg;
  }
  if (!NORMS) return;
  block_norms(srms, srho, sbad, ((q[0] + q[1]) + (q[2] + q[3])) + q[4], q[0], bad, st);
}

// The fine level's step-begin arrays, for a prolongation that begins its
// next smoothing step.
struct BeginArgs {
  double* rec2;
  float* rec32;
  double* old;
  const double* cbrt_vol;
  unsigned long long* dt_key;
};

// down_kernel (mg.h:66-88) with the parent offsets precomputed.  BEGIN: the
// fine level's next smoothing step begins here (step_begin_core on the new
// state while it is in registers) instead of in a separate pass that reads
// the level's state again; every thread reaches the block reduction.
template <bool BEGIN, bool MIXED, bool SEG, bool DW>
__global__ void __launch_bounds__(kNodeThreads) k_prolong(int32_t nf, const int32_t* __restrict__ n2mg,
                                                          const double4_32a* __restrict__ dvec,
                                                          double* __restrict__ frec, const double* __restrict__ fres,
                                                          const double* __restrict__ cres,
                                                          const DevStatus* __restrict__ st,
                                                          const int32_t* __restrict__ mesh_id,
                                                          const SegStop* __restrict__ seg_stop, BeginArgs B) {
  if (st->halt) return;  // the same for every thread of the launch
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < nf && !(seg_stop && seg_stop[mesh_id[i]].halt);  // not a stopped mesh of a batch
  double x[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  if (live) {
    const int64_t c = n2mg[i];
    const double4_32a d = dvec[i];
    // The record's first four values as one 32-byte access, the fifth alone.
    double4_32a* r4 = reinterpret_cast<double4_32a*>(frec + 8 * i);
    double4_32a v = r4[0];
    double v4 = frec[8 * i + 4];
    const double* cr = cres + 5 * c;
    const double* fr = fres + 5 * i;
    v.x -= d.w * (cr[0] - fr[0]);
    v.y -= d.x * (cr[1] - fr[1]);
    v.z -= d.y * (cr[2] - fr[2]);
    v.w -= d.z * (cr[3] - fr[3]);
    v4 -= d.w * (cr[4] - fr[4]);
    r4[0] = v;
    frec[8 * i + 4] = v4;
    x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w; x[4] = v4;
  }
  if (BEGIN) step_begin_core<MIXED, SEG, DW>(i, live, x, frec, B.rec2, B.rec32, B.old, B.cbrt_vol, B.dt_key, mesh_id);
}

// Far-field terms w.F_ff of every folded boundary row for a new freestream
// (the same arithmetic as the setup's fold, so a retargeted solver holds the
// bits a fresh one would).
__global__ void k_bnd_ffw(int32_t nrows, double* __restrict__ bdata, mgcfd_freestream ff) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  double* row = bdata + 12 * r;
  const double w0 = row[0], w1 = row[1], w2 = row[2];
  const double* fv = ff.ff_variable;
  const double* rows[4] = {ff.ff_flux_contribution_momentum_x, ff.ff_flux_contribution_momentum_y,
                           ff.ff_flux_contribution_momentum_z, ff.ff_flux_contribution_density_energy};
  row[6] = __dadd_rn(__dadd_rn(__dmul_rn(w0, fv[1]), __dmul_rn(w1, fv[2])), __dmul_rn(w2, fv[3]));
  for (int q = 0; q < 4; q++)
    row[7 + q] = __dadd_rn(__dadd_rn(__dmul_rn(w0, rows[q][0]), __dmul_rn(w1, rows[q][1])), __dmul_rn(w2, rows[q][2]));
}

// Fused increment: b-side copies of the edge data in b_list order.
__global__ void k_bside(int32_t ne, const int32_t* __restrict__ b_list, const int2* __restrict__ e2n,
                        const float4* __restrict__ w4f, int32_t* __restrict__ b_nbr, float4* __restrict__ b_w4f) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ne) return;
  const int32_t e = b_list[j];
  b_nbr[j] = e2n[e].x;
  b_w4f[j] = w4f[e];
}

// End of a V-cycle under a stop rule: count it, record the level-0 density
// residual norm sqrt(sum(res_rho^2) / N0) and stop further work (not an
// error) when the rule is met.  One thread.
__global__ void k_cycle_end(DevStatus* st, double n0, int32_t max_cycles, double drop) {
  if (st->halt) return;
  const int c = ++st->cycles_done;
  const double rho = sqrt(st->rho_acc / n0);
  if (c == 1) st->rho_first = rho;
  st->rho_last = rho;
  if (c >= max_cycles || (drop > 0.0 && c > 1 && rho <= drop * st->rho_first)) {
    st->stopped = 1;
    st->halt = 1;
  }
}

// The same per mesh of a batched solver, one thread per mesh: a mesh that
// met the rule, or failed (min_dt < 0, NaN/Inf), stops changing.
__global__ void k_cycle_end_seg(int32_t nseg, SegStop* __restrict__ ss, const double* __restrict__ seg_rho,
                                const double* __restrict__ n0, const int* __restrict__ seg_neg,
                                const int* __restrict__ seg_bad, int32_t max_cycles, double drop) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nseg || ss[m].halt) return;
  if (seg_neg[m] || seg_bad[m]) {
    ss[m].halt = 1;
    return;
  }
  const int c = ++ss[m].cycles_done;
  const double rho = sqrt(seg_rho[m] / n0[m]);
  if (c == 1) ss[m].rho_first = rho;
  ss[m].rho_last = rho;
  if (c >= max_cycles || (drop > 0.0 && c > 1 && rho <= drop * ss[m].rho_first)) {
    ss[m].stopped = 1;
    ss[m].halt = 1;
  }
}

// Fetch helpers: scatter the renumbered rows [off, off + n) back to input
// order (rows of one mesh, or of the whole level when off = 0).
__global__ void k_unpermute(int32_t n, int32_t off, int32_t width, int32_t stride, const double* __restrict__ src,
                            const int32_t* __restrict__ perm, double* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * width) return;
  const int64_t i = off + t / width, k = t % width;
  dst[(int64_t)(perm[i] - off) * width + k] = src[i * stride + k];
}

// time_stepping_kernels.h:63 with each node's own mesh's last min_dt.
__global__ void k_step_factors(int32_t n, int32_t off, const double* __restrict__ vol,
                               const unsigned long long* __restrict__ keys, const int32_t* __restrict__ mesh_id,
                               const int32_t* __restrict__ perm, double* __restrict__ dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t i = off + t;
  const unsigned long long k = keys[mesh_id ? mesh_id[i] : 0];
  dst[perm[i] - off] = dkey_inv(k) / vol[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side.


namespace {

int grid(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

int edge_threads(const mgcfd_solver* s) { return s->opt.block_size > 0 ? s->opt.block_size : 128; }

// Launchers indexed by the kernels' compile-time variants.
template <bool G, bool L, bool M, bool S>
void launch_update(int grid_n, cudaStream_t st, const UpdateArgs& A) {
  k_update<G, L, M, S><<<grid_n, kNodeThreads, 0, st>>>(A);
}
using UpdateFn = void (*)(int, cudaStream_t, const UpdateArgs&);
const UpdateFn kUpdate[16] = {
    launch_update<0, 0, 0, 0>, launch_update<0, 0, 0, 1>, launch_update<0, 0, 1, 0>, launch_update<0, 0, 1, 1>,
    launch_update<0, 1, 0, 0>, launch_update<0, 1, 0, 1>, launch_update<0, 1, 1, 0>, launch_update<0, 1, 1, 1>,
    launch_update<1, 0, 0, 0>, launch_update<1, 0, 0, 1>, launch_update<1, 0, 1, 0>, launch_update<1, 0, 1, 1>,
    launch_update<1, 1, 0, 0>, launch_update<1, 1, 0, 1>, launch_update<1, 1, 1, 0>, launch_update<1, 1, 1, 1>};

template <bool G, bool L, bool S>
void launch_update_dw(int grid_n, cudaStream_t st, const UpdateArgs& A) {
  k_update<G, L, false, S, false, false, 0, true><<<grid_n, kNodeThreads, 0, st>>>(A);
}
const UpdateFn kUpdateDW[8] = {launch_update_dw<0, 0, 0>, launch_update_dw<0, 0, 1>, launch_update_dw<0, 1, 0>,
                               launch_update_dw<0, 1, 1>, launch_update_dw<1, 0, 0>, launch_update_dw<1, 0, 1>,
                               launch_update_dw<1, 1, 0>, launch_update_dw<1, 1, 1>};

template <bool L, bool S>
void launch_update_dw_fused(int grid_n, cudaStream_t st, const UpdateArgs& A) {
  k_update<true, L, false, S, false, true, 0, true><<<grid_n, kNodeThreads, 0, st>>>(A);
}
const UpdateFn kUpdateDWFused[4] = {launch_update_dw_fused<0, 0>, launch_update_dw_fused<0, 1>,
                                    launch_update_dw_fused<1, 0>, launch_update_dw_fused<1, 1>};

template <bool L, bool S>
void launch_update_pair(int grid_n, cudaStream_t st, const UpdateArgs& A) {
  k_update<true, L, true, S, true><<<grid_n, kNodeThreads, 0, st>>>(A);
}
const UpdateFn kUpdatePair[4] = {launch_update_pair<0, 0>, launch_update_pair<0, 1>, launch_update_pair<1, 0>,
                                 launch_update_pair<1, 1>};

template <bool L, bool S, bool P, int V = 0>
void launch_update_fused(int grid_n, cudaStream_t st, const UpdateArgs& A) {
  k_update<true, L, true, S, P, true, V><<<grid_n, kNodeThreads, 0, st>>>(A);
}
// Indexed by variant (0 per-node loop, 1 staged ids, 2 edge-parallel) * 8 +
// last * 4 + seg * 2 + pair.
const UpdateFn kUpdateFused[24] = {
    launch_update_fused<0, 0, 0, 0>, launch_update_fused<0, 0, 1, 0>, launch_update_fused<0, 1, 0, 0>,
    launch_update_fused<0, 1, 1, 0>, launch_update_fused<1, 0, 0, 0>, launch_update_fused<1, 0, 1, 0>,
    launch_update_fused<1, 1, 0, 0>, launch_update_fused<1, 1, 1, 0>, launch_update_fused<0, 0, 0, 1>,
    launch_update_fused<0, 0, 1, 1>, launch_update_fused<0, 1, 0, 1>, launch_update_fused<0, 1, 1, 1>,
    launch_update_fused<1, 0, 0, 1>, launch_update_fused<1, 0, 1, 1>, launch_update_fused<1, 1, 0, 1>,
    launch_update_fused<1, 1, 1, 1>, launch_update_fused<0, 0, 0, 2>, launch_update_fused<0, 0, 1, 2>,
    launch_update_fused<0, 1, 0, 2>, launch_update_fused<0, 1, 1, 2>, launch_update_fused<1, 0, 0, 2>,
    launch_update_fused<1, 0, 1, 2>, launch_update_fused<1, 1, 0, 2>, launch_update_fused<1, 1, 1, 2>};

template <bool M, bool S, bool W = false>
void launch_step_begin(const DevLevel& D, unsigned long long* key, const DevStatus* st, const SegStop* ss,
                       cudaStream_t stream) {
  k_step_begin<M, S, W><<<grid(D.n, kNodeThreads), kNodeThreads, 0, stream>>>(D.n, D.rec, D.rec2, D.rec32, D.old,
                                                                               D.cbrt_vol, key, st, D.mesh_id, ss);
}
using StepFn = void (*)(const DevLevel&, unsigned long long*, const DevStatus*, const SegStop*, cudaStream_t);
// Indexed by precision (FP64, MIXED, DW) * 2 + seg.
const StepFn kStepBegin[6] = {launch_step_begin<0, 0>, launch_step_begin<0, 1>, launch_step_begin<1, 0>,
                              launch_step_begin<1, 1>, launch_step_begin<0, 0, 1>, launch_step_begin<0, 1, 1>};

// The level's min_dt key and, after a step, the copy of the key it used
// (for the step factors a fetch reports).
unsigned long long* level_key(mgcfd_solver* s, int level) {
  return s->nseg > 1 ? s->seg_keys + (size_t)level * s->nseg : &s->st->dt_key[level];
}
unsigned long long* level_key_used(mgcfd_solver* s, int level) {
  return s->nseg > 1 ? s->seg_keys + ((size_t)kMaxLevels + level) * s->nseg : &s->st->dt_key_used[level];
}

template <bool B, bool M, bool S, bool W>
void launch_prolong(const DevLevel& F, const DevLevel& Cl, const DevStatus* st, const SegStop* ss,
                    unsigned long long* key, cudaStream_t stream) {
  const BeginArgs b{F.rec2, F.rec32, F.old, F.cbrt_vol, key};
  k_prolong<B, M, S, W><<<grid(F.n, kNodeThreads), kNodeThreads, 0, stream>>>(F.n, F.n2mg, F.dvec, F.rec, F.res,
                                                                               Cl.res, st, F.mesh_id, ss, b);
}
using ProlongFn = void (*)(const DevLevel&, const DevLevel&, const DevStatus*, const SegStop*, unsigned long long*,
                           cudaStream_t);
// With the fine level's step begin, indexed by precision (FP64, MIXED, DW) * 2 + seg.
const ProlongFn kProlongBegin[6] = {launch_prolong<1, 0, 0, 0>, launch_prolong<1, 0, 1, 0>,
                                   launch_prolong<1, 1, 0, 0>, launch_prolong<1, 1, 1, 0>,
                                   launch_prolong<1, 0, 0, 1>, launch_prolong<1, 0, 1, 1>};

int precision_index(const mgcfd_solver* s) {
  return s->opt.precision == MGCFD_PRECISION_DW ? 2 : s->opt.precision == MGCFD_PRECISION_MIXED ? 1 : 0;
}

// Where the level-0 norms (calc_rms_kernel, count_bad_vals) are taken: in
// the last RK stage, or -- for plain multi-level solvers with the fused
// stage, whose warps finish at uneven times and idle at the stage's block
// reduction -- in the restriction that follows, which reads the same state
// and residuals (measured: 203.1 -> 206.4 V-cycles/s at 8M nodes; the FP64
// stage loses 1% the same way, so it keeps them).
bool norms_in_restrict(const mgcfd_solver* s) { return s->fused && s->nseg == 1 && s->L.size() > 1; }

// One smoothing step at `level` (euler3d.cpp:467-550).
int enqueue_smooth(mgcfd_solver* s, int level) {
  DevLevel& D = s->L[(size_t)level];
  const bool mixed = s->opt.precision == MGCFD_PRECISION_MIXED;
  const bool dw = s->opt.precision == MGCFD_PRECISION_DW;
  const bool timing = s->opt.time_kernels && level == 0;
  const bool seg = s->nseg > 1;
  unsigned long long* key = level_key(s, level);
  if (!s->begun) {  // no prolongation began this step: its own begin pass
    CK(cudaMemsetAsync(key, 0xff, sizeof(unsigned long long) * (size_t)s->nseg, s->stream));
    kStepBegin[2 * precision_index(s) + (seg ? 1 : 0)](D, key, s->st, seg ? s->seg_stop : nullptr, s->stream);
    s->launches++;
  }
  s->begun = false;
  if (level == 0) {
    CK(cudaMemsetAsync(&s->st->rms_acc, 0, 2 * sizeof(double), s->stream));  // rms_acc, rho_acc
    if (seg) {
      CK(cudaMemsetAsync(s->seg_rms, 0, sizeof(double) * (size_t)s->nseg, s->stream));
      CK(cudaMemsetAsync(s->seg_rho, 0, sizeof(double) * (size_t)s->nseg, s->stream));
    }
  }
  const int et = edge_threads(s);
  const bool pair = mixed && s->opt.accumulation == MGCFD_ACCUM_PAIR32;
  for (int rk = 0; rk < kRK; rk++) {
    const bool last = rk == kRK - 1;
    // Level-0 timing events wrap the flux sweep (the fused stage when the
    // flux is computed inside the node kernel).
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    const bool time_this = timing && D.ne > 0;
    if (time_this) {
      if (!s->spare.empty()) { ev = s->spare.back(); s->spare.pop_back(); }
      else {
        CK(cudaEventCreate(&ev.first));
        CK(cudaEventCreate(&ev.second));
      }
      CK(cudaEventRecord(ev.first, s->stream));
    }
    if (D.ne > 0 && s->coloured) {
      for (size_t c = 0; c + 1 < D.colour_off.size(); c++) {
        const int32_t lo = D.colour_off[c], cnt = D.colour_off[c + 1] - lo;
        if (cnt == 0) continue;
        k_flux_f64_coloured<<<grid(cnt, et), et, 0, s->stream>>>(cnt, D.e2n + lo, D.w4 + lo, D.rec, D.flux, s->st);
        s->launches++;
      }
      if (time_this) {
        CK(cudaEventRecord(ev.second, s->stream));
        s->pending.push_back(ev);
      }
    } else if (D.ne > 0 && !s->fused) {
      const int g = grid(D.ne, et);
      if (dw) {
        if (s->gather) k_flux_dw<true><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4dw, D.rec2, D.flux, D.fe, s->st);
        else k_flux_dw<false><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4dw, D.rec2, D.flux, D.fe, s->st);
      } else if (mixed) {
        if (s->gather) k_flux_mixed<true><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4f, D.rec32, D.flux, D.fe32, s->st);
        else k_flux_mixed<false><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4f, D.rec32, D.flux, D.fe32, s->st);
      } else {
        if (s->gather) k_flux_f64<true><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4, D.rec, D.flux, D.fe, s->st);
        else k_flux_f64<false><<<g, et, 0, s->stream>>>(D.ne, D.e2n, D.w4, D.rec, D.flux, D.fe, s->st);
      }
      s->launches++;
      if (time_this) {
        CK(cudaEventRecord(ev.second, s->stream));
        s->pending.push_back(ev);
      }
    }
    UpdateArgs A;
    A.n = D.n; A.level0 = level == 0 && !norms_in_restrict(s); A.inv_div = 1.0 / (double)(kRK + 1 - rk);
    A.rec = D.rec; A.rec2 = D.rec2; A.rec32 = D.rec32; A.old = D.old; A.flux = D.flux; A.fe = D.fe; A.fe32 = D.fe32;
    A.a_off = D.a_off; A.b_off = D.b_off; A.b_list = D.b_list; A.inv_vol = D.inv_vol; A.bidx = D.bidx;
    A.bdata = D.bdata; A.res = D.res; A.dt_key = key; A.st = s->st;
    A.mesh_id = D.mesh_id; A.seg_neg = s->seg_neg; A.seg_bad = s->seg_bad; A.seg_rms = s->seg_rms;
    A.seg_rho = s->seg_rho;
    A.seg_stop = seg ? s->seg_stop : nullptr;
    A.e2n = D.e2n; A.w4f = D.w4f; A.b_nbr = D.b_nbr; A.b_w4f = D.b_w4f;
    A.rec2_in = nullptr; A.off2 = D.off2; A.ent2 = D.ent2; A.w4dw = D.w4dw;
    if (s->fused && dw) {
      // Stage rk reads the primitives of stage rk and writes those of rk + 1
      // into the other buffer: k_step_begin fills rec2 for stage 0.
      A.rec2_in = (rk & 1) ? D.rec2b : D.rec2;
      A.rec2 = (rk & 1) ? D.rec2 : D.rec2b;
      A.rec32_in = nullptr;
      kUpdateDWFused[(last ? 2 : 0) | (seg ? 1 : 0)](grid(D.n, kNodeThreads), s->stream, A);
      if (time_this) {
        CK(cudaEventRecord(ev.second, s->stream));
        s->pending.push_back(ev);
      }
    } else if (s->fused) {
      // Stage rk reads the primitives of stage rk and writes those of rk + 1
      // into the other buffer: k_step_begin fills rec32 for stage 0.
      A.rec32_in = (rk & 1) ? D.rec32b : D.rec32;
      A.rec32 = (rk & 1) ? D.rec32 : D.rec32b;
      kUpdateFused[8 * s->fused_variant + ((last ? 4 : 0) | (seg ? 2 : 0) | (pair ? 1 : 0))](grid(D.n, kNodeThreads),
                                                                                           s->stream, A);
      if (time_this) {
        CK(cudaEventRecord(ev.second, s->stream));
        s->pending.push_back(ev);
      }
    } else if (mixed && s->gather && pair) {
      A.rec32_in = nullptr;
      kUpdatePair[(last ? 2 : 0) | (seg ? 1 : 0)](grid(D.n, kNodeThreads), s->stream, A);
    } else if (dw) {
      A.rec32_in = nullptr;
      kUpdateDW[(s->gather ? 4 : 0) | (last ? 2 : 0) | (seg ? 1 : 0)](grid(D.n, kNodeThreads), s->stream, A);
    } else {
      A.rec32_in = nullptr;
      kUpdate[(s->gather ? 8 : 0) | (last ? 4 : 0) | (mixed ? 2 : 0) | (seg ? 1 : 0)](grid(D.n, kNodeThreads), s->stream, A);
    }
    s->launches++;
    if (s->opt.measure_mem_bound && D.ne > 0) {
      k_stream<<<grid(D.ne, et), et, 0, s->stream>>>(D.ne, D.e2n, D.w4, D.rec, D.dummy, s->st);
      s->launches++;
    }
  }
  // The key this step used, for the step factors a fetch reports (a
  // prolongation may begin this level's next step before the fetch).
  CK(cudaMemcpyAsync(level_key_used(s, level), key, sizeof(unsigned long long) * (size_t)s->nseg,
                     cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaGetLastError());
  s->steps++;
  return MGCFD_OK;
}

// One iteration of the reference's while loop (euler3d.cpp:458-640).
int enqueue_iteration(mgcfd_solver* s) {
  const int levels = (int)s->L.size();
  const int64_t cycle0 = s->cycle;
  int r = enqueue_smooth(s, s->level);
  if (r) return r;
  if (levels <= 1) {
    s->cycle++;
  } else if (s->up) {
    s->level++;
    DevLevel& F = s->L[(size_t)s->level - 1];
    DevLevel& Cl = s->L[(size_t)s->level];
    const SegStop* ss = s->nseg > 1 ? s->seg_stop : nullptr;
    if (s->level == 1 && norms_in_restrict(s))  // level-0 norms of the step just smoothed
      k_restrict<true><<<grid(Cl.n, kNodeThreads), kNodeThreads, 0, s->stream>>>(Cl.n, Cl.ch_off, Cl.ch_list, F.rec,
                                                                                 Cl.rec, F.res, s->st, Cl.mesh_id, ss);
    else
      k_restrict<false><<<grid(Cl.n, kNodeThreads), kNodeThreads, 0, s->stream>>>(Cl.n, Cl.ch_off, Cl.ch_list, F.rec,
                                                                                  Cl.rec, nullptr, s->st, Cl.mesh_id, ss);
    s->launches++;
    if (s->level == levels - 1) s->up = false;
  } else {
    s->level--;
    DevLevel& F = s->L[(size_t)s->level];
    DevLevel& Cl = s->L[(size_t)s->level + 1];
    // The fine level's next smoothing step begins in the prolongation.
    unsigned long long* key = level_key(s, s->level);
    CK(cudaMemsetAsync(key, 0xff, sizeof(unsigned long long) * (size_t)s->nseg, s->stream));
    kProlongBegin[2 * precision_index(s) + (s->nseg > 1 ? 1 : 0)](F, Cl, s->st, s->nseg > 1 ? s->seg_stop : nullptr,
                                                                   key, s->stream);
    s->begun = true;
    s->launches++;
    if (s->level == 0) {
      s->up = true;
      s->cycle++;
    }
  }
  if (s->cycle != cycle0 && s->stop_max_cycles > 0) {  // a V-cycle just ended
    if (s->nseg > 1)
      k_cycle_end_seg<<<(unsigned)((s->nseg + 127) / 128), 128, 0, s->stream>>>(
          s->nseg, s->seg_stop, s->seg_rho, s->seg_n0, s->seg_neg, s->seg_bad, s->stop_max_cycles, s->stop_drop);
    else
      k_cycle_end<<<1, 1, 0, s->stream>>>(s->st, (double)s->L[0].n, s->stop_max_cycles, s->stop_drop);
    s->launches++;
  }
  CK(cudaGetLastError());
  return MGCFD_OK;
}

int enqueue_cycle(mgcfd_solver* s) {
  const int64_t target = s->cycle + 1;
  while (s->cycle < target) {
    int r = enqueue_iteration(s);
    if (r) return r;
  }
  return MGCFD_OK;
}

int collect_timings(mgcfd_solver* s) {
  for (auto& ev : s->pending) {
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, ev.first, ev.second));
    s->flux_ms += ms;
    s->flux_sweeps++;
    s->spare.push_back(ev);
  }
  s->pending.clear();
  return MGCFD_OK;
}

int read_status(mgcfd_solver* s) {
  if (s->nseg > 1) {  // batched: per-mesh outcome, the batch itself keeps going
    std::vector<int> neg((size_t)s->nseg), bad((size_t)s->nseg);
    CK(cudaMemcpy(neg.data(), s->seg_neg, sizeof(int) * neg.size(), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(bad.data(), s->seg_bad, sizeof(int) * bad.size(), cudaMemcpyDeviceToHost));
    for (int m = 0; m < s->nseg; m++)
      s->seg_status[(size_t)m] = neg[(size_t)m] ? MGCFD_ERR_NEGATIVE_DT : bad[(size_t)m] ? MGCFD_ERR_BAD_VALUES : MGCFD_OK;
    return MGCFD_OK;
  }
  DevStatus h;
  CK(cudaMemcpy(&h, s->st, sizeof(h), cudaMemcpyDeviceToHost));
  if (h.neg_dt) {
    double m = 0.0;
    for (int l = 0; l < (int)s->L.size(); l++) {
      unsigned long long k = h.dt_key[l];
      if (k != ~0ull) {
        unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
        double v;
        std::memcpy(&v, &u, 8);
        if (v < m) m = v;
      }
    }
    char buf[128];
    std::snprintf(buf, sizeof buf, "Fatal error during 'step factor' calculation, min_dt = %.5e", m);
    s->status = set_error(MGCFD_ERR_NEGATIVE_DT, buf);
  } else if (h.bad_count > 0) {
    s->status = set_error(MGCFD_ERR_BAD_VALUES, "Bad variable values detected, aborting");
  }
  return s->status;
}

int init_state(mgcfd_solver* s) {
  const double* v = s->ff.ff_variable;
  for (auto& D : s->L) {
    if (s->nseg > 1)
      k_init_state_seg<<<grid(D.n, kNodeThreads), kNodeThreads, 0, s->stream>>>(D.n, D.rec, D.mesh_id, s->seg_ffvar);
    else
      k_init_state<<<grid(D.n, kNodeThreads), kNodeThreads, 0, s->stream>>>(D.n, D.rec, v[0], v[1], v[2], v[3], v[4]);
    CK(cudaMemsetAsync(D.old, 0, sizeof(double) * 5 * (size_t)D.n, s->stream));
    CK(cudaMemsetAsync(D.res, 0, sizeof(double) * 5 * (size_t)D.n, s->stream));
    if (D.flux) CK(cudaMemsetAsync(D.flux, 0, sizeof(double) * 5 * (size_t)D.n, s->stream));
    if (D.dummy) CK(cudaMemsetAsync(D.dummy, 0, sizeof(double) * 5 * (size_t)D.n, s->stream));
  }
  CK(cudaMemsetAsync(s->st, 0, sizeof(DevStatus), s->stream));
  CK(cudaMemsetAsync(s->st->dt_key, 0xff, sizeof(s->st->dt_key), s->stream));
  CK(cudaMemsetAsync(s->st->dt_key_used, 0xff, sizeof(s->st->dt_key_used), s->stream));
  if (s->nseg > 1) {
    const size_t ns = (size_t)s->nseg;
    CK(cudaMemsetAsync(s->seg_keys, 0xff, sizeof(unsigned long long) * 2 * kMaxLevels * ns, s->stream));
    CK(cudaMemsetAsync(s->seg_neg, 0, sizeof(int) * ns, s->stream));
    CK(cudaMemsetAsync(s->seg_bad, 0, sizeof(int) * ns, s->stream));
    CK(cudaMemsetAsync(s->seg_rms, 0, sizeof(double) * ns, s->stream));
    CK(cudaMemsetAsync(s->seg_rho, 0, sizeof(double) * ns, s->stream));
    if (s->seg_stop) CK(cudaMemsetAsync(s->seg_stop, 0, sizeof(SegStop) * ns, s->stream));
  }
  s->seg_status.assign((size_t)s->nseg, MGCFD_OK);
  // The first V-cycle's first step begins here; every later V-cycle's
  // begins in the prolongation that ends the one before, so every V-cycle
  // (and the captured graph) has the same launches.  A one-level solver has
  // no prolongation: each of its steps begins on its own.
  s->begun = s->L.size() > 1;
  if (s->begun)
    kStepBegin[2 * precision_index(s) + (s->nseg > 1 ? 1 : 0)](s->L[0], level_key(s, 0), s->st, nullptr, s->stream);
  CK(cudaGetLastError());
  s->cycle = 0; s->level = 0; s->up = true; s->steps = 0; s->launches = 0;
  s->flux_ms = 0.0; s->flux_sweeps = 0; s->status = MGCFD_OK;
  for (auto& ev : s->pending) s->spare.push_back(ev);
  s->pending.clear();
  return MGCFD_OK;
}

void free_solver(mgcfd_solver* s) {
  if (!s) return;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  for (auto& ev : s->pending) { cudaEventDestroy(ev.first); cudaEventDestroy(ev.second); }
  for (auto& ev : s->spare) { cudaEventDestroy(ev.first); cudaEventDestroy(ev.second); }
  for (void* p : s->allocs) cudaFreeAsync(p, s->stream);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->owns_stream) cudaStreamDestroy(s->stream);
  delete s;
}

}  // namespace

namespace {
// COLOURED increment: greedy edge colouring of one level on the host (each
// edge takes the smallest colour that neither end node has used yet, in the
// level's sorted edge order), then the level's edges and weights reordered on
// the device into colour classes.  At most 64 classes (a node with more edges
// than that fails the set-up with MGCFD_ERR_INVALID); a lattice needs 7.
int colour_edges(mgcfd_solver* s, DevLevel& D) {
  D.colour_off.assign(1, 0);
  if (D.ne == 0) return MGCFD_OK;
  std::vector<int2> e2n((size_t)D.ne);
  CK(cudaMemcpyAsync(e2n.data(), D.e2n, sizeof(int2) * e2n.size(), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  std::vector<uint64_t> used((size_t)D.n, 0);
  std::vector<uint8_t> col((size_t)D.ne);
  int ncol = 0;
  for (size_t e = 0; e < e2n.size(); e++) {
    const uint64_t free_mask = ~(used[(size_t)e2n[e].x] | used[(size_t)e2n[e].y]);
    if (!free_mask) return set_error(MGCFD_ERR_INVALID, "coloured increment: a node has more than 64 edges");
    const int c = __builtin_ctzll(free_mask);
    col[e] = (uint8_t)c;
    used[(size_t)e2n[e].x] |= 1ull << c;
    used[(size_t)e2n[e].y] |= 1ull << c;
    ncol = std::max(ncol, c + 1);
  }
  std::vector<int32_t> off((size_t)ncol + 1, 0), idx((size_t)D.ne);
  for (uint8_t c : col) off[(size_t)c + 1]++;
  for (int c = 0; c < ncol; c++) off[(size_t)c + 1] += off[(size_t)c];
  std::vector<int32_t> fill(off.begin(), off.end() - 1);
  for (size_t e = 0; e < col.size(); e++) idx[(size_t)fill[col[e]]++] = (int32_t)e;  // stable within a colour
  int32_t* d_idx = nullptr;
  int2* e2n_tmp = nullptr;
  double4_32a* w4_tmp = nullptr;
  CK(cudaMallocAsync(reinterpret_cast<void**>(&d_idx), sizeof(int32_t) * idx.size(), s->stream));
  CK(cudaMallocAsync(reinterpret_cast<void**>(&e2n_tmp), sizeof(int2) * idx.size(), s->stream));
  CK(cudaMallocAsync(reinterpret_cast<void**>(&w4_tmp), sizeof(double4_32a) * idx.size(), s->stream));
  CK(cudaMemcpyAsync(d_idx, idx.data(), sizeof(int32_t) * idx.size(), cudaMemcpyHostToDevice, s->stream));
  k_gather_edges<<<grid(D.ne, 256), 256, 0, s->stream>>>(D.ne, d_idx, D.e2n, D.w4, e2n_tmp, w4_tmp);
  CK(cudaMemcpyAsync(D.e2n, e2n_tmp, sizeof(int2) * idx.size(), cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaMemcpyAsync(D.w4, w4_tmp, sizeof(double4_32a) * idx.size(), cudaMemcpyDeviceToDevice, s->stream));
  CK(cudaFreeAsync(d_idx, s->stream));
  CK(cudaFreeAsync(e2n_tmp, s->stream));
  CK(cudaFreeAsync(w4_tmp, s->stream));
  CK(cudaStreamSynchronize(s->stream));  // idx's host buffer
  CK(cudaGetLastError());
  D.colour_off = off;
  return MGCFD_OK;
}

// DW precision: one level's primitives as pair words (written by the node
// kernels) and its edge weights split into pairs, from the FP64 weights.
// FUSED: also the second primitive buffer and the per-node neighbour table
// (nb2, w2 from off2), from the CSR tables a_off, b_off and b_list.
int build_dw_tables(mgcfd_solver* s, DevLevel& D) {
  int r;
  if ((r = s->alloc(&D.rec2, 8 * (size_t)D.n)) || (r = s->alloc(&D.w4dw, (size_t)D.ne))) return r;
  const int64_t nw = 4 * (int64_t)D.ne;
  if (nw) {
    unsigned int* bad = nullptr;
    unsigned int nbad = 0;
    CK(cudaMallocAsync(&bad, sizeof(unsigned int), s->stream));
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned int), s->stream));
    k_split_weights<<<grid(nw, 256), 256, 0, s->stream>>>(nw, reinterpret_cast<const double*>(D.w4),
                                                          reinterpret_cast<double*>(D.w4dw), bad);
    CK(cudaMemcpyAsync(&nbad, bad, sizeof(unsigned int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaFreeAsync(bad, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (nbad)
      return set_error(MGCFD_ERR_INVALID, std::to_string(nbad) + " edge weight components outside the DW form's "
                                          "range [2^-70, 2^70); use FP64 precision for this mesh");
  }
  if (s->fused) {
    if ((r = s->alloc(&D.rec2b, 8 * (size_t)D.n)) || (r = s->alloc(&D.off2, (size_t)D.n + 1)) ||
        (r = s->alloc(&D.ent2, 2 * (size_t)D.ne)))
      return r;
    k_dw_offsets<<<grid((int64_t)D.n + 1, 256), 256, 0, s->stream>>>(D.n, D.a_off, D.b_off, D.off2);
    if (D.ne) {
      k_dw_table_a<<<grid(D.ne, 256), 256, 0, s->stream>>>(D.ne, D.e2n, D.a_off, D.off2, D.ent2);
      k_dw_table_b<<<grid(D.ne, 256), 256, 0, s->stream>>>(D.ne, D.e2n, D.b_list, D.a_off, D.b_off, D.off2, D.ent2);
    }
  }
  CK(cudaGetLastError());
  return MGCFD_OK;
}

// Increment strategy: AUTO is FP64 atomics for FP64, and the fused
// node-centric stage for mixed precision and DW (the fastest of each,
// measured; DW at 8M nodes: fused 248, gather 177, atomic 125 V-cycles/s).
int resolve_increment(mgcfd_solver* s) {
  const int inc = s->opt.increment;
  const bool mixed = s->opt.precision == MGCFD_PRECISION_MIXED;
  if (inc < MGCFD_INCREMENT_AUTO || inc > MGCFD_INCREMENT_COLOURED)
    return set_error(MGCFD_ERR_INVALID, "unknown increment strategy");
  const bool dw = s->opt.precision == MGCFD_PRECISION_DW;
  if (inc == MGCFD_INCREMENT_FUSED && !mixed && !dw)
    return set_error(MGCFD_ERR_INVALID, "the fused increment needs mixed or DW precision");
  if (dw && (s->opt.stage_neighbour_ids || s->opt.edge_parallel_stage))
    return set_error(MGCFD_ERR_INVALID, "the staged and edge-parallel fused variants are mixed-precision forms");
  if (inc == MGCFD_INCREMENT_COLOURED && s->opt.precision != MGCFD_PRECISION_FP64)
    return set_error(MGCFD_ERR_INVALID, "the coloured increment is an FP64 strategy");
  s->coloured = inc == MGCFD_INCREMENT_COLOURED;
  s->fused = inc == MGCFD_INCREMENT_FUSED || (inc == MGCFD_INCREMENT_AUTO && (mixed || dw));
  s->gather = s->fused || inc == MGCFD_INCREMENT_GATHER;
  s->fused_variant = !s->fused ? 0 : s->opt.edge_parallel_stage ? 2 : s->opt.stage_neighbour_ids ? 1 : 0;
  return MGCFD_OK;
}
}  // namespace

extern "C" void mgcfd_solver_default_options(mgcfd_solver_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = MGCFD_PRECISION_FP64;
  o->increment = MGCFD_INCREMENT_AUTO;
  o->renumber = MGCFD_RENUMBER_SPATIAL;
  o->use_graph = 1;
}

extern "C" int mgcfd_solver_create(int32_t nlevels, const mgcfd_level_view* levels, double mach, double aoa_deg,
                                   const mgcfd_solver_options* opt, void* stream, mgcfd_solver** out) {
  if (!out) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_create: null output");
  *out = nullptr;
  if (nlevels < 1 || nlevels > kMaxLevels) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_create: 1..16 levels supported");
  std::unique_ptr<mgcfd_solver, void (*)(mgcfd_solver*)> s(new (std::nothrow) mgcfd_solver(), free_solver);
  if (!s) return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  int r0;
  if (opt) s->opt = *opt; else mgcfd_solver_default_options(&s->opt);
  if (s->opt.precision < MGCFD_PRECISION_FP64 || s->opt.precision > MGCFD_PRECISION_DW)
    return set_error(MGCFD_ERR_INVALID, "unknown precision");
  if (s->opt.accumulation != MGCFD_ACCUM_FP64 && s->opt.accumulation != MGCFD_ACCUM_PAIR32)
    return set_error(MGCFD_ERR_INVALID, "unknown accumulation");
  if (s->opt.block_size < 0 || s->opt.block_size > 1024 || (s->opt.block_size % 32) != 0)
    return set_error(MGCFD_ERR_INVALID, "block_size must be 0 or a multiple of 32 up to 1024");
  if ((r0 = resolve_increment(s.get()))) return r0;
  s->stream = static_cast<cudaStream_t>(stream);
  CK(cudaGetDevice(&s->device));
  if (!s->stream) {
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->owns_stream = true;
  }
  mgcfd_freestream_init(mach, aoa_deg, &s->ff);

  keep_freed_memory(s->device);
  s->L.resize((size_t)nlevels);
  size_t max_n = 0;
  for (int l = 0; l < nlevels; l++) max_n = std::max(max_n, (size_t)levels[l].nnodes);
  int r;
  const bool host_setup = s->opt.host_setup || s->opt.renumber == MGCFD_RENUMBER_RCM;
  if (!host_setup) {
    if ((r = validate_views(nlevels, levels, false))) return r;
    if ((r = device_prepare(s.get(), {MeshInput{levels, s->ff}}))) return r;
  }
  std::vector<PreparedLevel> P;
  if (host_setup) {
    s->seg_noff.assign((size_t)nlevels, std::vector<int32_t>(2, 0));
    for (int l = 0; l < nlevels; l++) s->seg_noff[(size_t)l][1] = levels[l].nnodes;
    try {
      r = prepare_mesh(nlevels, levels, s->ff, s->opt.renumber, s->opt.precision == MGCFD_PRECISION_MIXED, &P);
    } catch (const std::bad_alloc&) {
      return set_error(MGCFD_ERR_NOMEM, "host allocation failed while preparing the mesh");
    }
    if (r) return r;
  }
  const bool mixed = s->opt.precision == MGCFD_PRECISION_MIXED;
  for (int l = 0; host_setup && l < nlevels; l++) {
    PreparedLevel& p = P[(size_t)l];
    DevLevel& D = s->L[(size_t)l];
    D.n = p.n; D.ne = p.ne; D.nb = p.nb; D.nbrows = p.nb;
    if (l > 0) D.nfine = P[(size_t)l - 1].n;
    if ((r = s->alloc(&D.rec, 8 * (size_t)p.n)) || (r = s->alloc(&D.old, 5 * (size_t)p.n)) ||
        (r = s->alloc(&D.res, 5 * (size_t)p.n)) || (r = s->alloc(&D.inv_vol, (size_t)p.n)) ||
        (r = s->alloc(&D.cbrt_vol, (size_t)p.n)) ||
        (r = s->upload(&D.vol, p.vol.data(), (size_t)p.n)) ||
        (r = s->upload(&D.e2n, p.e2n.data(), (size_t)p.ne)) ||
        (r = s->upload(&D.bidx, p.bidx.data(), (size_t)p.n)) ||
        (r = s->upload(&D.bdata, p.bdata.data(), p.bdata.size())) ||
        (r = s->upload(&D.perm, p.perm.data(), (size_t)p.n)))
      return r;
    k_vol_constants<<<grid(p.n, kNodeThreads), kNodeThreads, 0, s->stream>>>(p.n, D.vol, D.inv_vol, D.cbrt_vol);
    if (mixed) {
      std::vector<float> w4f((size_t)p.ne * 4);
      for (size_t k = 0; k < w4f.size(); k++) w4f[k] = (float)p.w4[k];
      if ((r = s->alloc(&D.rec32, 8 * (size_t)p.n)) || (r = s->upload(&D.w4f, w4f.data(), (size_t)p.ne))) return r;
      // Compute-bound only on the FP64 path; mixed still needs FP64 weights for the -b probe.
      if (s->opt.measure_mem_bound && (r = s->upload(&D.w4, p.w4.data(), (size_t)p.ne))) return r;
      CK(cudaStreamSynchronize(s->stream));  // w4f host buffer goes out of scope
    } else {
      if ((r = s->upload(&D.w4, p.w4.data(), (size_t)p.ne))) return r;
    }
    if (s->gather) {
      if ((r = s->upload(&D.a_off, p.a_off.data(), (size_t)p.n + 1)) ||
          (r = s->upload(&D.b_off, p.b_off.data(), (size_t)p.n + 1)) ||
          (r = s->upload(&D.b_list, p.b_list.data(), (size_t)p.ne)))
        return r;
      if (s->fused) r = build_fused_tables(s.get(), D);
      else if (mixed) r = s->alloc(&D.fe32, 5 * (size_t)p.ne);
      else r = s->alloc(&D.fe, 5 * (size_t)p.ne);
      if (r) return r;
    } else {
      if ((r = s->alloc(&D.flux, 5 * (size_t)p.n))) return r;
    }
    if (s->opt.measure_mem_bound && (r = s->alloc(&D.dummy, 5 * (size_t)p.n))) return r;
    if (!p.n2mg.empty() && ((r = s->upload(&D.n2mg, p.n2mg.data(), (size_t)p.n)) ||
                            (r = s->upload(&D.dvec, p.dvec.data(), (size_t)p.n))))
      return r;
    if (!p.ch_off.empty() && ((r = s->upload(&D.ch_off, p.ch_off.data(), p.ch_off.size())) ||
                              (r = s->upload(&D.ch_list, p.ch_list.data(), p.ch_list.size()))))
      return r;
    // The host vectors of this level die at the end of create: finish the copies first.
    CK(cudaStreamSynchronize(s->stream));
  }
  for (auto& D : s->L) {
    if (s->coloured && (r = colour_edges(s.get(), D))) return r;
    if (s->opt.precision == MGCFD_PRECISION_DW && (r = build_dw_tables(s.get(), D))) return r;
  }
  if ((r = s->alloc(&s->st, 1)) || (r = s->alloc(&s->fetch_buf, 5 * max_n))) return r;
  if ((r = init_state(s.get()))) return r;
  CK(cudaStreamSynchronize(s->stream));
  *out = s.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_batch_create(int32_t nmeshes, int32_t nlevels, const mgcfd_level_view* const* levels,
                                  const double* mach, const double* aoa_deg, const mgcfd_solver_options* opt,
                                  void* stream, mgcfd_solver** out) {
  if (!out) return set_error(MGCFD_ERR_INVALID, "mgcfd_batch_create: null output");
  *out = nullptr;
  if (nmeshes < 1 || !levels || !mach || !aoa_deg) return set_error(MGCFD_ERR_INVALID, "mgcfd_batch_create: no meshes");
  if (nlevels < 1 || nlevels > kMaxLevels) return set_error(MGCFD_ERR_INVALID, "mgcfd_batch_create: 1..16 levels supported");
  std::unique_ptr<mgcfd_solver, void (*)(mgcfd_solver*)> s(new (std::nothrow) mgcfd_solver(), free_solver);
  if (!s) return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  int r0;
  if (opt) s->opt = *opt; else mgcfd_solver_default_options(&s->opt);
  if (s->opt.precision < MGCFD_PRECISION_FP64 || s->opt.precision > MGCFD_PRECISION_DW)
    return set_error(MGCFD_ERR_INVALID, "unknown precision");
  if (s->opt.accumulation != MGCFD_ACCUM_FP64 && s->opt.accumulation != MGCFD_ACCUM_PAIR32)
    return set_error(MGCFD_ERR_INVALID, "unknown accumulation");
  if (s->opt.block_size < 0 || s->opt.block_size > 1024 || (s->opt.block_size % 32) != 0)
    return set_error(MGCFD_ERR_INVALID, "block_size must be 0 or a multiple of 32 up to 1024");
  if (s->opt.renumber == MGCFD_RENUMBER_RCM || s->opt.host_setup)
    return set_error(MGCFD_ERR_INVALID, "batched solvers are set up on the device (renumber none or spatial)");
  if ((r0 = resolve_increment(s.get()))) return r0;
  if (s->coloured) return set_error(MGCFD_ERR_INVALID, "the coloured increment is for single-mesh solvers");
  s->stream = static_cast<cudaStream_t>(stream);
  CK(cudaGetDevice(&s->device));
  if (!s->stream) {
    CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->owns_stream = true;
  }
  keep_freed_memory(s->device);
  int r;
  std::vector<MeshInput> meshes((size_t)nmeshes);
  s->seg_ff.resize((size_t)nmeshes);
  std::vector<double> ffvar(5 * (size_t)nmeshes);
  int64_t total0 = 0;
  for (int m = 0; m < nmeshes; m++) {
    if ((r = validate_views(nlevels, levels[m], false))) return r;
    mgcfd_freestream_init(mach[m], aoa_deg[m], &s->seg_ff[(size_t)m]);
    meshes[(size_t)m] = MeshInput{levels[m], s->seg_ff[(size_t)m]};
    for (int k = 0; k < 5; k++) ffvar[5 * (size_t)m + k] = s->seg_ff[(size_t)m].ff_variable[k];
    total0 += levels[m][0].nnodes;
  }
  if (total0 > 2147483647ll) return set_error(MGCFD_ERR_INVALID, "batch too large for int32 node ids");
  s->ff = s->seg_ff[0];
  s->nseg = nmeshes;
  s->L.resize((size_t)nlevels);
  if ((r = device_prepare(s.get(), meshes))) return r;
  for (auto& D : s->L)
    if (s->opt.precision == MGCFD_PRECISION_DW && (r = build_dw_tables(s.get(), D))) return r;
  size_t max_n = 0;
  for (auto& D : s->L) max_n = std::max(max_n, (size_t)D.n);
  const size_t ns = (size_t)nmeshes;
  if ((r = s->alloc(&s->st, 1)) || (r = s->alloc(&s->fetch_buf, 5 * max_n)) ||
      (r = s->alloc(&s->seg_keys, 2 * kMaxLevels * ns)) || (r = s->alloc(&s->seg_neg, ns)) ||
      (r = s->alloc(&s->seg_bad, ns)) || (r = s->alloc(&s->seg_rms, ns)) || (r = s->alloc(&s->seg_rho, ns)) ||
      (r = s->upload(&s->seg_ffvar, ffvar.data(), 5 * ns)))
    return r;
  CK(cudaStreamSynchronize(s->stream));  // ffvar host buffer
  if ((r = init_state(s.get()))) return r;
  CK(cudaStreamSynchronize(s->stream));
  *out = s.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_solver_reset(mgcfd_solver* s) {
  if (!s) return set_error(MGCFD_ERR_INVALID, "null solver");
  CK(cudaStreamSynchronize(s->stream));
  return init_state(s);
}

extern "C" int mgcfd_solver_run(mgcfd_solver* s, int32_t ncycles) {
  if (!s) return set_error(MGCFD_ERR_INVALID, "null solver");
  if (ncycles < 0) return set_error(MGCFD_ERR_INVALID, "negative cycle count");
  if (s->status) return s->status;
  if (s->level != 0 || !s->up) return set_error(MGCFD_ERR_INVALID, "solver is not at a V-cycle boundary");
  const bool use_graph = s->opt.use_graph && !s->opt.time_kernels;
  for (int32_t c = 0; c < ncycles; c++) {
    if (use_graph) {
      if (!s->graph) {
        // Capture one V-cycle; its launch sequence is the same every cycle.
        cudaGraph_t g;
        const int64_t l0 = s->launches, st0 = s->steps, c0 = s->cycle;
        CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int r = enqueue_cycle(s);
        cudaError_t ce = cudaStreamEndCapture(s->stream, &g);
        if (r) return r;
        if (ce != cudaSuccess) return set_error(MGCFD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        cudaError_t ie = cudaGraphInstantiate(&s->graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return set_error(MGCFD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        s->launches_per_cycle = s->launches - l0;
        s->launches = l0; s->steps = st0; s->cycle = c0;
      }
      CK(cudaGraphLaunch(s->graph, s->stream));
      s->launches += s->launches_per_cycle;
      s->steps += (int64_t)(s->L.size() <= 1 ? 1 : 2 * s->L.size() - 2);
      s->cycle++;
    } else {
      int r = enqueue_cycle(s);
      if (r) return r;
    }
  }
  return MGCFD_OK;
}

int mgcfd::build_fused_tables(mgcfd_solver* s, DevLevel& D) {
  if (s->opt.precision == MGCFD_PRECISION_DW) return MGCFD_OK;  // its own tables: build_dw_tables
  int r;
  if ((r = s->alloc(&D.rec32b, 8 * (size_t)D.n)) || (r = s->alloc(&D.b_nbr, (size_t)D.ne)) ||
      (r = s->alloc(&D.b_w4f, (size_t)D.ne)))
    return r;
  if (D.ne > 0)
    k_bside<<<(unsigned)((D.ne + 255) / 256), 256, 0, s->stream>>>(D.ne, D.b_list, D.e2n, D.w4f, D.b_nbr, D.b_w4f);
  CK(cudaGetLastError());
  return MGCFD_OK;
}

int mgcfd::solver_retarget(mgcfd_solver* s, double mach, double aoa_deg) {
  if (!s || s->nseg > 1) return set_error(MGCFD_ERR_INVALID, "retarget: plain solvers only");
  int r = mgcfd_freestream_init(mach, aoa_deg, &s->ff);
  if (r) return r;
  for (auto& D : s->L)
    if (D.nbrows > 0)
      k_bnd_ffw<<<(unsigned)((D.nbrows + 127) / 128), 128, 0, s->stream>>>(D.nbrows, D.bdata, s->ff);
  CK(cudaGetLastError());
  return init_state(s);
}

int mgcfd::solver_set_stop_rule(mgcfd_solver* s, int32_t max_cycles, double residual_drop) {
  if (!s || max_cycles < 1 || s->graph || s->cycle > 0)
    return set_error(MGCFD_ERR_INVALID, "stop rule: before the solver's first cycle only");
  if (s->nseg > 1 && !s->seg_stop) {
    const size_t ns = (size_t)s->nseg;
    std::vector<double> n0(ns);
    for (size_t m = 0; m < ns; m++) n0[m] = (double)(s->seg_noff[0][m + 1] - s->seg_noff[0][m]);
    int r;
    if ((r = s->alloc(&s->seg_stop, ns)) || (r = s->upload(&s->seg_n0, n0.data(), ns))) return r;
    CK(cudaMemsetAsync(s->seg_stop, 0, sizeof(SegStop) * ns, s->stream));
    CK(cudaStreamSynchronize(s->stream));  // n0's host buffer
  }
  s->stop_max_cycles = max_cycles;
  s->stop_drop = residual_drop;
  return MGCFD_OK;
}

extern "C" int mgcfd_solver_step(mgcfd_solver* s, int32_t* smoothed_level, int64_t* cycles_done) {
  if (!s) return set_error(MGCFD_ERR_INVALID, "null solver");
  if (s->status) return s->status;
  const int level = s->level;
  int r = enqueue_iteration(s);
  if (r) return r;
  if (smoothed_level) *smoothed_level = level;
  if (cycles_done) *cycles_done = s->cycle;
  return MGCFD_OK;
}

extern "C" int mgcfd_solver_synchronize(mgcfd_solver* s) {
  if (!s) return set_error(MGCFD_ERR_INVALID, "null solver");
  CK(cudaStreamSynchronize(s->stream));
  int r = collect_timings(s);
  if (r) return r;
  return read_status(s);
}

namespace {
int fetch_rows(mgcfd_solver* s, int32_t level, int32_t q, int32_t off, int32_t n, double* host_out) {
  DevLevel& D = s->L[(size_t)level];
  const int T = 256;
  int width = 5;
  const unsigned long long* keys = level_key_used(s, level);
  switch (q) {
    case MGCFD_Q_VARIABLES:
      k_unpermute<<<grid((int64_t)n * 5, T), T, 0, s->stream>>>(n, off, 5, 8, D.rec, D.perm, s->fetch_buf);
      break;
    case MGCFD_Q_FLUXES:
      if (D.flux) k_unpermute<<<grid((int64_t)n * 5, T), T, 0, s->stream>>>(n, off, 5, 5, D.flux, D.perm, s->fetch_buf);
      else CK(cudaMemsetAsync(s->fetch_buf, 0, sizeof(double) * 5 * (size_t)n, s->stream));
      break;
    case MGCFD_Q_RESIDUALS:
      k_unpermute<<<grid((int64_t)n * 5, T), T, 0, s->stream>>>(n, off, 5, 5, D.res, D.perm, s->fetch_buf);
      break;
    case MGCFD_Q_OLD_VARIABLES:
      k_unpermute<<<grid((int64_t)n * 5, T), T, 0, s->stream>>>(n, off, 5, 5, D.old, D.perm, s->fetch_buf);
      break;
    case MGCFD_Q_VOLUMES:
      width = 1;
      k_unpermute<<<grid(n, T), T, 0, s->stream>>>(n, off, 1, 1, D.vol, D.perm, s->fetch_buf);
      break;
    case MGCFD_Q_STEP_FACTORS:
      width = 1;
      k_step_factors<<<grid(n, T), T, 0, s->stream>>>(n, off, D.vol, keys, D.mesh_id, D.perm, s->fetch_buf);
      break;
    default:
      return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch: unknown quantity");
  }
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(host_out, s->fetch_buf, sizeof(double) * (size_t)width * (size_t)n, cudaMemcpyDeviceToHost,
                     s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return MGCFD_OK;
}
}  // namespace

extern "C" int mgcfd_solver_fetch(mgcfd_solver* s, int32_t level, int32_t q, double* host_out) {
  if (!s || !host_out) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch: null argument");
  if (level < 0 || level >= (int)s->L.size()) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch: bad level");
  return fetch_rows(s, level, q, 0, s->L[(size_t)level].n, host_out);
}

extern "C" int mgcfd_solver_fetch_mesh(mgcfd_solver* s, int32_t mesh, int32_t level, int32_t q, double* host_out) {
  if (!s || !host_out) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch_mesh: null argument");
  if (level < 0 || level >= (int)s->L.size()) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch_mesh: bad level");
  if (mesh < 0 || mesh >= s->nseg) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_fetch_mesh: bad mesh");
  const int32_t off = s->seg_noff[(size_t)level][(size_t)mesh];
  return fetch_rows(s, level, q, off, s->seg_noff[(size_t)level][(size_t)mesh + 1] - off, host_out);
}

extern "C" int mgcfd_solver_num_meshes(const mgcfd_solver* s) { return s ? s->nseg : 0; }

extern "C" int mgcfd_solver_mesh_status(mgcfd_solver* s, int32_t mesh, double* rms_l0, double* rho_rms_l0) {
  if (!s || mesh < 0 || mesh >= s->nseg) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_mesh_status: bad mesh");
  int r = mgcfd_solver_synchronize(s);
  if (r && s->nseg > 1) return r;
  double acc[2] = {0.0, 0.0};
  const double n0 = (double)(s->seg_noff[0][(size_t)mesh + 1] - s->seg_noff[0][(size_t)mesh]);
  if (s->nseg > 1) {
    CK(cudaMemcpy(&acc[0], s->seg_rms + mesh, sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&acc[1], s->seg_rho + mesh, sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    CK(cudaMemcpy(acc, &s->st->rms_acc, 2 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (rms_l0) *rms_l0 = std::sqrt(acc[0] / n0);      // euler3d.cpp:537
  if (rho_rms_l0) *rho_rms_l0 = std::sqrt(acc[1] / n0);
  return s->nseg > 1 ? s->seg_status[(size_t)mesh] : r;
}

extern "C" int mgcfd_solver_get_stats(mgcfd_solver* s, mgcfd_solver_stats* o) {
  if (!s || !o) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_get_stats: null argument");
  int r = mgcfd_solver_synchronize(s);
  std::memset(o, 0, sizeof(*o));
  o->cycles = s->cycle;
  o->smoothing_steps = s->steps;
  o->flux_sweeps_l0 = s->flux_sweeps;
  o->flux_ms_l0 = s->flux_ms;
  o->kernel_launches = s->launches;
  o->device_bytes = s->device_bytes;
  DevStatus h;
  CK(cudaMemcpy(&h, s->st, sizeof(h), cudaMemcpyDeviceToHost));
  o->rms_l0 = std::sqrt(h.rms_acc / (double)s->L[0].n);  // euler3d.cpp:537
  o->status = r;
  return MGCFD_OK;
}

extern "C" int mgcfd_solver_table(mgcfd_solver* s, int32_t level, int32_t table, void* out, int64_t cap,
                                  int64_t* bytes) {
  if (!s || !bytes) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_table: null argument");
  if (level < 0 || level >= (int)s->L.size()) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_table: bad level");
  const DevLevel& D = s->L[(size_t)level];
  const void* src = nullptr;
  int64_t n = 0;
  switch (table) {
    case MGCFD_T_PERM: src = D.perm; n = 4ll * D.n; break;
    case MGCFD_T_EDGES: src = D.e2n; n = 8ll * D.ne; break;
    case MGCFD_T_WEIGHTS: src = D.w4; n = D.w4 ? 32ll * D.ne : 0; break;
    case MGCFD_T_VOLUMES: src = D.vol; n = 8ll * D.n; break;
    case MGCFD_T_INV_VOL: src = D.inv_vol; n = 8ll * D.n; break;
    case MGCFD_T_CBRT_VOL: src = D.cbrt_vol; n = 8ll * D.n; break;
    case MGCFD_T_BIDX: src = D.bidx; n = 4ll * D.n; break;
    case MGCFD_T_BDATA: src = D.bdata; n = 96ll * D.nbrows; break;
    case MGCFD_T_N2MG: src = D.n2mg; n = D.n2mg ? 4ll * D.n : 0; break;
    case MGCFD_T_DVEC: src = D.dvec; n = D.dvec ? 32ll * D.n : 0; break;
    case MGCFD_T_CH_OFF: src = D.ch_off; n = D.ch_off ? 4ll * (D.n + 1) : 0; break;
    case MGCFD_T_CH_LIST: src = D.ch_list; n = D.ch_list ? 4ll * D.nfine : 0; break;
    case MGCFD_T_A_OFF: src = D.a_off; n = D.a_off ? 4ll * (D.n + 1) : 0; break;
    case MGCFD_T_B_OFF: src = D.b_off; n = D.b_off ? 4ll * (D.n + 1) : 0; break;
    case MGCFD_T_B_LIST: src = D.b_list; n = D.b_list ? 4ll * D.ne : 0; break;
    case MGCFD_T_WEIGHTS32: src = D.w4f; n = D.w4f ? 16ll * D.ne : 0; break;
    default: return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_table: unknown table");
  }
  *bytes = src ? n : 0;
  if (!src || n == 0 || !out) return MGCFD_OK;  // out == NULL: size query
  if (cap < n) return set_error(MGCFD_ERR_INVALID, "mgcfd_solver_table: output too small");
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(out, src, (size_t)n, cudaMemcpyDeviceToHost));
  return MGCFD_OK;
}

extern "C" void mgcfd_solver_destroy(mgcfd_solver* s) { free_solver(s); }

extern "C" int mgcfd_solve(int32_t nlevels, const mgcfd_level_view* levels, double mach, double aoa_deg,
                           int32_t ncycles, const mgcfd_solver_options* opt, double* const* out_variables) {
  if (!out_variables) return set_error(MGCFD_ERR_INVALID, "mgcfd_solve: null output");
  mgcfd_solver* s = nullptr;
  int r = mgcfd_solver_create(nlevels, levels, mach, aoa_deg, opt, nullptr, &s);
  if (r) return r;
  r = mgcfd_solver_run(s, ncycles);
  if (!r) r = mgcfd_solver_synchronize(s);
  for (int l = 0; !r && l < nlevels; l++)
    if (out_variables[l]) r = mgcfd_solver_fetch(s, l, MGCFD_Q_VARIABLES, out_variables[l]);
  mgcfd_solver_destroy(s);
  return r;
}
