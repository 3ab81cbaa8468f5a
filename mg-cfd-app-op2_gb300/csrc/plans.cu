// Execution plans of the per-loop entry points: what OP2's CUDA backend
// builds and caches for an indirect loop the first time it runs (op_plan_get:
// a block partition and colouring per loop, set and map), re-designed for
// GB300.  A plan holds only integer structure derived from a map, never data
// values, and is cached per (device, map pointer, set sizes) for the life of
// the process (or until mgcfd_op_plans_release).
//
// Edge plan (compute_flux_edge_kernel, flux.h:41-208; euler3d.cpp:498-503).
// Naively, every edge gathers both end nodes' states, recomputes their
// primitives (one reciprocal and two square roots each), recomputes |w| and
// issues ten FP64 atomics at the caller's node numbering.  On a mesh whose
// node ids are scattered those atomics hit random HBM rows (about 28 G
// atomics/s on GB300, 8.5 ms for 24M edges).  The plan instead holds
//   * an internal node order with locality: the caller's own order when its
//     edges already join nearby ids, else a Cuthill-McKee order built on the
//     device (breadth-first levels from a low-degree node, each level's nodes
//     ordered by their earliest neighbour in the previous level, ties by id);
//   * the valid edges in that order, oriented a <= b and sorted by (a, b),
//     each with its caller edge index (complemented when the orientation
//     flipped, which negates the weight: flux(b, a, -w) = -flux(a, b, w));
//   * per edge, the last weight seen as (-w/2 or w/2, -|w|*smoothing/2), used
//     again while the caller's weight keeps the same bits (an integer
//     compare), so |w| is recomputed only when the weight changes;
//   * work space for the nodes' primitives in internal order and, when the
//     order is not the caller's, the internal increments.
// A call then runs three kernels: primitives of every node once (gathered
// from the caller's state), the edge fluxes with FP64 atomics into internal
// rows that sit close together (so they resolve in L2), and the addition of
// the internal increments onto the caller's flux rows (each caller row
// gathers its internal row: the order is a bijection, no atomics).  With the
// caller's own order the last step is skipped and the atomics go straight to
// the caller's rows.
//
// Children plan (up_pre_kernel / up_kernel, mg.h:29-52; euler3d.cpp:581-588).
// The fine-to-coarse map's children of every coarse node as a CSR list
// (children ordered by fine id), so up_kernel becomes a gather per coarse
// node -- no atomics, deterministic -- with the reference's per-call effect:
// coarse += sum of its children, count += number of children.
//
// Plans are built on the caller's stream and synchronise it (the level-by-
// level breadth-first search reads each level's size on the host), so the
// first call on a map blocks, and a first call made while the stream is
// capturing a CUDA graph runs the plan-free kernels instead.  Calls that use
// the same plan share its work space: run them in stream order, as OP2 runs
// its loops.  Map entries out of range are left out of a plan and reported
// as skipped on every call, as the plan-free kernels do.
#include <cub/cub.cuh>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "common.h"
#include "device_math.cuh"
#include "dw_math.cuh"
#include "plans.h"
#include "solver_internal.h"

namespace mgcfd {

struct EdgePlan {
  int32_t ne = 0, nn = 0;
  int32_t nvalid = 0;       // edges with both ends in range
  int64_t nbad = 0;         // edges skipped (an end out of range)
  bool permuted = false;    // internal order differs from the caller's
  int32_t* perm = nullptr;  // [nn] internal node -> caller node (permuted only)
  int32_t* pos = nullptr;   // [nn] caller node -> internal node (permuted only)
  int2* e2n = nullptr;      // [nvalid] internal (a, b), a <= b, sorted
  int32_t* eref = nullptr;  // [nvalid] caller edge index, complemented when flipped
  double4_32a* memo = nullptr;  // [nvalid] (h, wfac) of the last weight seen
  double memo_sc = NAN;     // smoothing coefficient of the memo (NaN: never used)
  double* rec = nullptr;    // [nn][8] state + primitives, internal order
  double* fl = nullptr;     // [nn][5] internal increments (permuted only)
  // DW form (built on the first call with DW flux precision): each internal
  // node's entries -- its a-side edges, then its b-side ones -- a memo of its
  // own and the pair-word buffers.
  bool dw_built = false;
  int32_t* off2 = nullptr;          // [nn + 1] each node's entries in ent2
  int2* ent2 = nullptr;             // [2 nvalid] (neighbour, edge; bit 31 set on the b side)
  int32_t* inv_e = nullptr;        // [ne] caller edge -> internal edge (bit 31: flipped; kNoEdge: left out)
  double* wcopy = nullptr;          // [ne][3] the caller's weights of the last DW call, caller order
  double4_32a* memo_dw = nullptr;   // [nvalid] (h, wfac) of those weights as pair words
  double memo_dw_sc = NAN;          // smoothing coefficient of memo_dw (NaN: never used)
  double* rec2 = nullptr;           // [nn][8] pair-word primitives, internal order
  int64_t bytes = 0;
};

struct ChildPlan {
  int32_t nf = 0, nc = 0;
  int64_t nbad = 0;             // fine nodes whose map entry is out of range
  int32_t* ch_off = nullptr;    // [nc + 1]
  int32_t* ch_list = nullptr;   // [nf - nbad] fine ids, by coarse node then fine id
  int64_t bytes = 0;
};

struct VolPlan {
  int32_t n = 0;
  double* vcopy = nullptr;  // [n] the volumes the roots were taken of (bits)
  double* root = nullptr;   // [n] cbrt of those volumes
  int64_t bytes = 0;
};

namespace {

constexpr int kT = 256;
constexpr int kMaxComponents = 64;  // breadth-first searches before the rest is appended in id order
// Breadth-first levels at most (each reads its size on the host): a mesh
// whose graph is a long chain stops there and the rest follows in id order,
// so the first call never takes more than a fraction of a second per level
// cap; results do not depend on the order, only locality does.
constexpr int kMaxBfsLevels = 16384;

int grid(int64_t n, int t = kT) { return (int)((n + t - 1) / t); }

int bits_for(int64_t n) {  // bits needed to hold 0..n
  int b = 1;
  while (b < 63 && (1ll << b) <= n) b++;
  return b;
}

// Stream-ordered scratch for one plan build, freed at the end of the build.
struct Scratch {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t st) : s(st) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
  template <class T>
  int get(T** p, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, count * sizeof(T) + 16, s);
    if (e != cudaSuccess) return set_error(MGCFD_ERR_NOMEM, std::string("plan scratch: ") + cudaGetErrorString(e));
    ptrs.push_back(q);
    *p = static_cast<T*>(q);
    return MGCFD_OK;
  }
};

template <class T>
int plan_alloc(T** p, size_t count, int64_t* bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
  if (e != cudaSuccess) return set_error(MGCFD_ERR_NOMEM, std::string("plan memory: ") + cudaGetErrorString(e));
  *p = static_cast<T*>(q);
  *bytes += (int64_t)(count * sizeof(T) + 16);
  return MGCFD_OK;
}

__device__ __forceinline__ bool in_range(int32_t i, int32_t n) { return (uint32_t)i < (uint32_t)n; }

// ---- edge plan build ------------------------------------------------------

// counts[0] += valid edges, counts[1] += valid edges joining ids more than
// `window` apart.
__global__ void k_edge_census(int32_t ne, int32_t nn, int32_t window, const int32_t* __restrict__ e2n,
                              unsigned long long* __restrict__ counts) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int valid = 0, far = 0;
  if (e < ne) {
    const int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
    valid = in_range(a, nn) && in_range(b, nn);
    far = valid && (a > b ? a - b : b - a) > window;
  }
  valid = __reduce_add_sync(0xffffffffu, valid);
  far = __reduce_add_sync(0xffffffffu, far);
  if ((threadIdx.x & 31) == 0) {
    if (valid) atomicAdd(counts, (unsigned long long)valid);
    if (far) atomicAdd(counts + 1, (unsigned long long)far);
  }
}

// Both directions of every valid non-loop edge, keyed by the source node
// (invalid slots get the sentinel nn and sort last).
__global__ void k_adj_pairs(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, uint32_t* __restrict__ key,
                            int32_t* __restrict__ val, int32_t* __restrict__ deg) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
  const bool ok = in_range(a, nn) && in_range(b, nn) && a != b;
  key[2 * e] = ok ? (uint32_t)a : (uint32_t)nn;
  val[2 * e] = ok ? b : 0;
  key[2 * e + 1] = ok ? (uint32_t)b : (uint32_t)nn;
  val[2 * e + 1] = ok ? a : 0;
  if (ok) {
    atomicAdd(deg + a, 1);
    atomicAdd(deg + b, 1);
  }
}

// The start of the next breadth-first search: the unplaced node of smallest
// (degree, id) among nodes with at least one neighbour.
__global__ void k_pick_start(int32_t nn, const int32_t* __restrict__ state, const int32_t* __restrict__ off,
                             unsigned long long* __restrict__ best) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long k = ~0ull;
  if (i < nn && state[i] == -1) {
    const int32_t d = off[i + 1] - off[i];
    if (d > 0) k = ((unsigned long long)d << 32) | (unsigned long long)i;
  }
  k = warp_min_u64(k);
  if ((threadIdx.x & 31) == 0 && k != ~0ull) atomicMin(best, k);
}

__global__ void k_place_one(const unsigned long long* __restrict__ best, int32_t pos, int32_t* __restrict__ state,
                            int32_t* __restrict__ order) {
  const int32_t v = (int32_t)(*best & 0xffffffffull);
  state[v] = pos;
  order[pos] = v;
}

// One breadth-first step: every unplaced neighbour of the level [lb, le)
// records the earliest position of a neighbour in the level and is listed
// once as a candidate of the next level.  state: -1 unplaced, -2 listed,
// >= 0 position.
__global__ void k_expand(int32_t lb, int32_t le, const int32_t* __restrict__ order, const int32_t* __restrict__ off,
                         const int32_t* __restrict__ adj, int32_t* __restrict__ state, int32_t* __restrict__ parent,
                         int32_t* __restrict__ cand, int32_t* __restrict__ ncand) {
  const int64_t j = lb + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= le) return;
  const int32_t u = order[j];
  for (int32_t k = off[u]; k < off[u + 1]; k++) {
    const int32_t v = adj[k];
    const int32_t sv = state[v];
    if (sv >= 0) continue;
    atomicMin(parent + v, (int32_t)j);
    if (sv == -1 && atomicCAS(state + v, -1, -2) == -1) cand[atomicAdd(ncand, 1)] = v;
  }
}

__global__ void k_cand_keys(int32_t n, const int32_t* __restrict__ cand, const int32_t* __restrict__ parent,
                            unsigned long long* __restrict__ key) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t v = cand[k];
  key[k] = ((unsigned long long)parent[v] << 32) | (unsigned long long)v;
}

__global__ void k_place_level(int32_t n, int32_t base, const unsigned long long* __restrict__ key,
                              int32_t* __restrict__ state, int32_t* __restrict__ order) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int32_t v = (int32_t)(key[k] & 0xffffffffull);
  state[v] = base + (int32_t)k;
  order[base + k] = v;
}

// Nodes no search reached (isolated nodes, or components past the limit)
// follow in id order.
__global__ void k_unplaced_flags(int32_t nn, const int32_t* __restrict__ state, int32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nn) flag[i] = state[i] < 0 ? 1 : 0;
}

__global__ void k_place_rest(int32_t nn, int32_t base, const int32_t* __restrict__ flag,
                             const int32_t* __restrict__ rank, int32_t* __restrict__ state,
                             int32_t* __restrict__ order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn || !flag[i]) return;
  const int32_t p = base + rank[i];
  state[i] = p;
  order[p] = (int32_t)i;
}

__global__ void k_iota(int32_t n, int32_t* __restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t)i;
}

// Internal endpoints of every edge; invalid edges sort last.
__global__ void k_edge_keys(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, const int32_t* __restrict__ pos,
                            unsigned long long* __restrict__ key, int32_t* __restrict__ val) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
  unsigned long long k = ~0ull;
  if (in_range(a, nn) && in_range(b, nn)) {
    const int32_t pa = pos ? pos[a] : a, pb = pos ? pos[b] : b;
    const uint32_t lo = (uint32_t)min(pa, pb), hi = (uint32_t)max(pa, pb);
    k = ((unsigned long long)lo << 32) | hi;
  }
  key[e] = k;
  val[e] = (int32_t)e;
}

__global__ void k_edge_final(int32_t nvalid, const unsigned long long* __restrict__ key,
                             const int32_t* __restrict__ val, const int32_t* __restrict__ e2n,
                             const int32_t* __restrict__ pos, int2* __restrict__ pe2n, int32_t* __restrict__ eref) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nvalid) return;
  const int32_t e = val[k];
  const int32_t a = e2n[2 * (int64_t)e];
  const int32_t pa = pos ? pos[a] : a;
  const int32_t lo = (int32_t)(key[k] >> 32), hi = (int32_t)(key[k] & 0xffffffffull);
  pe2n[k] = make_int2(lo, hi);
  eref[k] = (pa == lo) ? e : ~e;  // a became the high end: the edge is flipped
}

__global__ void k_fill_i32(int64_t n, int32_t v, int32_t* __restrict__ p) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void k_fill_u64(int64_t n, unsigned long long v, unsigned long long* __restrict__ p) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// ---- edge plan kernels -------------------------------------------------------

// Primitives of every node in internal order.
template <bool PERM>
__global__ void __launch_bounds__(kT) k_plan_prims(int32_t nn, const int32_t* __restrict__ perm,
                                                   const double* __restrict__ var, double* __restrict__ rec) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const int64_t c = PERM ? (int64_t)perm[i] : i;
  const double* x = var + 5 * c;
  const NodePrim p = node_prim(x[0], x[1], x[2], x[3], x[4]);
  double4_32a* r = reinterpret_cast<double4_32a*>(rec + 8 * i);
  r[0] = make_double4_32a(p.rho, p.mx, p.my, p.mz);
  r[1] = make_double4_32a(p.rhoE, p.p, p.s, p.rinv);
}

__device__ __forceinline__ NodePrim plan_rec(const double* rec, int64_t i) {
  const double4_32a* r = reinterpret_cast<const double4_32a*>(rec + 8 * i);
  const double4_32a x = r[0], y = r[1];
  NodePrim p;
  p.rho = x.x; p.mx = x.y; p.my = x.z; p.mz = x.w;
  p.rhoE = y.x; p.p = y.y; p.s = y.z; p.rinv = y.w;
  return p;
}

// The bits of -w/2 (w/2 when `pos`) from those of w, on the integer pipe:
// exact for normal w whose half is still normal; other inputs report false.
__device__ __forceinline__ bool half_bits(double w, bool pos, unsigned long long* out) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  *out = (b - (1ull << 52)) ^ (pos ? 0ull : 0x8000000000000000ull);
  return e > 1u && e < 0x7ffu;
}

// compute_flux_edge_kernel over the plan's edges.  The weight term comes from
// the memo when the caller's weight has the bits it was made from.
template <bool PERM>
__global__ void __launch_bounds__(128) k_plan_flux(int32_t ne, const int2* __restrict__ e2n,
                                                   const int32_t* __restrict__ eref, const double* __restrict__ ewt,
                                                   double4_32a* __restrict__ memo, int memo_valid, double sc,
                                                   const double* __restrict__ rec, double* __restrict__ acc) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int2 ab = e2n[e];
  const int32_t r = eref[e];
  const bool flip = r < 0;
  const int64_t ce = flip ? (int64_t)~r : (int64_t)r;
  const double wx = ewt[3 * ce], wy = ewt[3 * ce + 1], wz = ewt[3 * ce + 2];
  double4_32a m = memo[e];
  unsigned long long hx, hy, hz;
  const bool exact = half_bits(wx, flip, &hx) & half_bits(wy, flip, &hy) & half_bits(wz, flip, &hz);
  const bool hit = memo_valid && exact && hx == (unsigned long long)__double_as_longlong(m.x) &&
                   hy == (unsigned long long)__double_as_longlong(m.y) &&
                   hz == (unsigned long long)__double_as_longlong(m.z);
  if (!hit) {
    const double h = flip ? 0.5 : -0.5;
    const double mag = sqrt(fma(wz, wz, fma(wy, wy, wx * wx)));
    m = make_double4_32a(h * wx, h * wy, h * wz, -(mag * sc) * 0.5);
    memo[e] = m;
  }
  const NodePrim a = plan_rec(rec, ab.x);
  const NodePrim b = plan_rec(rec, ab.y);
  double f[5];
  edge_flux(a, b, m.x, m.y, m.z, m.w, f);
  double* fa = acc + 5 * (int64_t)ab.x;
  double* fb = acc + 5 * (int64_t)ab.y;
#pragma unroll
  for (int k = 0; k < 5; k++) {
    atomicAdd(fa + k, f[k]);
    atomicAdd(fb + k, negate(f[k]));
  }
}

// The internal increments onto the caller's rows: one thread per (caller
// node, variable), so the caller's flux is read and written coalesced and
// only the internal rows are gathered (five neighbouring threads share a
// row).  A bijection: no atomics.
__global__ void k_plan_gather(int64_t n5, const int32_t* __restrict__ pos, const double* __restrict__ fl,
                              double* __restrict__ flux) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n5) return;
  const int64_t c = j / 5;
  flux[j] += fl[5 * (int64_t)pos[c] + (j - 5 * c)];
}

// ---- edge plan, DW form ---------------------------------------------------------

__global__ void k_count_ends(int32_t nv, const int2* __restrict__ e2n, int32_t* __restrict__ cnt_a,
                             int32_t* __restrict__ cnt_b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nv) return;
  const int2 ab = e2n[e];
  atomicAdd(cnt_a + ab.x, 1);
  atomicAdd(cnt_b + ab.y, 1);
}

__global__ void k_b_keys(int32_t nv, const int2* __restrict__ e2n, uint32_t* __restrict__ key,
                         int32_t* __restrict__ val) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nv) return;
  key[e] = (uint32_t)e2n[e].y;
  val[e] = (int32_t)e;
}

__global__ void k_off2(int32_t nn, const int32_t* __restrict__ a_off, const int32_t* __restrict__ b_off,
                       int32_t* __restrict__ off2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= nn) off2[i] = a_off[i] + b_off[i];
}

// Node a's entries start at a_off[a] + b_off[a]; the edges are sorted by a,
// so edge e is its (e - a_off[a])-th a-side entry.
__global__ void k_ent_a(int32_t nv, const int2* __restrict__ e2n, const int32_t* __restrict__ a_off,
                        const int32_t* __restrict__ b_off, int2* __restrict__ ent2) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nv) return;
  const int2 ab = e2n[e];
  ent2[(int64_t)a_off[ab.x] + b_off[ab.x] + (e - a_off[ab.x])] = make_int2(ab.y, (int32_t)e);
}

// blist: the edges sorted by b (stable: ties in edge order).  Node b's b-side
// entries follow its a-side ones: entry j of blist lands at a_off[b+1] + j.
__global__ void k_ent_b(int32_t nv, const int2* __restrict__ e2n, const int32_t* __restrict__ blist,
                        const int32_t* __restrict__ a_off, int2* __restrict__ ent2) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nv) return;
  const int32_t e = blist[j];
  const int2 ab = e2n[e];
  ent2[(int64_t)a_off[ab.y + 1] + j] = make_int2(ab.x, (int32_t)((uint32_t)e | 0x80000000u));
}

constexpr int32_t kNoEdge = 0x7fffffff;  // inv_e of a caller edge left out of the plan

__global__ void k_inv_e(int32_t nv, const int32_t* __restrict__ eref, int32_t* __restrict__ inv) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nv) return;
  const int32_t r = eref[e];
  inv[r < 0 ? ~r : r] = (int32_t)((uint32_t)e | (r < 0 ? 0x80000000u : 0u));
}

// The weights of the DW form, in the caller's edge order (coalesced): each
// caller edge whose weight bits differ from the copy of the last DW call (or
// every edge, after a change of smoothing coefficient) gets its (h, wfac)
// recomputed -- the FP64 plan's formula -- and stored as pair words at its
// internal position.  Unchanged weights cost a compare.
__global__ void k_plan_weights_dw(int32_t ne, const int32_t* __restrict__ inv, const double* __restrict__ ewt,
                                  double* __restrict__ wcopy, double4_32a* __restrict__ memo_dw, int force,
                                  double sc) {
  const int64_t ce = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (ce >= ne) return;
  const int32_t r = inv[ce];
  if (r == kNoEdge) return;
  const double wx = ewt[3 * ce], wy = ewt[3 * ce + 1], wz = ewt[3 * ce + 2];
  double* c = wcopy + 3 * ce;
  const bool same = __double_as_longlong(wx) == __double_as_longlong(c[0]) &&
                    __double_as_longlong(wy) == __double_as_longlong(c[1]) &&
                    __double_as_longlong(wz) == __double_as_longlong(c[2]);
  if (same && !force) return;
  const bool flip = r < 0;
  const double h = flip ? 0.5 : -0.5;
  const double mag = sqrt(fma(wz, wz, fma(wy, wy, wx * wx)));
  memo_dw[r & 0x7fffffff] = make_double4_32a(dw_pack(dw_split(h * wx)), dw_pack(dw_split(h * wy)),
                                             dw_pack(dw_split(h * wz)), dw_pack(dw_split(-(mag * sc) * 0.5)));
  c[0] = wx;
  c[1] = wy;
  c[2] = wz;
}

// Pair-word primitives of every node in internal order (no FP64 instruction).
template <bool PERM>
__global__ void __launch_bounds__(kT) k_plan_prims_dw(int32_t nn, const int32_t* __restrict__ perm,
                                                      const double* __restrict__ var, double* __restrict__ rec2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double* x = var + 5 * (PERM ? (int64_t)perm[i] : i);
  store_prim_dw(rec2, i, node_prim_dw(x[0], x[1], x[2], x[3], x[4]));
}

// compute_flux_edge_kernel in the DW form, node-centric: each node sums the
// fluxes of its edges with itself as end a (h negated on the b side) in
// node_flux_dw's factored form and adds the total to its caller row once --
// every caller row is one node's, so no atomics, and the same bits each call.
template <bool PERM>
__global__ void __launch_bounds__(128, 8) k_plan_flux_dw(int32_t nn, const int32_t* __restrict__ perm,
                                                         const int32_t* __restrict__ off2,
                                                         const int2* __restrict__ ent2,
                                                         const double4_32a* __restrict__ memo_dw,
                                                         const double* __restrict__ rec2, double* __restrict__ flux) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const dwf s_me = dw_unpack(rec2[8 * i + 6]);
  NodeFluxDW acc;
  node_flux_dw_init(acc);
  const int32_t k0 = off2[i], k1 = off2[i + 1];
  for (int32_t j = k0; j < k1; j++) {
    const int2 en = ent2[j];
    const NodePrimDW o = load_prim_dw(rec2, en.x);
    const double4_32a w = memo_dw[en.y & 0x7fffffff];
    const uint32_t sg = (uint32_t)en.y & 0x80000000u;
    dwf hx = dw_unpack(w.x), hy = dw_unpack(w.y), hz = dw_unpack(w.z);
    hx = dwf{__uint_as_float(__float_as_uint(hx.h) ^ sg), __uint_as_float(__float_as_uint(hx.l) ^ sg)};
    hy = dwf{__uint_as_float(__float_as_uint(hy.h) ^ sg), __uint_as_float(__float_as_uint(hy.l) ^ sg)};
    hz = dwf{__uint_as_float(__float_as_uint(hz.h) ^ sg), __uint_as_float(__float_as_uint(hz.l) ^ sg)};
    node_flux_dw_edge(acc, s_me, o, hx, hy, hz, dw_unpack(w.w));
  }
  double F[5];
  node_flux_dw_finish(acc, load_prim_dw(rec2, i), F);
  double* row = flux + 5 * (PERM ? (int64_t)perm[i] : i);
#pragma unroll
  for (int k = 0; k < 5; k++) row[k] += F[k];
}

// ---- children plan -------------------------------------------------------------

__global__ void k_child_pairs(int32_t nf, int32_t nc, const int32_t* __restrict__ map, uint32_t* __restrict__ key,
                              int32_t* __restrict__ val, int32_t* __restrict__ cnt,
                              unsigned long long* __restrict__ nbad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  const int32_t c = map[i];
  const bool ok = in_range(c, nc);
  key[i] = ok ? (uint32_t)c : (uint32_t)nc;
  val[i] = (int32_t)i;
  if (ok) atomicAdd(cnt + c, 1);
  else atomicAdd(nbad, 1ull);
}

// up_pre_kernel (mg.h:29-39): every coarse node with a child starts from zero.
__global__ void k_child_pre(int32_t nc, const int32_t* __restrict__ off, double* __restrict__ cv,
                            int32_t* __restrict__ scratch) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc || off[c + 1] == off[c]) return;
#pragma unroll
  for (int k = 0; k < 5; k++) cv[5 * c + k] = 0.0;
  scratch[c] = 0;
}

// up_kernel (mg.h:41-52) as a gather: the children's states added to the
// coarse state in child order, and the count raised by the number of children.
__global__ void k_child_up(int32_t nc, const int32_t* __restrict__ off, const int32_t* __restrict__ list,
                           const double* __restrict__ fv, double* __restrict__ cv, int32_t* __restrict__ scratch) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int32_t lo = off[c], hi = off[c + 1];
  if (hi == lo) return;
  double s[5];
#pragma unroll
  for (int k = 0; k < 5; k++) s[k] = cv[5 * c + k];
  for (int32_t j = lo; j < hi; j++) {
    const double* x = fv + 5 * (int64_t)list[j];
#pragma unroll
    for (int k = 0; k < 5; k++) s[k] += x[k];
  }
#pragma unroll
  for (int k = 0; k < 5; k++) cv[5 * c + k] = s[k];
  scratch[c] += hi - lo;
}

// ---- cache -----------------------------------------------------------------------

struct Key {
  int device;
  const void* map;
  int64_t n_from, n_to;
  int kind;
  bool operator<(const Key& o) const {
    return std::tie(device, map, n_from, n_to, kind) < std::tie(o.device, o.map, o.n_from, o.n_to, o.kind);
  }
};

enum { kEdgePlan = 0, kChildPlan = 1, kVolPlan = 2 };

std::mutex g_mu;
std::map<Key, EdgePlan*> g_edge;
std::map<Key, ChildPlan*> g_child;
std::map<Key, VolPlan*> g_vol;
int g_mode = MGCFD_PLANS_AUTO;
std::atomic<int> g_flux_dw{0};  // mgcfd_op_flux_precision: DW form of the flux through plans

void free_edge_plan(EdgePlan* P) {
  if (!P) return;
  for (void* p : {(void*)P->perm, (void*)P->pos, (void*)P->e2n, (void*)P->eref, (void*)P->memo, (void*)P->rec,
                  (void*)P->fl, (void*)P->off2, (void*)P->ent2, (void*)P->inv_e, (void*)P->wcopy, (void*)P->memo_dw,
                  (void*)P->rec2})
    if (p) cudaFree(p);
  delete P;
}

void free_child_plan(ChildPlan* P) {
  if (!P) return;
  if (P->ch_off) cudaFree(P->ch_off);
  if (P->ch_list) cudaFree(P->ch_list);
  delete P;
}

void free_vol_plan(VolPlan* P) {
  if (!P) return;
  if (P->vcopy) cudaFree(P->vcopy);
  if (P->root) cudaFree(P->root);
  delete P;
}

void free_plan(EdgePlan* P) { free_edge_plan(P); }
void free_plan(ChildPlan* P) { free_child_plan(P); }
void free_plan(VolPlan* P) { free_vol_plan(P); }

template <class F>
int cub_call(Scratch& S, F&& f) {
  size_t bytes = 0;
  CK(f(nullptr, bytes));
  char* t = nullptr;
  int r = S.get(&t, bytes);
  if (r) return r;
  CK(f(t, bytes));
  return MGCFD_OK;
}

// Cuthill-McKee order of the nodes (pos: caller node -> position; order:
// position -> caller node) from the valid edges of `e2n`.
int cm_order(const int32_t* e2n, int32_t ne, int32_t nn, cudaStream_t s, Scratch& S, int32_t* pos, int32_t* order) {
  int r;
  const int64_t np = 2 * (int64_t)ne;
  uint32_t *k_in, *k_out;
  int32_t *v_in, *adj, *deg, *off, *parent, *cand, *ncand;
  unsigned long long *ckey, *ckey_out, *best;
  if ((r = S.get(&k_in, (size_t)np)) || (r = S.get(&k_out, (size_t)np)) || (r = S.get(&v_in, (size_t)np)) ||
      (r = S.get(&adj, (size_t)np)) || (r = S.get(&deg, (size_t)nn + 1)) || (r = S.get(&off, (size_t)nn + 1)) ||
      (r = S.get(&parent, (size_t)nn)) || (r = S.get(&cand, (size_t)nn)) || (r = S.get(&ncand, 1)) ||
      (r = S.get(&ckey, (size_t)nn)) || (r = S.get(&ckey_out, (size_t)nn)) || (r = S.get(&best, 1)))
    return r;
  CK(cudaMemsetAsync(deg, 0, sizeof(int32_t) * ((size_t)nn + 1), s));
  if (ne > 0) k_adj_pairs<<<grid(ne), kT, 0, s>>>(ne, nn, e2n, k_in, v_in, deg);
  const int kb = bits_for(nn);
  if (np > 0 &&
      (r = cub_call(S, [&](void* t, size_t& b) {
         return cub::DeviceRadixSort::SortPairs(t, b, k_in, k_out, v_in, adj, (int)np, 0, kb, s);
       })))
    return r;
  if ((r = cub_call(S, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, deg, off, nn + 1, s); })))
    return r;
  CK(cudaMemsetAsync(pos, 0xff, sizeof(int32_t) * (size_t)nn, s));  // state -1: unplaced
  CK(cudaMemsetAsync(parent, 0x7f, sizeof(int32_t) * (size_t)nn, s));
  int32_t placed = 0;
  char* sort_tmp = nullptr;
  size_t sort_bytes = 0;
  int32_t* ncand_h = nullptr;
  unsigned long long* best_h = nullptr;
  struct HostFree {
    int32_t** a; unsigned long long** b;
    ~HostFree() {
      if (*a) cudaFreeHost(*a);
      if (*b) cudaFreeHost(*b);
    }
  } hf{&ncand_h, &best_h};
  CK(cudaMallocHost(&ncand_h, sizeof(int32_t)));
  CK(cudaMallocHost(&best_h, sizeof(unsigned long long)));
  int bfs_levels = 0;
  for (int comp = 0; comp < kMaxComponents && placed < nn && bfs_levels < kMaxBfsLevels; comp++) {
    k_fill_u64<<<1, 1, 0, s>>>(1, ~0ull, best);
    k_pick_start<<<grid(nn), kT, 0, s>>>(nn, pos, off, best);
    CK(cudaMemcpyAsync(best_h, best, sizeof(*best_h), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (*best_h == ~0ull) break;  // only nodes without neighbours are left
    k_place_one<<<1, 1, 0, s>>>(best, placed, pos, order);
    int32_t lb = placed, le = placed + 1;
    placed = le;
    while (lb < le && ++bfs_levels <= kMaxBfsLevels) {
      CK(cudaMemsetAsync(ncand, 0, sizeof(int32_t), s));
      k_expand<<<grid(le - lb), kT, 0, s>>>(lb, le, order, off, adj, pos, parent, cand, ncand);
      CK(cudaMemcpyAsync(ncand_h, ncand, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      const int32_t nc = *ncand_h;
      if (nc <= 0) break;
      if (nc > nn - placed) return set_error(MGCFD_ERR_CUDA, "plan: breadth-first search over-counted a level");
      k_cand_keys<<<grid(nc), kT, 0, s>>>(nc, cand, parent, ckey);
      const int eb = 32 + kb;
      size_t need = 0;
      CK(cub::DeviceRadixSort::SortKeys(nullptr, need, ckey, ckey_out, nc, 0, eb, s));
      if (need > sort_bytes) {  // one buffer for every level, grown when a level needs more
        sort_bytes = need;
        if ((r = S.get(&sort_tmp, sort_bytes))) return r;
      }
      CK(cub::DeviceRadixSort::SortKeys(sort_tmp, need, ckey, ckey_out, nc, 0, eb, s));
      k_place_level<<<grid(nc), kT, 0, s>>>(nc, placed, ckey_out, pos, order);
      lb = placed;
      placed += nc;
      le = placed;
    }
  }
  if (placed < nn) {
    int32_t *flag, *rank;
    if ((r = S.get(&flag, (size_t)nn + 1)) || (r = S.get(&rank, (size_t)nn + 1))) return r;
    k_unplaced_flags<<<grid(nn), kT, 0, s>>>(nn, pos, flag);
    if ((r = cub_call(S, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, flag, rank, nn, s); })))
      return r;
    k_place_rest<<<grid(nn), kT, 0, s>>>(nn, placed, flag, rank, pos, order);
  }
  CK(cudaGetLastError());
  return MGCFD_OK;
}

int build_edge_plan(const int32_t* e2n, int32_t ne, int32_t nn, int mode, cudaStream_t s, EdgePlan* P) {
  Scratch S(s);
  int r;
  P->ne = ne;
  P->nn = nn;
  unsigned long long* counts;
  if ((r = S.get(&counts, 2))) return r;
  CK(cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), s));
  const int32_t window = std::max<int32_t>(65536, nn / 128);
  if (ne > 0) k_edge_census<<<grid(ne), kT, 0, s>>>(ne, nn, window, e2n, counts);
  unsigned long long h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  P->nvalid = (int32_t)h[0];
  P->nbad = (int64_t)ne - (int64_t)h[0];
  // Reorder when more than a tenth of the edges join far-apart ids: their
  // atomics and gathers would miss L2.
  P->permuted = mode == MGCFD_PLANS_REORDER || (mode == MGCFD_PLANS_AUTO && h[1] * 10 > h[0]);
  int32_t* pos = nullptr;
  if (P->permuted) {
    if ((r = plan_alloc(&P->pos, (size_t)nn, &P->bytes)) || (r = plan_alloc(&P->perm, (size_t)nn, &P->bytes))) return r;
    pos = P->pos;
    if ((r = cm_order(e2n, ne, nn, s, S, pos, P->perm))) return r;
  }
  unsigned long long *key, *key_out;
  int32_t *val, *val_out;
  if ((r = S.get(&key, (size_t)ne + 1)) || (r = S.get(&key_out, (size_t)ne + 1)) || (r = S.get(&val, (size_t)ne + 1)) ||
      (r = S.get(&val_out, (size_t)ne + 1)))
    return r;
  if (ne > 0) {
    k_edge_keys<<<grid(ne), kT, 0, s>>>(ne, nn, e2n, pos, key, val);
    if ((r = cub_call(S, [&](void* t, size_t& b) {
           return cub::DeviceRadixSort::SortPairs(t, b, key, key_out, val, val_out, ne, 0, 64, s);
         })))
      return r;
  }
  const size_t nv = (size_t)std::max(P->nvalid, 1);
  if ((r = plan_alloc(&P->e2n, nv, &P->bytes)) || (r = plan_alloc(&P->eref, nv, &P->bytes)) ||
      (r = plan_alloc(&P->memo, nv, &P->bytes)) || (r = plan_alloc(&P->rec, 8 * (size_t)std::max(nn, 1), &P->bytes)))
    return r;
  if (P->permuted && (r = plan_alloc(&P->fl, 5 * (size_t)std::max(nn, 1), &P->bytes))) return r;
  if (P->nvalid > 0)
    k_edge_final<<<grid(P->nvalid), kT, 0, s>>>(P->nvalid, key_out, val_out, e2n, pos, P->e2n, P->eref);
  // A memo of all-ones bits (a NaN) matches no weight until first written.
  CK(cudaMemsetAsync(P->memo, 0xff, sizeof(double4_32a) * nv, s));
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return MGCFD_OK;
}

// The DW form's tables of an edge plan: per internal node its a-side edges
// (the sorted edge list's runs) then its b-side ones (a stable sort by b).
int build_edge_plan_dw(EdgePlan* P, cudaStream_t s) {
  Scratch S(s);
  int r;
  const int32_t nn = P->nn, nv = P->nvalid;
  int32_t *cnt_a, *cnt_b, *a_off, *b_off, *val, *val_out;
  uint32_t *key, *key_out;
  if ((r = S.get(&cnt_a, (size_t)nn + 1)) || (r = S.get(&cnt_b, (size_t)nn + 1)) ||
      (r = S.get(&a_off, (size_t)nn + 1)) || (r = S.get(&b_off, (size_t)nn + 1)) ||
      (r = S.get(&key, (size_t)nv + 1)) || (r = S.get(&key_out, (size_t)nv + 1)) ||
      (r = S.get(&val, (size_t)nv + 1)) || (r = S.get(&val_out, (size_t)nv + 1)))
    return r;
  CK(cudaMemsetAsync(cnt_a, 0, sizeof(int32_t) * ((size_t)nn + 1), s));
  CK(cudaMemsetAsync(cnt_b, 0, sizeof(int32_t) * ((size_t)nn + 1), s));
  if (nv > 0) k_count_ends<<<grid(nv), kT, 0, s>>>(nv, P->e2n, cnt_a, cnt_b);
  if ((r = cub_call(S, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, cnt_a, a_off, nn + 1, s); })) ||
      (r = cub_call(S, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, cnt_b, b_off, nn + 1, s); })))
    return r;
  if (nv > 0) {
    k_b_keys<<<grid(nv), kT, 0, s>>>(nv, P->e2n, key, val);
    if ((r = cub_call(S, [&](void* t, size_t& b) {
           return cub::DeviceRadixSort::SortPairs(t, b, key, key_out, val, val_out, nv, 0, bits_for(nn), s);
         })))
      return r;
  }
  const size_t nv1 = (size_t)std::max(nv, 1);
  const size_t ne1 = (size_t)std::max(P->ne, 1);
  if ((r = plan_alloc(&P->off2, (size_t)nn + 1, &P->bytes)) || (r = plan_alloc(&P->ent2, 2 * nv1, &P->bytes)) ||
      (r = plan_alloc(&P->inv_e, ne1, &P->bytes)) || (r = plan_alloc(&P->wcopy, 3 * ne1, &P->bytes)) ||
      (r = plan_alloc(&P->memo_dw, nv1, &P->bytes)) || (r = plan_alloc(&P->rec2, 8 * (size_t)std::max(nn, 1), &P->bytes)))
    return r;
  k_off2<<<grid((int64_t)nn + 1), kT, 0, s>>>(nn, a_off, b_off, P->off2);
  if (nv > 0) {
    k_ent_a<<<grid(nv), kT, 0, s>>>(nv, P->e2n, a_off, b_off, P->ent2);
    k_ent_b<<<grid(nv), kT, 0, s>>>(nv, P->e2n, val_out, a_off, P->ent2);
  }
  // Caller edges left out of the plan stay kNoEdge.
  if (P->ne > 0) k_fill_i32<<<grid(P->ne), kT, 0, s>>>(P->ne, kNoEdge, P->inv_e);
  if (nv > 0) k_inv_e<<<grid(nv), kT, 0, s>>>(nv, P->eref, P->inv_e);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  P->dw_built = true;
  return MGCFD_OK;
}

int build_child_plan(const int32_t* map, int32_t nf, int32_t nc, cudaStream_t s, ChildPlan* P) {
  Scratch S(s);
  int r;
  P->nf = nf;
  P->nc = nc;
  uint32_t *key, *key_out;
  int32_t *val, *cnt;
  unsigned long long* nbad;
  if ((r = S.get(&key, (size_t)nf + 1)) || (r = S.get(&key_out, (size_t)nf + 1)) || (r = S.get(&val, (size_t)nf + 1)) ||
      (r = S.get(&cnt, (size_t)nc + 1)) || (r = S.get(&nbad, 1)))
    return r;
  if ((r = plan_alloc(&P->ch_off, (size_t)nc + 1, &P->bytes)) ||
      (r = plan_alloc(&P->ch_list, (size_t)std::max(nf, 1), &P->bytes)))
    return r;
  CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)nc + 1), s));
  CK(cudaMemsetAsync(nbad, 0, sizeof(unsigned long long), s));
  if (nf > 0) {
    k_child_pairs<<<grid(nf), kT, 0, s>>>(nf, nc, map, key, val, cnt, nbad);
    const int kb = bits_for(nc);
    if ((r = cub_call(S, [&](void* t, size_t& b) {
           return cub::DeviceRadixSort::SortPairs(t, b, key, key_out, val, P->ch_list, nf, 0, kb, s);
         })))
      return r;
  }
  if ((r = cub_call(S, [&](void* t, size_t& b) { return cub::DeviceScan::ExclusiveSum(t, b, cnt, P->ch_off, nc + 1, s); })))
    return r;
  unsigned long long hb = 0;
  CK(cudaMemcpyAsync(&hb, nbad, sizeof(hb), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  P->nbad = (int64_t)hb;
  CK(cudaGetLastError());
  return MGCFD_OK;
}

// calculate_dt_kernel (time_stepping_kernels.h:13-32) with the volume's
// cube root taken from the plan while the volume keeps the bits it had when
// the root was taken (a bit compare per node), else computed and kept: the
// same bits as cbrt on every call.  node_prim and the division stay per call.
__global__ void k_plan_calculate_dt(int32_t n, const double* __restrict__ var, const double* __restrict__ vol,
                                    double* __restrict__ vcopy, double* __restrict__ root, double* __restrict__ dt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = vol[i];
    double c;
    if (__double_as_longlong(v) == __double_as_longlong(vcopy[i])) {
      c = root[i];
    } else {
      c = cbrt(v);
      root[i] = c;
      vcopy[i] = v;
    }
    const double* x = var + 5 * i;
    const NodePrim p = node_prim(x[0], x[1], x[2], x[3], x[4]);
    dt[i] = 0.5 * (c / p.s);
  }
}

// A volume plan starts with every copied volume and root set to the
// all-ones bit pattern (a NaN): the first call takes every root, and a volume
// with exactly those bits would read that NaN, as cbrt would give a NaN.
int build_vol_plan(int32_t n, cudaStream_t s, VolPlan* P) {
  int r;
  P->n = n;
  if ((r = plan_alloc(&P->vcopy, (size_t)n, &P->bytes)) || (r = plan_alloc(&P->root, (size_t)n, &P->bytes))) return r;
  CK(cudaMemsetAsync(P->vcopy, 0xff, sizeof(double) * (size_t)n, s));
  CK(cudaMemsetAsync(P->root, 0xff, sizeof(double) * (size_t)n, s));
  return MGCFD_OK;
}

// Finds or builds a plan.  *out = nullptr (and MGCFD_OK) when plans are off,
// or when none exists yet and the stream is capturing a graph.
template <class P, class Build>
int get_plan(std::map<Key, P*>& cache, const Key& k, cudaStream_t s, Build build, P** out) {
  *out = nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_mode == MGCFD_PLANS_OFF) return MGCFD_OK;
  auto it = cache.find(k);
  if (it != cache.end()) {
    *out = it->second;
    return MGCFD_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) return MGCFD_OK;
  P* p = new (std::nothrow) P();
  if (!p) return set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  int r = build(p);
  if (r) {
    cudaStreamSynchronize(s);
    free_plan(p);
    return r;
  }
  cache[k] = p;
  *out = p;
  return MGCFD_OK;
}

}  // namespace

int edge_plan_get(const int32_t* e2n, int32_t ne, int32_t nn, cudaStream_t s, EdgePlan** out) {
  *out = nullptr;
  if (ne > (1 << 30)) return MGCFD_OK;  // both directions of every edge must fit one sort's int count
  int dev = 0;
  CK(cudaGetDevice(&dev));
  return get_plan(g_edge, Key{dev, e2n, ne, nn, kEdgePlan}, s,
                  [&](EdgePlan* p) { return build_edge_plan(e2n, ne, nn, g_mode, s, p); }, out);
}

int edge_plan_flux(EdgePlan* P, const double* var, const double* ewt, double sc, double* flux, cudaStream_t s,
                   int64_t* skipped) {
  *skipped = P->nbad;
  if (P->nn == 0) return MGCFD_OK;
  bool dw = g_flux_dw.load();
  if (dw && !P->dw_built) {
    // The DW tables are built on the first DW call (synchronising the
    // stream); a first DW call during graph capture runs the FP64 form.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
      dw = false;
    } else {
      std::lock_guard<std::mutex> lock(g_mu);
      int r;
      if (!P->dw_built && (r = build_edge_plan_dw(P, s))) return r;
    }
  }
  if (dw) {
    // The DW form: three kernels, no atomics, no work space of FP64 rows.
    const bool force = !(P->memo_dw_sc == sc);  // the first DW call (NaN) or a new smoothing coefficient
    P->memo_dw_sc = sc;
    if (P->nvalid > 0)
      k_plan_weights_dw<<<grid(P->ne), kT, 0, s>>>(P->ne, P->inv_e, ewt, P->wcopy, P->memo_dw, force ? 1 : 0, sc);
    if (P->permuted) {
      k_plan_prims_dw<true><<<grid(P->nn), kT, 0, s>>>(P->nn, P->perm, var, P->rec2);
      k_plan_flux_dw<true><<<grid(P->nn, 128), 128, 0, s>>>(P->nn, P->perm, P->off2, P->ent2, P->memo_dw, P->rec2, flux);
    } else {
      k_plan_prims_dw<false><<<grid(P->nn), kT, 0, s>>>(P->nn, nullptr, var, P->rec2);
      k_plan_flux_dw<false><<<grid(P->nn, 128), 128, 0, s>>>(P->nn, nullptr, P->off2, P->ent2, P->memo_dw, P->rec2,
                                                            flux);
    }
    CK(cudaGetLastError());
    return MGCFD_OK;
  }
  const bool memo_valid = P->memo_sc == sc;  // false for NaN: never used yet
  P->memo_sc = sc;
  if (P->permuted) {
    CK(cudaMemsetAsync(P->fl, 0, sizeof(double) * 5 * (size_t)P->nn, s));
    k_plan_prims<true><<<grid(P->nn), kT, 0, s>>>(P->nn, P->perm, var, P->rec);
    if (P->nvalid > 0)
      k_plan_flux<true><<<grid(P->nvalid, 128), 128, 0, s>>>(P->nvalid, P->e2n, P->eref, ewt, P->memo,
                                                             memo_valid ? 1 : 0, sc, P->rec, P->fl);
    k_plan_gather<<<grid(5 * (int64_t)P->nn), kT, 0, s>>>(5 * (int64_t)P->nn, P->pos, P->fl, flux);
  } else {
    k_plan_prims<false><<<grid(P->nn), kT, 0, s>>>(P->nn, nullptr, var, P->rec);
    if (P->nvalid > 0)
      k_plan_flux<false><<<grid(P->nvalid, 128), 128, 0, s>>>(P->nvalid, P->e2n, P->eref, ewt, P->memo,
                                                              memo_valid ? 1 : 0, sc, P->rec, flux);
  }
  CK(cudaGetLastError());
  return MGCFD_OK;
}

int child_plan_get(const int32_t* map, int32_t nf, int32_t nc, cudaStream_t s, ChildPlan** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  return get_plan(g_child, Key{dev, map, nf, nc, kChildPlan}, s,
                  [&](ChildPlan* p) { return build_child_plan(map, nf, nc, s, p); }, out);
}

int child_plan_up_pre(ChildPlan* P, double* cv, int32_t* scratch, cudaStream_t s, int64_t* skipped) {
  *skipped = P->nbad;
  if (P->nc > 0) k_child_pre<<<grid(P->nc), kT, 0, s>>>(P->nc, P->ch_off, cv, scratch);
  CK(cudaGetLastError());
  return MGCFD_OK;
}

int child_plan_up(ChildPlan* P, const double* fv, double* cv, int32_t* scratch, cudaStream_t s, int64_t* skipped) {
  *skipped = P->nbad;
  if (P->nc > 0) k_child_up<<<grid(P->nc, 128), 128, 0, s>>>(P->nc, P->ch_off, P->ch_list, fv, cv, scratch);
  CK(cudaGetLastError());
  return MGCFD_OK;
}

bool edge_plan_permuted(const EdgePlan* P) { return P->permuted; }

int vol_plan_get(const double* vol, int32_t n, cudaStream_t s, VolPlan** out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  return get_plan(g_vol, Key{dev, vol, n, n, kVolPlan}, s, [&](VolPlan* p) { return build_vol_plan(n, s, p); },
                  out);
}

int vol_plan_calculate_dt(VolPlan* P, const double* var, const double* vol, double* dt, cudaStream_t s) {
  if (P->n > 0) k_plan_calculate_dt<<<grid(P->n), kT, 0, s>>>(P->n, var, vol, P->vcopy, P->root, dt);
  CK(cudaGetLastError());
  return MGCFD_OK;
}

}  // namespace mgcfd

extern "C" int mgcfd_op_plans_mode(int32_t mode) {
  if (mode < MGCFD_PLANS_OFF || mode > MGCFD_PLANS_CALLER_ORDER)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_op_plans_mode: unknown mode");
  std::lock_guard<std::mutex> lock(mgcfd::g_mu);
  mgcfd::g_mode = mode;
  return MGCFD_OK;
}

extern "C" int mgcfd_op_flux_precision(int32_t precision) {
  if (precision != MGCFD_PRECISION_FP64 && precision != MGCFD_PRECISION_DW)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_op_flux_precision: FP64 or DW");
  mgcfd::g_flux_dw.store(precision == MGCFD_PRECISION_DW ? 1 : 0);
  return MGCFD_OK;
}

extern "C" int mgcfd_op_plans_release(void) {
  std::lock_guard<std::mutex> lock(mgcfd::g_mu);
  cudaError_t e = cudaDeviceSynchronize();
  for (auto& kv : mgcfd::g_edge) mgcfd::free_edge_plan(kv.second);
  for (auto& kv : mgcfd::g_child) mgcfd::free_child_plan(kv.second);
  for (auto& kv : mgcfd::g_vol) mgcfd::free_vol_plan(kv.second);
  mgcfd::g_edge.clear();
  mgcfd::g_child.clear();
  mgcfd::g_vol.clear();
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("mgcfd_op_plans_release: ") + cudaGetErrorString(e));
  return MGCFD_OK;
}

extern "C" int mgcfd_op_plan_release(const void* map) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("mgcfd_op_plan_release: ") + cudaGetErrorString(e));
  std::lock_guard<std::mutex> lock(mgcfd::g_mu);
  for (auto it = mgcfd::g_edge.begin(); it != mgcfd::g_edge.end();) {
    if (it->first.device == dev && it->first.map == map) {
      mgcfd::free_edge_plan(it->second);
      it = mgcfd::g_edge.erase(it);
    } else {
      ++it;
    }
  }
  for (auto it = mgcfd::g_child.begin(); it != mgcfd::g_child.end();) {
    if (it->first.device == dev && it->first.map == map) {
      mgcfd::free_child_plan(it->second);
      it = mgcfd::g_child.erase(it);
    } else {
      ++it;
    }
  }
  for (auto it = mgcfd::g_vol.begin(); it != mgcfd::g_vol.end();) {
    if (it->first.device == dev && it->first.map == map) {
      mgcfd::free_vol_plan(it->second);
      it = mgcfd::g_vol.erase(it);
    } else {
      ++it;
    }
  }
  return MGCFD_OK;
}

extern "C" int mgcfd_op_plans_info(int64_t* edge_plans, int64_t* child_plans, int64_t* reordered,
                                   int64_t* device_bytes) {
  std::lock_guard<std::mutex> lock(mgcfd::g_mu);
  int64_t re = 0, bytes = 0;
  for (auto& kv : mgcfd::g_edge) {
    re += kv.second->permuted ? 1 : 0;
    bytes += kv.second->bytes;
  }
  for (auto& kv : mgcfd::g_child) bytes += kv.second->bytes;
  for (auto& kv : mgcfd::g_vol) bytes += kv.second->bytes;
  if (edge_plans) *edge_plans = (int64_t)mgcfd::g_edge.size();
  if (child_plans) *child_plans = (int64_t)mgcfd::g_child.size();
  if (reordered) *reordered = re;
  if (device_bytes) *device_bytes = bytes;
  return MGCFD_OK;
}
