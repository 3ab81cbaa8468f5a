// Device-side mesh preparation: everything prepare_mesh() (setup.cpp) does on
// the host, built on the GPU from the uploaded level arrays, with identical
// results:
//   * node order: Morton keys of the coordinates (same quantisation), stable
//     radix sort;
//   * geometry: calculate_cell_volumes + dampen_ewt (misc.h:40-84) per edge
//     with explicitly rounded operations, and each node's volume summed over
//     its incident edges in increasing edge id -- the reference's sequential
//     order, so volumes are bit-identical to the reference (the mixed-
//     precision form computes the per-edge geometry in FP32 and sums the
//     volumes in FP64);
//   * edges oriented a < b and stably sorted by (a, b); CSR tables by counting
//     and prefix sums;
//   * boundary entries folded per node in entry order; multigrid tables.
//
// A batch of meshes is prepared as one: per level, the meshes' arrays are
// concatenated (mesh m's nodes, edges and boundary entries start at its
// segment offsets) and every kernel and sort runs once over the whole level.
// Maps stay mesh-local in the input and become global by adding the mesh's
// node offset; a kernel finds an element's mesh by binary search over the
// offsets.  Sorting by global node ids equals sorting each mesh by its local
// ids, because meshes occupy consecutive id ranges; the one per-mesh sort key,
// the Morton code, is sorted first and then stably by mesh.  The tables of
// mesh m are therefore those of mesh m prepared alone, shifted by its offsets.
//
// Every kernel that reads an input map checks the entry against the target
// set size of its mesh first; an out-of-range entry is recorded and replaced
// by an in-range one, and setup fails with MGCFD_ERR_INVALID after the last
// kernel.
#include <cub/cub.cuh>

#include <climits>
#include <cmath>
#include <cstring>

#include "device_math.cuh"
#include "setup.h"
#include "solver_internal.h"

namespace mgcfd {
namespace {

constexpr int T = 256;
inline int nblk(int64_t n) { return (int)((n + T - 1) / T); }

int bits_for(int64_t n) {  // number of bits needed to hold values 0..n
  int b = 1;
  while (b < 63 && (int64_t(1) << b) <= n) b++;
  return b;
}

// Setup scratch: a bump allocator over stream-ordered chunks of at least
// 64 MiB, so that the many temporaries of a setup cost a handful of
// allocation calls.  Everything is released when the setup ends.
struct Temp {
  static constexpr size_t kChunk = 64ull << 20;
  cudaStream_t stream;
  std::vector<void*> chunks;
  char* cur = nullptr;
  size_t left = 0;
  explicit Temp(cudaStream_t s) : stream(s) {}
  ~Temp() {
    for (void* p : chunks) cudaFreeAsync(p, stream);
  }
  template <class X>
  int get(X** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    const size_t bytes = (count * sizeof(X) + 255) & ~size_t(255);
    if (bytes > left) {
      const size_t size = bytes > kChunk ? bytes : kChunk;
      void* c = nullptr;
      cudaError_t e = cudaMallocAsync(&c, size, stream);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(MGCFD_ERR_NOMEM, std::string("setup scratch allocation failed: ") + cudaGetErrorString(e));
      }
      chunks.push_back(c);
      cur = static_cast<char*>(c);
      left = size;
    }
    *p = reinterpret_cast<X*>(cur);
    cur += bytes;
    left -= bytes;
    return MGCFD_OK;
  }
};

// Segment table of one level: offsets of each mesh's nodes, edges and
// boundary entries ([nseg + 1] each), per-mesh flags and free streams.
constexpr int32_t kHasVolumes = 1;  // the mesh came with volumes (legacy datasets)
struct Seg {
  int32_t nseg;
  const int32_t* noff;
  const int32_t* eoff;
  const int32_t* boff;
  const int32_t* flags;
  const mgcfd_freestream* ff;
};

// The segment of global index i: the largest m with off[m] <= i.  Segments
// may be empty (edges, boundary entries); i is below off[nseg].
__device__ __forceinline__ int32_t seg_of(const int32_t* __restrict__ off, int32_t nseg, int64_t i) {
  int32_t lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int32_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ bool ok_index(int32_t i, int32_t n, unsigned* err) {
  if ((uint32_t)i < (uint32_t)n) return true;
  atomicAdd(err, 1u);
  return false;
}

// out[i] = segment of (idx ? idx[i] : i).
__global__ void k_seg_of(int32_t n, const int32_t* __restrict__ off, int32_t nseg, const int32_t* __restrict__ idx,
                         int32_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = seg_of(off, nseg, idx ? idx[i] : i);
}

// ---- node order -------------------------------------------------------------

// Per-mesh bounding boxes as ordered keys: lo[3m + d], hi[3m + d].  A warp
// whose nodes share one mesh reduces first; warps of the block's first mesh
// combine in shared memory, so the common case costs one global atomic per
// block and dimension (a handful of addresses take every update).
__global__ void k_bbox(int32_t n, const double* __restrict__ xyz, Seg g, unsigned long long* __restrict__ lo,
                       unsigned long long* __restrict__ hi) {
  __shared__ unsigned long long s_lo[3], s_hi[3];
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x;
  const int32_t mb = seg_of(g.noff, g.nseg, i0);  // the block's first mesh
  if (threadIdx.x < 3) { s_lo[threadIdx.x] = ~0ull; s_hi[threadIdx.x] = 0ull; }
  __syncthreads();
  const int64_t i = i0 + threadIdx.x;
  const bool in = i < n;
  const int32_t m = in ? seg_of(g.noff, g.nseg, i) : -1;
  const int32_t m0 = __shfl_sync(0xffffffffu, m, 0);
  const bool uniform = __all_sync(0xffffffffu, m == m0 || m < 0);
  for (int d = 0; d < 3; d++) {
    const unsigned long long k = in ? dkey(xyz[3 * i + d]) : 0ull;
    if (uniform) {
      const unsigned long long kmin = warp_min_u64(in ? k : ~0ull);
      const unsigned long long kmax = ~warp_min_u64(in ? ~k : ~0ull);
      if ((threadIdx.x & 31) == 0 && m0 >= 0) {
        if (m0 == mb) {
          atomicMin(&s_lo[d], kmin);
          atomicMax(&s_hi[d], kmax);
        } else {
          atomicMin(&lo[3 * m0 + d], kmin);
          atomicMax(&hi[3 * m0 + d], kmax);
        }
      }
    } else if (in) {
      atomicMin(&lo[3 * m + d], k);
      atomicMax(&hi[3 * m + d], k);
    }
  }
  __syncthreads();
  if (threadIdx.x < 3 && s_lo[threadIdx.x] != ~0ull) {
    atomicMin(&lo[3 * mb + threadIdx.x], s_lo[threadIdx.x]);
    atomicMax(&hi[3 * mb + threadIdx.x], s_hi[threadIdx.x]);
  }
}

// Each mesh's quantisation per dimension (as spatial_order() in setup.cpp):
// box[6m + d] = the low end, box[6m + 3 + d] = 2097151 / span or 0.
__global__ void k_box_scale(int32_t nseg, const unsigned long long* __restrict__ lo,
                            const unsigned long long* __restrict__ hi, double* __restrict__ box) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * nseg) return;
  const int m = t / 3, d = t % 3;
  const double a = dkey_inv(lo[3 * m + d]), b = dkey_inv(hi[3 * m + d]);
  const double span = __dsub_rn(b, a);
  box[6 * m + d] = a;
  box[6 * m + 3 + d] = (b > a && isfinite(span)) ? __ddiv_rn(2097151.0, span) : 0.0;
}

__device__ __forceinline__ uint64_t spread3(uint64_t x) {
  x &= 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

// Same quantisation as spatial_order() in setup.cpp, against the node's own
// mesh's box.
__global__ void k_morton(int32_t n, const double* __restrict__ xyz, Seg g, const double* __restrict__ box,
                         unsigned long long* __restrict__ key, int32_t* __restrict__ val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* bx = box + 6 * seg_of(g.noff, g.nseg, i);
  uint64_t q[3];
  for (int d = 0; d < 3; d++) {
    double t = __dmul_rn(__dsub_rn(xyz[3 * i + d], bx[d]), bx[3 + d]);
    if (!(t > 0.0)) t = 0.0;
    if (t > 2097151.0) t = 2097151.0;
    q[d] = (uint64_t)t;
  }
  key[i] = (spread3(q[2]) << 2) | (spread3(q[1]) << 1) | spread3(q[0]);
  val[i] = (int32_t)i;
}

__global__ void k_iota(int32_t n, int32_t* __restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (int32_t)i;
}

__global__ void k_inverse(int32_t n, const int32_t* __restrict__ perm, int32_t* __restrict__ inv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) inv[perm[i]] = (int32_t)i;
}

// ---- geometry (misc.h:40-84) ---------------------------------------------------

__device__ __forceinline__ double sq3(double a, double b, double c) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// FP32 geometry of the mixed-precision form, the same steps in FP32 (IEEE
// round-to-nearest; setup.cpp computes the same on the host): the coordinate
// differences and the input weights are taken in FP64 and rounded once.
__device__ __forceinline__ float sq3f(float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c));
}

// Per edge: global input end nodes (-1 where the entry is out of range),
// volume contribution tv and damped weights w (F32: computed in FP32 and
// stored widened, for the mixed-precision form).
template <bool F32>
__global__ void k_edge_geometry(int32_t ne, Seg g, const int32_t* __restrict__ e2n, const double* __restrict__ xyz,
                                const double* __restrict__ ewt_in, int32_t* __restrict__ ge2n,
                                double* __restrict__ tv, double* __restrict__ w, unsigned* __restrict__ err) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int32_t m = seg_of(g.eoff, g.nseg, e);
  const int32_t base = g.noff[m], nn = g.noff[m + 1] - base;
  const int32_t la = e2n[2 * e], lb = e2n[2 * e + 1];
  const bool va = ok_index(la, nn, err), vb = ok_index(lb, nn, err);
  const int32_t a = va ? base + la : -1, b = vb ? base + lb : -1;
  ge2n[2 * e] = a;
  ge2n[2 * e + 1] = b;
  const double* wi = ewt_in + 3 * e;
  if (g.flags[m] & kHasVolumes) {  // weights used as read (euler3d.cpp:416-431 skipped)
    tv[e] = 0.0;
    for (int i = 0; i < 3; i++) w[3 * e + i] = __dmul_rn(wi[i], 1e-7);
    return;
  }
  if (!va || !vb) {
    tv[e] = 0.0;
    for (int i = 0; i < 3; i++) w[3 * e + i] = 0.0;
    return;
  }
  double d[3];
  for (int i = 0; i < 3; i++) d[i] = __dsub_rn(xyz[3 * (int64_t)b + i], xyz[3 * (int64_t)a + i]);
  if (F32) {
    float df[3], wf[3];
    for (int i = 0; i < 3; i++) { df[i] = d2f_bits(d[i]); wf[i] = d2f_bits(wi[i]); }
    const float dist = __fsqrt_rn(sq3f(df[0], df[1], df[2]));
    const float area = __fsqrt_rn(sq3f(wf[0], wf[1], wf[2]));
    tv[e] = f2d_bits(__fmul_rn(__fmul_rn((float)((1.0 / 3.0) * 0.5), dist), area));
    for (int i = 0; i < 3; i++)
      w[3 * e + i] = f2d_bits(__fmul_rn(__fdiv_rn(__fmul_rn(__fdiv_rn(df[i], dist), area), dist), 1e-7f));
    return;
  }
  const double dist = __dsqrt_rn(sq3(d[0], d[1], d[2]));
  const double area = __dsqrt_rn(sq3(wi[0], wi[1], wi[2]));
  tv[e] = __dmul_rn(__dmul_rn((1.0 / 3.0) * 0.5, dist), area);
  for (int i = 0; i < 3; i++) w[3 * e + i] = __dmul_rn(__ddiv_rn(__dmul_rn(__ddiv_rn(d[i], dist), area), dist), 1e-7);
}

// Incidence pairs (node, edge) in edge order; a stable sort by node keeps
// each node's edges in increasing id.
__global__ void k_incidence(int32_t ne, int32_t nn, const int32_t* __restrict__ ge2n, int32_t* __restrict__ key,
                            int32_t* __restrict__ val, int32_t* __restrict__ cnt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int k = 0; k < 2; k++) {
    int32_t v = ge2n[2 * e + k];
    if (v < 0) v = nn;  // sentinel: sorts last, never summed
    key[2 * e + k] = v;
    val[2 * e + k] = (int32_t)e;
    if (v < nn) atomicAdd(cnt + v, 1);
  }
}

// Volumes of the meshes that came without them, at input node ids.
__global__ void k_volumes(int32_t nn, Seg g, const int32_t* __restrict__ off, const int32_t* __restrict__ edges,
                          const double* __restrict__ tv, double* __restrict__ vol) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  if (g.flags[seg_of(g.noff, g.nseg, i)] & kHasVolumes) return;
  double v = 0.0;  // zero_1d_array_kernel, then OP_INC in edge order
  for (int32_t j = off[i]; j < off[i + 1]; j++) v = __dadd_rn(v, tv[edges[j]]);
  vol[i] = v;
}

__global__ void k_node_constants(int32_t nn, const int32_t* __restrict__ perm, const double* __restrict__ vol_in,
                                 double* __restrict__ vol, double* __restrict__ inv_vol,
                                 double* __restrict__ cbrt_vol) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double v = vol_in[perm[i]];
  vol[i] = v;
  inv_vol[i] = __ddiv_rn(1.0, v);
  cbrt_vol[i] = cbrt(v);
}

// ---- edges -------------------------------------------------------------------

__global__ void k_edge_keys(int32_t ne, const int32_t* __restrict__ ge2n, const int32_t* __restrict__ inv,
                            unsigned long long* __restrict__ key, int32_t* __restrict__ val,
                            unsigned char* __restrict__ flip) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int32_t a = ge2n[2 * e], b = ge2n[2 * e + 1];
  a = a >= 0 ? inv[a] : 0;  // out-of-range maps were recorded by k_edge_geometry
  b = b >= 0 ? inv[b] : 0;
  const bool f = a > b;
  const uint32_t lo = f ? b : a, hi = f ? a : b;
  key[e] = ((unsigned long long)lo << 32) | hi;
  val[e] = (int32_t)e;
  flip[e] = f;
}

template <bool F32>
__global__ void k_edge_finalize(int32_t ne, Seg g, const unsigned long long* __restrict__ key,
                                const int32_t* __restrict__ order, const double* __restrict__ w,
                                const unsigned char* __restrict__ flip, int2* __restrict__ e2n,
                                double* __restrict__ w4, int32_t* __restrict__ acnt, int32_t* __restrict__ bcnt) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ne) return;
  const int64_t e = order[k];
  const double sc = g.ff[seg_of(g.eoff, g.nseg, e)].smoothing_coefficient;
  const int32_t a = (int32_t)(key[k] >> 32), b = (int32_t)(key[k] & 0xffffffffu);
  e2n[k] = make_int2(a, b);
  double x = w[3 * e], y = w[3 * e + 1], z = w[3 * e + 2];
  if (flip[e]) { x = -x; y = -y; z = -z; }
  if (F32) {  // the FP32 weights, stored widened (exact)
    const float xf = d2f_bits(x), yf = d2f_bits(y), zf = d2f_bits(z);
    const float mag = __fsqrt_rn(sq3f(xf, yf, zf));
    w4[4 * k + 0] = f2d_bits(__fmul_rn(-0.5f, xf));
    w4[4 * k + 1] = f2d_bits(__fmul_rn(-0.5f, yf));
    w4[4 * k + 2] = f2d_bits(__fmul_rn(-0.5f, zf));
    w4[4 * k + 3] = f2d_bits(__fmul_rn(__fmul_rn(-mag, d2f_bits(sc)), 0.5f));
  } else {
    const double mag = __dsqrt_rn(sq3(x, y, z));
    w4[4 * k + 0] = __dmul_rn(-0.5, x);
    w4[4 * k + 1] = __dmul_rn(-0.5, y);
    w4[4 * k + 2] = __dmul_rn(-0.5, z);
    w4[4 * k + 3] = __dmul_rn(__dmul_rn(-mag, sc), 0.5);
  }
  atomicAdd(acnt + a, 1);
  atomicAdd(bcnt + b, 1);
}

__global__ void k_b_pairs(int32_t ne, const int2* __restrict__ e2n, int32_t* __restrict__ key,
                          int32_t* __restrict__ val) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ne) return;
  key[k] = e2n[k].y;
  val[k] = (int32_t)k;
}

__global__ void k_to_float(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// ---- boundary -----------------------------------------------------------------

__global__ void k_bnd_keys(int32_t nb, int32_t nn, Seg g, const int32_t* __restrict__ b2n,
                           const int32_t* __restrict__ grp, const int32_t* __restrict__ inv,
                           int32_t* __restrict__ key, int32_t* __restrict__ val, int32_t* __restrict__ cnt,
                           unsigned* __restrict__ err) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int32_t m = seg_of(g.boff, g.nseg, k);
  const int32_t base = g.noff[m];
  const int32_t n = b2n[k];
  const int gr = grp[k];
  int32_t node = nn;  // sentinel: ignored entry
  if (ok_index(n, g.noff[m + 1] - base, err) && gr <= 7) {
    node = inv[base + n];
    atomicAdd(cnt + node, 1);
  }
  key[k] = node;
  val[k] = (int32_t)k;
}

// Folded boundary rows (flux.h:14-39 is linear in the weight), entries in order.
__global__ void k_bnd_fold(int32_t nn, Seg g, const int32_t* __restrict__ off, const int32_t* __restrict__ entries,
                           const int32_t* __restrict__ grp, const double* __restrict__ bwt,
                           const int32_t* __restrict__ row_of, int32_t* __restrict__ bidx,
                           double* __restrict__ bdata) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const int32_t lo = off[i], hi = off[i + 1];
  if (hi == lo) { bidx[i] = -1; return; }
  double wff[3] = {0.0, 0.0, 0.0}, wwall[3] = {0.0, 0.0, 0.0};
  for (int32_t j = lo; j < hi; j++) {
    const int32_t k = entries[j];
    double* dst = grp[k] <= 2 ? wwall : wff;
    for (int c = 0; c < 3; c++) dst[c] = __dadd_rn(dst[c], __dmul_rn(bwt[3 * (int64_t)k + c], 1e-7));
  }
  const int32_t r = row_of[i];
  bidx[i] = r;
  double* row = bdata + 12 * (int64_t)r;
  for (int c = 0; c < 3; c++) { row[c] = wff[c]; row[3 + c] = wwall[c]; }
  const mgcfd_freestream& ff = g.ff[seg_of(g.noff, g.nseg, i)];
  const double* fv = ff.ff_variable;
  const double* rows[4] = {ff.ff_flux_contribution_momentum_x, ff.ff_flux_contribution_momentum_y,
                           ff.ff_flux_contribution_momentum_z, ff.ff_flux_contribution_density_energy};
  row[6] = __dadd_rn(__dadd_rn(__dmul_rn(wff[0], fv[1]), __dmul_rn(wff[1], fv[2])), __dmul_rn(wff[2], fv[3]));
  for (int q = 0; q < 4; q++)
    row[7 + q] = __dadd_rn(__dadd_rn(__dmul_rn(wff[0], rows[q][0]), __dmul_rn(wff[1], rows[q][1])),
                           __dmul_rn(wff[2], rows[q][2]));
  row[11] = 0.0;
}

__global__ void k_copy1(const int32_t* __restrict__ src, unsigned* __restrict__ dst) { *dst = (unsigned)*src; }

__global__ void k_nonempty(int32_t nn, const int32_t* __restrict__ off, int32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nn) flag[i] = off[i + 1] > off[i] ? 1 : 0;
}

// ---- multigrid ----------------------------------------------------------------

// Fine node f (new global id) of mesh m: its coarse node (new global id),
// the distance vector to it (mg.h:76) and a (coarse, fine) pair for the
// child lists.
__global__ void k_mg(int32_t nf, int32_t nseg, const int32_t* __restrict__ noff_f, const int32_t* __restrict__ noff_c,
                     const int32_t* __restrict__ perm_f, const int32_t* __restrict__ n2mg_in,
                     const int32_t* __restrict__ inv_c, const double* __restrict__ xf, const double* __restrict__ xc,
                     int32_t* __restrict__ n2mg, double* __restrict__ dvec, int32_t* __restrict__ key,
                     int32_t* __restrict__ val, int32_t* __restrict__ cnt, unsigned* __restrict__ err) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t m = seg_of(noff_f, nseg, f);
  const int32_t cbase = noff_c[m];
  const int32_t fin = perm_f[f];
  const int32_t cin = n2mg_in[fin];
  int32_t c = cbase;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  if (ok_index(cin, noff_c[m + 1] - cbase, err)) {
    const int64_t cg = (int64_t)cbase + cin;
    c = inv_c[cg];
    dx = fabs(__dsub_rn(xf[3 * (int64_t)fin], xc[3 * cg]));
    dy = fabs(__dsub_rn(xf[3 * (int64_t)fin + 1], xc[3 * cg + 1]));
    dz = fabs(__dsub_rn(xf[3 * (int64_t)fin + 2], xc[3 * cg + 2]));
  }
  n2mg[f] = c;
  dvec[4 * f + 0] = dx;
  dvec[4 * f + 1] = dy;
  dvec[4 * f + 2] = dz;
  dvec[4 * f + 3] = __dsqrt_rn(sq3(dx, dy, dz));  // mg.h:76
  key[f] = c;
  val[f] = (int32_t)f;
  atomicAdd(cnt + c, 1);
}

// ---- helpers ------------------------------------------------------------------

template <class K>
int sort_pairs(Temp& tmp, const K* kin, K* kout, const int32_t* vin, int32_t* vout, int64_t n, int end_bit,
               cudaStream_t s) {
  if (n == 0) return MGCFD_OK;
  size_t bytes = 0;
  CK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, kin, kout, vin, vout, (int)n, 0, end_bit, s));
  void* t = nullptr;
  int r = tmp.get(reinterpret_cast<char**>(&t), bytes);
  if (r) return r;
  CK(cub::DeviceRadixSort::SortPairs(t, bytes, kin, kout, vin, vout, (int)n, 0, end_bit, s));
  return MGCFD_OK;
}

// Exclusive prefix sum of cnt[0..n) into off[0..n] (off[n] = total).
int offsets(Temp& tmp, int32_t* cnt, int32_t* off, int64_t n, cudaStream_t s) {
  size_t bytes = 0;
  CK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt, off, (int)(n + 1), s));
  void* t = nullptr;
  int r = tmp.get(reinterpret_cast<char**>(&t), bytes);
  if (r) return r;
  CK(cub::DeviceScan::ExclusiveSum(t, bytes, cnt, off, (int)(n + 1), s));  // cnt[n] is zero
  return MGCFD_OK;
}

// One level's input arrays on the device, the meshes concatenated.
struct LevelIn {
  double *xyz = nullptr, *ewt = nullptr, *bwt = nullptr, *vol = nullptr;
  int32_t *e2n = nullptr, *b2n = nullptr, *grp = nullptr, *n2mg = nullptr;
  int32_t* inv = nullptr;  // input node id -> new node id (global)
};

}  // namespace

int device_prepare(mgcfd_solver* s, const std::vector<MeshInput>& meshes) {
  cudaStream_t st = s->stream;
  Temp tmp(st);
  const bool mixed = s->opt.precision == MGCFD_PRECISION_MIXED;
  const int nseg = (int)meshes.size();
  const int nlevels = (int)s->L.size();
  int r;

  // Segment tables, checked to fit the 32-bit ids (incidence pairs: 2 per edge).
  const size_t per = 4 * (size_t)nseg + 3;  // noff | eoff | boff | flags
  std::vector<int32_t> meta(per * (size_t)nlevels, 0);
  s->seg_noff.assign((size_t)nlevels, std::vector<int32_t>((size_t)nseg + 1, 0));
  bool any_computed_volumes = false;
  for (int l = 0; l < nlevels; l++) {
    int32_t* M = meta.data() + per * (size_t)l;
    int64_t n = 0, ne = 0, nb = 0;
    for (int m = 0; m < nseg; m++) {
      const mgcfd_level_view& v = meshes[(size_t)m].levels[l];
      n += v.nnodes; ne += v.nedges; nb += v.nbnd;
      if (n >= INT32_MAX || 2 * ne >= INT32_MAX || nb >= INT32_MAX)
        return set_error(MGCFD_ERR_INVALID, "level " + std::to_string(l) + ": more than 2^31 nodes, "
                                            "2^30 edges or 2^31 boundary entries in one solver");
      M[m + 1] = (int32_t)n;
      M[nseg + 1 + m + 1] = (int32_t)ne;
      M[2 * (nseg + 1) + m + 1] = (int32_t)nb;
      M[3 * (nseg + 1) + m] = v.volumes ? kHasVolumes : 0;
      any_computed_volumes |= !v.volumes;
      s->seg_noff[(size_t)l][(size_t)m + 1] = (int32_t)n;
    }
  }
  std::vector<mgcfd_freestream> ffs((size_t)nseg);
  for (int m = 0; m < nseg; m++) ffs[(size_t)m] = meshes[(size_t)m].ff;
  int32_t* dmeta;
  mgcfd_freestream* dff;
  unsigned* fin;  // fin[0]: out-of-range map entries; fin[1 + l]: folded boundary rows of level l
  if ((r = tmp.get(&dmeta, meta.size())) || (r = tmp.get(&dff, (size_t)nseg)) ||
      (r = tmp.get(&fin, 1 + (size_t)nlevels)))
    return r;
  unsigned* err = fin;
  CK(cudaMemcpyAsync(dmeta, meta.data(), 4 * meta.size(), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dff, ffs.data(), sizeof(mgcfd_freestream) * (size_t)nseg, cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(fin, 0, sizeof(unsigned) * (1 + (size_t)nlevels), st));
  auto seg = [&](int l) {
    const int32_t* M = dmeta + per * (size_t)l;
    return Seg{nseg, M, M + (nseg + 1), M + 2 * (nseg + 1), M + 3 * (nseg + 1), dff};
  };
  auto total = [&](int l, int which) { return meta[per * (size_t)l + (size_t)which * (nseg + 1) + (size_t)nseg]; };

  // Upload every level's inputs before the first kernel: a copy from pageable
  // host memory may wait for the work queued ahead of it on the stream.
  std::vector<LevelIn> in((size_t)nlevels);
  for (int l = 0; l < nlevels; l++) {
    LevelIn& I = in[(size_t)l];
    const int32_t N = total(l, 0), NE = total(l, 1), NB = total(l, 2);
    if ((r = tmp.get(&I.xyz, 3 * (size_t)N)) || (r = tmp.get(&I.e2n, 2 * (size_t)NE)) ||
        (r = tmp.get(&I.ewt, 3 * (size_t)NE)) || (r = tmp.get(&I.b2n, (size_t)NB)) ||
        (r = tmp.get(&I.grp, (size_t)NB)) || (r = tmp.get(&I.bwt, 3 * (size_t)NB)) ||
        (r = tmp.get(&I.vol, (size_t)N)) || (r = tmp.get(&I.inv, (size_t)N)) ||
        (l + 1 < nlevels && (r = tmp.get(&I.n2mg, (size_t)N))))
      return r;
    for (int m = 0; m < nseg; m++) {
      const mgcfd_level_view& v = meshes[(size_t)m].levels[l];
      const int64_t noff = s->seg_noff[(size_t)l][(size_t)m];
      const int64_t eoff = meta[per * (size_t)l + (size_t)(nseg + 1) + (size_t)m];
      const int64_t boff = meta[per * (size_t)l + 2 * (size_t)(nseg + 1) + (size_t)m];
      CK(cudaMemcpyAsync(I.xyz + 3 * noff, v.coords, 24 * (size_t)v.nnodes, cudaMemcpyHostToDevice, st));
      if (v.nedges) {
        CK(cudaMemcpyAsync(I.e2n + 2 * eoff, v.edge_to_nodes, 8 * (size_t)v.nedges, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(I.ewt + 3 * eoff, v.edge_weights, 24 * (size_t)v.nedges, cudaMemcpyHostToDevice, st));
      }
      if (v.nbnd) {
        CK(cudaMemcpyAsync(I.b2n + boff, v.bnd_to_node, 4 * (size_t)v.nbnd, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(I.grp + boff, v.bnd_group, 4 * (size_t)v.nbnd, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(I.bwt + 3 * boff, v.bnd_weights, 24 * (size_t)v.nbnd, cudaMemcpyHostToDevice, st));
      }
      if (v.volumes) CK(cudaMemcpyAsync(I.vol + noff, v.volumes, 8 * (size_t)v.nnodes, cudaMemcpyHostToDevice, st));
      if (I.n2mg)
        CK(cudaMemcpyAsync(I.n2mg + noff, v.node_to_mg, 4 * (size_t)v.nnodes, cudaMemcpyHostToDevice, st));
    }
  }

  for (int l = 0; l < nlevels; l++) {
    DevLevel& D = s->L[(size_t)l];
    LevelIn& I = in[(size_t)l];
    const Seg g = seg(l);
    const int32_t N = total(l, 0), NE = total(l, 1), NB = total(l, 2);
    D.n = N; D.ne = NE; D.nb = NB;
    if ((r = s->alloc(&D.perm, (size_t)N)) || (r = s->alloc(&D.vol, (size_t)N)) ||
        (r = s->alloc(&D.inv_vol, (size_t)N)) || (r = s->alloc(&D.cbrt_vol, (size_t)N)) ||
        (r = s->alloc(&D.e2n, (size_t)NE)) || (r = s->alloc(&D.bidx, (size_t)N)) ||
        (r = s->alloc(&D.bdata, 12 * (size_t)(NB > 0 ? NB : 1))))
      return r;
    double* w4all = nullptr;
    if (mixed) { if ((r = tmp.get(&w4all, 4 * (size_t)NE))) return r; }
    else { if ((r = s->alloc(&D.w4, (size_t)NE))) return r; w4all = reinterpret_cast<double*>(D.w4); }
    if (s->gather && ((r = s->alloc(&D.a_off, (size_t)N + 1)) || (r = s->alloc(&D.b_off, (size_t)N + 1)) ||
                      (r = s->alloc(&D.b_list, (size_t)NE))))
      return r;
    if (nseg > 1) {
      if ((r = s->alloc(&D.mesh_id, (size_t)N))) return r;
      k_seg_of<<<nblk(N), T, 0, st>>>(N, g.noff, nseg, nullptr, D.mesh_id);
    }

    // Node order: Morton codes within each mesh, then stably by mesh.
    if (s->opt.renumber == MGCFD_RENUMBER_SPATIAL) {
      unsigned long long *lo, *hi, *key, *key2;
      int32_t *val, *val2;
      if ((r = tmp.get(&lo, 3 * (size_t)nseg)) || (r = tmp.get(&hi, 3 * (size_t)nseg)) ||
          (r = tmp.get(&key, (size_t)N)) || (r = tmp.get(&key2, (size_t)N)) || (r = tmp.get(&val, (size_t)N)) ||
          (r = tmp.get(&val2, (size_t)N)))
        return r;
      CK(cudaMemsetAsync(lo, 0xff, 24 * (size_t)nseg, st));
      CK(cudaMemsetAsync(hi, 0, 24 * (size_t)nseg, st));
      double* box;
      if ((r = tmp.get(&box, 6 * (size_t)nseg))) return r;
      k_bbox<<<nblk(N), T, 0, st>>>(N, I.xyz, g, lo, hi);
      k_box_scale<<<nblk(3 * (int64_t)nseg), T, 0, st>>>(nseg, lo, hi, box);
      k_morton<<<nblk(N), T, 0, st>>>(N, I.xyz, g, box, key, val);
      if (nseg == 1) {
        if ((r = sort_pairs(tmp, key, key2, val, D.perm, N, 63, st))) return r;
      } else {
        int32_t *mkey, *mkey2;
        if ((r = tmp.get(&mkey, (size_t)N)) || (r = tmp.get(&mkey2, (size_t)N))) return r;
        if ((r = sort_pairs(tmp, key, key2, val, val2, N, 63, st))) return r;
        k_seg_of<<<nblk(N), T, 0, st>>>(N, g.noff, nseg, val2, mkey);
        if ((r = sort_pairs(tmp, mkey, mkey2, val2, D.perm, N, bits_for(nseg - 1), st))) return r;
      }
    } else {
      k_iota<<<nblk(N), T, 0, st>>>(N, D.perm);
    }
    k_inverse<<<nblk(N), T, 0, st>>>(N, D.perm, I.inv);

    // Geometry and volumes.
    double *tv, *wd;
    int32_t* ge2n;
    if ((r = tmp.get(&tv, (size_t)NE)) || (r = tmp.get(&wd, 3 * (size_t)NE)) || (r = tmp.get(&ge2n, 2 * (size_t)NE)))
      return r;
    if (NE && mixed) k_edge_geometry<true><<<nblk(NE), T, 0, st>>>(NE, g, I.e2n, I.xyz, I.ewt, ge2n, tv, wd, err);
    else if (NE) k_edge_geometry<false><<<nblk(NE), T, 0, st>>>(NE, g, I.e2n, I.xyz, I.ewt, ge2n, tv, wd, err);
    if (any_computed_volumes) {
      int32_t *ikey, *ival, *ikey2, *ival2, *cnt, *off;
      if ((r = tmp.get(&ikey, 2 * (size_t)NE)) || (r = tmp.get(&ival, 2 * (size_t)NE)) ||
          (r = tmp.get(&ikey2, 2 * (size_t)NE)) || (r = tmp.get(&ival2, 2 * (size_t)NE)) ||
          (r = tmp.get(&cnt, (size_t)N + 1)) || (r = tmp.get(&off, (size_t)N + 1)))
        return r;
      CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)N + 1), st));
      if (NE) k_incidence<<<nblk(NE), T, 0, st>>>(NE, N, ge2n, ikey, ival, cnt);
      if ((r = sort_pairs(tmp, ikey, ikey2, ival, ival2, 2 * (int64_t)NE, bits_for(N), st))) return r;
      if ((r = offsets(tmp, cnt, off, N, st))) return r;
      k_volumes<<<nblk(N), T, 0, st>>>(N, g, off, ival2, tv, I.vol);
    }
    k_node_constants<<<nblk(N), T, 0, st>>>(N, D.perm, I.vol, D.vol, D.inv_vol, D.cbrt_vol);

    // Edges: orientation, order, weights, CSR.
    {
      unsigned long long *key, *key2;
      int32_t *val, *order, *acnt, *bcnt;
      unsigned char* flip;
      if ((r = tmp.get(&key, (size_t)NE)) || (r = tmp.get(&key2, (size_t)NE)) || (r = tmp.get(&val, (size_t)NE)) ||
          (r = tmp.get(&order, (size_t)NE)) || (r = tmp.get(&flip, (size_t)NE)) ||
          (r = tmp.get(&acnt, (size_t)N + 1)) || (r = tmp.get(&bcnt, (size_t)N + 1)))
        return r;
      CK(cudaMemsetAsync(acnt, 0, sizeof(int32_t) * ((size_t)N + 1), st));
      CK(cudaMemsetAsync(bcnt, 0, sizeof(int32_t) * ((size_t)N + 1), st));
      if (NE) {
        k_edge_keys<<<nblk(NE), T, 0, st>>>(NE, ge2n, I.inv, key, val, flip);
        if ((r = sort_pairs(tmp, key, key2, val, order, NE, 32 + bits_for(N), st))) return r;
        if (mixed) k_edge_finalize<true><<<nblk(NE), T, 0, st>>>(NE, g, key2, order, wd, flip, D.e2n, w4all, acnt, bcnt);
        else k_edge_finalize<false><<<nblk(NE), T, 0, st>>>(NE, g, key2, order, wd, flip, D.e2n, w4all, acnt, bcnt);
      }
      if (s->gather) {
        int32_t *bkey, *bval, *bkey2;
        if ((r = tmp.get(&bkey, (size_t)NE)) || (r = tmp.get(&bval, (size_t)NE)) || (r = tmp.get(&bkey2, (size_t)NE)))
          return r;
        if ((r = offsets(tmp, acnt, D.a_off, N, st)) || (r = offsets(tmp, bcnt, D.b_off, N, st))) return r;
        if (NE) {
          k_b_pairs<<<nblk(NE), T, 0, st>>>(NE, D.e2n, bkey, bval);
          if ((r = sort_pairs(tmp, bkey, bkey2, bval, D.b_list, NE, bits_for(N), st))) return r;
        }
      }
    }

    // Boundary entries folded per node.
    {
      int32_t *key, *val, *key2, *val2, *cnt, *off, *flag, *row;
      if ((r = tmp.get(&key, (size_t)NB)) || (r = tmp.get(&val, (size_t)NB)) || (r = tmp.get(&key2, (size_t)NB)) ||
          (r = tmp.get(&val2, (size_t)NB)) || (r = tmp.get(&cnt, (size_t)N + 1)) ||
          (r = tmp.get(&off, (size_t)N + 1)) || (r = tmp.get(&flag, (size_t)N + 1)) ||
          (r = tmp.get(&row, (size_t)N + 1)))
        return r;
      CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)N + 1), st));
      if (NB) {
        k_bnd_keys<<<nblk(NB), T, 0, st>>>(NB, N, g, I.b2n, I.grp, I.inv, key, val, cnt, err);
        if ((r = sort_pairs(tmp, key, key2, val, val2, NB, bits_for(N), st))) return r;
      }
      if ((r = offsets(tmp, cnt, off, N, st))) return r;
      CK(cudaMemsetAsync(flag, 0, sizeof(int32_t) * ((size_t)N + 1), st));
      k_nonempty<<<nblk(N), T, 0, st>>>(N, off, flag);
      if ((r = offsets(tmp, flag, row, N, st))) return r;
      k_bnd_fold<<<nblk(N), T, 0, st>>>(N, g, off, val2, I.grp, I.bwt, row, D.bidx, D.bdata);
      k_copy1<<<1, 1, 0, st>>>(row + N, fin + 1 + l);
    }
    if (mixed) {
      if ((r = s->alloc(&D.w4f, (size_t)NE))) return r;
      if (NE) k_to_float<<<nblk(4 * (int64_t)NE), T, 0, st>>>(4 * (int64_t)NE, w4all, reinterpret_cast<float*>(D.w4f));
      if (s->opt.measure_mem_bound) {
        if ((r = s->alloc(&D.w4, (size_t)NE))) return r;
        if (NE) CK(cudaMemcpyAsync(D.w4, w4all, 32 * (size_t)NE, cudaMemcpyDeviceToDevice, st));
      }
    }
    // Per-level state.
    if ((r = s->alloc(&D.rec, 8 * (size_t)N)) || (r = s->alloc(&D.old, 5 * (size_t)N)) ||
        (r = s->alloc(&D.res, 5 * (size_t)N)))
      return r;
    if (mixed && (r = s->alloc(&D.rec32, 8 * (size_t)N))) return r;
    if (s->fused) {
      if ((r = build_fused_tables(s, D))) return r;
    } else if (s->gather) {
      if (mixed ? (r = s->alloc(&D.fe32, 5 * (size_t)NE)) : (r = s->alloc(&D.fe, 5 * (size_t)NE))) return r;
    }
    else if ((r = s->alloc(&D.flux, 5 * (size_t)N))) return r;
    if (s->opt.measure_mem_bound && (r = s->alloc(&D.dummy, 5 * (size_t)N))) return r;
    CK(cudaGetLastError());
  }

  // Multigrid tables.
  for (int l = 0; l + 1 < nlevels; l++) {
    DevLevel& F = s->L[(size_t)l];
    DevLevel& Cl = s->L[(size_t)l + 1];
    const int32_t NF = F.n, NC = Cl.n;
    if ((r = s->alloc(&F.n2mg, (size_t)NF)) || (r = s->alloc(&F.dvec, (size_t)NF)) ||
        (r = s->alloc(&Cl.ch_off, (size_t)NC + 1)) || (r = s->alloc(&Cl.ch_list, (size_t)NF)))
      return r;
    Cl.nfine = NF;
    int32_t *key, *val, *key2, *cnt;
    if ((r = tmp.get(&key, (size_t)NF)) || (r = tmp.get(&val, (size_t)NF)) || (r = tmp.get(&key2, (size_t)NF)) ||
        (r = tmp.get(&cnt, (size_t)NC + 1)))
      return r;
    CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)NC + 1), st));
    k_mg<<<nblk(NF), T, 0, st>>>(NF, nseg, seg(l).noff, seg(l + 1).noff, F.perm, in[(size_t)l].n2mg,
                                 in[(size_t)l + 1].inv, in[(size_t)l].xyz, in[(size_t)l + 1].xyz, F.n2mg,
                                 reinterpret_cast<double*>(F.dvec), key, val, cnt, err);
    if ((r = sort_pairs(tmp, key, key2, val, Cl.ch_list, NF, bits_for(NC), st))) return r;
    if ((r = offsets(tmp, cnt, Cl.ch_off, NC, st))) return r;
  }
  CK(cudaGetLastError());
  std::vector<unsigned> h_fin(1 + (size_t)nlevels, 0);
  CK(cudaMemcpyAsync(h_fin.data(), fin, sizeof(unsigned) * h_fin.size(), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int l = 0; l < nlevels; l++) s->L[(size_t)l].nbrows = (int32_t)h_fin[1 + (size_t)l];
  if (h_fin[0])
    return set_error(MGCFD_ERR_INVALID, "mesh has " + std::to_string(h_fin[0]) + " map entries out of range");
  return MGCFD_OK;
}

}  // namespace mgcfd
