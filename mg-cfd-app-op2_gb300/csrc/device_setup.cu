// Device-side mesh preparation: everything prepare_mesh() (setup.cpp) does on
// the host, built on the GPU from the uploaded level arrays, with identical
// results:
//   * node order: Morton keys of the coordinates (same quantisation), stable
//     radix sort;
//   * geometry: calculate_cell_volumes + dampen_ewt (misc.h:40-84) per edge
//     with explicitly rounded operations, and each node's volume summed over
//     its incident edges in increasing edge id -- the reference's sequential
//     order, so volumes are bit-identical to the reference;
//   * edges oriented a < b and stably sorted by (a, b); CSR tables by counting
//     and prefix sums;
//   * boundary entries folded per node in entry order; multigrid tables.
// Every kernel that reads an input map checks the entry against the target
// set size first; an out-of-range entry is recorded and skipped, and setup
// fails with MGCFD_ERR_INVALID after the last kernel.
#include <cub/cub.cuh>

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

// Temporary device memory for the setup, freed (stream-ordered) at the end.
// Setup scratch: a bump allocator over stream-ordered chunks of at least
// 64 MiB, so that the many small temporaries of a setup cost a handful of
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

// Independent per-mesh setup work of a batch runs on up to kLanes streams,
// so that the many small kernels of small meshes overlap; the level-wide
// arrays are allocated on the solver's stream, which forks to the lanes and
// joins them again.  One mesh: the solver's stream alone.
struct Lanes {
  static constexpr int kLanes = 8;
  cudaStream_t main;
  std::vector<cudaStream_t> streams;
  std::vector<std::unique_ptr<Temp>> temps;
  std::vector<cudaEvent_t> events;  // events[0]: fork point on main; events[1 + k]: lane k done
  explicit Lanes(cudaStream_t m) : main(m) {}
  ~Lanes() {
    temps.clear();  // frees enqueued on the lanes
    for (size_t k = 0; k < streams.size(); k++)
      if (streams[k] != main) cudaStreamDestroy(streams[k]);
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
  int init(int nseg) {
    const int k = nseg > 1 ? std::min(nseg, kLanes) : 1;
    for (int i = 0; i < k; i++) {
      cudaStream_t sm = main;
      if (k > 1) CK(cudaStreamCreateWithFlags(&sm, cudaStreamNonBlocking));
      streams.push_back(sm);
      temps.emplace_back(new Temp(sm));
    }
    events.resize((size_t)k + 1);
    for (auto& e : events) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return MGCFD_OK;
  }
  cudaStream_t stream(int m) const { return streams[(size_t)m % streams.size()]; }
  Temp& temp(int m) { return *temps[(size_t)m % temps.size()]; }
  int fork() {
    if (streams.size() < 2) return MGCFD_OK;
    CK(cudaEventRecord(events[0], main));
    for (cudaStream_t sm : streams) CK(cudaStreamWaitEvent(sm, events[0], 0));
    return MGCFD_OK;
  }
  int join() {
    if (streams.size() < 2) return MGCFD_OK;
    for (size_t k = 0; k < streams.size(); k++) {
      CK(cudaEventRecord(events[1 + k], streams[k]));
      CK(cudaStreamWaitEvent(main, events[1 + k], 0));
    }
    return MGCFD_OK;
  }
};

__device__ __forceinline__ bool ok_index(int32_t i, int32_t n, unsigned* err) {
  if ((uint32_t)i < (uint32_t)n) return true;
  atomicAdd(err, 1u);
  return false;
}

// ---- node order -------------------------------------------------------------

__global__ void k_bbox(int32_t n, const double* __restrict__ xyz, unsigned long long* __restrict__ box) {
  __shared__ unsigned long long lo[3], hi[3];
  if (threadIdx.x < 3) { lo[threadIdx.x] = ~0ull; hi[threadIdx.x] = 0ull; }
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    for (int d = 0; d < 3; d++) {
      const unsigned long long k = dkey(xyz[3 * i + d]);
      atomicMin(&lo[d], k);
      atomicMax(&hi[d], k);
    }
  __syncthreads();
  if (threadIdx.x < 3) {
    atomicMin(&box[threadIdx.x], lo[threadIdx.x]);
    atomicMax(&box[3 + threadIdx.x], hi[threadIdx.x]);
  }
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

// Same quantisation as spatial_order() in setup.cpp.
__global__ void k_morton(int32_t n, const double* __restrict__ xyz, const unsigned long long* __restrict__ box,
                         unsigned long long* __restrict__ key, int32_t* __restrict__ val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t q[3];
  for (int d = 0; d < 3; d++) {
    const double lo = dkey_inv(box[d]), hi = dkey_inv(box[3 + d]);
    const double span = __dsub_rn(hi, lo);
    const double scale = (hi > lo && isfinite(span)) ? __ddiv_rn(2097151.0, span) : 0.0;
    double t = __dmul_rn(__dsub_rn(xyz[3 * i + d], lo), scale);
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

__global__ void k_edge_geometry(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n,
                                const double* __restrict__ xyz, const double* __restrict__ ewt_in, int legacy,
                                double* __restrict__ tv, double* __restrict__ w, unsigned* __restrict__ err) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
  const double* wi = ewt_in + 3 * e;
  if (legacy) {  // weights used as read (euler3d.cpp:416-431 skipped)
    for (int i = 0; i < 3; i++) w[3 * e + i] = __dmul_rn(wi[i], 1e-7);
    ok_index(a, nn, err);
    ok_index(b, nn, err);
    return;
  }
  if (!ok_index(a, nn, err) || !ok_index(b, nn, err)) {
    tv[e] = 0.0;
    for (int i = 0; i < 3; i++) w[3 * e + i] = 0.0;
    return;
  }
  double d[3];
  for (int i = 0; i < 3; i++) d[i] = __dsub_rn(xyz[3 * (int64_t)b + i], xyz[3 * (int64_t)a + i]);
  const double dist = __dsqrt_rn(sq3(d[0], d[1], d[2]));
  const double area = __dsqrt_rn(sq3(wi[0], wi[1], wi[2]));
  tv[e] = __dmul_rn(__dmul_rn((1.0 / 3.0) * 0.5, dist), area);
  for (int i = 0; i < 3; i++) w[3 * e + i] = __dmul_rn(__ddiv_rn(__dmul_rn(__ddiv_rn(d[i], dist), area), dist), 1e-7);
}

// Incidence pairs (node, edge) in edge order; a stable sort by node keeps
// each node's edges in increasing id.
__global__ void k_incidence(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, int32_t* __restrict__ key,
                            int32_t* __restrict__ val, int32_t* __restrict__ cnt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int k = 0; k < 2; k++) {
    int32_t v = e2n[2 * e + k];
    if ((uint32_t)v >= (uint32_t)nn) v = nn;  // sentinel: sorts last, never summed
    key[2 * e + k] = v;
    val[2 * e + k] = (int32_t)e;
    if (v < nn) atomicAdd(cnt + v, 1);
  }
}

__global__ void k_volumes(int32_t nn, const int32_t* __restrict__ off, const int32_t* __restrict__ edges,
                          const double* __restrict__ tv, double* __restrict__ vol) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
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

__global__ void k_edge_keys(int32_t ne, int32_t nn, const int32_t* __restrict__ e2n, const int32_t* __restrict__ inv,
                            unsigned long long* __restrict__ key, int32_t* __restrict__ val,
                            unsigned char* __restrict__ flip) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int32_t a = e2n[2 * e], b = e2n[2 * e + 1];
  a = (uint32_t)a < (uint32_t)nn ? inv[a] : 0;  // out-of-range maps were recorded by k_edge_geometry
  b = (uint32_t)b < (uint32_t)nn ? inv[b] : 0;
  const bool f = a > b;
  const uint32_t lo = f ? b : a, hi = f ? a : b;
  key[e] = ((unsigned long long)lo << 32) | hi;
  val[e] = (int32_t)e;
  flip[e] = f;
}

__global__ void k_edge_finalize(int32_t ne, int32_t node_off, const unsigned long long* __restrict__ key,
                                const int32_t* __restrict__ order, const double* __restrict__ w,
                                const unsigned char* __restrict__ flip, double sc, int2* __restrict__ e2n,
                                double* __restrict__ w4, int32_t* __restrict__ acnt, int32_t* __restrict__ bcnt) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ne) return;
  const int64_t e = order[k];
  const int32_t a = (int32_t)(key[k] >> 32), b = (int32_t)(key[k] & 0xffffffffu);
  e2n[k] = make_int2(a + node_off, b + node_off);
  double x = w[3 * e], y = w[3 * e + 1], z = w[3 * e + 2];
  if (flip[e]) { x = -x; y = -y; z = -z; }
  const double mag = __dsqrt_rn(sq3(x, y, z));
  w4[4 * k + 0] = __dmul_rn(-0.5, x);
  w4[4 * k + 1] = __dmul_rn(-0.5, y);
  w4[4 * k + 2] = __dmul_rn(-0.5, z);
  w4[4 * k + 3] = __dmul_rn(__dmul_rn(-mag, sc), 0.5);
  atomicAdd(acnt + a, 1);
  atomicAdd(bcnt + b, 1);
}

__global__ void k_b_pairs(int32_t ne, const int2* __restrict__ e2n, int32_t node_off, int32_t* __restrict__ key,
                          int32_t* __restrict__ val) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ne) return;
  key[k] = e2n[k].y - node_off;
  val[k] = (int32_t)k;
}

__global__ void k_to_float(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)x[i];
}

// ---- boundary -----------------------------------------------------------------

__global__ void k_bnd_keys(int32_t nb, int32_t nn, const int32_t* __restrict__ b2n, const int32_t* __restrict__ grp,
                           const int32_t* __restrict__ inv, int32_t* __restrict__ key, int32_t* __restrict__ val,
                           int32_t* __restrict__ cnt, unsigned* __restrict__ err) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int32_t n = b2n[k];
  const int g = grp[k];
  int32_t node = nn;  // sentinel: ignored entry
  if (ok_index(n, nn, err) && g <= 7) {
    node = inv[n];
    atomicAdd(cnt + node, 1);
  }
  key[k] = node;
  val[k] = (int32_t)k;
}

// Folded boundary rows (flux.h:14-39 is linear in the weight), entries in order.
__global__ void k_bnd_fold(int32_t nn, const int32_t* __restrict__ off, const int32_t* __restrict__ entries,
                           const int32_t* __restrict__ grp, const double* __restrict__ bwt,
                           const int32_t* __restrict__ row_of, const int32_t* __restrict__ row_base,
                           mgcfd_freestream ff,
                           int32_t* __restrict__ bidx,
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
  const int32_t r = row_of[i] + *row_base;
  bidx[i] = r;
  double* row = bdata + 12 * (int64_t)r;
  for (int c = 0; c < 3; c++) { row[c] = wff[c]; row[3 + c] = wwall[c]; }
  const double* fv = ff.ff_variable;
  const double* rows[4] = {ff.ff_flux_contribution_momentum_x, ff.ff_flux_contribution_momentum_y,
                           ff.ff_flux_contribution_momentum_z, ff.ff_flux_contribution_density_energy};
  row[6] = __dadd_rn(__dadd_rn(__dmul_rn(wff[0], fv[1]), __dmul_rn(wff[1], fv[2])), __dmul_rn(wff[2], fv[3]));
  for (int q = 0; q < 4; q++)
    row[7 + q] = __dadd_rn(__dadd_rn(__dmul_rn(wff[0], rows[q][0]), __dmul_rn(wff[1], rows[q][1])),
                           __dmul_rn(wff[2], rows[q][2]));
  row[11] = 0.0;
}

__global__ void k_copy1(const int32_t* __restrict__ src, int32_t* __restrict__ dst) { *dst = *src; }

// base[0] = 0, base[m + 1] = base[m] + count[m] for a handful of meshes.
__global__ void k_exclusive_scan_small(int32_t n, const int32_t* __restrict__ count, int32_t* __restrict__ base) {
  int32_t acc = 0;
  base[0] = 0;
  for (int32_t m = 0; m < n; m++) {
    acc += count[m];
    base[m + 1] = acc;
  }
}

__global__ void k_nonempty(int32_t nn, const int32_t* __restrict__ off, int32_t* __restrict__ flag) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nn) flag[i] = off[i + 1] > off[i] ? 1 : 0;
}

// ---- multigrid ----------------------------------------------------------------

__global__ void k_mg(int32_t nf, int32_t nc, int32_t coarse_off, const int32_t* __restrict__ perm_f,
                     const int32_t* __restrict__ n2mg_in,
                     const int32_t* __restrict__ inv_c, const double* __restrict__ xf, const double* __restrict__ xc,
                     int32_t* __restrict__ n2mg, double* __restrict__ dvec, int32_t* __restrict__ key,
                     int32_t* __restrict__ val, int32_t* __restrict__ cnt, unsigned* __restrict__ err) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int32_t fin = perm_f[f];
  const int32_t cin = n2mg_in[fin];
  int32_t c = 0;
  double dx = 0.0, dy = 0.0, dz = 0.0;
  if (ok_index(cin, nc, err)) {
    c = inv_c[cin];
    dx = fabs(__dsub_rn(xf[3 * (int64_t)fin], xc[3 * (int64_t)cin]));
    dy = fabs(__dsub_rn(xf[3 * (int64_t)fin + 1], xc[3 * (int64_t)cin + 1]));
    dz = fabs(__dsub_rn(xf[3 * (int64_t)fin + 2], xc[3 * (int64_t)cin + 2]));
  }
  n2mg[f] = c + coarse_off;
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

// Per mesh and level: the arrays kept until the multigrid tables are built.
struct LevelTmp {
  int32_t* perm = nullptr;  // local new id -> local input id
  int32_t* inv = nullptr;   // local input id -> local new id
  double* xyz = nullptr;
  int32_t* n2mg_in = nullptr;
  // the level's input arrays on the device
  int32_t *e2n_in = nullptr, *b2n_in = nullptr, *grp_in = nullptr;
  double *ewt_in = nullptr, *bwt_in = nullptr, *vol_in = nullptr;
  // boundary fold inputs, kept for the fold pass after the lanes join
  int32_t *b_off = nullptr, *b_entries = nullptr, *b_row = nullptr;
};

__global__ void k_offset_copy(int32_t n, const int32_t* __restrict__ src, int32_t add, int32_t* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] + add;
}

__global__ void k_fill(int32_t n, int32_t value, int32_t* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = value;
}

}  // namespace

int device_prepare(mgcfd_solver* s, const std::vector<MeshInput>& meshes) {
  cudaStream_t st = s->stream;
  Temp tmp(st);
  Lanes lanes(st);
  if (int r0 = lanes.init((int)meshes.size())) return r0;
  unsigned* err = nullptr;
  int r = tmp.get(&err, 1);
  if (r) return r;
  CK(cudaMemsetAsync(err, 0, sizeof(unsigned), st));
  const bool mixed = s->opt.precision == MGCFD_PRECISION_MIXED;
  const int nseg = (int)meshes.size();
  const int nlevels = (int)s->L.size();
  std::vector<std::vector<LevelTmp>> lt((size_t)nseg, std::vector<LevelTmp>((size_t)nlevels));
  s->seg_noff.assign((size_t)nlevels, std::vector<int32_t>((size_t)nseg + 1, 0));
  std::vector<std::vector<int32_t>> seg_eoff((size_t)nlevels, std::vector<int32_t>((size_t)nseg + 1, 0));
  for (int l = 0; l < nlevels; l++)
    for (int m = 0; m < nseg; m++) {
      const mgcfd_level_view& v = meshes[(size_t)m].levels[l];
      s->seg_noff[(size_t)l][(size_t)m + 1] = s->seg_noff[(size_t)l][(size_t)m] + v.nnodes;
      seg_eoff[(size_t)l][(size_t)m + 1] = seg_eoff[(size_t)l][(size_t)m] + v.nedges;
    }

  for (int l = 0; l < nlevels; l++) {
    DevLevel& D = s->L[(size_t)l];
    const int32_t N = s->seg_noff[(size_t)l][(size_t)nseg], NE = seg_eoff[(size_t)l][(size_t)nseg];
    int64_t NB = 0;
    for (int m = 0; m < nseg; m++) NB += meshes[(size_t)m].levels[l].nbnd;
    D.n = N; D.ne = NE; D.nb = (int32_t)NB;
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
    if (nseg > 1 && (r = s->alloc(&D.mesh_id, (size_t)N))) return r;
    // Folded boundary rows of mesh m start at row_base[m]; the offsets stay on
    // the device, so the meshes' setup work is queued without host round trips.
    int32_t *row_base, *rows_tot;
    if ((r = tmp.get(&row_base, (size_t)nseg + 1)) || (r = tmp.get(&rows_tot, (size_t)nseg))) return r;
    if ((r = lanes.fork())) return r;

    // Upload every mesh's input arrays first: a copy from pageable host
    // memory may wait for the stream, so the copies go ahead of the kernels.
    for (int m = 0; m < nseg; m++) {
      const cudaStream_t st = lanes.stream(m);
      Temp& tmp = lanes.temp(m);
      const mgcfd_level_view& v = meshes[(size_t)m].levels[l];
      LevelTmp& T_ = lt[(size_t)m][(size_t)l];
      const int32_t n = v.nnodes, ne = v.nedges, nb = v.nbnd;
      if ((r = tmp.get(&T_.xyz, 3 * (size_t)n)) || (r = tmp.get(&T_.e2n_in, 2 * (size_t)ne)) ||
          (r = tmp.get(&T_.ewt_in, 3 * (size_t)ne)) || (r = tmp.get(&T_.b2n_in, (size_t)nb)) ||
          (r = tmp.get(&T_.grp_in, (size_t)nb)) || (r = tmp.get(&T_.bwt_in, 3 * (size_t)nb)) ||
          (r = tmp.get(&T_.vol_in, (size_t)n)))
        return r;
      CK(cudaMemcpyAsync(T_.xyz, v.coords, 24 * (size_t)n, cudaMemcpyHostToDevice, st));
      if (ne) {
        CK(cudaMemcpyAsync(T_.e2n_in, v.edge_to_nodes, 8 * (size_t)ne, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(T_.ewt_in, v.edge_weights, 24 * (size_t)ne, cudaMemcpyHostToDevice, st));
      }
      if (nb) {
        CK(cudaMemcpyAsync(T_.b2n_in, v.bnd_to_node, 4 * (size_t)nb, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(T_.grp_in, v.bnd_group, 4 * (size_t)nb, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(T_.bwt_in, v.bnd_weights, 24 * (size_t)nb, cudaMemcpyHostToDevice, st));
      }
      if (v.volumes) CK(cudaMemcpyAsync(T_.vol_in, v.volumes, 8 * (size_t)n, cudaMemcpyHostToDevice, st));
      if (v.node_to_mg) {
        if ((r = tmp.get(&T_.n2mg_in, (size_t)n))) return r;
        CK(cudaMemcpyAsync(T_.n2mg_in, v.node_to_mg, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
      }
    }

    for (int m = 0; m < nseg; m++) {
      const cudaStream_t st = lanes.stream(m);
      Temp& tmp = lanes.temp(m);
      const mgcfd_level_view& v = meshes[(size_t)m].levels[l];
      const mgcfd_freestream& ff = meshes[(size_t)m].ff;
      const double sc = ff.smoothing_coefficient;
      LevelTmp& T_ = lt[(size_t)m][(size_t)l];
      const int32_t n = v.nnodes, ne = v.nedges, nb = v.nbnd;
      const int32_t noff = s->seg_noff[(size_t)l][(size_t)m], eoff = seg_eoff[(size_t)l][(size_t)m];
      const int32_t *e2n_in = T_.e2n_in, *b2n_in = T_.b2n_in, *grp_in = T_.grp_in;
      const double *ewt_in = T_.ewt_in, *bwt_in = T_.bwt_in;
      if (nseg > 1) k_fill<<<nblk(n), T, 0, st>>>(n, m, D.mesh_id + noff);

      // Node order (local to the mesh).
      if ((r = tmp.get(&T_.perm, (size_t)n)) || (r = tmp.get(&T_.inv, (size_t)n))) return r;
      if (s->opt.renumber == MGCFD_RENUMBER_SPATIAL) {
        unsigned long long *box, *key, *key2;
        int32_t* val;
        if ((r = tmp.get(&box, 6)) || (r = tmp.get(&key, (size_t)n)) || (r = tmp.get(&key2, (size_t)n)) ||
            (r = tmp.get(&val, (size_t)n)))
          return r;
        CK(cudaMemsetAsync(box, 0xff, 3 * sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(box + 3, 0, 3 * sizeof(unsigned long long), st));
        k_bbox<<<nblk(n), T, 0, st>>>(n, T_.xyz, box);
        k_morton<<<nblk(n), T, 0, st>>>(n, T_.xyz, box, key, val);
        if ((r = sort_pairs(tmp, key, key2, val, T_.perm, n, 63, st))) return r;
      } else {
        k_iota<<<nblk(n), T, 0, st>>>(n, T_.perm);
      }
      k_inverse<<<nblk(n), T, 0, st>>>(n, T_.perm, T_.inv);
      k_offset_copy<<<nblk(n), T, 0, st>>>(n, T_.perm, noff, D.perm + noff);

      // Geometry and volumes.
      double *tv, *wd;
      double* vol_in = T_.vol_in;
      if ((r = tmp.get(&tv, (size_t)ne)) || (r = tmp.get(&wd, 3 * (size_t)ne))) return r;
      if (ne) k_edge_geometry<<<nblk(ne), T, 0, st>>>(ne, n, e2n_in, T_.xyz, ewt_in, v.volumes != nullptr, tv, wd, err);
      if (!v.volumes) {
        int32_t *ikey, *ival, *ikey2, *ival2, *cnt, *off;
        if ((r = tmp.get(&ikey, 2 * (size_t)ne)) || (r = tmp.get(&ival, 2 * (size_t)ne)) ||
            (r = tmp.get(&ikey2, 2 * (size_t)ne)) || (r = tmp.get(&ival2, 2 * (size_t)ne)) ||
            (r = tmp.get(&cnt, (size_t)n + 1)) || (r = tmp.get(&off, (size_t)n + 1)))
          return r;
        CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)n + 1), st));
        if (ne) k_incidence<<<nblk(ne), T, 0, st>>>(ne, n, e2n_in, ikey, ival, cnt);
        if ((r = sort_pairs(tmp, ikey, ikey2, ival, ival2, 2 * (int64_t)ne, bits_for(n), st))) return r;
        if ((r = offsets(tmp, cnt, off, n, st))) return r;
        k_volumes<<<nblk(n), T, 0, st>>>(n, off, ival2, tv, vol_in);
      }
      k_node_constants<<<nblk(n), T, 0, st>>>(n, T_.perm, vol_in, D.vol + noff, D.inv_vol + noff, D.cbrt_vol + noff);

      // Edges: orientation, order, weights, CSR.
      {
        unsigned long long *key, *key2;
        int32_t *val, *order, *acnt, *bcnt;
        unsigned char* flip;
        if ((r = tmp.get(&key, (size_t)ne)) || (r = tmp.get(&key2, (size_t)ne)) || (r = tmp.get(&val, (size_t)ne)) ||
            (r = tmp.get(&order, (size_t)ne)) || (r = tmp.get(&flip, (size_t)ne)) ||
            (r = tmp.get(&acnt, (size_t)n + 1)) || (r = tmp.get(&bcnt, (size_t)n + 1)))
          return r;
        CK(cudaMemsetAsync(acnt, 0, sizeof(int32_t) * ((size_t)n + 1), st));
        CK(cudaMemsetAsync(bcnt, 0, sizeof(int32_t) * ((size_t)n + 1), st));
        if (ne) {
          k_edge_keys<<<nblk(ne), T, 0, st>>>(ne, n, e2n_in, T_.inv, key, val, flip);
          if ((r = sort_pairs(tmp, key, key2, val, order, ne, 32 + bits_for(n), st))) return r;
          k_edge_finalize<<<nblk(ne), T, 0, st>>>(ne, noff, key2, order, wd, flip, sc, D.e2n + eoff,
                                                  w4all + 4 * (size_t)eoff, acnt, bcnt);
        }
        if (s->gather) {
          int32_t *aoff, *boff, *bkey, *bval, *bkey2, *blist;
          if ((r = tmp.get(&aoff, (size_t)n + 1)) || (r = tmp.get(&boff, (size_t)n + 1)) ||
              (r = tmp.get(&bkey, (size_t)ne)) || (r = tmp.get(&bval, (size_t)ne)) ||
              (r = tmp.get(&bkey2, (size_t)ne)) || (r = tmp.get(&blist, (size_t)ne)))
            return r;
          if ((r = offsets(tmp, acnt, aoff, n, st)) || (r = offsets(tmp, bcnt, boff, n, st))) return r;
          k_offset_copy<<<nblk(n), T, 0, st>>>(n, aoff, eoff, D.a_off + noff);
          k_offset_copy<<<nblk(n), T, 0, st>>>(n, boff, eoff, D.b_off + noff);
          if (ne) {
            k_b_pairs<<<nblk(ne), T, 0, st>>>(ne, D.e2n + eoff, noff, bkey, bval);
            if ((r = sort_pairs(tmp, bkey, bkey2, bval, blist, ne, bits_for(n), st))) return r;
            k_offset_copy<<<nblk(ne), T, 0, st>>>(ne, blist, eoff, D.b_list + eoff);
          }
        }
      }

      // Boundary entries folded per node.
      {
        int32_t *key, *val, *key2, *val2, *cnt, *off, *flag, *row;
        if ((r = tmp.get(&key, (size_t)nb)) || (r = tmp.get(&val, (size_t)nb)) || (r = tmp.get(&key2, (size_t)nb)) ||
            (r = tmp.get(&val2, (size_t)nb)) || (r = tmp.get(&cnt, (size_t)n + 1)) ||
            (r = tmp.get(&off, (size_t)n + 1)) || (r = tmp.get(&flag, (size_t)n + 1)) ||
            (r = tmp.get(&row, (size_t)n + 1)))
          return r;
        CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)n + 1), st));
        if (nb) {
          k_bnd_keys<<<nblk(nb), T, 0, st>>>(nb, n, b2n_in, grp_in, T_.inv, key, val, cnt, err);
          if ((r = sort_pairs(tmp, key, key2, val, val2, nb, bits_for(n), st))) return r;
        }
        if ((r = offsets(tmp, cnt, off, n, st))) return r;
        CK(cudaMemsetAsync(flag, 0, sizeof(int32_t) * ((size_t)n + 1), st));
        k_nonempty<<<nblk(n), T, 0, st>>>(n, off, flag);
        if ((r = offsets(tmp, flag, row, n, st))) return r;
        k_copy1<<<1, 1, 0, st>>>(row + n, rows_tot + m);
        T_.b_off = off;
        T_.b_entries = val2;
        T_.b_row = row;
      }
    }
    // Row offsets of every mesh's folded boundary rows, then the fold.
    if ((r = lanes.join())) return r;
    k_exclusive_scan_small<<<1, 1, 0, st>>>(nseg, rows_tot, row_base);
    if ((r = lanes.fork())) return r;
    for (int m = 0; m < nseg; m++) {
      const LevelTmp& T_ = lt[(size_t)m][(size_t)l];
      const int32_t n = meshes[(size_t)m].levels[l].nnodes, noff = s->seg_noff[(size_t)l][(size_t)m];
      k_bnd_fold<<<nblk(n), T, 0, lanes.stream(m)>>>(n, T_.b_off, T_.b_entries, T_.grp_in, T_.bwt_in, T_.b_row,
                                                   row_base + m, meshes[(size_t)m].ff, D.bidx + noff, D.bdata);
    }
    if ((r = lanes.join())) return r;
    CK(cudaMemcpyAsync(&D.nbrows, row_base + nseg, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (s->gather) {
      k_fill<<<1, 1, 0, st>>>(1, NE, D.a_off + N);
      k_fill<<<1, 1, 0, st>>>(1, NE, D.b_off + N);
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
    if ((r = s->alloc(&F.n2mg, (size_t)F.n)) || (r = s->alloc(&F.dvec, (size_t)F.n)) ||
        (r = s->alloc(&Cl.ch_off, (size_t)Cl.n + 1)) || (r = s->alloc(&Cl.ch_list, (size_t)F.n)))
      return r;
    Cl.nfine = F.n;
    if ((r = lanes.fork())) return r;
    for (int m = 0; m < nseg; m++) {
      const cudaStream_t st = lanes.stream(m);
      Temp& tmp = lanes.temp(m);
      const int32_t nf = meshes[(size_t)m].levels[l].nnodes, nc = meshes[(size_t)m].levels[l + 1].nnodes;
      const int32_t noff_f = s->seg_noff[(size_t)l][(size_t)m], noff_c = s->seg_noff[(size_t)l + 1][(size_t)m];
      int32_t *key, *val, *key2, *cnt, *off, *list;
      if ((r = tmp.get(&key, (size_t)nf)) || (r = tmp.get(&val, (size_t)nf)) || (r = tmp.get(&key2, (size_t)nf)) ||
          (r = tmp.get(&cnt, (size_t)nc + 1)) || (r = tmp.get(&off, (size_t)nc + 1)) || (r = tmp.get(&list, (size_t)nf)))
        return r;
      CK(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ((size_t)nc + 1), st));
      const LevelTmp& TF = lt[(size_t)m][(size_t)l];
      const LevelTmp& TC = lt[(size_t)m][(size_t)l + 1];
      k_mg<<<nblk(nf), T, 0, st>>>(nf, nc, noff_c, TF.perm, TF.n2mg_in, TC.inv, TF.xyz, TC.xyz, F.n2mg + noff_f,
                                   reinterpret_cast<double*>(F.dvec) + 4 * (size_t)noff_f, key, val, cnt, err);
      if ((r = sort_pairs(tmp, key, key2, val, list, nf, bits_for(nc), st))) return r;
      if ((r = offsets(tmp, cnt, off, nc, st))) return r;
      k_offset_copy<<<nblk(nf), T, 0, st>>>(nf, list, noff_f, Cl.ch_list + noff_f);
      k_offset_copy<<<nblk(nc), T, 0, st>>>(nc, off, noff_f, Cl.ch_off + noff_c);
    }
    if ((r = lanes.join())) return r;
    k_fill<<<1, 1, 0, st>>>(1, F.n, Cl.ch_off + Cl.n);
  }
  CK(cudaGetLastError());
  unsigned h_err = 0;
  CK(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (h_err) return set_error(MGCFD_ERR_INVALID, "mesh has " + std::to_string(h_err) + " map entries out of range");
  return MGCFD_OK;
}

}  // namespace mgcfd
