// Internal state of the device solver, shared by solver.cu (kernels and the
// V-cycle driver) and device_setup.cu (building the per-level tables on the
// GPU).  Device memory comes from the stream-ordered allocator
// (cudaMallocAsync on the solver's stream) so that repeated solves reuse
// pooled memory instead of paying for cudaMalloc each time.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "common.h"

constexpr int kMaxLevels = 16;
constexpr int kMaxDevices = 64;

#define CK(call)                                                                                         \
  do {                                                                                                   \
    cudaError_t e_ = (call);                                                                             \
    if (e_ != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct DevStatus {
  unsigned long long dt_key[kMaxLevels];  // order-preserving key of each level's min_dt (the step
                                           // begun last: a prolongation begins its fine level's next step)
  unsigned long long dt_key_used[kMaxLevels];  // the key each level's last finished step used
  int halt;                                // non-zero: stop all further work
  int neg_dt;                              // min_dt < 0 seen
  int bad_count;                           // NaN/Inf count at level 0
  int stopped;                             // the stop rule ended the solve (not an error)
  double rms_acc;                          // sum of residual^2, last level-0 step
  double rho_acc;                          // its density part
  // Stop rule (solvers run by the server): V-cycles completed and the
  // level-0 density residual norm of the first and the latest of them.
  int cycles_done;
  int pad;
  double rho_first;
  double rho_last;
};

// Per-mesh stop rule of a batched solver (the serving loop's cohorts): like
// DevStatus's cycles_done / rho_first / rho_last / stopped, one per mesh, and
// `halt`, which every batched node kernel checks for its node's mesh.
struct SegStop {
  int halt;         // non-zero: this mesh's state no longer changes
  int stopped;      // the stop rule ended this mesh's solve (not an error)
  int cycles_done;
  int pad;
  double rho_first;
  double rho_last;
};

struct DevLevel {
  int32_t n = 0, ne = 0, nb = 0;
  int32_t nbrows = 0;  // folded boundary rows in bdata
  int32_t nfine = 0;   // fine nodes (length of ch_list) when this level has a finer one
  double* rec = nullptr;
  float* rec32 = nullptr;
  float* rec32b = nullptr;  // second FP32 primitive buffer (fused stages ping-pong)
  double* old = nullptr;
  double* flux = nullptr;
  double* res = nullptr;
  double* dummy = nullptr;
  double* inv_vol = nullptr;
  double* cbrt_vol = nullptr;
  double* vol = nullptr;
  int2* e2n = nullptr;
  double4_32a* w4 = nullptr;
  float4* w4f = nullptr;
  double* rec2 = nullptr;         // DW: [N][8] node primitives as pair words (dw_math.cuh)
  double4_32a* w4dw = nullptr;    // DW: [E] w4 as pair words
  double* rec2b = nullptr;        // DW fused: second primitive buffer (stages ping-pong)
  int32_t* off2 = nullptr;        // DW fused: [N+1] each node's entries in ent2 (a_off + b_off)
  int2* ent2 = nullptr;           // DW fused: [2E] a node's a-side edges, then its b-side ones: (neighbour,
                                  // edge index, bit 31 set on the b side)
  double* fe = nullptr;     // [E][5] per-edge fluxes, FP64 gather
  float* fe32 = nullptr;    // [E][5] per-edge fluxes, mixed-precision gather
  int32_t* a_off = nullptr;
  int32_t* b_off = nullptr;
  int32_t* b_list = nullptr;
  int32_t* b_nbr = nullptr;   // fused: end a of each edge in b_list order
  float4* b_w4f = nullptr;    // fused: w4f of each edge in b_list order
  int32_t* bidx = nullptr;
  double* bdata = nullptr;
  int32_t* n2mg = nullptr;
  double4_32a* dvec = nullptr;
  int32_t* ch_off = nullptr;
  int32_t* ch_list = nullptr;
  int32_t* perm = nullptr;
  int32_t* mesh_id = nullptr;  // [n] mesh of each node (batched solvers only)
  std::vector<int32_t> colour_off;  // COLOURED: edges [colour_off[c], colour_off[c+1]) share no node
};

struct mgcfd_solver {
  mgcfd_solver_options opt{};
  mgcfd_freestream ff{};
  cudaStream_t stream = nullptr;
  bool owns_stream = false;  // graph capture needs a non-legacy stream
  int device = 0;
  std::vector<DevLevel> L;
  std::vector<void*> allocs;
  DevStatus* st = nullptr;
  double* fetch_buf = nullptr;
  int64_t device_bytes = 0;
  // Batched solvers: nseg meshes concatenated per level (nseg == 1: plain).
  int nseg = 1;
  std::vector<std::vector<int32_t>> seg_noff;    // [level][nseg + 1] node offsets
  std::vector<mgcfd_freestream> seg_ff;          // per mesh
  unsigned long long* seg_keys = nullptr;        // [2][kMaxLevels][nseg] min_dt keys, then the keys used
  int* seg_neg = nullptr;                        // [nseg] min_dt < 0 seen
  int* seg_bad = nullptr;                        // [nseg] NaN/Inf count at level 0
  double* seg_rms = nullptr;                     // [nseg] sum of residual^2, last level-0 step
  double* seg_rho = nullptr;                     // [nseg] its density part
  double* seg_ffvar = nullptr;                   // [nseg][5] freestream states
  SegStop* seg_stop = nullptr;                   // [nseg] per-mesh stop rule (when installed)
  double* seg_n0 = nullptr;                      // [nseg] level-0 node counts, for the norms
  std::vector<int> seg_status;                   // host copy after synchronize
  // V-cycle state (euler3d.cpp:452-457).
  int64_t cycle = 0;
  int level = 0;
  bool up = true;
  int64_t steps = 0;
  int64_t launches = 0;
  int64_t launches_per_cycle = 0;
  bool begun = false;   // the next smoothing step's begin is already enqueued (by a prolongation or set-up)
  bool gather = false;  // node-side CSR tables exist (GATHER or FUSED)
  bool fused = false;   // FUSED: flux and update in one node-centric kernel
  bool coloured = false;  // COLOURED: one flux launch per colour class, plain increments
  int fused_variant = 0;  // FUSED: 0 per-node edge loop, 1 neighbour ids staged by cp.async, 2 edge-parallel
  cudaGraphExec_t graph = nullptr;
  // Kernel timing.
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending, spare;
  double flux_ms = 0.0;
  int64_t flux_sweeps = 0;
  int status = MGCFD_OK;
  // Stop rule evaluated on the device at the end of every V-cycle (0 = off):
  // stop after stop_max_cycles cycles, or once the level-0 density residual
  // norm is at most stop_drop times that of the first cycle.
  int32_t stop_max_cycles = 0;
  double stop_drop = 0.0;

  template <class T>
  int alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return MGCFD_OK;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(p), count * sizeof(T), stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return mgcfd::set_error(MGCFD_ERR_NOMEM, "device allocation of " + std::to_string(count * sizeof(T)) +
                                            " bytes failed: " + cudaGetErrorString(e));
    }
    allocs.push_back(*p);
    device_bytes += (int64_t)(count * sizeof(T));
    return MGCFD_OK;
  }
  template <class T>
  int upload(T** p, const void* src, size_t count) {
    int r = alloc(p, count);
    if (r) return r;
    if (count) CK(cudaMemcpyAsync(*p, src, count * sizeof(T), cudaMemcpyHostToDevice, stream));
    return MGCFD_OK;
  }
};

namespace mgcfd {
struct MeshInput {
  const mgcfd_level_view* levels;  // s->L.size() levels
  mgcfd_freestream ff;
};
// Builds every per-level device table of `s` on the GPU from one or more
// meshes (concatenated per level, each renumbered on its own), device_setup.cu.
// For one mesh the results equal prepare_mesh() in setup.cpp.
int device_prepare(mgcfd_solver* s, const std::vector<MeshInput>& meshes);

// FUSED increment: the second FP32 primitive buffer and the b-side copies
// (b_nbr, b_w4f) of a level whose e2n, w4f and b_list are in place.
int build_fused_tables(mgcfd_solver* s, DevLevel& D);

// Re-initialises a plain solver for a new freestream (Mach, angle of
// attack): far-field boundary terms, state and counters, as a fresh solver
// on the same mesh would have them.  Stream-ordered.
int solver_retarget(mgcfd_solver* s, double mach, double aoa_deg);

// Installs the device-side stop rule before the solver's first run (the
// V-cycle graph is captured with it).  On a batched solver it applies to
// every mesh separately: a mesh that meets it (or fails) stops changing
// while the others go on.
int solver_set_stop_rule(mgcfd_solver* s, int32_t max_cycles, double residual_drop);
}  // namespace mgcfd
