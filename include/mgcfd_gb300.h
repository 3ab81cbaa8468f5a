/*
 * mgcfd_gb300 -- C ABI of the GB300-native MG-CFD multigrid Euler hot path.
 *
 * Reference: warwick-hpsc/MG-CFD-app-OP2.  In the reference every step of the
 * V-cycle is an OP2 parallel loop,
 *     op_par_loop(kernel, "name", set, op_arg_dat(...), ...)
 * over an elemental kernel with plain pointer arguments (for example
 * compute_flux_edge_kernel, flux.h:41-46).  OP2's code generator turns each
 * such call into a backend-specific host stub.  This library is what such a
 * stub binds to on GB300:
 *
 *   1. Per-loop entry points (mgcfd_op_*), one per op_par_loop of the hot
 *      path.  Arguments are device pointers to arrays in exactly the layout
 *      of the OP2 dats and maps they replace (row-major [set size][dim],
 *      0-based int32 maps), the set size, and the CUDA stream (cudaStream_t
 *      passed as void*, NULL = default stream).  The call enqueues work and
 *      returns; increments land in unspecified order (FP64 atomics), so
 *      sums differ from OP2's sequential order only by rounding.  Mapped
 *      loops also take the size of the set the map points into; an element
 *      whose map entry is out of range is skipped and counted (see
 *      mgcfd_op_map_errors) instead of being dereferenced.
 *   2. A device-resident solver (mgcfd_solver_*) that owns a whole multigrid
 *      mesh in HBM and runs complete V-cycles (euler3d.cpp:452-641) with
 *      renumbered, fused kernels and no host synchronisation inside a cycle.
 *   3. Host helpers: synthetic meshes, the input.dat + HDF5 mesh layout
 *      (euler3d.cpp:243-336, io.h:28-205) and the far-field state
 *      (euler3d.cpp:157-189).
 *
 * Conventions: every function returns an int status (MGCFD_OK = 0); no C++
 * exception crosses the ABI; mgcfd_last_error() gives a message for the last
 * failure on the calling thread.  The reference prints and exits where this
 * library returns MGCFD_ERR_NEGATIVE_DT (euler3d.cpp:480-484) or
 * MGCFD_ERR_BAD_VALUES (euler3d.cpp:539-548).
 */
#ifndef MGCFD_GB300_H
#define MGCFD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MGCFD_ABI_VERSION 1

enum {
  MGCFD_OK = 0,
  MGCFD_ERR_INVALID = 1,      /* bad argument, size or call order */
  MGCFD_ERR_CUDA = 2,         /* CUDA runtime error (message in mgcfd_last_error) */
  MGCFD_ERR_NOMEM = 3,        /* host or device allocation failed */
  MGCFD_ERR_IO = 4,           /* file missing, unreadable or malformed */
  MGCFD_ERR_NEGATIVE_DT = 5,  /* min_dt < 0 (euler3d.cpp:480-484) */
  MGCFD_ERR_BAD_VALUES = 6,   /* NaN/Inf in level-0 variables (euler3d.cpp:539-548) */
  MGCFD_ERR_TIMEOUT = 7,      /* a bounded device-side wait gave up */
  MGCFD_ERR_BUDGET = 8        /* request exceeds the configured HBM budget */
};

int mgcfd_abi_version(void);
const char* mgcfd_status_string(int status);
const char* mgcfd_last_error(void);

/* ------------------------------------------------------------------------ */
/* Far-field state: global.h:4-14 values computed as euler3d.cpp:157-189,   */
/* with Mach and angle of attack (degrees) as run-time inputs (the          */
/* reference fixes them in const.h:32-33 at 1.2 and 0.0).                   */
typedef struct mgcfd_freestream {
  double smoothing_coefficient;                 /* euler3d.cpp:47: double(0.2f) */
  double ff_variable[5];
  double ff_flux_contribution_momentum_x[3];
  double ff_flux_contribution_momentum_y[3];
  double ff_flux_contribution_momentum_z[3];
  double ff_flux_contribution_density_energy[3];
} mgcfd_freestream;

int mgcfd_freestream_init(double mach, double aoa_deg, mgcfd_freestream* out);

/* ------------------------------------------------------------------------ */
/* Host meshes.                                                             */
typedef struct mgcfd_level_view {
  int32_t nnodes, nedges, nbnd, n_axis;  /* n_axis: lattice size for synthetic meshes, else 0 */
  const double* coords;         /* [nnodes][3]  "node_coordinates"   */
  const int32_t* edge_to_nodes; /* [nedges][2]  "edge-->node", 0-based */
  const int32_t* bnd_to_node;   /* [nbnd]       "bnd_node-->node"    */
  const int32_t* bnd_group;     /* [nbnd]       "bnd_node-->group"   */
  const double* edge_weights;   /* [nedges][3]  "edge_weights"       */
  const double* bnd_weights;    /* [nbnd][3]    "bnd_node_weights"   */
  const int32_t* node_to_mg;    /* [nnodes]     "node-->mg_node" (NULL on the coarsest level) */
  const double* volumes;        /* [nnodes] legacy-mode dual volumes ("areas", euler3d.cpp:292-299);
                                   NULL = compute them from the edges (euler3d.cpp:416-431) */
} mgcfd_level_view;

typedef struct mgcfd_host_mesh mgcfd_host_mesh;

/* Seeded jittered-lattice mesh (n^3 nodes on level 0, `nlevels` levels). */
int mgcfd_host_mesh_generate(int n, int nlevels, uint64_t seed, mgcfd_host_mesh** out);
/* Read an input.dat deck (io.h:28-205 semantics, base_array_index default 1)
 * and its per-level HDF5 files; input_dir may be NULL or "" (euler3d.cpp:84-100).
 * legacy_mode selects the ".renumbered"/"edge_weights.recalculated"/"areas"
 * datasets of euler3d.cpp:247-309; legacy volumes are used as read and the
 * edge weights are not re-oriented (euler3d.cpp:416-431 is skipped). */
int mgcfd_host_mesh_load(const char* input_file, const char* input_dir, int legacy_mode,
                         mgcfd_host_mesh** out);
/* Write "<dir>/<prefix>L<l>.h5" per level and "<dir>/input.dat".  With
 * legacy_datasets != 0 the files also hold the legacy-mode datasets
 * ("*.renumbered", "areas", "edge_weights.recalculated"; euler3d.cpp:247-309). */
int mgcfd_host_mesh_write(const mgcfd_host_mesh* mesh, const char* dir, const char* prefix,
                          int32_t legacy_datasets);
/* A host mesh holding copies of the caller's level arrays (any mesh, not only
 * a synthetic lattice), e.g. to write it in the reference's layout. */
int mgcfd_host_mesh_from_views(int32_t nlevels, const mgcfd_level_view* levels, mgcfd_host_mesh** out);
int mgcfd_host_mesh_num_levels(const mgcfd_host_mesh* mesh);
/* Views stay valid until the mesh is destroyed. */
int mgcfd_host_mesh_level(const mgcfd_host_mesh* mesh, int level, mgcfd_level_view* out);
void mgcfd_host_mesh_destroy(mgcfd_host_mesh* mesh);

/* Mesh renumbering as a standalone step.  Replaces the reference's -n option
 * (config.h:119,366; op_renumber(p_edge_to_nodes[0]) at euler3d.cpp:377, a
 * Scotch reordering of the level-0 nodes inside OP2) with the solver's own
 * orders, method = MGCFD_RENUMBER_SPATIAL (Morton curve of the coordinates)
 * or MGCFD_RENUMBER_RCM (reverse Cuthill-McKee of the edge graph).
 *
 * mgcfd_renumber_nodes writes perm_out[new] = old for one node set.
 * mgcfd_host_mesh_renumber returns a new mesh with every level relabelled:
 * node data permuted, edge endpoints and boundary entries mapped through the
 * inverse permutation (edges keep their direction and are ordered by the new
 * (min, max) endpoint pair, boundary entries by node; ties keep input order),
 * and node-->mg_node mapped on both sides.  The input mesh is not changed. */
int mgcfd_renumber_nodes(int method, int32_t nnodes, const double* coords, int32_t nedges,
                         const int32_t* edge_to_nodes, int32_t* perm_out);
int mgcfd_host_mesh_renumber(const mgcfd_host_mesh* mesh, int method, mgcfd_host_mesh** out);

/* HDF5 subset used by the reference's files (op_decl_*_hdf5 and
 * op_fetch_data_hdf5_file in euler3d.cpp).  dims receives up to 2 extents. */
int mgcfd_h5_dataset_shape(const char* path, const char* name, int64_t dims[2], int* rank);
int mgcfd_h5_read_f64(const char* path, const char* name, double* out, int64_t nelems);
int mgcfd_h5_read_i32(const char* path, const char* name, int32_t* out, int64_t nelems);
/* Writes a new file holding one [rows][cols] float64 dataset with OP2's
 * "size"/"dim"/"type" attributes (the op_fetch_data_hdf5_file layout). */
int mgcfd_h5_write_f64(const char* path, const char* name, const double* data, int64_t rows, int64_t cols);

/* ------------------------------------------------------------------------ */
/* Per-loop drop-in entry points (device pointers, OP2 dat layout).         */
/* Each replaces one op_par_loop of euler3d.cpp; the elemental kernel it    */
/* implements is cited.                                                     */

/* initialize_variables_kernel, misc.h:10-16; loop euler3d.cpp:414-415. */
int mgcfd_op_initialize_variables(int32_t nnodes, const mgcfd_freestream* ff, double* variables, void* stream);
/* zero_5d/3d/1d_array_kernel, misc.h:18-38; euler3d.cpp:416-424. */
int mgcfd_op_zero(int32_t n, int32_t dim, double* array, void* stream);
/* calculate_cell_volumes, misc.h:40-76; euler3d.cpp:425-431 (edge weights OP_RW,
 * volumes OP_INC). */
int mgcfd_op_calculate_cell_volumes(int32_t nedges, int32_t nnodes, const int32_t* edge_to_nodes,
                                    const double* coords, double* edge_weights, double* volumes, void* stream);
/* dampen_ewt, misc.h:78-84; euler3d.cpp:436-441 (n elements of dim 3). */
int mgcfd_op_dampen_ewt(int32_t n, double* weights, void* stream);
/* copy_double_kernel, copy_double_kernel.h:6-13; euler3d.cpp:467-469. */
int mgcfd_op_copy_double(int32_t nnodes, const double* variables, double* old_variables, void* stream);
/* calculate_dt_kernel, time_stepping_kernels.h:13-32; euler3d.cpp:472-475. */
int mgcfd_op_calculate_dt(int32_t nnodes, const double* variables, const double* volumes, double* dt,
                          void* stream);
/* get_min_dt_kernel with OP_MIN, time_stepping_kernels.h:34-41; euler3d.cpp:476-479.
 * Writes min(DBL_MAX, dt[0..n)) to the device scalar *min_dt (NaNs ignored,
 * as `dt < min` is false for them). */
int mgcfd_op_get_min_dt(int32_t nnodes, const double* dt, double* min_dt, void* stream);
/* compute_step_factor_kernel, time_stepping_kernels.h:43-64; euler3d.cpp:485-489.
 * min_dt is a device scalar. */
int mgcfd_op_compute_step_factor(int32_t nnodes, const double* variables, const double* volumes,
                                 const double* min_dt, double* step_factors, void* stream);
/* compute_flux_edge_kernel, flux.h:41-208; euler3d.cpp:498-503 (both ends OP_INC). */
int mgcfd_op_compute_flux_edge(int32_t nedges, int32_t nnodes, const int32_t* edge_to_nodes,
                               const double* variables, const double* edge_weights,
                               double smoothing_coefficient, double* fluxes, void* stream);
/* compute_bnd_node_flux_kernel, flux.h:14-39; euler3d.cpp:505-509. */
int mgcfd_op_compute_bnd_node_flux(int32_t nbnd, int32_t nnodes, const int32_t* bnd_to_node,
                                   const int32_t* bnd_group,
                                   const double* bnd_weights, const double* variables,
                                   const mgcfd_freestream* ff, double* fluxes, void* stream);
/* time_step_kernel, time_stepping_kernels.h:66-86; euler3d.cpp:511-516. */
int mgcfd_op_time_step(int32_t nnodes, int32_t rk_cycle, const double* step_factors, double* fluxes,
                       const double* old_variables, double* variables, void* stream);
/* unstructured_stream_kernel, unstructured_stream.h:7-57; euler3d.cpp:518-525. */
int mgcfd_op_unstructured_stream(int32_t nedges, int32_t nnodes, const int32_t* edge_to_nodes,
                                 const double* variables, const double* edge_weights, double* fluxes,
                                 void* stream);
/* residual_kernel, validation.h:27-35; euler3d.cpp:528-531. */
int mgcfd_op_residual(int32_t nnodes, const double* old_variables, const double* variables,
                      double* residuals, void* stream);
/* calc_rms_kernel with OP_INC, validation.h:37-44; euler3d.cpp:533-537.
 * Adds sum(residual^2) to the device scalar *rms. */
int mgcfd_op_calc_rms(int32_t nnodes, const double* residuals, double* rms, void* stream);
/* count_bad_vals with OP_INC, validation.h:102-115; euler3d.cpp:539-544.
 * Adds the NaN/Inf count to the device scalar *count. */
int mgcfd_op_count_bad_vals(int32_t nnodes, const double* variables, int32_t* count, void* stream);
/* up_pre_kernel, mg.h:29-39; euler3d.cpp:581-583 (over fine nodes). */
int mgcfd_op_up_pre(int32_t nfine, int32_t ncoarse, const int32_t* node_to_mg, double* coarse_variables,
                    int32_t* up_scratch, void* stream);
/* up_kernel, mg.h:41-52; euler3d.cpp:585-588. */
int mgcfd_op_up(int32_t nfine, int32_t ncoarse, const int32_t* node_to_mg, const double* fine_variables,
                double* coarse_variables, int32_t* up_scratch, void* stream);
/* up_post_kernel, mg.h:54-64; euler3d.cpp:590-592 (over coarse nodes). */
int mgcfd_op_up_post(int32_t ncoarse, double* coarse_variables, const int32_t* up_scratch, void* stream);
/* down_kernel, mg.h:66-88; euler3d.cpp:626-631. */
int mgcfd_op_down(int32_t nfine, int32_t ncoarse, const int32_t* node_to_mg, double* fine_variables,
                  const double* fine_residuals, const double* fine_coords, const double* coarse_residuals,
                  const double* coarse_coords, void* stream);
/* Restriction (up_pre + up + up_post) that allocates nothing.  It has no
 * counterpart in the reference: the reference, like mgcfd_op_up*, needs a
 * caller-provided per-coarse-node count buffer (p_up_scratch).  This variant
 * is for callers that cannot call cudaMalloc -- a host framework that owns
 * all device memory through its own allocator, or code that must not
 * allocate between time steps -- and keeps the counts in a fixed device
 * array inside the library instead.  Limit: ncoarse <= 1,048,576 (larger
 * levels are rejected with MGCFD_ERR_INVALID); the 4 MiB array stays
 * resident on every GPU that loads the library until the process exits.
 * Every call shares the array and clears the part it uses; calls that
 * overlap on the GPU race and give wrong results.  The first call on each
 * device looks up the array's address (cudaGetSymbolAddress); make it
 * before any stream capture (inside one it fails with MGCFD_ERR_INVALID).
 * Calls outside a capture look the address up again, so it stays right
 * after a cudaDeviceReset.  Out-of-range map entries are skipped and
 * counted in mgcfd_op_map_errors. */
int mgcfd_op_restrict_noalloc(int32_t nfine, int32_t ncoarse, const int32_t* node_to_mg,
                              const double* fine_variables, double* coarse_variables, void* stream);
/* Execution plans of the per-loop entry points.  As OP2's CUDA backend builds
 * and caches a plan for an indirect loop on its first call (op_plan_get),
 * mgcfd_op_compute_flux_edge and mgcfd_op_up_pre / mgcfd_op_up build one per
 * map on first use and reuse it on every later call with the same map
 * pointer and set sizes:
 *   - edge flux: a locality order of the nodes (the caller's own when its
 *     edges join nearby ids, else a Cuthill-McKee order built on the GPU),
 *     the edges sorted in it, and work space; each call computes every
 *     node's primitives once, the edge fluxes with FP64 atomics that stay in
 *     L2, and adds the increments onto the caller's rows.  |w| is kept per
 *     edge and recomputed only when the weight's bits change;
 *   - restriction: the children of every coarse node, so up_kernel is a
 *     gather with no atomics (results independent of scheduling);
 *   - mgcfd_op_calculate_dt: per vol dat (pointer and node count), each
 *     node's cube root of its volume with the volume's bits beside it; a call
 *     takes the root again only where the bits changed, so results are those
 *     of cbrt on every call.
 * A map plan holds integer structure derived from the map only: the map's
 * contents must not change while it is cached (OP2 maps are immutable too).
 * Building a plan synchronises the caller's stream; a first call made while
 * the stream captures a CUDA graph runs the plan-free kernel instead.  Calls
 * on the same map share the plan's work space: issue them in stream order.
 * Before freeing a map, or reusing its memory for another map, release its
 * plans with mgcfd_op_plan_release(map) (plans on the current device built
 * from that pointer, a vol dat's included); mgcfd_op_plans_release frees
 * every plan.  Both
 * synchronise the device.  mgcfd_op_plans_mode selects how plans built
 * from then on order the nodes (AUTO: the caller's order unless more than a
 * tenth of the edges join ids over max(65536, N/128) apart; REORDER: always
 * the Cuthill-McKee order; CALLER_ORDER: never) or switches plans off (OFF:
 * plan-free kernels for every later call).  mgcfd_op_plans_info reports the
 * plans held (any pointer may be NULL).  These have no counterpart in the
 * reference's source: OP2 does this inside its runtime. */
enum { MGCFD_PLANS_OFF = 0, MGCFD_PLANS_AUTO = 1, MGCFD_PLANS_REORDER = 2, MGCFD_PLANS_CALLER_ORDER = 3 };
int mgcfd_op_plans_mode(int32_t mode);
int mgcfd_op_plan_release(const void* map);
int mgcfd_op_plans_release(void);
int mgcfd_op_plans_info(int64_t* edge_plans, int64_t* child_plans, int64_t* reordered, int64_t* device_bytes);
/* Arithmetic of mgcfd_op_compute_flux_edge calls that run through a plan:
 * MGCFD_PRECISION_FP64 (the default) or MGCFD_PRECISION_DW, the solver's
 * double-word form (see the solver section).  DW: the primitives and the edge
 * fluxes in float-float pairs on the FP32 pipes; each node sums its edges'
 * fluxes in pairs and adds the total to its row of fluxes once in FP64 -- no
 * atomics, the same bits on every call -- within the FP64 bar of the
 * reference (1e-10).  The pairs have binary32's exponent range: weights
 * should lie in [2^-70, 2^70).  Plan-free calls stay FP64.  A plan builds
 * its DW tables on its first DW call (synchronising the stream); a first DW
 * call made while the stream captures a CUDA graph runs the FP64 form.
 * Process-wide, like mgcfd_op_plans_mode; other precisions are refused. */
int mgcfd_op_flux_precision(int32_t precision);
/* Number of elements the mapped entry points above skipped because a map
 * entry was outside [0, set size) since the last reset; reset != 0 zeroes the
 * counter.  Reads a device counter: call after the streams used are idle. */
int mgcfd_op_map_errors(int64_t* count, int32_t reset);
/* identify_differences + count_non_zeros, validation.h:46-100; euler3d.cpp:689-699.
 * Adds the number of values of `test` that differ from `master` by more than
 * the reference's tolerance to the device scalar *count. */
int mgcfd_op_count_differences(int32_t nnodes, const double* test, const double* master, int32_t* count,
                               void* stream);

/* ------------------------------------------------------------------------ */
/* Device-resident multigrid solver.                                        */
/* FP64: every operation in binary64.  MIXED: FP32 edge-flux arithmetic and
 * geometry, FP64 node sums, time step and norms.  DW: the state, the time
 * step, the norms and min_dt in binary64; the node primitives, the edge
 * fluxes and their per-node sums in double-word arithmetic on the FP32 pipes
 * (each value an unevaluated pair of binary32 numbers, 48 significand bits,
 * built from error-free TwoSum / TwoProd steps), with the primitives and the
 * edge weights stored as such pairs.  Within the same 1e-10 relative bar of
 * the FP64 reference as FP64; the exponent range of the pairs is binary32's,
 * and set-up refuses (MGCFD_ERR_INVALID) a mesh with edge weights outside
 * [2^-70, 2^70).  DW takes the FUSED (AUTO), ATOMIC or GATHER increment. */
enum { MGCFD_PRECISION_FP64 = 0, MGCFD_PRECISION_MIXED = 1, MGCFD_PRECISION_DW = 2 };
/* How the edge fluxes reach the nodes.  ATOMIC: each edge adds +f / -f to its
 * end nodes with FP64 atomics.  GATHER: each edge stores f, then each node
 * sums its edges' f in a fixed order (deterministic).  FUSED (mixed precision
 * and DW): one node-centric kernel per RK stage computes the flux of every
 * edge at both of its end nodes, sums them in a fixed order and applies the
 * time step (deterministic).  In mixed precision it computes each FP32 flux
 * from the same inputs in the same order as GATHER and sums exactly as GATHER
 * does -- GATHER's results
 * bit for bit, with no per-edge flux array and one launch per stage. */
/* COLOURED (FP64, single-mesh solvers): each level's edges are split at set-up
 * into colour classes in which no two edges share a node (greedy, at most 64
 * classes); each class is one launch whose edges add +f / -f to their end
 * nodes with plain loads and stores -- no atomics, and the same sums in the
 * same order on every run.  Measured slower than ATOMIC on GB300 (each class
 * streams the node records and flux rows again), so AUTO does not pick it. */
enum {
  MGCFD_INCREMENT_AUTO = 0,
  MGCFD_INCREMENT_ATOMIC = 1,
  MGCFD_INCREMENT_GATHER = 2,
  MGCFD_INCREMENT_FUSED = 3,
  MGCFD_INCREMENT_COLOURED = 4
};
enum { MGCFD_RENUMBER_NONE = 0, MGCFD_RENUMBER_SPATIAL = 1, MGCFD_RENUMBER_RCM = 2 };
/* Node-residual accumulation in mixed precision.  FP64: every FP32 edge flux
 * is widened exactly and added in FP64.  PAIR32: the fluxes enter an
 * unevaluated FP32 pair (hi, lo) through error-free TwoSum steps (Knuth,
 * TAOCP vol. 2, 4.2.2) and the pair is added once in FP64 -- within 2^-48 of
 * the exact sum, and no FP64 add per edge. */
enum { MGCFD_ACCUM_FP64 = 0, MGCFD_ACCUM_PAIR32 = 1 };
enum {
  MGCFD_Q_VARIABLES = 0,    /* [N][5] */
  MGCFD_Q_FLUXES = 1,       /* [N][5] */
  MGCFD_Q_STEP_FACTORS = 2, /* [N]    */
  MGCFD_Q_VOLUMES = 3,      /* [N]    */
  MGCFD_Q_RESIDUALS = 4,    /* [N][5] */
  MGCFD_Q_OLD_VARIABLES = 5 /* [N][5] */
};

typedef struct mgcfd_solver_options {
  int32_t precision;         /* MGCFD_PRECISION_*                                   */
  int32_t increment;         /* MGCFD_INCREMENT_*; AUTO = ATOMIC for FP64 and FUSED
                                for MIXED (the fastest of each on GB300)           */
  int32_t renumber;          /* MGCFD_RENUMBER_*                                    */
  int32_t use_graph;         /* capture one V-cycle as a CUDA graph and replay it  */
  int32_t measure_mem_bound; /* also run unstructured_stream each RK stage (-b)   */
  int32_t block_size;        /* threads per block of the edge kernels (a multiple
                                of 32 up to 1024); 0 = default (128)               */
  int32_t time_kernels;      /* record CUDA events around level-0 flux sweeps      */
  int32_t host_setup;        /* build the mesh tables on the host instead of the GPU
                                (always on for MGCFD_RENUMBER_RCM); same results      */
  int32_t accumulation;      /* MGCFD_ACCUM_*: how mixed precision sums the FP32
                                edge fluxes of a node (gather increment only)      */
  int32_t stage_neighbour_ids; /* FUSED only: copy each block's neighbour ids into
                                shared memory with cp.async before the edge loop
                                (same results; measured slower on GB300, off by
                                default)                                           */
  int32_t edge_parallel_stage; /* FUSED only: each block computes all its nodes'
                                edge ends at once into shared memory, then every
                                node sums its own in the gather order (same
                                results)                                           */
  int32_t reserved[5];
} mgcfd_solver_options;

typedef struct mgcfd_solver_stats {
  int64_t cycles;            /* V-cycles completed since create/reset             */
  int64_t smoothing_steps;   /* smoothing steps (euler3d.cpp:467-550)             */
  int64_t flux_sweeps_l0;    /* level-0 edge-flux launches timed                  */
  double flux_ms_l0;         /* summed CUDA-event time of those launches          */
  int64_t kernel_launches;   /* kernels this solver enqueued since create/reset   */
  int64_t device_bytes;      /* HBM held by the solver                             */
  double rms_l0;             /* last level-0 sqrt(sum res^2 / N) (euler3d.cpp:537) */
  int32_t status;            /* sticky device status (MGCFD_OK or an error)       */
  int32_t ncolors_reserved;
} mgcfd_solver_stats;

typedef struct mgcfd_solver mgcfd_solver;

void mgcfd_solver_default_options(mgcfd_solver_options* opt);
/* Copies the mesh to the device (renumbered per opt->renumber), computes
 * volumes and re-oriented, damped weights (euler3d.cpp:413-441) and sets the
 * flow to freestream.  `stream` is used for every later launch. */
int mgcfd_solver_create(int32_t nlevels, const mgcfd_level_view* levels, double mach, double aoa_deg,
                        const mgcfd_solver_options* opt, void* stream, mgcfd_solver** out);
/* Batched solves (many independent meshes in one launch per stage): the
 * meshes are concatenated per level, each renumbered on its own, and every
 * kernel of the V-cycle covers all of them.  All meshes need the same number
 * of levels; each has its own Mach number and angle of attack, its own
 * min_dt (euler3d.cpp:476-479 per mesh) and its own outcome: a mesh that hits
 * min_dt < 0 or NaN/Inf is marked failed (mgcfd_solver_mesh_status) while the
 * others continue.  levels[m] points at mesh m's nlevels level views.  The
 * returned solver works with every mgcfd_solver_* call; fetch returns the
 * concatenated level, fetch_mesh one mesh. */
int mgcfd_batch_create(int32_t nmeshes, int32_t nlevels, const mgcfd_level_view* const* levels, const double* mach,
                       const double* aoa_deg, const mgcfd_solver_options* opt, void* stream, mgcfd_solver** out);
int mgcfd_solver_num_meshes(const mgcfd_solver* s);
/* Copy one mesh's quantity of one level to host memory in that mesh's input order. */
int mgcfd_solver_fetch_mesh(mgcfd_solver* s, int32_t mesh, int32_t level, int32_t quantity, double* host_out);
/* Synchronises; returns mesh `mesh`'s status (MGCFD_OK, MGCFD_ERR_NEGATIVE_DT
 * or MGCFD_ERR_BAD_VALUES) and its last level-0 residual norms (all
 * variables as euler3d.cpp:537, and density only); either output may be NULL.
 * A plain (one-mesh) solver is mesh 0. */
int mgcfd_solver_mesh_status(mgcfd_solver* s, int32_t mesh, double* rms_l0, double* rho_rms_l0);
/* Back to the state right after create (freestream, counters zeroed). */
int mgcfd_solver_reset(mgcfd_solver* s);
/* Enqueue `ncycles` V-cycles (euler3d.cpp:458-641).  Asynchronous. */
int mgcfd_solver_run(mgcfd_solver* s, int32_t ncycles);
/* Enqueue one iteration of the reference's V-cycle loop (euler3d.cpp:458-640):
 * one smoothing step at the current level followed by its restriction or
 * prolongation.  *smoothed_level (may be NULL) receives the level smoothed and
 * *cycles_done the number of completed V-cycles afterwards.  The level-0
 * state after a step that smoothed level 0 is the state euler3d.cpp:552-571
 * writes with -I. */
int mgcfd_solver_step(mgcfd_solver* s, int32_t* smoothed_level, int64_t* cycles_done);
/* Wait for enqueued work; returns the sticky status. */
int mgcfd_solver_synchronize(mgcfd_solver* s);
/* Copy a per-node quantity of one level to host memory in the caller's
 * (input) node order.  Synchronises. */
int mgcfd_solver_fetch(mgcfd_solver* s, int32_t level, int32_t quantity, double* host_out);
int mgcfd_solver_get_stats(mgcfd_solver* s, mgcfd_solver_stats* out);
/* Internal per-level tables, for inspection and tests (renumbered order). */
enum {
  MGCFD_T_PERM = 0,      /* int32 [N]      new id -> input id                           */
  MGCFD_T_EDGES = 1,     /* int32 [E][2]   (a, b), a < b, sorted                         */
  MGCFD_T_WEIGHTS = 2,   /* f64   [E][4]   (-wx/2, -wy/2, -wz/2, -|w|*smoothing/2)       */
  MGCFD_T_VOLUMES = 3,   /* f64   [N]                                                    */
  MGCFD_T_INV_VOL = 4,   /* f64   [N]                                                    */
  MGCFD_T_CBRT_VOL = 5,  /* f64   [N]                                                    */
  MGCFD_T_BIDX = 6,      /* int32 [N]      boundary row or -1                            */
  MGCFD_T_BDATA = 7,     /* f64   [rows][12]                                             */
  MGCFD_T_N2MG = 8,      /* int32 [N]      coarse parent (not on the coarsest level)      */
  MGCFD_T_DVEC = 9,      /* f64   [N][4]                                                 */
  MGCFD_T_CH_OFF = 10,   /* int32 [N+1]    children offsets (not on the finest level)     */
  MGCFD_T_CH_LIST = 11,  /* int32 [N_fine]                                                */
  MGCFD_T_A_OFF = 12,    /* int32 [N+1]    gather strategy only                          */
  MGCFD_T_B_OFF = 13,    /* int32 [N+1]    gather strategy only                          */
  MGCFD_T_B_LIST = 14,   /* int32 [E]      gather strategy only                          */
  MGCFD_T_WEIGHTS32 = 15 /* f32   [E][4]   the same as WEIGHTS, mixed precision only      */
};
/* Copies table `table` of `level` into host_out if capacity_bytes suffices;
 * *bytes receives the table's size (0 if the table does not exist).  With
 * host_out == NULL only the size is returned. */
int mgcfd_solver_table(mgcfd_solver* s, int32_t level, int32_t table, void* host_out, int64_t capacity_bytes,
                       int64_t* bytes);
void mgcfd_solver_destroy(mgcfd_solver* s);

/* ------------------------------------------------------------------------ */
/* Serving: solves of different meshes and freestream conditions arrive at  */
/* any time and run concurrently on one GPU (continuous batching at V-cycle */
/* granularity).  A worker thread admits queued requests in arrival order    */
/* when a slot (CUDA stream) is free and the HBM budget covers the request's */
/* estimated footprint, advances every admitted request one V-cycle at a    */
/* time, and retires it when its level-0 density residual has dropped below */
/* residual_drop times its first value, it fails (min_dt < 0, NaN/Inf), or  */
/* max_cycles is reached.  A request's arithmetic is that of a solver       */
/* running alone, so with MGCFD_INCREMENT_GATHER or _FUSED its result is    */
/* identical alone and in any mix.                                           */
/* Cohorts (batch_max_meshes > 1): small requests -- at most                 */
/* batch_max_nodes level-0 nodes -- that wait next to each other in the     */
/* queue with the same number of levels are admitted together as one        */
/* batched solver (mgcfd_batch_create: one launch per V-cycle stage for all */
/* of them, one slot), each with its own stop rule: a request that meets it */
/* or fails stops changing while the others go on; the cohort's results are */
/* copied out when its last request has stopped.  Batched kernels do the    */
/* arithmetic of the solver alone, so results stay identical.               */
typedef struct mgcfd_server_options {
  int64_t hbm_budget_bytes;  /* admission budget for all active requests          */
  int32_t max_active;        /* concurrent requests (one stream each)              */
  int32_t precision;         /* MGCFD_PRECISION_*                                  */
  int32_t increment;         /* MGCFD_INCREMENT_*                                  */
  int32_t max_cycles;        /* V-cycles per request at most                       */
  double residual_drop;      /* stop when rho_rms <= residual_drop * first rho_rms */
  int32_t accumulation;      /* MGCFD_ACCUM_* for mixed precision                 */
  int32_t batch_max_meshes;  /* requests per cohort (<= 64); 0 or 1: no cohorts    */
  int32_t batch_max_nodes;   /* level-0 nodes of a request that may join a cohort  */
  int32_t reserved[5];
} mgcfd_server_options;

typedef struct mgcfd_request_result {
  int64_t id;
  int32_t status;            /* MGCFD_OK, _NEGATIVE_DT, _BAD_VALUES, _BUDGET, ... */
  int32_t cycles;            /* V-cycles run                                       */
  double submit_s, admit_s, finish_s;  /* seconds since the server started       */
  double rho_rms_first, rho_rms_last;  /* level-0 density residual norms         */
  double device_begin_s, device_end_s; /* GPU timestamps (CUDA events, seconds since
                                          the server started) of the request's first
                                          V-cycle chunk starting and its last one
                                          ending; -1 if it never ran               */
} mgcfd_request_result;

typedef struct mgcfd_server_stats {
  int64_t submitted, completed, failed;
  int64_t active, pending;
  int64_t used_bytes, peak_bytes, peak_active;  /* used_bytes includes idle cached solvers */
  int64_t cache_hits;                           /* requests that reused a resident mesh   */
  int64_t cached_solvers;                       /* idle solvers held for reuse            */
  int64_t cohorts;                              /* batched solvers admitted               */
  int64_t cohort_requests;                      /* requests admitted inside them          */
} mgcfd_server_stats;

typedef struct mgcfd_server mgcfd_server;

void mgcfd_server_default_options(mgcfd_server_options* opt);
int mgcfd_server_create(const mgcfd_server_options* opt, mgcfd_server** out);
/* Queue a solve.  The level arrays must stay valid until the request has
 * completed; out_variables_l0 (may be NULL) receives the final level-0
 * variables [N0][5] in input order.  mesh_key != 0 names the mesh: requests
 * with the same key reuse its resident device tables (the caller guarantees
 * the arrays are the same mesh); 0 uploads and sets up the mesh afresh. */
int mgcfd_server_submit(mgcfd_server* server, int32_t nlevels, const mgcfd_level_view* levels, double mach,
                        double aoa_deg, int64_t mesh_key, double* out_variables_l0, int64_t* id);
/* Move up to `capacity` completed results into out; *count receives how many. */
int mgcfd_server_poll(mgcfd_server* server, mgcfd_request_result* out, int32_t capacity, int32_t* count);
/* Wait until no request is queued or running (MGCFD_ERR_TIMEOUT after timeout_s). */
int mgcfd_server_drain(mgcfd_server* server, double timeout_s);
int mgcfd_server_get_stats(mgcfd_server* server, mgcfd_server_stats* out);
/* Finishes every queued and running request, then frees the server. */
void mgcfd_server_destroy(mgcfd_server* server);
/* The device footprint the server charges against hbm_budget_bytes for a
 * request on this mesh (state, tables and setup scratch at its peak). */
int mgcfd_request_estimate_bytes(int32_t nlevels, const mgcfd_level_view* levels, int32_t precision,
                                 int32_t increment, int64_t* bytes);

/* One full solve through host buffers: upload the mesh, initialise, run
 * ncycles V-cycles, download every level's variables (file order) into
 * out_variables[l] (host, [N_l][5]).  The reference-facing end-to-end call. */
int mgcfd_solve(int32_t nlevels, const mgcfd_level_view* levels, double mach, double aoa_deg, int32_t ncycles,
                const mgcfd_solver_options* opt, double* const* out_variables);

#ifdef __cplusplus
}
#endif
#endif
