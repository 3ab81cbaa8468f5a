/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * CPU restatement of MG-CFD's multigrid Euler hot path (reference
 * warwick-hpsc/MG-CFD-app-OP2), used only by tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg as the checker.  The product never links or
 * calls it.
 *
 * Pinning: the sequential restatement reproduces the reference binary built
 * from the unmodified reference sources against the OP2 stand-in
 * (oracle/_ref/euler3d_ref) bit for bit on the committed golden meshes; the
 * fixtures and the script that made them are in tests/golden/.
 *
 * Element order, floating-point operation order and the V-cycle schedule
 * follow the reference exactly (file:line citations at each function in
 * mgcfd_oracle.c).  Build with -ffp-contract=off and without -ffast-math.
 */
#ifndef MGCFD_ORACLE_H
#define MGCFD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_freestream {
  double smoothing_coefficient;
  double ff_variable[5];
  double ff_flux_contribution_momentum_x[3];
  double ff_flux_contribution_momentum_y[3];
  double ff_flux_contribution_momentum_z[3];
  double ff_flux_contribution_density_energy[3];
} orc_freestream;

void orc_freestream_init(double mach, double aoa_deg, orc_freestream* ff);

/* ---- single loops, sequential element order (one op_par_loop each) ---- */
void orc_loop_initialize_variables(int nnodes, const orc_freestream* ff, double* variables);
void orc_loop_calculate_cell_volumes(int nedges, const int* e2n, const double* coords,
                                     double* ewt, double* volumes);
void orc_loop_dampen_ewt(int n, double* weights);
void orc_loop_copy_double(int nnodes, const double* variables, double* old_variables);
void orc_loop_calculate_dt(int nnodes, const double* variables, const double* volumes, double* dt);
double orc_loop_get_min_dt(int nnodes, const double* dt);
void orc_loop_compute_step_factor(int nnodes, const double* variables, const double* volumes,
                                  double min_dt, double* step_factors);
void orc_loop_compute_flux_edge(int nedges, const int* e2n, const double* variables,
                                const double* ewt, double smoothing_coefficient, double* fluxes);
void orc_loop_compute_bnd_node_flux(int nbnd, const int* b2n, const int* groups, const double* bwt,
                                    const double* variables, const orc_freestream* ff, double* fluxes);
void orc_loop_time_step(int nnodes, int rk_cycle, const double* step_factors, double* fluxes,
                        const double* old_variables, double* variables);
void orc_loop_residual(int nnodes, const double* old_variables, const double* variables, double* residuals);
double orc_loop_calc_rms(int nnodes, const double* residuals);
int orc_loop_count_bad_vals(int nnodes, const double* variables);
void orc_loop_up_pre(int nfine, const int* n2mg, double* coarse_variables, int* up_scratch);
void orc_loop_up(int nfine, const int* n2mg, const double* fine_variables, double* coarse_variables, int* up_scratch);
void orc_loop_up_post(int ncoarse, double* coarse_variables, const int* up_scratch);
void orc_loop_down(int nfine, const int* n2mg, double* fine_variables, const double* fine_residuals,
                   const double* fine_coords, const double* coarse_residuals, const double* coarse_coords);
void orc_loop_unstructured_stream(int nedges, const int* e2n, const double* variables,
                                  const double* ewt, double* fluxes);
void orc_loop_identify_differences(int nnodes, const double* test, const double* master, double* diff);
int orc_loop_count_non_zeros(int nnodes, const double* values);

/* ---- whole-run driver (euler3d.cpp:413-641) ---- */
typedef struct orc_mesh orc_mesh;

orc_mesh* orc_mesh_create(int nlevels);
/* Copies the arrays.  n2mg may be NULL on the coarsest level. */
int orc_mesh_set_level(orc_mesh* m, int level, int nnodes, int nedges, int nbnd,
                       const double* coords, const int* e2n, const int* b2n, const int* bgroup,
                       const double* ewt, const double* bwt, const int* n2mg);
/* Legacy mode (euler3d.cpp:292-299): use these volumes ("areas") and skip
 * calculate_cell_volumes.  Copies the array. */
int orc_mesh_set_volumes(orc_mesh* m, int level, const double* volumes);
/* Runs init (euler3d.cpp:413-441) then `ncycles` V-cycles (:452-641).
 * nthreads <= 1: sequential seq-backend order (the parity oracle).
 * nthreads > 1: OpenMP loops over coloured edges (a timing baseline only;
 *               summation order differs from seq).
 * measure_mem_bound != 0 also runs unstructured_stream (the reference's -b).
 * Returns 0, 1 for min_dt < 0 (euler3d.cpp:480-484) or 2 for NaN/Inf at
 * level 0 (euler3d.cpp:539-548).  *runtime_s receives the V-cycle wall time
 * (the region euler3d.cpp:450-647 times). */
int orc_run(orc_mesh* m, double mach, double aoa_deg, int ncycles, int nthreads,
            int measure_mem_bound, double* runtime_s);
/* what: 0 variables [N][5], 1 fluxes [N][5], 2 step factors [N], 3 volumes [N],
 *       4 residuals [N][5], 5 edge weights after init [E][3],
 *       6 boundary weights after init [B][3], 7 old variables [N][5]. */
int orc_get(const orc_mesh* m, int level, int what, double* out);
/* Number of smoothing steps the last orc_run performed. */
long orc_smoothing_steps(const orc_mesh* m);
void orc_mesh_destroy(orc_mesh* m);

#ifdef __cplusplus
}
#endif
#endif
