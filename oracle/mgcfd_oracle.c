/* ORACLE TEST INFRASTRUCTURE -- not part of the product.
 *
 * CPU restatement of the MG-CFD multigrid Euler hot path.  See
 * mgcfd_oracle.h for its role and how it is pinned.  Every function cites the
 * reference file:line it restates; floating-point expressions keep the
 * reference's association order so that, compiled with -ffp-contract=off, the
 * sequential run reproduces the reference's seq build bit for bit.
 */
#include "mgcfd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_GAMMA 1.4
#define ORC_RK 3
#define ORC_PI 3.1415926535897931 /* const.h:43 */

/* euler3d.cpp:157-189 (far-field state and its flux tensor). */
void orc_freestream_init(double mach, double aoa_deg, orc_freestream* ff) {
  const double angle = (ORC_PI / 180.0) * aoa_deg;
  ff->smoothing_coefficient = (double)0.2f; /* euler3d.cpp:47 */
  ff->ff_variable[0] = 1.4;
  const double pressure = 1.0;
  const double sos = sqrt(ORC_GAMMA * pressure / ff->ff_variable[0]);
  const double speed = mach * sos;
  const double vx = speed * cos(angle);
  const double vy = speed * sin(angle);
  const double vz = 0.0;
  ff->ff_variable[1] = ff->ff_variable[0] * vx;
  ff->ff_variable[2] = ff->ff_variable[0] * vy;
  ff->ff_variable[3] = ff->ff_variable[0] * vz;
  ff->ff_variable[4] = ff->ff_variable[0] * (0.5 * (speed * speed)) + (pressure / (ORC_GAMMA - 1.0));
  /* inlined_funcs.h:70-96 applied to (rho, momentum, rhoE, p, velocity). */
  const double mx = ff->ff_variable[1], my = ff->ff_variable[2], mz = ff->ff_variable[3];
  ff->ff_flux_contribution_momentum_x[0] = vx * mx + pressure;
  ff->ff_flux_contribution_momentum_x[1] = vx * my;
  ff->ff_flux_contribution_momentum_x[2] = vx * mz;
  ff->ff_flux_contribution_momentum_y[0] = ff->ff_flux_contribution_momentum_x[1];
  ff->ff_flux_contribution_momentum_y[1] = vy * my + pressure;
  ff->ff_flux_contribution_momentum_y[2] = vy * mz;
  ff->ff_flux_contribution_momentum_z[0] = ff->ff_flux_contribution_momentum_x[2];
  ff->ff_flux_contribution_momentum_z[1] = ff->ff_flux_contribution_momentum_y[2];
  ff->ff_flux_contribution_momentum_z[2] = vz * mz + pressure;
  const double de_p = ff->ff_variable[4] + pressure;
  ff->ff_flux_contribution_density_energy[0] = vx * de_p;
  ff->ff_flux_contribution_density_energy[1] = vy * de_p;
  ff->ff_flux_contribution_density_energy[2] = vz * de_p;
}

/* Primitive state of one node: inlined_funcs.h:98-130 (non-IDIVIDE path). */
typedef struct {
  double rho, mx, my, mz, rhoE;
  double vx, vy, vz;
  double speed_sqd, pressure, speed_of_sound;
  double fcx[3], fcy[3], fcz[3], fcde[3];
} orc_node_state;

static inline void orc_primitives(const double* v, orc_node_state* s) {
  s->rho = v[0];
  s->mx = v[1]; s->my = v[2]; s->mz = v[3];
  s->rhoE = v[4];
  s->vx = s->mx / s->rho; /* inlined_funcs.h:119-124 */
  s->vy = s->my / s->rho;
  s->vz = s->mz / s->rho;
  s->speed_sqd = s->vx * s->vx + s->vy * s->vy + s->vz * s->vz;               /* :98-101 */
  s->pressure = (ORC_GAMMA - 1.0) * (s->rhoE - 0.5 * s->rho * s->speed_sqd); /* :103-106 */
  s->speed_of_sound = sqrt(ORC_GAMMA * s->pressure / s->rho);                 /* :125-128 */
}

/* inlined_funcs.h:70-96 */
static inline void orc_flux_contribution(orc_node_state* s) {
  s->fcx[0] = s->vx * s->mx + s->pressure;
  s->fcx[1] = s->vx * s->my;
  s->fcx[2] = s->vx * s->mz;
  s->fcy[0] = s->fcx[1];
  s->fcy[1] = s->vy * s->my + s->pressure;
  s->fcy[2] = s->vy * s->mz;
  s->fcz[0] = s->fcx[2];
  s->fcz[1] = s->fcy[2];
  s->fcz[2] = s->vz * s->mz + s->pressure;
  const double de_p = s->rhoE + s->pressure;
  s->fcde[0] = s->vx * de_p;
  s->fcde[1] = s->vy * de_p;
  s->fcde[2] = s->vz * de_p;
}

/* flux.h:41-208: central flux plus scalar dissipation on one edge. */
static inline void orc_flux_edge(const double* va, const double* vb, const double* w, double sc,
                                 double* fa, double* fb) {
  const double ewt = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  orc_node_state b, a;
  orc_primitives(vb, &b);
  const double speed_b = sqrt(b.speed_sqd);
  orc_flux_contribution(&b);
  orc_primitives(va, &a);
  const double speed_a = sqrt(a.speed_sqd);
  orc_flux_contribution(&a);
  const double factor_a = -ewt * sc * 0.5 * (speed_a + sqrt(b.speed_sqd) + a.speed_of_sound + b.speed_of_sound);
  const double factor_b = -ewt * sc * 0.5 * (speed_b + sqrt(a.speed_sqd) + b.speed_of_sound + a.speed_of_sound);
  const double fx = -0.5 * w[0], fy = -0.5 * w[1], fz = -0.5 * w[2];

  fa[0] += factor_a * (a.rho - b.rho) + fx * (a.mx + b.mx) + fy * (a.my + b.my) + fz * (a.mz + b.mz);
  fa[4] += factor_a * (a.rhoE - b.rhoE) + fx * (a.fcde[0] + b.fcde[0]) + fy * (a.fcde[1] + b.fcde[1]) +
           fz * (a.fcde[2] + b.fcde[2]);
  fa[1] += factor_a * (a.mx - b.mx) + fx * (a.fcx[0] + b.fcx[0]) + fy * (a.fcx[1] + b.fcx[1]) +
           fz * (a.fcx[2] + b.fcx[2]);
  fa[2] += factor_a * (a.my - b.my) + fx * (a.fcy[0] + b.fcy[0]) + fy * (a.fcy[1] + b.fcy[1]) +
           fz * (a.fcy[2] + b.fcy[2]);
  fa[3] += factor_a * (a.mz - b.mz) + fx * (a.fcz[0] + b.fcz[0]) + fy * (a.fcz[1] + b.fcz[1]) +
           fz * (a.fcz[2] + b.fcz[2]);

  fb[0] += factor_b * (b.rho - a.rho) - fx * (a.mx + b.mx) - fy * (a.my + b.my) - fz * (a.mz + b.mz);
  fb[4] += factor_b * (b.rhoE - a.rhoE) - fx * (a.fcde[0] + b.fcde[0]) - fy * (a.fcde[1] + b.fcde[1]) -
           fz * (a.fcde[2] + b.fcde[2]);
  fb[1] += factor_b * (b.mx - a.mx) - fx * (a.fcx[0] + b.fcx[0]) - fy * (a.fcx[1] + b.fcx[1]) -
           fz * (a.fcx[2] + b.fcx[2]);
  fb[2] += factor_b * (b.my - a.my) - fx * (a.fcy[0] + b.fcy[0]) - fy * (a.fcy[1] + b.fcy[1]) -
           fz * (a.fcy[2] + b.fcy[2]);
  fb[3] += factor_b * (b.mz - a.mz) - fx * (a.fcz[0] + b.fcz[0]) - fy * (a.fcz[1] + b.fcz[1]) -
           fz * (a.fcz[2] + b.fcz[2]);
}

/* flux.h:14-39 with flux_boundary.elem_func:9-54 (g <= 2, solid wall) and
 * flux_wall.elem_func:8-76 (g == 3 or 4 <= g <= 7, far field). */
static inline void orc_bnd_flux(int g, const double* w, const double* vb, const orc_freestream* ff,
                                double* fb) {
  orc_node_state b;
  if (g <= 2) {
    orc_primitives(vb, &b);
    fb[0] += 0.0;
    fb[1] += w[0] * b.pressure;
    fb[2] += w[1] * b.pressure;
    fb[3] += w[2] * b.pressure;
    fb[4] += 0.0;
  } else if (g == 3 || (g >= 4 && g <= 7)) {
    orc_primitives(vb, &b);
    orc_flux_contribution(&b);
    const double fx = 0.5 * w[0], fy = 0.5 * w[1], fz = 0.5 * w[2];
    const double* fv = ff->ff_variable;
    fb[0] += fx * (fv[1] + b.mx) + fy * (fv[2] + b.my) + fz * (fv[3] + b.mz);
    fb[4] += fx * (ff->ff_flux_contribution_density_energy[0] + b.fcde[0]) +
             fy * (ff->ff_flux_contribution_density_energy[1] + b.fcde[1]) +
             fz * (ff->ff_flux_contribution_density_energy[2] + b.fcde[2]);
    fb[1] += fx * (ff->ff_flux_contribution_momentum_x[0] + b.fcx[0]) +
             fy * (ff->ff_flux_contribution_momentum_x[1] + b.fcx[1]) +
             fz * (ff->ff_flux_contribution_momentum_x[2] + b.fcx[2]);
    fb[2] += fx * (ff->ff_flux_contribution_momentum_y[0] + b.fcy[0]) +
             fy * (ff->ff_flux_contribution_momentum_y[1] + b.fcy[1]) +
             fz * (ff->ff_flux_contribution_momentum_y[2] + b.fcy[2]);
    fb[3] += fx * (ff->ff_flux_contribution_momentum_z[0] + b.fcz[0]) +
             fy * (ff->ff_flux_contribution_momentum_z[1] + b.fcz[1]) +
             fz * (ff->ff_flux_contribution_momentum_z[2] + b.fcz[2]);
  }
}

/* ------------------------------------------------------------------------ */
/* Loops.                                                                   */

/* misc.h:10-16 */
void orc_loop_initialize_variables(int nnodes, const orc_freestream* ff, double* variables) {
  for (int n = 0; n < nnodes; n++)
    for (int j = 0; j < 5; j++) variables[5 * (size_t)n + j] = ff->ff_variable[j];
}

/* misc.h:40-76 over edges (euler3d.cpp:425-431). */
static inline void orc_cell_volume_edge(const double* c1, const double* c2, double* ewt, double* vol1,
                                        double* vol2) {
  double d[3];
  double dist = 0.0;
  for (int i = 0; i < 3; i++) {
    d[i] = c2[i] - c1[i];
    dist += d[i] * d[i];
  }
  dist = sqrt(dist);
  double area = 0.0;
  for (int i = 0; i < 3; i++) area += ewt[i] * ewt[i];
  area = sqrt(area);
  const double tetra_volume = (1.0 / 3.0) * 0.5 * dist * area;
  *vol1 += tetra_volume;
  *vol2 += tetra_volume;
  for (int i = 0; i < 3; i++) ewt[i] = (d[i] / dist) * area;
  for (int i = 0; i < 3; i++) ewt[i] /= dist;
}

void orc_loop_calculate_cell_volumes(int nedges, const int* e2n, const double* coords, double* ewt,
                                     double* volumes) {
  for (int e = 0; e < nedges; e++) {
    const int a = e2n[2 * (size_t)e], b = e2n[2 * (size_t)e + 1];
    orc_cell_volume_edge(coords + 3 * (size_t)a, coords + 3 * (size_t)b, ewt + 3 * (size_t)e, volumes + a,
                         volumes + b);
  }
}

/* misc.h:78-84 */
void orc_loop_dampen_ewt(int n, double* w) {
  for (size_t i = 0; i < 3 * (size_t)n; i++) w[i] *= 1e-7;
}

/* copy_double_kernel.h:6-13 */
void orc_loop_copy_double(int nnodes, const double* v, double* old) {
  memcpy(old, v, sizeof(double) * 5 * (size_t)nnodes);
}

/* time_stepping_kernels.h:13-32 */
static inline double orc_dt(const double* v, double vol) {
  orc_node_state s;
  orc_primitives(v, &s);
  return 0.5 * (cbrt(vol) / (sqrt(s.speed_sqd) + s.speed_of_sound));
}

void orc_loop_calculate_dt(int nnodes, const double* v, const double* vol, double* dt) {
  for (int n = 0; n < nnodes; n++) dt[n] = orc_dt(v + 5 * (size_t)n, vol[n]);
}

/* time_stepping_kernels.h:34-41 with OP_MIN starting at DBL_MAX (euler3d.cpp:476-479). */
double orc_loop_get_min_dt(int nnodes, const double* dt) {
  double m = DBL_MAX;
  for (int n = 0; n < nnodes; n++)
    if (dt[n] < m) m = dt[n];
  return m;
}

/* time_stepping_kernels.h:43-64 (the primitive arithmetic there is unused). */
void orc_loop_compute_step_factor(int nnodes, const double* v, const double* vol, double min_dt, double* sf) {
  (void)v;
  for (int n = 0; n < nnodes; n++) sf[n] = min_dt / vol[n];
}

/* euler3d.cpp:498-503 */
void orc_loop_compute_flux_edge(int nedges, const int* e2n, const double* v, const double* ewt, double sc,
                                double* flux) {
  for (int e = 0; e < nedges; e++) {
    const int a = e2n[2 * (size_t)e], b = e2n[2 * (size_t)e + 1];
    orc_flux_edge(v + 5 * (size_t)a, v + 5 * (size_t)b, ewt + 3 * (size_t)e, sc, flux + 5 * (size_t)a,
                  flux + 5 * (size_t)b);
  }
}

/* euler3d.cpp:505-509 */
void orc_loop_compute_bnd_node_flux(int nbnd, const int* b2n, const int* groups, const double* bwt,
                                    const double* v, const orc_freestream* ff, double* flux) {
  for (int i = 0; i < nbnd; i++) {
    const int n = b2n[i];
    orc_bnd_flux(groups[i], bwt + 3 * (size_t)i, v + 5 * (size_t)n, ff, flux + 5 * (size_t)n);
  }
}

/* time_stepping_kernels.h:66-86 */
void orc_loop_time_step(int nnodes, int rk, const double* sf, double* flux, const double* old, double* v) {
  for (int n = 0; n < nnodes; n++) {
    const double factor = sf[n] / (double)(ORC_RK + 1 - rk);
    double* f = flux + 5 * (size_t)n;
    const double* o = old + 5 * (size_t)n;
    double* x = v + 5 * (size_t)n;
    for (int j = 0; j < 5; j++) x[j] = o[j] + factor * f[j];
    for (int j = 0; j < 5; j++) f[j] = 0.0;
  }
}

/* validation.h:27-35 */
void orc_loop_residual(int nnodes, const double* old, const double* v, double* res) {
  for (size_t i = 0; i < 5 * (size_t)nnodes; i++) res[i] = v[i] - old[i];
}

/* validation.h:37-44 with OP_INC from 0.0 (euler3d.cpp:533-537, before the sqrt). */
double orc_loop_calc_rms(int nnodes, const double* res) {
  double rms = 0.0;
  for (size_t i = 0; i < 5 * (size_t)nnodes; i++) rms += res[i] * res[i];
  return rms;
}

/* validation.h:102-115 */
int orc_loop_count_bad_vals(int nnodes, const double* v) {
  int count = 0;
  for (size_t i = 0; i < 5 * (size_t)nnodes; i++)
    if (isnan(v[i]) || isinf(v[i])) count += 1;
  return count;
}

/* mg.h:29-39 over fine nodes (euler3d.cpp:581-583). */
void orc_loop_up_pre(int nfine, const int* n2mg, double* cv, int* scratch) {
  for (int n = 0; n < nfine; n++) {
    const int c = n2mg[n];
    for (int j = 0; j < 5; j++) cv[5 * (size_t)c + j] = 0.0;
    scratch[c] = 0;
  }
}

/* mg.h:41-52 (euler3d.cpp:585-588). */
void orc_loop_up(int nfine, const int* n2mg, const double* fv, double* cv, int* scratch) {
  for (int n = 0; n < nfine; n++) {
    const int c = n2mg[n];
    for (int j = 0; j < 5; j++) cv[5 * (size_t)c + j] += fv[5 * (size_t)n + j];
    scratch[c] += 1;
  }
}

/* mg.h:54-64 (euler3d.cpp:590-592). */
void orc_loop_up_post(int ncoarse, double* cv, const int* scratch) {
  for (int c = 0; c < ncoarse; c++) {
    const double avg = scratch[c] == 0 ? 1.0 : 1.0 / (double)scratch[c];
    for (int j = 0; j < 5; j++) cv[5 * (size_t)c + j] *= avg;
  }
}

/* mg.h:66-88 (euler3d.cpp:626-631). */
void orc_loop_down(int nfine, const int* n2mg, double* fv, const double* fres, const double* fcoord,
                   const double* cres, const double* ccoord) {
  for (int n = 0; n < nfine; n++) {
    const int c = n2mg[n];
    const double* x = fcoord + 3 * (size_t)n;
    const double* xa = ccoord + 3 * (size_t)c;
    const double* r = fres + 5 * (size_t)n;
    const double* ra = cres + 5 * (size_t)c;
    double* v = fv + 5 * (size_t)n;
    const double dx = fabs(x[0] - xa[0]);
    const double dy = fabs(x[1] - xa[1]);
    const double dz = fabs(x[2] - xa[2]);
    const double dm = sqrt(dx * dx + dy * dy + dz * dz);
    v[0] -= dm * (ra[0] - r[0]);
    v[1] -= dx * (ra[1] - r[1]);
    v[2] -= dy * (ra[2] - r[2]);
    v[3] -= dz * (ra[3] - r[3]);
    v[4] -= dm * (ra[4] - r[4]);
  }
}

/* unstructured_stream.h:7-57 (euler3d.cpp:518-525). */
void orc_loop_unstructured_stream(int nedges, const int* e2n, const double* v, const double* ewt, double* flux) {
  for (int e = 0; e < nedges; e++) {
    const double* va = v + 5 * (size_t)e2n[2 * (size_t)e];
    const double* vb = v + 5 * (size_t)e2n[2 * (size_t)e + 1];
    double* fa = flux + 5 * (size_t)e2n[2 * (size_t)e];
    double* fb = flux + 5 * (size_t)e2n[2 * (size_t)e + 1];
    const double* w = ewt + 3 * (size_t)e;
    const double pa = va[0], pea = va[4], max = va[1], may = va[2], maz = va[3];
    const double pb = vb[0], peb = vb[4], mbx = vb[1], mby = vb[2], mbz = vb[3];
    const double p_a_val = pb + w[0], pe_a_val = peb + w[1], mx_a_val = mbx + w[2];
    fa[0] += p_a_val;
    fa[1] += mx_a_val;
    fa[2] += mby;
    fa[3] += mbz;
    fa[4] += pe_a_val;
    fb[0] += pa;
    fb[1] += max;
    fb[2] += may;
    fb[3] += maz;
    fb[4] += pea;
  }
}

/* validation.h:46-89 */
void orc_loop_identify_differences(int nnodes, const double* test, const double* master, double* diff) {
  const double acceptable_relative_difference = 10.0e-8;
  for (size_t i = 0; i < 5 * (size_t)nnodes; i++) {
    double acceptable = master[i] * acceptable_relative_difference;
    if (acceptable < 0.0) acceptable *= -1.0;
    if (acceptable < 3.0e-19) acceptable = 3.0e-19;
    double d = test[i] - master[i];
    if (d < 0.0) d *= -1.0;
    diff[i] = d > acceptable ? d : 0.0;
  }
}

/* validation.h:91-100 */
int orc_loop_count_non_zeros(int nnodes, const double* values) {
  int count = 0;
  for (size_t i = 0; i < 5 * (size_t)nnodes; i++)
    if (values[i] > 0.0) count++;
  return count;
}

/* ------------------------------------------------------------------------ */
/* Whole-run driver.                                                        */

typedef struct {
  int nnodes, nedges, nbnd;
  double *coords, *ewt, *bwt;
  double *ewt_in, *bwt_in; /* weights as read; init rewrites ewt/bwt from these each run */
  double* legacy_vol;      /* legacy-mode volumes, or NULL */
  int *e2n, *b2n, *bgroup, *n2mg;
  double *var, *old, *res, *vol, *sf, *flux, *dummy;
  int* up_scratch;
  /* OpenMP edge colouring: edges grouped by colour, colour offsets. */
  int ncolors;
  int* color_offsets;
  int* color_edges;
  int bnd_ncolors;
  int* bnd_color_offsets;
  int* bnd_color_entries;
} orc_level;

struct orc_mesh {
  int nlevels;
  orc_level* L;
  long steps;
};

orc_mesh* orc_mesh_create(int nlevels) {
  if (nlevels < 1) return NULL;
  orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
  m->nlevels = nlevels;
  m->L = (orc_level*)calloc((size_t)nlevels, sizeof(orc_level));
  return m;
}

static void* orc_dup(const void* p, size_t n) {
  void* q = malloc(n ? n : 1);
  if (p && n) memcpy(q, p, n);
  return q;
}

int orc_mesh_set_level(orc_mesh* m, int l, int nnodes, int nedges, int nbnd, const double* coords,
                       const int* e2n, const int* b2n, const int* bgroup, const double* ewt, const double* bwt,
                       const int* n2mg) {
  if (!m || l < 0 || l >= m->nlevels) return -1;
  orc_level* L = &m->L[l];
  L->nnodes = nnodes; L->nedges = nedges; L->nbnd = nbnd;
  L->coords = (double*)orc_dup(coords, sizeof(double) * 3 * (size_t)nnodes);
  L->e2n = (int*)orc_dup(e2n, sizeof(int) * 2 * (size_t)nedges);
  L->b2n = (int*)orc_dup(b2n, sizeof(int) * (size_t)nbnd);
  L->bgroup = (int*)orc_dup(bgroup, sizeof(int) * (size_t)nbnd);
  L->ewt_in = (double*)orc_dup(ewt, sizeof(double) * 3 * (size_t)nedges);
  L->bwt_in = (double*)orc_dup(bwt, sizeof(double) * 3 * (size_t)nbnd);
  L->ewt = (double*)orc_dup(ewt, sizeof(double) * 3 * (size_t)nedges);
  L->bwt = (double*)orc_dup(bwt, sizeof(double) * 3 * (size_t)nbnd);
  L->n2mg = n2mg ? (int*)orc_dup(n2mg, sizeof(int) * (size_t)nnodes) : NULL;
  size_t nv = 5 * (size_t)nnodes;
  L->var = (double*)calloc(nv, sizeof(double));
  L->old = (double*)calloc(nv, sizeof(double));
  L->res = (double*)calloc(nv, sizeof(double));
  L->flux = (double*)calloc(nv, sizeof(double));
  L->dummy = (double*)calloc(nv, sizeof(double));
  L->vol = (double*)calloc((size_t)nnodes, sizeof(double));
  L->sf = (double*)calloc((size_t)nnodes, sizeof(double));
  L->up_scratch = (int*)calloc((size_t)nnodes, sizeof(int));
  return 0;
}

/* Greedy colouring of elements touching up to two nodes so that no two
 * elements of one colour share a node; used only by the OpenMP baseline. */
static void orc_colour(int nelem, int arity, const int* nodes, int nnodes, int* ncolors_out, int** offsets_out,
                       int** order_out) {
  uint64_t* used = (uint64_t*)calloc((size_t)nnodes, sizeof(uint64_t));
  int* colour = (int*)malloc(sizeof(int) * (size_t)(nelem ? nelem : 1));
  int ncol = 0;
  for (int e = 0; e < nelem; e++) {
    uint64_t u = 0;
    for (int k = 0; k < arity; k++) u |= used[nodes[arity * (size_t)e + k]];
    int c = 0;
    while (c < 63 && (u >> c) & 1u) c++;
    colour[e] = c;
    for (int k = 0; k < arity; k++) used[nodes[arity * (size_t)e + k]] |= (1ull << c);
    if (c + 1 > ncol) ncol = c + 1;
  }
  int* off = (int*)calloc((size_t)ncol + 1, sizeof(int));
  for (int e = 0; e < nelem; e++) off[colour[e] + 1]++;
  for (int c = 0; c < ncol; c++) off[c + 1] += off[c];
  int* fill = (int*)malloc(sizeof(int) * (size_t)(ncol ? ncol : 1));
  for (int c = 0; c < ncol; c++) fill[c] = off[c];
  int* order = (int*)malloc(sizeof(int) * (size_t)(nelem ? nelem : 1));
  for (int e = 0; e < nelem; e++) order[fill[colour[e]]++] = e;
  free(fill);
  free(colour);
  free(used);
  *ncolors_out = ncol;
  *offsets_out = off;
  *order_out = order;
}

static double orc_wall(void) {
  struct timeval t;
  gettimeofday(&t, NULL);
  return (double)t.tv_sec + 1e-6 * (double)t.tv_usec;
}

/* Edge flux loop, OpenMP over colours (baseline only). */
static void orc_flux_edge_omp(orc_level* L, double sc) {
  for (int c = 0; c < L->ncolors; c++) {
    const int lo = L->color_offsets[c], hi = L->color_offsets[c + 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = lo; i < hi; i++) {
      const int e = L->color_edges[i];
      const int a = L->e2n[2 * (size_t)e], b = L->e2n[2 * (size_t)e + 1];
      orc_flux_edge(L->var + 5 * (size_t)a, L->var + 5 * (size_t)b, L->ewt + 3 * (size_t)e, sc,
                    L->flux + 5 * (size_t)a, L->flux + 5 * (size_t)b);
    }
  }
}

static void orc_bnd_flux_omp(orc_level* L, const orc_freestream* ff) {
  for (int c = 0; c < L->bnd_ncolors; c++) {
    const int lo = L->bnd_color_offsets[c], hi = L->bnd_color_offsets[c + 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = lo; i < hi; i++) {
      const int k = L->bnd_color_entries[i];
      const int n = L->b2n[k];
      orc_bnd_flux(L->bgroup[k], L->bwt + 3 * (size_t)k, L->var + 5 * (size_t)n, ff, L->flux + 5 * (size_t)n);
    }
  }
}

static void orc_stream_omp(orc_level* L) {
  for (int c = 0; c < L->ncolors; c++) {
    const int lo = L->color_offsets[c], hi = L->color_offsets[c + 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = lo; i < hi; i++) {
      const int e = L->color_edges[i];
      orc_loop_unstructured_stream(1, L->e2n + 2 * (size_t)e, L->var, L->ewt + 3 * (size_t)e, L->dummy);
    }
  }
}

int orc_run(orc_mesh* m, double mach, double aoa_deg, int ncycles, int nthreads, int measure_mem_bound,
            double* runtime_s) {
  orc_freestream ff;
  orc_freestream_init(mach, aoa_deg, &ff);
  const int par = nthreads > 1;
#ifdef _OPENMP
  if (par) omp_set_num_threads(nthreads);
#endif
  const int levels = m->nlevels;
  m->steps = 0;

  /* Initialisation, euler3d.cpp:413-441. */
  for (int l = 0; l < levels; l++) {
    orc_level* L = &m->L[l];
    memcpy(L->ewt, L->ewt_in, sizeof(double) * 3 * (size_t)L->nedges);
    memcpy(L->bwt, L->bwt_in, sizeof(double) * 3 * (size_t)L->nbnd);
    orc_loop_initialize_variables(L->nnodes, &ff, L->var);
    memset(L->flux, 0, sizeof(double) * 5 * (size_t)L->nnodes);
    memset(L->dummy, 0, sizeof(double) * 5 * (size_t)L->nnodes);
    memset(L->vol, 0, sizeof(double) * (size_t)L->nnodes);
    memset(L->up_scratch, 0, sizeof(int) * (size_t)L->nnodes);
    if (L->legacy_vol) memcpy(L->vol, L->legacy_vol, sizeof(double) * (size_t)L->nnodes);
    else orc_loop_calculate_cell_volumes(L->nedges, L->e2n, L->coords, L->ewt, L->vol);
    if (par && L->color_offsets == NULL) {
      orc_colour(L->nedges, 2, L->e2n, L->nnodes, &L->ncolors, &L->color_offsets, &L->color_edges);
      orc_colour(L->nbnd, 1, L->b2n, L->nnodes, &L->bnd_ncolors, &L->bnd_color_offsets, &L->bnd_color_entries);
    }
  }
  for (int l = 0; l < levels; l++) {
    orc_loop_dampen_ewt(m->L[l].nedges, m->L[l].ewt);
    orc_loop_dampen_ewt(m->L[l].nbnd, m->L[l].bwt);
  }

  const double t0 = orc_wall();
  int level = 0, up = 1, i = 0, status = 0;
  while (i < ncycles) {
    orc_level* L = &m->L[level];
    const int N = L->nnodes;
    /* euler3d.cpp:467-489 */
    double min_dt = DBL_MAX;
    if (!par) {
      orc_loop_copy_double(N, L->var, L->old);
      orc_loop_calculate_dt(N, L->var, L->vol, L->sf);
      min_dt = orc_loop_get_min_dt(N, L->sf);
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(min : min_dt)
#endif
      for (int n = 0; n < N; n++) {
        for (int j = 0; j < 5; j++) L->old[5 * (size_t)n + j] = L->var[5 * (size_t)n + j];
        const double dt = orc_dt(L->var + 5 * (size_t)n, L->vol[n]);
        L->sf[n] = dt;
        if (dt < min_dt) min_dt = dt;
      }
    }
    if (min_dt < 0.0f) { status = 1; break; }
    if (!par) {
      orc_loop_compute_step_factor(N, L->var, L->vol, min_dt, L->sf);
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
      for (int n = 0; n < N; n++) L->sf[n] = min_dt / L->vol[n];
    }
    /* euler3d.cpp:492-526 */
    for (int rk = 0; rk < ORC_RK; rk++) {
      if (!par) {
        orc_loop_compute_flux_edge(L->nedges, L->e2n, L->var, L->ewt, ff.smoothing_coefficient, L->flux);
        orc_loop_compute_bnd_node_flux(L->nbnd, L->b2n, L->bgroup, L->bwt, L->var, &ff, L->flux);
        orc_loop_time_step(N, rk, L->sf, L->flux, L->old, L->var);
        if (measure_mem_bound) orc_loop_unstructured_stream(L->nedges, L->e2n, L->var, L->ewt, L->dummy);
      } else {
        orc_flux_edge_omp(L, ff.smoothing_coefficient);
        orc_bnd_flux_omp(L, &ff);
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int n = 0; n < N; n++) orc_loop_time_step(1, rk, L->sf + n, L->flux + 5 * (size_t)n,
                                                       L->old + 5 * (size_t)n, L->var + 5 * (size_t)n);
        if (measure_mem_bound) orc_stream_omp(L);
      }
    }
    /* euler3d.cpp:528-550 */
    if (!par) {
      orc_loop_residual(N, L->old, L->var, L->res);
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
      for (int n = 0; n < N; n++)
        for (int j = 0; j < 5; j++) L->res[5 * (size_t)n + j] = L->var[5 * (size_t)n + j] - L->old[5 * (size_t)n + j];
    }
    m->steps++;
    if (level == 0) {
      int bad = 0;
      if (!par) {
        (void)orc_loop_calc_rms(N, L->res);
        bad = orc_loop_count_bad_vals(N, L->var);
      } else {
        double rms = 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(+ : rms, bad)
#endif
        for (int n = 0; n < N; n++)
          for (int j = 0; j < 5; j++) {
            const double r = L->res[5 * (size_t)n + j], v = L->var[5 * (size_t)n + j];
            rms += r * r;
            if (isnan(v) || isinf(v)) bad += 1;
          }
        (void)rms;
      }
      if (bad > 0) { status = 2; break; }
    }
    /* euler3d.cpp:573-640 */
    if (levels <= 1) {
      i++;
    } else if (up) {
      level++;
      orc_level* C = &m->L[level];
      orc_loop_up_pre(L->nnodes, L->n2mg, C->var, C->up_scratch);
      orc_loop_up(L->nnodes, L->n2mg, L->var, C->var, C->up_scratch);
      orc_loop_up_post(C->nnodes, C->var, C->up_scratch);
      if (level == levels - 1) up = 0;
    } else {
      level--;
      orc_level* F = &m->L[level];
      orc_level* C = &m->L[level + 1];
      if (!par) {
        orc_loop_down(F->nnodes, F->n2mg, F->var, F->res, F->coords, C->res, C->coords);
      } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int n = 0; n < F->nnodes; n++)
          orc_loop_down(1, F->n2mg + n, F->var + 5 * (size_t)n, F->res + 5 * (size_t)n, F->coords + 3 * (size_t)n,
                        C->res, C->coords);
      }
      if (level == 0) {
        up = 1;
        i++;
      }
    }
  }
  if (runtime_s) *runtime_s = orc_wall() - t0;
  return status;
}

int orc_get(const orc_mesh* m, int level, int what, double* out) {
  if (!m || level < 0 || level >= m->nlevels) return -1;
  const orc_level* L = &m->L[level];
  const size_t n = (size_t)L->nnodes;
  switch (what) {
    case 0: memcpy(out, L->var, sizeof(double) * 5 * n); return 0;
    case 1: memcpy(out, L->flux, sizeof(double) * 5 * n); return 0;
    case 2: memcpy(out, L->sf, sizeof(double) * n); return 0;
    case 3: memcpy(out, L->vol, sizeof(double) * n); return 0;
    case 4: memcpy(out, L->res, sizeof(double) * 5 * n); return 0;
    case 5: memcpy(out, L->ewt, sizeof(double) * 3 * (size_t)L->nedges); return 0;
    case 6: memcpy(out, L->bwt, sizeof(double) * 3 * (size_t)L->nbnd); return 0;
    case 7: memcpy(out, L->old, sizeof(double) * 5 * n); return 0;
    default: return -1;
  }
}

int orc_mesh_set_volumes(orc_mesh* m, int l, const double* volumes) {
  if (!m || l < 0 || l >= m->nlevels) return -1;
  orc_level* L = &m->L[l];
  free(L->legacy_vol);
  L->legacy_vol = volumes ? (double*)orc_dup(volumes, sizeof(double) * (size_t)L->nnodes) : NULL;
  return 0;
}

long orc_smoothing_steps(const orc_mesh* m) { return m ? m->steps : 0; }

void orc_mesh_destroy(orc_mesh* m) {
  if (!m) return;
  for (int l = 0; l < m->nlevels; l++) {
    orc_level* L = &m->L[l];
    free(L->coords); free(L->ewt); free(L->bwt); free(L->ewt_in); free(L->bwt_in); free(L->legacy_vol); free(L->e2n); free(L->b2n); free(L->bgroup); free(L->n2mg);
    free(L->var); free(L->old); free(L->res); free(L->vol); free(L->sf); free(L->flux); free(L->dummy);
    free(L->up_scratch);
    free(L->color_offsets); free(L->color_edges); free(L->bnd_color_offsets); free(L->bnd_color_entries);
  }
  free(m->L);
  free(m);
}
