// Execution plans of the per-loop entry points (plans.cu): cached per map
// (or per vol dat), built on first use.  Internal to the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mgcfd {

struct EdgePlan;
struct ChildPlan;

// *out = nullptr (status MGCFD_OK) when plans are switched off, or when no
// plan exists yet and `s` is capturing a CUDA graph: the caller then runs its
// plan-free kernel.  A new plan is built on `s` and synchronises it.
int edge_plan_get(const int32_t* e2n, int32_t ne, int32_t nn, cudaStream_t s, EdgePlan** out);
// compute_flux_edge_kernel over the plan; *skipped = edges left out of the plan.
int edge_plan_flux(EdgePlan* P, const double* var, const double* ewt, double sc, double* flux, cudaStream_t s,
                   int64_t* skipped);
bool edge_plan_permuted(const EdgePlan* P);

int child_plan_get(const int32_t* map, int32_t nf, int32_t nc, cudaStream_t s, ChildPlan** out);
// up_pre_kernel / up_kernel over the plan; *skipped = fine nodes out of range.
int child_plan_up_pre(ChildPlan* P, double* cv, int32_t* scratch, cudaStream_t s, int64_t* skipped);
int child_plan_up(ChildPlan* P, const double* fv, double* cv, int32_t* scratch, cudaStream_t s, int64_t* skipped);

struct VolPlan;
// calculate_dt_kernel's volume cube roots, cached per vol dat and checked
// against the volumes' bits on every call.
int vol_plan_get(const double* vol, int32_t n, cudaStream_t s, VolPlan** out);
int vol_plan_calculate_dt(VolPlan* P, const double* var, const double* vol, double* dt, cudaStream_t s);

}  // namespace mgcfd
